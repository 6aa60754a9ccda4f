"""Generates tests/golden/coupling.npz from the REFERENCE itself:
t4mesh::mesh_coupling::bind_surface and update_surface
(core/containers/t4mesh/util/t4mesh_mesh_coupling.h:129-275) compiled from
the unmodified headers into oracle/_ref/libotfem_ref.so (oracle/ref/
ref_coupling.cpp).

Two meshes: a 6x3x3 jittered block beam (seed 2) and an unstructured
Delaunay mesh of a jittered 6x3x3 lattice (seed 5, tests/helpers.py
irregular_mesh).  Points per mesh: 300 uniform in the bounding box (some near
the jittered boundary fall outside every tet), the centroids of 50 tet faces
(on faces shared by two tets: both embed the point), 20 node positions
(shared by every tet around the node) and 5 points far outside.  Stored: the
binding (tet index, -1 unbound; barycentric w1, w2, w3) at the rest shape,
and the bound points moved by update_surface for a deformed copy of the mesh
(a bend, a twist and a translation of the rest coordinates).

Usage: python tests/golden/make_coupling.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from helpers import beam, irregular_mesh  # noqa: E402
from oracle import build as obuild  # noqa: E402
from oracle import pyoracle as po  # noqa: E402


def points_for(tets, coord, seed):
    rng = np.random.default_rng(seed)
    lo, hi = coord.min(0), coord.max(0)
    inside = rng.uniform(lo + 1e-3, hi - 1e-3, (300, 3))
    faces = coord[tets[rng.choice(tets.shape[0], 50, replace=False)][:, :3]].mean(1)
    nodes = coord[rng.choice(coord.shape[0], 20, replace=False)]
    far = rng.uniform(hi + 0.05, hi + 0.5, (5, 3))
    return np.vstack([inside, faces, nodes, far])


def deformed(coord):
    x = coord - coord.min(0)
    L = x[:, 0].max()
    s = x[:, 0] / L
    out = coord.copy()
    out[:, 1] += 0.05 * s ** 2                   # bend
    a = 0.3 * s                                  # twist about the beam axis
    c = coord[:, 1:] - coord[:, 1:].mean(0)
    out[:, 1] += c[:, 0] * (np.cos(a) - 1) - c[:, 1] * np.sin(a)
    out[:, 2] += c[:, 0] * np.sin(a) + c[:, 1] * (np.cos(a) - 1)
    return out + np.array([0.01, -0.02, 0.03])


def main():
    if obuild.build_reference() is None:
        raise SystemExit("reference tree not available: cannot regenerate the coupling fixture")
    arrays = {}
    for name, (tets, coord, fixed) in (("blocks", beam(6, 3, 3, jitter_seed=2)),
                                       ("delaunay", irregular_mesh((6, 3, 3), seed=5))):
        pts = points_for(tets, coord, 3)
        tet, bary = po.coupling_bind(tets, coord, pts)
        bound = tet >= 0
        moved_coord = deformed(coord)
        moved = pts.copy()
        moved[bound] = po.coupling_update(tets, moved_coord, tet[bound], bary[bound])
        arrays.update({f"{name}_tets": tets, f"{name}_coord": coord, f"{name}_points": pts, f"{name}_tet": tet,
                       f"{name}_bary": bary, f"{name}_coord_deformed": moved_coord, f"{name}_moved": moved})
        print(f"{name}: {len(tets)} tets, {len(pts)} points, {bound.sum()} bound")
    path = os.path.join(HERE, "coupling.npz")
    np.savez_compressed(path, **arrays)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KB)")


if __name__ == "__main__":
    main()
