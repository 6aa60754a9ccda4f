"""Mesh coupling (t4mesh::mesh_coupling): surface points bound to the tets
that embed them and moved with the deformed mesh, against the reference
itself (tests/golden/coupling.npz: bind_surface and update_surface compiled
from the unmodified reference headers, tests/golden/make_coupling.py) and
against the CPU restatement in oracle/coupling_oracle.py (itself pinned to
that fixture)."""
import numpy as np
import pytest

from helpers import beam, golden, irregular_mesh
from oracle import coupling_oracle as co
from opentissue_gb300 import capi, fem

MESHES = ("blocks", "delaunay")


@pytest.mark.parametrize("name", MESHES)
def test_restatement_matches_the_reference_fixture(name):
    """The restatement against the reference build: the same tet for every
    point (the reference's spatial-hash query visits tets in index order and
    keeps the first that embeds a point, so on shared faces and at nodes the
    lowest tet index), weights and moved points to rounding."""
    g = golden("coupling")
    tets, coord, pts = g[f"{name}_tets"], g[f"{name}_coord"], g[f"{name}_points"]
    tet, bary = co.bind(tets, coord, pts)
    assert np.array_equal(tet, g[f"{name}_tet"])
    assert np.abs(bary - g[f"{name}_bary"]).max() <= 1e-12
    moved = co.update(tets, g[f"{name}_coord_deformed"], tet, bary, pts)
    ref = g[f"{name}_moved"]
    assert np.abs(moved - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.gpu
@pytest.mark.parametrize("name", MESHES)
def test_library_matches_the_reference_fixture(gpu, name):
    """otfem_surface_bind / otfem_surface_update against the reference build:
    bound tets identical (shared faces and nodes included), weights and moved
    points to rounding, unbound points kept where they were."""
    g = golden("coupling")
    tets, coord, pts = g[f"{name}_tets"], g[f"{name}_coord"], g[f"{name}_points"]
    mesh = fem.Mesh(tets, coord)
    fem.init(mesh, 5e5, 0.33, 1000.0, 1e30, 0.0, 0.0)
    b = fem.bind_surface(mesh, pts)
    tet, bary = b.binding()
    assert np.array_equal(tet, g[f"{name}_tet"])
    assert np.abs(bary - g[f"{name}_bary"]).max() <= 1e-12
    assert b.bound == int((g[f"{name}_tet"] >= 0).sum())
    mesh.coord = np.ascontiguousarray(g[f"{name}_coord_deformed"])
    mesh.upload(capi.COORD)
    moved = fem.update_surface(b)
    ref = g[f"{name}_moved"]
    assert np.abs(moved - ref).max() <= 1e-12 * np.abs(ref).max()
    b.close()
    mesh.close()

# ---- the restatement (CPU) ------------------------------------------------------


def test_oracle_barycentric_of_vertices_and_centroid():
    x = np.array([[0.0, 0, 0], [1.0, 0, 0], [0, 1.0, 0], [0, 0, 1.0]])
    for k in range(4):
        w = co.barycentric(x[0][None], x[1][None], x[2][None], x[3][None], x[k][None])[0]
        assert np.allclose(w, np.eye(4)[k], atol=1e-15)
    w = co.barycentric(x[0][None], x[1][None], x[2][None], x[3][None], x.mean(0)[None])[0]
    assert np.allclose(w, 0.25)


def test_oracle_bind_then_update_at_rest_returns_the_points():
    tets, coord, _ = beam(3, 2, 2, jitter_seed=1)
    rng = np.random.default_rng(0)
    pts = rng.uniform(coord.min(0) + 0.02, coord.max(0) - 0.02, (40, 3))
    tet, bary = co.bind(tets, coord, pts)
    assert (tet >= 0).all()
    assert np.allclose(co.update(tets, coord, tet, bary, pts), pts, atol=1e-13)

# ---- the GPU --------------------------------------------------------------------


def sample_points(coord, n, seed, outside=5):
    rng = np.random.default_rng(seed)
    lo, hi = coord.min(0), coord.max(0)
    pts = rng.uniform(lo + 1e-3, hi - 1e-3, (n, 3))
    far = rng.uniform(hi + 0.05, hi + 0.5, (outside, 3))  # outside every tet
    return np.vstack([pts, far])


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["blocks", "delaunay"])
def test_bind_matches_restatement(gpu, kind):
    if kind == "blocks":
        tets, coord, fixed = beam(6, 3, 3, jitter_seed=2)
    else:
        tets, coord, fixed = irregular_mesh((6, 3, 3), seed=5)
    mesh = fem.Mesh(tets, coord, fixed=fixed.astype(bool))
    fem.init(mesh, 5e5, 0.33, 1000.0, 1e30, 0.0, 0.0)
    pts = sample_points(coord, 300, 3)
    b = fem.bind_surface(mesh, pts)
    tet, bary = b.binding()
    tet_o, bary_o = co.bind(tets, coord, pts)
    assert np.array_equal(tet, tet_o)
    assert np.abs(bary - bary_o).max() <= 1e-12
    assert b.bound == int((tet_o >= 0).sum()) and (tet[-5:] == -1).all()
    b.close()
    mesh.close()


@pytest.mark.gpu
def test_update_follows_the_deformed_mesh(gpu):
    tets, coord, fixed = beam(8, 3, 3, jitter_seed=4)
    mesh = fem.Mesh(tets, coord, fixed=fixed.astype(bool))
    fem.init(mesh, 5e5, 0.33, 1000.0, 1e30, 0.0, 0.0)
    pts = sample_points(coord, 500, 6)
    b = fem.bind_surface(mesh, pts)
    tet, bary = b.binding()
    p = capi.default_params(solver=capi.SOLVER_MIXED, max_iterations=2000, rtol=1e-6)
    for _ in range(10):
        f = np.zeros_like(coord)
        f[~fixed.astype(bool), 1] = -9.81 * mesh.mass[~fixed.astype(bool)] * 20.0
        mesh.f_external = f
        fem.simulate(mesh, 0.01, True, p)
    moved = fem.update_surface(b)
    ref = co.update(tets, mesh.coord, tet, bary, pts)
    assert np.abs(moved - ref).max() <= 1e-12 * np.abs(ref).max()
    assert np.abs(moved[:-5] - pts[:-5]).max() > 1e-3  # the mesh did move
    assert np.array_equal(moved[-5:], pts[-5:])        # unbound points stay
    # and the points are where the deformed tets put them: rebinding against
    # the deformed mesh finds the same tets and weights
    b2 = fem.bind_surface(mesh, moved[:-5])
    tet2, bary2 = b2.binding()
    same = tet2 == tet[:-5]
    assert same.mean() > 0.95 and np.abs(bary2[same] - bary[:-5][same]).max() < 1e-9
    b2.close()
    b.close()
    mesh.close()


@pytest.mark.gpu
def test_surface_argument_checks(gpu):
    tets, coord, fixed = beam(2, 2, 2)
    mesh = fem.Mesh(tets, coord, fixed=fixed.astype(bool))
    fem.init(mesh, 5e5, 0.33, 1000.0, 1e30, 0.0, 0.0)
    b = fem.bind_surface(mesh, coord[:3])
    lib = capi.lib()
    out = np.zeros((4, 3))
    assert lib.otfem_surface_update(b.s, out.ctypes.data_as(capi._dp), 4) == capi.ERR_INVALID_ARGUMENT
    bad = np.array([[np.nan, 0.0, 0.0]])
    s = capi.ctypes.c_void_p()
    assert lib.otfem_surface_bind(mesh.handle, bad.ctypes.data_as(capi._dp), 1, capi.ctypes.byref(s), None) == \
        capi.ERR_INVALID_ARGUMENT
    empty = fem.bind_surface(mesh, np.zeros((0, 3)))
    assert empty.bound == 0 and empty.update().shape == (0, 3)
    empty.close()
    b.close()
    mesh.close()
