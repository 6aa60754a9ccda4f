"""Generates the golden fixtures in tests/golden/ from the REFERENCE itself:
OpenTissue's unmodified FEM headers compiled behind the oracle C interface
(oracle/_ref/libotfem_ref.so, built by oracle/build.py where the reference
tree is present).  The committed .npz files are what the tests compare
against on machines without the reference.

Cases (all meshes from t4mesh::generate_blocks, edge 0.1 m, x = 0 face fixed,
gravity -9.81 in y applied as m_i * g to free nodes every step):
  config1        10x4x4, E=5e5, nu=0.33, rho=1000, dt=0.01, warping, fem::simulate
                 (20-iteration CG), 100 steps
  plastic        config1 with c_yield=1e-4, c_creep=50, c_max=1e-2, 30 steps
  nowarp         config1 without stiffness warping, 10 steps
  converged      16x6x6, nodes jittered by U[-0.01, 0.01] m (numpy PCG64 seed
                 7), relative-residual CG to 1e-6, 20 steps
  large          128x32x32, jittered (seed 20261203), converged CG to 1e-6,
                 3 steps; a fixed sample of 4096 nodes is stored

Usage: python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build as obuild  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

GRAVITY = -9.81


def beam(I, J, K, jitter_seed=None, jitter=0.01, edge=0.1):
    tets, coord = po.generate_blocks(I, J, K, edge, edge, edge, kind="reference")
    if jitter_seed is not None:
        rng = np.random.default_rng(jitter_seed)
        coord = coord + rng.uniform(-jitter, jitter, coord.shape)
    fixed = (np.arange(coord.shape[0]) < (J + 1) * (K + 1)).astype(np.uint8)  # grid index i == 0
    return tets, coord, fixed


def gravity_force(mass, fixed):
    f = np.zeros((mass.shape[0], 3))
    free = fixed == 0
    f[free, 1] = GRAVITY * mass[free]
    return f


def step_hash(x, v):
    return hashlib.sha256(np.ascontiguousarray(x).tobytes() + np.ascontiguousarray(v).tobytes()).hexdigest()


def run_reference(tets, coord, fixed, steps, material=(5e5, 0.33, 1000.0, 1e30, 0.0, 0.0), dt=0.01,
                  warp=True, converged=False, rtol=1e-6, keep=(), sample=None):
    m = po.OracleMesh(tets, coord, coord, fixed, kind="reference")
    m.init(*material)
    mass = m.get(po.MASS)
    out = {"mass": mass, "hashes": [], "iterations": [], "rel_residual": []}
    for s in range(1, steps + 1):
        m.set(po.F_EXTERNAL, gravity_force(mass, fixed))
        if converged:
            it, rr = m.simulate_converged(dt, warp, 2.0, rtol, 100000)
            out["iterations"].append(it)
            out["rel_residual"].append(rr)
        else:
            m.simulate(dt, warp)
        x, v = m.get(po.COORD), m.get(po.VELOCITY)
        out["hashes"].append(step_hash(x, v))
        if s in keep:
            out[f"x_{s}"] = x if sample is None else x[sample]
            out[f"v_{s}"] = v if sample is None else v[sample]
        if s == 1:
            out["re_1"] = m.re()
            out["f0_1"] = m.get(po.F0)
            out["b_1"] = m.get(po.B)
            if sample is None:
                rp, cols = m.k_pattern()
                out["k_row_ptr"], out["k_cols"] = rp, cols
                out["k_values_1"] = m.k_values()
                r, c, val = m.export_k()
                out["export_rows_1"], out["export_cols_1"], out["export_vals_1"] = r, c, val
    out["plastic_final"] = m.plastic()
    out["x_final"] = m.get(po.COORD) if sample is None else m.get(po.COORD)[sample]
    out["v_final"] = m.get(po.VELOCITY) if sample is None else m.get(po.VELOCITY)[sample]
    m.close()
    return out


def save(name, tets, coord, fixed, res, **meta):
    path = os.path.join(HERE, name + ".npz")
    arrays = {k: np.asarray(v) for k, v in res.items() if k != "hashes"}
    arrays["hashes"] = np.array(res["hashes"])
    np.savez_compressed(path, tets=tets, coord=coord, fixed=fixed, **arrays,
                        **{k: np.asarray(v) for k, v in meta.items()})
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KB)")


def main():
    if obuild.build_reference() is None:
        raise SystemExit("reference tree not available: cannot regenerate goldens")
    obuild.build_port()
    t, c, f = beam(10, 4, 4)
    save("config1", t, c, f, run_reference(t, c, f, 100, keep=(1, 10, 50, 100)), dt=0.01, steps=100)
    save("plastic", t, c, f, run_reference(t, c, f, 30, material=(5e5, 0.33, 1000.0, 1e-4, 50.0, 1e-2),
                                           keep=(1, 30)), dt=0.01, steps=30)
    save("nowarp", t, c, f, run_reference(t, c, f, 10, warp=False, keep=(1, 10)), dt=0.01, steps=10)
    t, c, f = beam(16, 6, 6, jitter_seed=7)
    save("converged", t, c, f, run_reference(t, c, f, 20, converged=True, keep=(1, 5, 20)), dt=0.01, steps=20,
         rtol=1e-6)
    t, c, f = beam(128, 32, 32, jitter_seed=20261203)
    sample = np.sort(np.random.default_rng(1).choice(c.shape[0], 4096, replace=False))
    res = run_reference(t, c, f, 3, converged=True, keep=(1, 2, 3), sample=sample)
    for k in ("re_1", "f0_1", "b_1", "mass", "plastic_final"):
        res.pop(k, None)
    np.savez_compressed(os.path.join(HERE, "large.npz"), sample=sample, hashes=np.array(res.pop("hashes")),
                        **{k: np.asarray(v) for k, v in res.items()}, I=128, J=32, K=32, seed=20261203,
                        dt=0.01, rtol=1e-6)
    print("wrote large.npz")


if __name__ == "__main__":
    main()
