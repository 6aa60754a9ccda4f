"""Generates the trajectory fixtures in tests/golden/ from the REFERENCE itself
(OpenTissue's unmodified FEM headers behind the oracle C interface,
oracle/_ref/libotfem_ref.so): the reference's fem::simulate pipeline
(fem_simulate.h:94-111, fem_position_update.h:25-39) with the CG replaced
by the relative-residual FP64 CG of the oracle's converged mode.

Each run is made twice: tightly converged (rel. residual 1e-10: the FP64
trajectory itself, x_s / v_s) and at the GPU solver's own tolerance 1e-6
(x6_s / v6_s: what the FP64 reference pipeline delivers with the same
stopping rule, and its deviation from the tight run).

Fixtures (meshes and loads from opentissue_gb300.workloads, so the tests and
the benchmark drive the same inputs):
  traj_beam128      128x32x32 jittered beam (seed 20261203), gravity, dt 0.01,
                    200 steps; x and v of 2,048 sampled nodes (and the whole
                    free end face's corner nodes) at steps 1, 50, 100, 200
  traj_beam64_sine  64x16x16 jittered beam (seed 20261208), gravity plus the
                    seeded sinusoidal tip load (SineTip seed 20261209), dt
                    0.01, 500 steps; x and v of 2,048 sampled nodes at steps
                    1, 100, 250, 500
  traj_batch        8 beams of the 256-beam batch (seed 20261203): the five
                    stiffest (E 4.6e6..5.0e6 Pa) and three others, dt 0.005,
                    gravity plus the constant tip force and, separately, the
                    sinusoidal tip force; x and v of 256 sampled free nodes
                    per beam (and the free end's corner nodes) at steps 1,
                    20, 40
Every sampled step also stores the largest displacement |x - x0| and the
largest |v| over all nodes (the scales the tests' relative bounds use) and
the FP64 pipeline's own errors at 1e-6 over all nodes.

Usage: python tests/golden/make_trajectories.py [name ...]
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build as obuild  # noqa: E402
from oracle import pyoracle as po  # noqa: E402
from opentissue_gb300 import workloads as wl  # noqa: E402

TIGHT = 1e-10
GPU_RTOL = 1e-6
MATERIAL = (5e5, 0.33, 1000.0, 1e30, 0.0, 0.0)
BATCH_BEAMS = (197, 213, 111, 195, 85, 0, 1, 2)
BATCH_KEEP = (1, 20, 40)


def run(tets, coord, fixed, steps, keep, forces, dt, rtol, material=MATERIAL):
    """Steps from rest; forces(k, mass) gives step k's (0-based) external
    forces.  Returns {step: (x, v)} at the kept steps and the iterations."""
    m = po.OracleMesh(tets, coord, coord, fixed, kind="reference")
    m.init(*material)
    mass = m.get(po.MASS)
    out, its = {}, []
    for k in range(steps):
        m.set(po.F_EXTERNAL, forces(k, mass))
        it, _ = m.simulate_converged(dt, True, 2.0, rtol, 100000)
        its.append(it)
        if k + 1 in keep:
            out[k + 1] = (m.get(po.COORD), m.get(po.VELOCITY))
    m.close()
    return out, np.array(its)


def sample_nodes(I, J, K, count, seed):
    n = (I + 1) * (J + 1) * (K + 1)
    free = np.arange((J + 1) * (K + 1), n)
    corners = [I * (J + 1) * (K + 1) + j * (K + 1) + k for j in (0, J) for k in (0, K)]
    pick = np.random.default_rng(seed).choice(free, count, replace=False)
    return np.unique(np.concatenate([pick, corners]))


def single(name, cfg, forces, keep):
    I, J, K = cfg["I"], cfg["J"], cfg["K"]
    tets, coord, fixed = wl.jittered_beam(I, J, K, cfg["seed"])
    ref_tets, ref_coord = po.generate_blocks(I, J, K, 0.1, 0.1, 0.1, kind="reference")
    assert np.array_equal(ref_tets, tets)
    sample = sample_nodes(I, J, K, 2048, cfg["seed"] + 1)
    t0 = time.time()
    tight, its = run(tets, coord, fixed, cfg["steps"], keep, forces, cfg["dt"], TIGHT)
    t1 = time.time()
    loose, its6 = run(tets, coord, fixed, cfg["steps"], keep, forces, cfg["dt"], GPU_RTOL)
    t2 = time.time()
    arrays = dict(sample=sample, keep=np.array(keep), iterations=its, iterations_rtol6=its6)
    for s in keep:
        x, v = tight[s]
        x6, v6 = loose[s]
        disp = np.abs(x - coord).max()
        vmax = np.abs(v).max()
        arrays[f"x_{s}"] = x[sample]
        arrays[f"v_{s}"] = v[sample]
        arrays[f"x6_{s}"] = x6[sample]
        arrays[f"v6_{s}"] = v6[sample]
        arrays[f"disp_{s}"] = disp
        arrays[f"vmax_{s}"] = vmax
        # the FP64 oracle stopped at the GPU's tolerance, against the tight run
        arrays[f"rtol6_x_err_{s}"] = np.abs(x6 - x).max() / disp
        arrays[f"rtol6_v_err_{s}"] = np.abs(v6 - v).max() / vmax
        print(f"{name} step {s}: disp {disp:.4e} vmax {vmax:.4e}  oracle@1e-6 vs @1e-10: "
              f"x {arrays[f'rtol6_x_err_{s}']:.2e} v {arrays[f'rtol6_v_err_{s}']:.2e}", flush=True)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays, I=I, J=J, K=K, seed=cfg["seed"], dt=cfg["dt"], steps=cfg["steps"],
                        rtol=TIGHT)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KB; {t1 - t0:.0f} s tight, {t2 - t1:.0f} s at 1e-6)")


def fixed_face(cfg):
    n = (cfg["I"] + 1) * (cfg["J"] + 1) * (cfg["K"] + 1)
    return (np.arange(n) < (cfg["J"] + 1) * (cfg["K"] + 1)).astype(np.uint8)


def beam128():
    cfg = wl.BEAM128
    fixed = fixed_face(cfg)
    single("traj_beam128", cfg, lambda k, mass: wl.gravity(mass, fixed), (1, 50, 100, 200))


def beam64_sine():
    cfg = wl.BEAM64_SINE
    load = wl.SineTip(cfg["I"], cfg["J"], cfg["K"], cfg["load_seed"])
    fixed = fixed_face(cfg)
    single("traj_beam64_sine", cfg, lambda k, mass: wl.gravity(mass, fixed) + load.force(k, cfg["dt"]),
           (1, 100, 250, 500))


def batch():
    cfg = wl.BATCH
    beams = wl.random_beams(cfg["count"], seed=cfg["seed"])
    freqs = wl.batch_tip_frequencies(cfg["count"])
    arrays = dict(beams=np.array(BATCH_BEAMS), keep=np.array(BATCH_KEEP))
    t0 = time.time()
    for b_i in BATCH_BEAMS:
        bm = beams[b_i]
        mat = (bm["young"], bm["poisson"], bm["density"], 1e30, 0.0, 0.0)
        for sine in (False, True):
            def forces(k, mass, bm=bm, sine=sine, b_i=b_i):
                s = np.sin(2 * np.pi * freqs[b_i] * k * cfg["dt"]) if sine else 1.0
                f = wl.gravity(mass, bm["fixed"]) + s * bm["tip_force"]
                f[bm["fixed"] == 1] = 0.0
                return f
            out, its = run(bm["tets"], bm["coord"], bm["fixed"], max(BATCH_KEEP), BATCH_KEEP, forces, cfg["dt"],
                           TIGHT, material=mat)
            out6, _ = run(bm["tets"], bm["coord"], bm["fixed"], max(BATCH_KEEP), BATCH_KEEP, forces, cfg["dt"],
                          GPU_RTOL, material=mat)
            tag = "sine" if sine else "const"
            free = np.flatnonzero(bm["fixed"] == 0)
            pick = np.random.default_rng(b_i).choice(free, min(256, free.size), replace=False)
            root = bm["coord"][bm["fixed"] == 1].mean(0)
            far = free[np.argmax(np.linalg.norm(bm["coord"][free] - root, axis=1))]  # at the free end
            sample = np.unique(np.concatenate([pick, [far]]))
            arrays[f"b{b_i}_sample"] = sample
            msg = []
            for s in BATCH_KEEP:
                x, v = out[s]
                x6, v6 = out6[s]
                disp, vmax = np.abs(x - bm["coord"]).max(), np.abs(v).max()
                arrays[f"b{b_i}_{tag}_x_{s}"] = x[sample]
                arrays[f"b{b_i}_{tag}_v_{s}"] = v[sample]
                arrays[f"b{b_i}_{tag}_disp_{s}"] = disp
                arrays[f"b{b_i}_{tag}_vmax_{s}"] = vmax
                arrays[f"b{b_i}_{tag}_rtol6_x_err_{s}"] = np.abs(x6 - x).max() / disp
                arrays[f"b{b_i}_{tag}_rtol6_v_err_{s}"] = np.abs(v6 - v).max() / vmax
                msg.append(f"s{s} x {np.abs(x6 - x).max() / disp:.1e} v {np.abs(v6 - v).max() / vmax:.1e}")
            print(f"batch beam {b_i} {bm['dims']} E {bm['young']:.3g} {tag}: {its.mean():.0f} it/step; "
                  f"oracle@1e-6 vs @1e-10: {'; '.join(msg)}", flush=True)
    path = os.path.join(HERE, "traj_batch.npz")
    np.savez_compressed(path, **arrays, count=cfg["count"], seed=cfg["seed"], dt=cfg["dt"], rtol=TIGHT)
    print(f"wrote {path} ({os.path.getsize(path) / 1024:.0f} KB; {time.time() - t0:.0f} s)")


def main():
    if obuild.build_reference() is None:
        raise SystemExit("reference tree not available: cannot regenerate the trajectory fixtures")
    names = sys.argv[1:] or ["beam64_sine", "batch", "beam128"]
    for n in names:
        {"beam128": beam128, "beam64_sine": beam64_sine, "batch": batch}[n]()


if __name__ == "__main__":
    main()
