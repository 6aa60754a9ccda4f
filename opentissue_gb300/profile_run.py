"""Profiling driver: a fixed sequence of library launches for `ncu`.

Builds a jittered block beam (x = 0 face fixed, gravity), runs `--steps`
matrix-free steps (OTFEM_SOLVER_MIXED, CG to rel. residual 1e-6) and then
`--sweeps` standalone element-apply sweeps, and prints the step statistics
and the autotuner's choice.  Run it plainly first, then under ncu, e.g.

  python opentissue_gb300/profile_run.py --dims 128 32 64 --steps 2 --sweeps 4
  ncu --set full --clock-control none -k regex:k_apply_sweep -s 150 -c 2 -o prof \\
      python opentissue_gb300/profile_run.py --dims 128 32 64 --steps 2 --sweeps 4

(the autotuner at otfem_init launches 15 apply sweeps per measured shape before
the step: 150 on a single mesh -- the two patch variants, the two tiled
variants at four tile sizes -- and 120 on a batch).  With --batch M the
mesh is a batch of the first M beams of the 256-beam workload (seed
20261203; dt 0.005, gravity and each beam's tip force), stepped by one
persistent launch per step.
"""
import argparse
import ctypes
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from opentissue_gb300 import build, capi  # noqa: E402
from opentissue_gb300.fem import generate_blocks  # noqa: E402


WARM_STARTS = {"previous": capi.WARM_START_PREVIOUS, "projected": capi.WARM_START_PROJECTED,
               "extrapolated": capi.WARM_START_EXTRAPOLATED}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dims", type=int, nargs=3, default=[128, 32, 32])
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--sweeps", type=int, default=4)
    ap.add_argument("--variant", type=int, default=-1, help="force an element-apply variant (0..3)")
    ap.add_argument("--solver", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--warm-start", default="previous", choices=["previous", "projected", "extrapolated"])
    ap.add_argument("--trace", action="store_true",
                    help="print the last step's phases and per-iteration breakdown (SM clock stamps)")
    ap.add_argument("--batch", type=int, default=0, help="a batch of the first M beams of the batch workload")
    args = ap.parse_args()
    build.build()
    lib = capi.lib()
    if args.batch:
        return run_batch(lib, args)
    I, J, K = args.dims
    tets, coord = generate_blocks(I, J, K, 0.1, 0.1, 0.1)
    coord = coord + np.random.default_rng(20261203).uniform(-0.01, 0.01, coord.shape)
    fixed = (np.arange(coord.shape[0]) < (J + 1) * (K + 1)).astype(np.uint8)
    N, T = coord.shape[0], tets.shape[0]
    dp = ctypes.POINTER(ctypes.c_double)
    desc = capi.MeshDesc(N, T, tets.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), coord.ctypes.data_as(dp),
                         coord.ctypes.data_as(dp), fixed.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    h = ctypes.c_void_p()
    capi.check(lib.otfem_create(ctypes.byref(desc), None, ctypes.byref(h)))
    capi.check(lib.otfem_init(h, 5e5, 0.33, 1000.0, 1e30, 0.0, 0.0))
    if args.variant >= 0:
        capi.check(lib.otfem_set_apply_variant(h, args.variant))
    variant = ctypes.c_int32()
    ms = np.zeros(capi.NUM_APPLY_VARIANTS)
    capi.check(lib.otfem_tuning(h, ctypes.byref(variant), ms.ctypes.data_as(dp)))
    mass = np.zeros(N)
    capi.check(lib.otfem_get_nodes(h, capi.MASS, mass.ctypes.data_as(dp), N))
    f = np.zeros((N, 3))
    f[fixed == 0, 1] = -9.81 * mass[fixed == 0]
    capi.check(lib.otfem_set_nodes(h, capi.F_EXTERNAL, f.ctypes.data_as(dp), f.size))
    solver = capi.SOLVER_MIXED if args.solver == "mixed" else capi.SOLVER_FP64
    warm = WARM_STARTS[args.warm_start]
    p = capi.default_params(solver=solver, max_iterations=5000, rtol=1e-6, graph=0, warm_start=warm)
    st = capi.StepStats()
    for _ in range(args.steps):
        capi.check(lib.otfem_simulate_ex(h, 0.01, 1, ctypes.byref(p), ctypes.byref(st)))
        print(f"step: iterations {st.iterations}, applies {st.applies}, rel. residual {st.rel_residual:.3e}")
    if args.trace:
        trace_report(lib, h, dp)
    if args.sweeps:
        capi.check(lib.otfem_apply_sweeps(h, solver, 0.01, args.sweeps))
    capi.check(lib.otfem_synchronize(h))
    print(f"tets {T}, nodes {N}, apply variant {variant.value}, sweep ms per variant {ms.tolist()}, "
          f"tuner sweeps {15 * tuning_rows(lib, h)}")
    capi.check(lib.otfem_destroy(h))


def run_batch(lib, args):
    from opentissue_gb300 import workloads as wl
    beams = wl.random_beams(wl.BATCH["count"], seed=wl.BATCH["seed"])[:args.batch]
    dp = ctypes.POINTER(ctypes.c_double)
    descs = (capi.MeshDesc * len(beams))()
    keep = []
    for k, b in enumerate(beams):
        t = np.ascontiguousarray(b["tets"], np.int32)
        c = np.ascontiguousarray(b["coord"], np.float64)
        f = np.ascontiguousarray(b["fixed"], np.uint8)
        keep += [t, c, f]
        descs[k] = capi.MeshDesc(c.shape[0], t.shape[0], t.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                 c.ctypes.data_as(dp), c.ctypes.data_as(dp), f.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    h = ctypes.c_void_p()
    capi.check(lib.otfem_batch_create(descs, len(beams), None, ctypes.byref(h)))
    e = np.array([b["young"] for b in beams])
    nu = np.array([b["poisson"] for b in beams])
    rho = np.array([b["density"] for b in beams])
    capi.check(lib.otfem_batch_init(h, e.ctypes.data_as(dp), nu.ctypes.data_as(dp), rho.ctypes.data_as(dp),
                                    1e30, 0.0, 0.0))
    if args.variant >= 0:
        capi.check(lib.otfem_set_apply_variant(h, args.variant))
    N = sum(b["coord"].shape[0] for b in beams)
    T = sum(b["tets"].shape[0] for b in beams)
    mass = np.zeros(N)
    capi.check(lib.otfem_get_nodes(h, capi.MASS, mass.ctypes.data_as(dp), N))
    f = wl.batch_forces(beams, mass, 0, 0.005, False)
    capi.check(lib.otfem_set_nodes(h, capi.F_EXTERNAL, f.ctypes.data_as(dp), f.size))
    warm = WARM_STARTS[args.warm_start]
    p = capi.default_params(solver=capi.SOLVER_MIXED, max_iterations=5000, rtol=1e-6, graph=0, warm_start=warm)
    st = capi.StepStats()
    for k in range(args.steps):
        f = wl.batch_forces(beams, mass, k, 0.005, False)
        capi.check(lib.otfem_set_nodes(h, capi.F_EXTERNAL, f.ctypes.data_as(dp), f.size))
        capi.check(lib.otfem_simulate_ex(h, 0.005, 1, ctypes.byref(p), ctypes.byref(st)))
        print(f"batch step: largest iteration count {st.iterations}, rel. residual {st.rel_residual:.3e}")
    if args.trace:
        batch_trace_report(lib, h, dp, len(beams))
    if args.sweeps:
        capi.check(lib.otfem_apply_sweeps(h, capi.SOLVER_MIXED, 0.005, args.sweeps))
    capi.check(lib.otfem_synchronize(h))
    variant = ctypes.c_int32()
    capi.check(lib.otfem_tuning(h, ctypes.byref(variant), None))
    print(f"batch of {len(beams)} beams: tets {T}, nodes {N}, apply variant {variant.value}, "
          f"tuner sweeps {15 * tuning_rows(lib, h)}")
    capi.check(lib.otfem_destroy(h))


def tuning_rows(lib, h):
    rows = ctypes.c_int32()
    capi.check(lib.otfem_tuning_search(h, 0, ctypes.byref(rows), None, None, None, None))
    return rows.value


def sm_mhz():
    import subprocess
    try:
        return float(subprocess.run(["nvidia-smi", "--query-gpu=clocks.max.sm", "--format=csv,noheader,nounits", "-i",
                                     "0"], capture_output=True, text=True, timeout=20).stdout.split()[0])
    except (OSError, ValueError, IndexError, subprocess.SubprocessError):
        return 2070.0


def batch_trace_report(lib, h, dp, meshes):
    """Per iteration of the last batch step: the meshes still iterating and
    the time of the iteration and of its apply sweep (middle CTA's stamps,
    microseconds), summed over groups of iterations."""
    mhz = sm_mhz()
    ph = np.zeros(8)
    capi.check(lib.otfem_solver_phases(h, ph.ctypes.data_as(dp)))
    tr = np.zeros((256, 10))
    rows = ctypes.c_int32()
    capi.check(lib.otfem_solver_trace(h, tr.ctypes.data_as(dp), 256, ctypes.byref(rows)))
    tr = tr[:rows.value]
    if rows.value == 0:
        return
    start = np.concatenate([[ph[2]], tr[:-1, 9]])
    it_us = (tr[:, 9] - start) / mhz
    sweep_us = (tr[:, 4] - start) / mhz
    print(f"batch phases (us): b {ph[0] / mhz:.1f}, start sweeps {(ph[1] - ph[0]) / mhz:.1f}, "
          f"start {(ph[2] - ph[1]) / mhz:.1f}, CG loop {(ph[3] - ph[2]) / mhz:.1f}, update {(ph[4] - ph[3]) / mhz:.1f}")
    for lo, hi in ((0, 5), (5, 10), (10, 20), (20, 40), (40, 80), (80, 256)):
        sel = slice(lo, min(hi, rows.value))
        if lo >= rows.value:
            break
        print(f"iterations {lo}-{min(hi, rows.value) - 1}: meshes iterating {tr[sel, 0].min():.0f}-{tr[sel, 0].max():.0f} "
              f"of {meshes}, per iteration {it_us[sel].mean():.1f} us (apply sweep {sweep_us[sel].mean():.1f} us), "
              f"{it_us[sel].sum():.0f} us in all")


def trace_report(lib, h, dp):
    """Phases of the last solve and the median of each part of a CG
    iteration, from the SM clock stamps of the middle CTA (microseconds at
    the SM clock the GPU reports as its maximum)."""
    import subprocess
    try:
        mhz = float(subprocess.run(["nvidia-smi", "--query-gpu=clocks.max.sm", "--format=csv,noheader,nounits", "-i", "0"],
                                   capture_output=True, text=True, timeout=20).stdout.split()[0])
    except (OSError, ValueError, IndexError, subprocess.SubprocessError):
        mhz = 2070.0
    ph = np.zeros(8)
    capi.check(lib.otfem_solver_phases(h, ph.ctypes.data_as(dp)))
    names = ["b", "initial residual and direction sweeps", "start (projection solved, |r| and |b|)", "CG loop",
             "position update"]
    for n, v in zip(names, np.diff(np.concatenate([[0.0], ph[:5]]))):
        print(f"phase {n}: {v / mhz:.1f} us")
    if ph[5] > 0:
        print(f"start detail: node pass {(ph[5] - ph[1]) / mhz:.1f} us, Gram sums {(ph[6] - ph[5]) / mhz:.1f} us, "
              f"coefficients {(ph[7] - ph[6]) / mhz:.1f} us, moving the start {(ph[2] - ph[7]) / mhz:.1f} us")
    tr = np.zeros((256, 10))
    rows = ctypes.c_int32()
    capi.check(lib.otfem_solver_trace(h, tr.ctypes.data_as(dp), 256, ctypes.byref(rows)))
    tr = tr[:rows.value]
    if rows.value > 2:
        prev = tr[:-1, 9]
        cur = tr[1:]
        parts = np.stack([cur[:, 4] - prev, cur[:, 5] - cur[:, 4], cur[:, 6] - cur[:, 5], cur[:, 7] - cur[:, 6],
                          cur[:, 8] - cur[:, 7], cur[:, 9] - cur[:, 8]], 1) / mhz
        med = np.median(parts, 0)
        labels = ["apply sweep", "barrier", "dot products", "grid sum", "vector update", "barrier"]
        print("iteration (median us): " + ", ".join(f"{l} {v:.2f}" for l, v in zip(labels, med)) +
              f"; total {med.sum():.1f}")


if __name__ == "__main__":
    main()
