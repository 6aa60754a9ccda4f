"""Benchmark of the stiffness-warped FEM step on GB300.

Workload (the metric's single-GPU configuration): a cantilever beam of
128x32x32 unit blocks, edge 0.1 m, 5 tets per block (655,360 tets, 140,481
nodes), every node jittered by U[-0.01, 0.01] m (numpy PCG64 seed 20261203),
x = 0 face fixed, E = 5e5 Pa, nu = 0.33, rho = 1000 kg/m^3, mass damping 2.0,
dt = 0.01 s, gravity -9.81 in y, stiffness warping on, CG to relative
residual 1e-6.  A "step" is one fem::simulate time step of the whole mesh.

Metric: tet-steps/s = tets x steps / seconds.  `value` is measured with the
mesh resident in HBM (device-side CUDA events around each step, L2 flushed
between steps); `e2e` goes through the C ABI with host buffers: each step
uploads coord, velocity and f_external and downloads coord and velocity, as
the drop-in fem::simulate does.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
With N > 1 (torchrun), every rank runs an independent replica of the
workload on its own GPU (the path does not shard); value sums all ranks.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # the metric's single-GPU configuration
    "beam128": dict(I=128, J=32, K=32, edge=0.1, seed=20261203, jitter=0.01, young=5e5, poisson=0.33,
                    density=1000.0, dt=0.01, rtol=1e-6, mass_damping=2.0,
                    name="cantilever 128x32x32 blocks, 5 tets/block (655,360 tets, 140,481 nodes), jittered "
                         "+/-0.1 edge, E=5e5 nu=0.33 rho=1000, dt=0.01, gravity, warping, CG to rel. residual 1e-6"),
    # a small case for tests of the launcher and the replica path
    "beam8": dict(I=8, J=3, K=3, edge=0.1, seed=5, jitter=0.01, young=5e5, poisson=0.33, density=1000.0, dt=0.01,
                  rtol=1e-6, mass_damping=2.0, name="cantilever 8x3x3 blocks (360 tets), test size"),
}
WORKLOAD = WORKLOADS["beam128"]
METRIC = "tet-steps/sec at rel. residual 1e-6: learned warm-start vs plain CG, 1 GB300"
# algorithmic bytes of one element-apply sweep: per tet 4 int32 connectivity,
# Re 9 fp32, B 9 fp32, V*D 3 fp32 = 100 B; per free node read p 12 B, write
# A p 12 B, diagonal 4 B = 28 B.  Per CG iteration the FP64 vectors add
# 5 x 24 B per free node.
BYTES_PER_TET_APPLY = 100
BYTES_PER_NODE_APPLY = 28
BYTES_PER_NODE_ITER = 120
L2_FLUSH_BYTES = 512 << 20


def build_mesh():
    from opentissue_gb300.fem import generate_blocks
    w = WORKLOAD
    tets, coord = generate_blocks(w["I"], w["J"], w["K"], w["edge"], w["edge"], w["edge"])
    rng = np.random.default_rng(w["seed"])
    coord = coord + rng.uniform(-w["jitter"] * w["edge"] / 0.1, w["jitter"] * w["edge"] / 0.1, coord.shape)
    fixed = (np.arange(coord.shape[0]) < (w["J"] + 1) * (w["K"] + 1)).astype(np.uint8)
    return tets, coord, fixed


def gravity(mass, fixed):
    f = np.zeros((mass.shape[0], 3))
    free = fixed == 0
    f[free, 1] = -9.81 * mass[free]
    return f


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.idx = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def dist_max(world, value):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if torch.cuda.is_available() and dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def oracle_sample(tets, coord, fixed, steps):
    """The CPU baseline: the C restatement of the reference (converged CG,
    same stopping rule), single thread, `steps` steps from rest."""
    from oracle import build as obuild
    from oracle import pyoracle as po
    obuild.build_port()
    w = WORKLOAD
    m = po.OracleMesh(tets, coord, coord, fixed)
    m.init(w["young"], w["poisson"], w["density"], 1e30, 0.0, 0.0)
    f = gravity(m.get(po.MASS), fixed)
    times, its = [], []
    for _ in range(steps):
        m.set(po.F_EXTERNAL, f)
        t0 = time.perf_counter()
        it, _ = m.simulate_converged(w["dt"], True, w["mass_damping"], w["rtol"], 100000)
        times.append(time.perf_counter() - t0)
        its.append(it)
    m.close()
    return times, its


def run_reference(args, world, rank):
    if rank != 0:
        return
    tets, coord, fixed = build_mesh()
    T = tets.shape[0]
    times, its = oracle_sample(tets, coord, fixed, args.warmup + args.steps)
    timed = times[args.warmup:]
    val = T * len(timed) / sum(timed)
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "tet-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(timed) / len(timed),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD["name"], "solver": "reference pipeline (fem::detail steps) with "
                       "relative-residual CG, FP64", "iterations_per_step": float(np.mean(its[args.warmup:]))},
            "cpu_baseline": {"value": val, "unit": "tet-steps/s", "cores": 1, "kind": "port",
                             "sample": f"{args.steps} timed steps after {args.warmup} warm-up steps of the full "
                                       "workload on one host core (the reference FEM path is single-threaded)"},
            "e2e": {"value": val, "unit": "tet-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import torch
    from opentissue_gb300 import build as ext_build
    from opentissue_gb300 import capi

    ext_build.build()
    lib = capi.lib()
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    tets, coord, fixed = build_mesh()
    T, N = tets.shape[0], coord.shape[0]
    n_free = int((fixed == 0).sum())
    w = WORKLOAD
    _dp = ctypes.POINTER(ctypes.c_double)
    desc = capi.MeshDesc(N, T, tets.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), coord.ctypes.data_as(_dp),
                         coord.ctypes.data_as(_dp), fixed.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    h = ctypes.c_void_p()
    capi.check(lib.otfem_create(ctypes.byref(desc), ctypes.c_void_p(stream.cuda_stream), ctypes.byref(h)))
    capi.check(lib.otfem_init(h, w["young"], w["poisson"], w["density"], 1e30, 0.0, 0.0))
    mass = np.zeros(N)
    capi.check(lib.otfem_get_nodes(h, capi.MASS, mass.ctypes.data_as(_dp), N))
    fext = gravity(mass, fixed)
    capi.check(lib.otfem_set_nodes(h, capi.F_EXTERNAL, fext.ctypes.data_as(_dp), fext.size))
    params = capi.default_params(solver=capi.SOLVER_MIXED, mass_damping=w["mass_damping"], rtol=w["rtol"],
                                 max_iterations=5000, refresh_period=16)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    stats = capi.StepStats()

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.fill_(1.0)

    def step():
        capi.check(lib.otfem_simulate_ex(h, w["dt"], 1, ctypes.byref(params), None))

    for _ in range(args.warmup):
        step()
    capi.check(lib.otfem_last_stats(h, ctypes.byref(stats)))
    torch.cuda.synchronize()

    # ---- device-resident timed region --------------------------------------
    n0 = ctypes.c_int64()
    capi.check(lib.otfem_launch_count(h, ctypes.byref(n0)))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    its, res, applies = [], [], []
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    dist_barrier(world)
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush_l2()
        ev[k][0].record(stream)
        step()
        ev[k][1].record(stream)
        capi.check(lib.otfem_last_stats(h, ctypes.byref(stats)))
        its.append(stats.iterations)
        res.append(stats.rel_residual)
        applies.append(stats.applies)
    torch.cuda.synchronize()
    dist_barrier(world)
    clocks = sampler.stop()
    n1 = ctypes.c_int64()
    capi.check(lib.otfem_launch_count(h, ctypes.byref(n1)))
    dev_s = sum(a.elapsed_time(b) for a, b in ev) / 1e3
    dev_s = dist_max(world, dev_s)

    # ---- roofline: the persistent CG kernel timed on its own ---------------
    cg_ms, cg_bytes = [], []
    for k in range(max(3, min(args.steps, 10))):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        flush_l2()
        e0.record(stream)
        capi.check(lib.otfem_simulate_phase(h, w["dt"], 1, ctypes.byref(params), capi.PHASE_ORIENT))
        e1.record(stream)
        capi.check(lib.otfem_simulate_phase(h, w["dt"], 1, ctypes.byref(params), capi.PHASE_SOLVE))
        e2.record(stream)
        capi.check(lib.otfem_last_stats(h, ctypes.byref(stats)))
        cg_ms.append(e1.elapsed_time(e2))
        cg_bytes.append(stats.applies * (BYTES_PER_TET_APPLY * T + BYTES_PER_NODE_APPLY * n_free)
                        + stats.iterations * BYTES_PER_NODE_ITER * n_free)
    cg_s = np.array(cg_ms) / 1e3
    achieved = float(np.mean(np.array(cg_bytes) / cg_s)) / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = peaks.get("hbm_gbs")
    peak_note = "measured" if peak else "fallback"
    peak = peak or 6800.0
    # DRAM bytes of one k_cg_mixed launch from an ncu capture of this workload,
    # scaled to this run's element-apply sweeps per launch
    traffic = None
    try:
        prof = json.load(open(os.path.join(ROOT, "profiles", "cg_dram_traffic.json")))
        traffic = prof["dram_bytes_per_launch"] / prof["applies_per_launch"] * float(np.mean(applies))
    except (OSError, ValueError, KeyError, ZeroDivisionError):
        traffic = None

    # ---- the element-apply sweep alone (the stiffness apply) ----------------
    variant = ctypes.c_int32()
    capi.check(lib.otfem_tuning(h, ctypes.byref(variant), None))
    sweep_ms = []
    for k in range(10):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush_l2()
        e0.record(stream)
        capi.check(lib.otfem_apply_sweeps(h, capi.SOLVER_MIXED, w["dt"], 1))
        e1.record(stream)
        torch.cuda.synchronize()
        sweep_ms.append(e0.elapsed_time(e1))
    sweep_bytes = BYTES_PER_TET_APPLY * T + BYTES_PER_NODE_APPLY * n_free
    sweep_gbs = sweep_bytes / (float(np.median(sweep_ms)) * 1e-3) / 1e9

    # ---- end to end through the C ABI with host buffers ---------------------
    pin_x = torch.empty((N, 3), dtype=torch.float64, pin_memory=True).numpy()
    pin_v = torch.empty((N, 3), dtype=torch.float64, pin_memory=True).numpy()
    pin_f = torch.empty((N, 3), dtype=torch.float64, pin_memory=True).numpy()
    capi.check(lib.otfem_get_nodes(h, capi.COORD, pin_x.ctypes.data_as(_dp), pin_x.size))
    capi.check(lib.otfem_get_nodes(h, capi.VELOCITY, pin_v.ctypes.data_as(_dp), pin_v.size))
    pin_f[:] = fext
    e2e_ms = []
    dist_barrier(world)
    for k in range(args.steps):
        flush_l2()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        capi.check(lib.otfem_set_nodes(h, capi.COORD, pin_x.ctypes.data_as(_dp), pin_x.size))
        capi.check(lib.otfem_set_nodes(h, capi.VELOCITY, pin_v.ctypes.data_as(_dp), pin_v.size))
        capi.check(lib.otfem_set_nodes(h, capi.F_EXTERNAL, pin_f.ctypes.data_as(_dp), pin_f.size))
        step()
        capi.check(lib.otfem_get_nodes(h, capi.COORD, pin_x.ctypes.data_as(_dp), pin_x.size))
        capi.check(lib.otfem_get_nodes(h, capi.VELOCITY, pin_v.ctypes.data_as(_dp), pin_v.size))
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_s = dist_max(world, sum(e2e_ms) / 1e3)
    dist_barrier(world)

    total_tet_steps = T * args.steps * world
    value = total_tet_steps / dev_s
    e2e_value = total_tet_steps / e2e_s
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "tet-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 element apply, f64 CG vectors and reductions",
        "data": "synthetic",
        "config": {"workload": WORKLOAD["name"], "warm_start": "previous velocity (plain CG)",
                   "solver": "matrix-free persistent CG (OTFEM_SOLVER_MIXED), CUDA graph per step",
                   "l2": "flushed (512 MiB write) before every timed step", "replicas": world,
                   "iterations_per_step": float(np.mean(its)), "max_rel_residual": float(np.max(res))},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": "k_cg_mixed", "peak_source": peak_note,
                     "algorithmic_bytes_per_launch": float(np.mean(cg_bytes)),
                     "kernel_ms": float(np.mean(cg_ms)),
                     "apply_sweep": {"kernel": "k_apply_sweep<float>", "variant": int(variant.value),
                                     "ms": float(np.median(sweep_ms)), "algorithmic_bytes": sweep_bytes,
                                     "achieved": sweep_gbs, "frac": sweep_gbs / peak,
                                     "l2": "flushed before each sweep"}},
        "e2e": {"value": e2e_value, "unit": "tet-steps/s", "h2d_bytes_per_step": 3 * 24 * N,
                "d2h_bytes_per_step": 2 * 24 * N},
        "gpu_launches": int(n1.value - n0.value),
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        times, cits = oracle_sample(tets, coord, fixed, args.cpu_steps)
        line["cpu_baseline"] = {"value": T * len(times) / sum(times), "unit": "tet-steps/s", "cores": 1,
                                "kind": "port",
                                "sample": f"{args.cpu_steps} steps of the full workload from rest, converged CG "
                                          f"({float(np.mean(cits)):.0f} iterations/step), one host core"}
    print(json.dumps(line), flush=True)
    capi.check(lib.otfem_destroy(h))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="beam128", choices=sorted(WORKLOADS))
    args = ap.parse_args()
    global WORKLOAD
    WORKLOAD = WORKLOADS[args.workload]
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
