"""Benchmark of the stiffness-warped FEM step on GB300.

Workload (the metric's single-GPU configuration): a cantilever beam of
128x32x32 unit blocks, edge 0.1 m, 5 tets per block (655,360 tets, 140,481
nodes), every node jittered by U[-0.01, 0.01] m (numpy PCG64 seed 20261203),
x = 0 face fixed, E = 5e5 Pa, nu = 0.33, rho = 1000 kg/m^3, mass damping 2.0,
dt = 0.01 s, gravity -9.81 in y, stiffness warping on, CG to relative
residual 1e-6.  A "step" is one fem::simulate time step of the whole mesh.

Metric: tet-steps/s = tets x steps / seconds.  `value` is the headline arm,
the extrapolated warm start (CG from the velocity the degree-4 polynomial
through the last five velocities predicts, Jacobi PCG), next to the plain CG
(the reference's method: previous-velocity start, no preconditioner), the
projected start (the least-energy point on the span of the last four
velocity changes) and the learned warm start (the trained network's
correction added to that search space) on the same trajectory; both measure
slower than the extrapolated start (config.projected, config.learned).  The
run first builds the network's training set with the plain solver on beams
of the workload's family (other jitter seeds; gravity, every other beam
with a sinusoidal tip load; 2M node samples) and trains it on the GPU
(Adam, lr 1e-3, batch 65,536, 60 epochs); both are timed outside the
measured steps and reported in config.training.

`value` is measured with the mesh resident in HBM (device-side CUDA events
around each step, L2 flushed between steps); `e2e` goes through the C ABI
with host buffers: each step takes coord, velocity and f_external from
page-locked host arrays and returns coord and velocity in them, as the
drop-in fem::simulate does (otfem_simulate_host: one graph per step whose
velocity and force uploads overlap the orientation kernel and whose two
downloads run at once; `e2e.staged` times the explicit copy sequence beside
it).

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
# Algorithmic bytes of one element-apply sweep, the canonical B-form in FP32:
# per tet 100 B (4 int32 node ids 16 B, Re as 9 fp32 36 B, B as 9 fp32 36 B,
# V*D 3 fp32 12 B), per free node 28 B (read p 12 B, write A p 12 B, the
# diagonal 4 B).  Every apply variant is scored against these bytes; the
# tets and staged variants actually read 80 B per tet (the rotation as a
# quaternion).  Per CG iteration the vector updates add 5 x 24 B = 120 B per
# free node.
BYTES_PER_TET_APPLY = 100
BYTES_PER_NODE_APPLY = 28
BYTES_PER_NODE_ITER = 120
L2_FLUSH_BYTES = 512 << 20


def build_mesh(seed=None):
    from opentissue_gb300.fem import generate_blocks
    w = WORKLOAD
    tets, coord = generate_blocks(w["I"], w["J"], w["K"], w["edge"], w["edge"], w["edge"])
    rng = np.random.default_rng(w["seed"] if seed is None else seed)
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


def oracle_batch_sample(beams, steps, threads=None):
    """The CPU baseline of the batch configuration: the C restatement of the
    reference (converged CG, rel. residual 1e-6), each beam an independent
    mesh, the beams spread over the host's cores (a pool of threads pulling
    beams; the oracle's calls release the interpreter lock), `steps` steps
    from rest under gravity and each beam's constant tip force, dt 0.005.
    Returns (tet-steps/s, threads, wall seconds)."""
    import concurrent.futures as cf
    from oracle import build as obuild
    from oracle import pyoracle as po
    from opentissue_gb300 import workloads as wl
    obuild.build_port()
    threads = threads or os.cpu_count() or 1

    def make(b):
        m = po.OracleMesh(b["tets"], b["coord"], b["coord"], b["fixed"])
        m.init(b["young"], b["poisson"], b["density"], 1e30, 0.0, 0.0)
        return m, wl.batch_forces([b], m.get(po.MASS), 0, 0.005, False, [0.0])

    def run(mf):
        m, f = mf
        for _ in range(steps):
            m.set(po.F_EXTERNAL, f)
            m.simulate_converged(0.005, True, WORKLOAD["mass_damping"], WORKLOAD["rtol"], 100000)

    order = sorted(beams, key=lambda b: -b["tets"].shape[0])  # largest first
    with cf.ThreadPoolExecutor(max_workers=threads) as pool:
        meshes = list(pool.map(make, order))  # set-up, untimed
        t0 = time.perf_counter()
        list(pool.map(run, meshes))
        wall = time.perf_counter() - t0
    for m, _ in meshes:
        m.close()
    T = sum(b["tets"].shape[0] for b in beams)
    return T * steps / wall, threads, wall


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


def load_fixture(name):
    """A trajectory of the reference's FP64 pipeline (tests/golden/traj_*.npz,
    made by tests/golden/make_trajectories.py from the reference build); None
    where it is absent."""
    try:
        return np.load(os.path.join(ROOT, "tests", "golden", name + ".npz"))
    except OSError:
        return None


class OracleError:
    """Largest relative error of a run against a fixture at its sampled steps:
    |x - x_ref| over the step's largest displacement and |v - v_ref| over its
    largest velocity (the fixture's scales over all nodes)."""

    def __init__(self, fix):
        self.fix = fix
        self.keep = [int(k) for k in fix["keep"]] if fix is not None else []
        self.errs = {}

    def wants(self, step):
        return step in self.keep

    def record(self, step, x, v):
        f = self.fix
        smp = f["sample"]
        ex = float(np.abs(x[smp] - f[f"x_{step}"]).max() / float(f[f"disp_{step}"]))
        ev = float(np.abs(v[smp] - f[f"v_{step}"]).max() / float(f[f"vmax_{step}"]))
        self.errs[step] = (ex, ev)

    def result(self):
        """Largest errors over the sampled steps, per step, and the FP64
        reference pipeline's own errors when stopped at rel. residual 1e-6
        (the same tolerance) at those steps."""
        if not self.errs:
            return None
        f = self.fix
        e6 = {k: (float(f[f"rtol6_x_err_{k}"]), float(f[f"rtol6_v_err_{k}"])) for k in self.errs}
        return {"x": max(e[0] for e in self.errs.values()), "v": max(e[1] for e in self.errs.values()),
                "steps": sorted(self.errs),
                "per_step": {str(k): {"x": e[0], "v": e[1], "fp64_rtol1e6_x": e6[k][0], "fp64_rtol1e6_v": e6[k][1]}
                             for k, e in sorted(self.errs.items())},
                "fp64_rtol1e6": {"x": max(e[0] for e in e6.values()), "v": max(e[1] for e in e6.values())}}


def get_xv(lib, capi, h, N):
    x = np.zeros((N, 3))
    v = np.zeros((N, 3))
    capi.check(lib.otfem_get_nodes(h, capi.COORD, x.ctypes.data_as(_dp), x.size))
    capi.check(lib.otfem_get_nodes(h, capi.VELOCITY, v.ctypes.data_as(_dp), v.size))
    return x, v


def train_warm_start(lib, capi, stream, args, rng):
    """Training set and training of the learned warm start (the network of
    the metric): (inputs, dv - dv_prev) pairs of the plain solver on beams of
    the workload's family (other jitter seeds; gravity, half of them with a
    sinusoidal tip load), Adam lr 1e-3, batch 65,536.  Returns the network
    and a summary."""
    from opentissue_gb300.warmstart import WarmStartNet
    w = WORKLOAD
    n_target = args.train_samples
    net = WarmStartNet(capacity=n_target, seed=args.seed)
    params = capi.default_params(solver=capi.SOLVER_MIXED, mass_damping=w["mass_damping"], rtol=w["rtol"],
                                 max_iterations=5000, refresh_period=16)
    t0 = time.perf_counter()
    beams = 0
    while net.num_samples() < n_target and beams < 64:
        tets, coord, fixed = build_mesh(seed=int(rng.integers(1 << 30)))
        h = make_handle(lib, capi, tets, coord, fixed, stream)
        WarmStartNet.collect(h)
        mass = get_mass(lib, capi, h, coord.shape[0])
        amp = 0.0 if beams % 2 == 0 else float(rng.uniform(0, 100))
        freq, d = float(rng.uniform(0.5, 5)), rng.normal(size=3)
        d /= np.linalg.norm(d)
        free = int((fixed == 0).sum())
        steps = args.train_steps
        frac = min(1.0, n_target / (2 * steps * free))
        for s in range(steps):
            f = gravity(mass, fixed) + tip_load(coord, amp, freq, d, s * w["dt"])
            capi.check(lib.otfem_set_nodes(h, capi.F_EXTERNAL, f.ctypes.data_as(_dp), f.size))
            capi.check(lib.otfem_simulate_ex(h, w["dt"], 1, ctypes.byref(params), None))
            net.add_samples(h, fraction=frac, seed=int(rng.integers(1 << 62)))
        capi.check(lib.otfem_destroy(h))
        beams += 1
    gen_s = time.perf_counter() - t0
    net.fit_normalization()
    loss0 = net.evaluate()
    t0 = time.perf_counter()
    loss = net.train(args.train_epochs, batch=65536, lr=1e-3, seed=args.seed)
    train_s = time.perf_counter() - t0
    return net, {"samples": net.num_samples(), "beams": beams, "epochs": args.train_epochs, "batch": 65536,
                 "lr": 1e-3, "loss_initial": loss0, "loss_final": loss, "generate_s": round(gen_s, 2),
                 "train_s": round(train_s, 2)}


_dp = ctypes.POINTER(ctypes.c_double)


def make_handle(lib, capi, tets, coord, fixed, stream):
    w = WORKLOAD
    desc = capi.MeshDesc(coord.shape[0], tets.shape[0], tets.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                         coord.ctypes.data_as(_dp), coord.ctypes.data_as(_dp),
                         fixed.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    h = ctypes.c_void_p()
    capi.check(lib.otfem_create(ctypes.byref(desc), ctypes.c_void_p(stream.cuda_stream), ctypes.byref(h)))
    capi.check(lib.otfem_init(h, w["young"], w["poisson"], w["density"], 1e30, 0.0, 0.0))
    return h


def get_mass(lib, capi, h, N):
    mass = np.zeros(N)
    capi.check(lib.otfem_get_nodes(h, capi.MASS, mass.ctypes.data_as(_dp), N))
    return mass


def tip_load(coord, amp, freq, d, t):
    w = WORKLOAD
    f = np.zeros_like(coord)
    if amp == 0.0:
        return f
    tip = np.arange(coord.shape[0]) >= w["I"] * (w["J"] + 1) * (w["K"] + 1)
    f[tip] = amp * np.sin(2 * np.pi * freq * t) * d / tip.sum()
    return f


def timed_steps(lib, capi, torch, stream, h, params, steps, forces, dt, flush_l2, stats_fn=None, after=None,
                first=0):
    """Steps with per-step external forces forces(k) (host arrays), timed on
    the device; after(step) runs on the host after each step's end event
    (outside the timing; step = first + k + 1).  Returns seconds and
    per-step iteration counts."""
    st = capi.StepStats()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    its = []
    for k in range(steps):
        f = forces(k)
        capi.check(lib.otfem_set_nodes(h, capi.F_EXTERNAL, f.ctypes.data_as(_dp), f.size))
        flush_l2()
        ev[k][0].record(stream)
        capi.check(lib.otfem_simulate_ex(h, dt, 1, ctypes.byref(params), ctypes.byref(st)))
        ev[k][1].record(stream)
        capi.check(lib.otfem_last_stats(h, ctypes.byref(st)))
        its.append(st.iterations if stats_fn is None else stats_fn())
        if after is not None:
            after(first + k + 1)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev) / 1e3, its


def run_inference_ab(lib, capi, torch, stream, net, args, flush_l2):
    """Learned vs plain CG (and the Jacobi and projected ablations) on the
    64x16x16 jittered beam under gravity and the seeded sinusoidal tip load
    (amplitude U[0,100] N, frequency U[0.5,5] Hz, direction uniform:
    workloads.SineTip), dt 0.01, from rest; positions and velocities checked
    against the reference's FP64 trajectory of the same run."""
    from opentissue_gb300 import workloads as wl
    cfg = wl.BEAM64_SINE
    I, J, K = cfg["I"], cfg["J"], cfg["K"]
    tets, coord, fixed = wl.jittered_beam(I, J, K, cfg["seed"])
    load = wl.SineTip(I, J, K, cfg["load_seed"])
    N = coord.shape[0]
    fix = load_fixture("traj_beam64_sine")
    w = WORKLOAD
    out = {}
    arms = (("plain", None, dict(preconditioner=capi.PRECONDITIONER_NONE)), ("plain_jacobi", None, {}),
            ("projected", None, dict(warm_start=capi.WARM_START_PROJECTED)),
            ("extrapolated", None, dict(warm_start=capi.WARM_START_EXTRAPOLATED, warm_history=4)),
            ("learned", net, dict(warm_start=capi.WARM_START_LEARNED)))
    for name, mlp, kw in arms:
        h = make_handle(lib, capi, tets, coord, fixed, stream)
        if mlp is not None:
            mlp.attach(h)
        mass = get_mass(lib, capi, h, N)
        g = gravity(mass, fixed)
        p = capi.default_params(solver=capi.SOLVER_MIXED, mass_damping=w["mass_damping"], rtol=w["rtol"],
                                max_iterations=5000, refresh_period=16, **kw)
        check = OracleError(fix)

        def after(step):
            if check.wants(step):
                check.record(step, *get_xv(lib, capi, h, N))
        sec, its = timed_steps(lib, capi, torch, stream, h, p, args.ab_steps, lambda k: g + load.force(k, cfg["dt"]),
                               cfg["dt"], flush_l2, after=after)
        x = np.zeros((N, 3))
        capi.check(lib.otfem_get_nodes(h, capi.COORD, x.ctypes.data_as(_dp), x.size))
        out[name] = {"tet_steps_per_s": tets.shape[0] * args.ab_steps / sec, "iterations_per_step": float(np.mean(its)),
                     "x": x, "oracle_error": check.result()}
        if mlp is not None:
            mlp.detach(h)
        capi.check(lib.otfem_destroy(h))
    disp = np.abs(out["plain"]["x"] - coord).max()
    res = {"workload": f"64x16x16 jittered beam ({tets.shape[0]} tets), gravity + tip load {load.amp:.1f} N "
                       f"sin(2 pi {load.freq:.2f} t), {args.ab_steps} steps from rest, dt 0.01, rel. residual 1e-6"}
    for k, v in out.items():
        res[k] = {"tet_steps_per_s": v["tet_steps_per_s"], "iterations_per_step": v["iterations_per_step"],
                  "oracle_error": v["oracle_error"]}
        if k != "plain":
            res[k]["position_difference_vs_plain"] = float(np.abs(v["x"] - out["plain"]["x"]).max() / disp)
    res["learned_over_plain"] = out["learned"]["tet_steps_per_s"] / out["plain"]["tet_steps_per_s"]
    res["learned_over_projected"] = out["learned"]["tet_steps_per_s"] / out["projected"]["tet_steps_per_s"]
    res["extrapolated_over_projected"] = (out["extrapolated"]["tet_steps_per_s"] /
                                          out["projected"]["tet_steps_per_s"])
    return res


def run_batch_workload(lib, capi, torch, stream, net, args, flush_l2):
    """256 beams of uneven size (nx U{8..64}, ny, nz U{3..16}), per-beam
    material, random fixed face, gravity plus a tip force, dt 0.005, one
    persistent launch per step: plain CG, Jacobi PCG, the projected and the
    extrapolated start under a constant tip force, then Jacobi PCG, projected,
    extrapolated and learned under a sinusoidal tip force."""
    from opentissue_gb300 import workloads as wl
    from opentissue_gb300.workloads import random_beams
    beams = random_beams(args.batch_meshes, seed=args.seed)
    descs = (capi.MeshDesc * len(beams))()
    keep = []
    for k, b in enumerate(beams):
        tets = np.ascontiguousarray(b["tets"], np.int32)
        coord = np.ascontiguousarray(b["coord"], np.float64)
        fixed = np.ascontiguousarray(b["fixed"], np.uint8)
        keep += [tets, coord, fixed]
        descs[k] = capi.MeshDesc(coord.shape[0], tets.shape[0], tets.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                 coord.ctypes.data_as(_dp), coord.ctypes.data_as(_dp),
                                 fixed.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    T = sum(b["tets"].shape[0] for b in beams)
    N = sum(b["coord"].shape[0] for b in beams)
    fixed_all = np.concatenate([b["fixed"] for b in beams])
    freqs = wl.batch_tip_frequencies(len(beams))
    # the reference's FP64 trajectories of eight of the beams (the full
    # 256-beam batch of the default workload only)
    fix = load_fixture("traj_batch") if (len(beams), args.seed) == (wl.BATCH["count"], wl.BATCH["seed"]) else None
    w = WORKLOAD
    res = {"workload": f"{len(beams)} beams, {T} tets, {N} nodes, dt 0.005, rel. residual 1e-6"}
    arms = (("plain_cg", capi.WARM_START_PREVIOUS, False, capi.PRECONDITIONER_NONE),
            ("plain", capi.WARM_START_PREVIOUS, False, capi.PRECONDITIONER_JACOBI),
            ("projected", capi.WARM_START_PROJECTED, False, capi.PRECONDITIONER_JACOBI),
            ("extrapolated", capi.WARM_START_EXTRAPOLATED, False, capi.PRECONDITIONER_JACOBI),
            ("plain_tip_sine", capi.WARM_START_PREVIOUS, True, capi.PRECONDITIONER_JACOBI),
            ("projected_tip_sine", capi.WARM_START_PROJECTED, True, capi.PRECONDITIONER_JACOBI),
            ("extrapolated_tip_sine", capi.WARM_START_EXTRAPOLATED, True, capi.PRECONDITIONER_JACOBI),
            ("learned_tip_sine", capi.WARM_START_LEARNED, True, capi.PRECONDITIONER_JACOBI))
    for name, warm, vary, pre in arms:
        h = ctypes.c_void_p()
        t0 = time.perf_counter()
        capi.check(lib.otfem_batch_create(descs, len(beams), ctypes.c_void_p(stream.cuda_stream), ctypes.byref(h)))
        e = np.array([b["young"] for b in beams])
        nu = np.array([b["poisson"] for b in beams])
        rho = np.array([b["density"] for b in beams])
        capi.check(lib.otfem_batch_init(h, e.ctypes.data_as(_dp), nu.ctypes.data_as(_dp), rho.ctypes.data_as(_dp),
                                        1e30, 0.0, 0.0))
        setup_s = time.perf_counter() - t0
        if warm == capi.WARM_START_LEARNED:
            net.attach(h)
        mass = get_mass(lib, capi, h, N)
        p = capi.default_params(solver=capi.SOLVER_MIXED, mass_damping=w["mass_damping"], rtol=w["rtol"],
                                max_iterations=5000, refresh_period=16, warm_start=warm, preconditioner=pre)

        def forces(k):
            return wl.batch_forces(beams, mass, k, 0.005, vary, freqs)
        noff = np.zeros(len(beams) + 1, np.int64)
        noff[1:] = np.cumsum([b["coord"].shape[0] for b in beams])
        errs = {}

        def after(step):
            if fix is None or step not in [int(k) for k in fix["keep"]]:
                return
            x, v = get_xv(lib, capi, h, N)
            tag = "sine" if vary else "const"
            ex = ev_ = 0.0
            ex6 = ev6 = 0.0
            for i in fix["beams"]:
                i = int(i)
                pre, smp = f"b{i}_{tag}_", noff[i] + fix[f"b{i}_sample"]
                xr, vr = fix[f"{pre}x_{step}"], fix[f"{pre}v_{step}"]
                ex = max(ex, float(np.abs(x[smp] - xr).max() / float(fix[f"{pre}disp_{step}"])))
                ev_ = max(ev_, float(np.abs(v[smp] - vr).max() / float(fix[f"{pre}vmax_{step}"])))
                ex6 = max(ex6, float(fix[f"{pre}rtol6_x_err_{step}"]))
                ev6 = max(ev6, float(fix[f"{pre}rtol6_v_err_{step}"]))
            errs[step] = (ex, ev_, ex6, ev6)
        steps = args.batch_steps
        pre_steps = args.lead_in + args.warmup
        timed_steps(lib, capi, torch, stream, h, p, pre_steps, forces, 0.005, flush_l2, after=after)
        sec, its = timed_steps(lib, capi, torch, stream, h, p, steps, lambda k: forces(k + pre_steps), 0.005,
                               flush_l2, after=after, first=pre_steps)
        done = pre_steps + steps
        last = max(int(k) for k in fix["keep"]) if fix is not None else 0
        st_ = capi.StepStats()
        while done < last:
            f = forces(done)
            capi.check(lib.otfem_set_nodes(h, capi.F_EXTERNAL, f.ctypes.data_as(_dp), f.size))
            capi.check(lib.otfem_simulate_ex(h, 0.005, 1, ctypes.byref(p), ctypes.byref(st_)))
            done += 1
            after(done)
        M = len(beams)
        mi = np.zeros(M, np.int32)
        capi.check(lib.otfem_batch_stats(h, mi.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), None, None, None))
        res[name] = {"tet_steps_per_s": T * steps / sec, "ms_per_step": 1e3 * sec / steps,
                     "max_iterations_per_step": float(np.mean(its)),
                     "mesh_iterations_last_step": {"mean": float(mi.mean()), "min": int(mi.min()), "max": int(mi.max())},
                     "setup_s": round(setup_s, 2)}
        if errs:
            res[name]["oracle_error"] = {
                "x": max(e[0] for e in errs.values()), "v": max(e[1] for e in errs.values()), "steps": sorted(errs),
                "beams": [int(i) for i in fix["beams"]],
                "fp64_rtol1e6": {"x": max(e[2] for e in errs.values()), "v": max(e[3] for e in errs.values())}}
        if name == "plain":
            # the element apply over all 4M tets (325 MB of tiles: beyond the
            # 129 MB L2, the HBM-bound regime), L2 flushed before each sweep
            variant = ctypes.c_int32()
            capi.check(lib.otfem_tuning(h, ctypes.byref(variant), None))
            n_free = int((fixed_all == 0).sum())
            nbytes = BYTES_PER_TET_APPLY * T + BYTES_PER_NODE_APPLY * n_free
            sweep_ms = []
            for _ in range(10):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                flush_l2()
                e0.record(stream)
                capi.check(lib.otfem_apply_sweeps(h, capi.SOLVER_MIXED, 0.005, 1))
                e1.record(stream)
                torch.cuda.synchronize()
                sweep_ms.append(e0.elapsed_time(e1))
            ms = float(np.median(sweep_ms))
            res["apply_sweep"] = {"variant": int(variant.value), "ms": ms, "algorithmic_bytes": nbytes,
                                  "achieved_gbs": nbytes / (ms * 1e-3) / 1e9, "l2": "flushed before each sweep"}
        if warm == capi.WARM_START_LEARNED:
            net.detach(h)
        capi.check(lib.otfem_destroy(h))
    if not args.no_cpu_baseline:
        # the reference's method on the host: every beam an independent mesh,
        # the beams spread over all host cores, 2 steps from rest
        val, threads, wall = oracle_batch_sample(beams, 2)
        res["cpu_baseline"] = {"value": val, "unit": "tet-steps/s", "cores": threads, "kind": "port",
                               "sample": f"2 steps from rest of all {len(beams)} beams (constant tip force), "
                                         f"converged CG, one beam per thread at a time, {wall:.1f} s wall"}
    res["projected_over_plain_cg"] = res["projected"]["tet_steps_per_s"] / res["plain_cg"]["tet_steps_per_s"]
    res["extrapolated_over_projected"] = res["extrapolated"]["tet_steps_per_s"] / res["projected"]["tet_steps_per_s"]
    res["learned_over_plain_tip_sine"] = res["learned_tip_sine"]["tet_steps_per_s"] / res["plain_tip_sine"]["tet_steps_per_s"]
    res["timed_steps"] = f"steps {args.lead_in + args.warmup + 1}..{args.lead_in + args.warmup + args.batch_steps}"
    return res


def run_ours(args, world, rank, local):
    import torch
    from opentissue_gb300 import build as ext_build
    from opentissue_gb300 import capi

    ext_build.build()
    lib = capi.lib()
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    rng = np.random.default_rng(args.seed + rank)
    w = WORKLOAD
    net, train_info = train_warm_start(lib, capi, stream, args, rng)

    tets, coord, fixed = build_mesh()
    T, N = tets.shape[0], coord.shape[0]
    n_free = int((fixed == 0).sum())
    def solver_params(**kw):
        base = dict(solver=capi.SOLVER_MIXED, mass_damping=w["mass_damping"], rtol=w["rtol"], max_iterations=5000,
                    refresh_period=16)
        base.update(kw)
        return capi.default_params(**base)
    # plain CG: the reference's method (no preconditioner, previous-velocity start) on the GPU
    plain = solver_params(preconditioner=capi.PRECONDITIONER_NONE)
    plain_jacobi = solver_params()
    projected = solver_params(warm_start=capi.WARM_START_PROJECTED)
    # the headline: CG from the velocity extrapolated by the degree-4
    # polynomial through the last five velocities (no extra element apply)
    extrapolated = solver_params(warm_start=capi.WARM_START_EXTRAPOLATED, warm_history=4)
    head = extrapolated
    # the same Jacobi PCG with every vector, reduction and scalar in FP64 and
    # the FP64 element apply (the precision the scope names for the CG
    # scalars, at FP64 cost)
    fp64_jacobi = solver_params(solver=capi.SOLVER_FP64)
    # the network's correction in place of the oldest history direction: the
    # same four search directions as the projected start
    learned_h3 = solver_params(warm_start=capi.WARM_START_LEARNED, warm_history=3)
    learned = solver_params(warm_start=capi.WARM_START_LEARNED)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.fill_(1.0)

    fix128 = load_fixture("traj_beam128") if args.workload == "beam128" else None

    def timed_run(h, params, continue_to_end=True):
        """The lead-in steps of the trajectory from rest and W warm-up steps,
        then K steps timed on the device (L2 flushed before each); the
        workload's gravity load.  The positions and velocities at the
        reference trajectory's sampled steps are compared with it, and (with
        continue_to_end) the run continues untimed to the trajectory's last
        step."""
        mass = get_mass(lib, capi, h, N)
        fext = gravity(mass, fixed)
        capi.check(lib.otfem_set_nodes(h, capi.F_EXTERNAL, fext.ctypes.data_as(_dp), fext.size))
        stats = capi.StepStats()
        check = OracleError(fix128)
        step = 0
        for _ in range(args.lead_in + args.warmup):
            capi.check(lib.otfem_simulate_ex(h, w["dt"], 1, ctypes.byref(params), None))
            step += 1
            if check.wants(step):
                check.record(step, *get_xv(lib, capi, h, N))
        torch.cuda.synchronize()
        n0 = ctypes.c_int64()
        capi.check(lib.otfem_launch_count(h, ctypes.byref(n0)))
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        its, res, applies = [], [], []
        dist_barrier(world)
        torch.cuda.synchronize()
        for k in range(args.steps):
            flush_l2()
            ev[k][0].record(stream)
            capi.check(lib.otfem_simulate_ex(h, w["dt"], 1, ctypes.byref(params), None))
            ev[k][1].record(stream)
            capi.check(lib.otfem_last_stats(h, ctypes.byref(stats)))
            its.append(stats.iterations)
            res.append(stats.rel_residual)
            applies.append(stats.applies)
            step += 1
            if check.wants(step):
                # after the step's end event: the host read is outside the timing
                check.record(step, *get_xv(lib, capi, h, N))
        torch.cuda.synchronize()
        dist_barrier(world)
        n1 = ctypes.c_int64()
        capi.check(lib.otfem_launch_count(h, ctypes.byref(n1)))
        dev_s = dist_max(world, sum(a.elapsed_time(b) for a, b in ev) / 1e3)
        x = np.zeros((N, 3))
        capi.check(lib.otfem_get_nodes(h, capi.COORD, x.ctypes.data_as(_dp), x.size))
        while continue_to_end and check.keep and step < max(check.keep):
            capi.check(lib.otfem_simulate_ex(h, w["dt"], 1, ctypes.byref(params), None))
            step += 1
            if check.wants(step):
                check.record(step, *get_xv(lib, capi, h, N))
        return {"dev_s": dev_s, "its": its, "res": res, "applies": applies, "launches": int(n1.value - n0.value),
                "x": x, "fext": fext, "oracle_error": check.result()}

    # ---- plain CG (the reference's method) and the headline arm, the
    # extrapolated start; then the projected start, the learned start (the
    # network's correction in the projected start's search space),
    # Jacobi-preconditioned CG and the other ablations, each on the same
    # trajectory
    h_plain = make_handle(lib, capi, tets, coord, fixed, stream)
    h_head = make_handle(lib, capi, tets, coord, fixed, stream)
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    r_plain = timed_run(h_plain, plain)
    # the headline handle stays at the timed steps' point of the trajectory:
    # the end-to-end steps below continue from there
    r_head = timed_run(h_head, head, continue_to_end=False)
    clocks = sampler.stop()
    ablations = {}
    for name, prm in (("projected", projected), ("learned", learned), ("plain_jacobi", plain_jacobi),
                      ("fp64_jacobi", fp64_jacobi), ("learned_history3", learned_h3)):
        h_ab = make_handle(lib, capi, tets, coord, fixed, stream)
        if prm.warm_start == capi.WARM_START_LEARNED:
            net.attach(h_ab)
        ablations[name] = timed_run(h_ab, prm)
        if prm.warm_start == capi.WARM_START_LEARNED:
            net.detach(h_ab)
        capi.check(lib.otfem_destroy(h_ab))
    disp = np.abs(r_plain["x"] - coord).max()
    pos_diff = float(np.abs(r_head["x"] - r_plain["x"]).max() / max(disp, 1e-300))
    r_learn = ablations["learned"]
    r_proj = ablations["projected"]

    # ---- roofline: the persistent CG kernel timed on its own ---------------
    cg_ms, cg_bytes, cg_applies = [], [], []
    stats = capi.StepStats()
    variant = ctypes.c_int32()
    capi.check(lib.otfem_tuning(h_plain, ctypes.byref(variant), None))
    tet_bytes = BYTES_PER_TET_APPLY
    for k in range(max(3, min(args.steps, 10))):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        flush_l2()
        e0.record(stream)
        capi.check(lib.otfem_simulate_phase(h_plain, w["dt"], 1, ctypes.byref(plain), capi.PHASE_ORIENT))
        e1.record(stream)
        capi.check(lib.otfem_simulate_phase(h_plain, w["dt"], 1, ctypes.byref(plain), capi.PHASE_SOLVE))
        e2.record(stream)
        capi.check(lib.otfem_last_stats(h_plain, ctypes.byref(stats)))
        cg_ms.append(e1.elapsed_time(e2))
        cg_applies.append(stats.applies)
        cg_bytes.append(stats.applies * (tet_bytes * T + BYTES_PER_NODE_APPLY * n_free)
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
    # scaled to the element-apply sweeps of the launches timed here
    traffic = None
    try:
        prof = json.load(open(os.path.join(ROOT, "profiles", "cg_dram_traffic.json")))
        traffic = prof["dram_bytes_per_launch"] / prof["applies_per_launch"] * float(np.mean(cg_applies))
    except (OSError, ValueError, KeyError, ZeroDivisionError):
        traffic = None

    # ---- the element-apply sweep alone (the stiffness apply) ----------------
    sweep_ms = []
    for k in range(10):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush_l2()
        e0.record(stream)
        capi.check(lib.otfem_apply_sweeps(h_plain, capi.SOLVER_MIXED, w["dt"], 1))
        e1.record(stream)
        torch.cuda.synchronize()
        sweep_ms.append(e0.elapsed_time(e1))
    sweep_bytes = tet_bytes * T + BYTES_PER_NODE_APPLY * n_free
    sweep_gbs = sweep_bytes / (float(np.median(sweep_ms)) * 1e-3) / 1e9

    # ---- end to end through the C ABI with host buffers (headline arm) -----
    # otfem_simulate_host on page-locked host arrays; beside it the copy
    # sequence (set coord, velocity, forces; step; get coord, velocity) from
    # the same state
    pin_x = torch.empty((N, 3), dtype=torch.float64, pin_memory=True).numpy()
    pin_v = torch.empty((N, 3), dtype=torch.float64, pin_memory=True).numpy()
    pin_f = torch.empty((N, 3), dtype=torch.float64, pin_memory=True).numpy()
    capi.check(lib.otfem_get_nodes(h_head, capi.COORD, pin_x.ctypes.data_as(_dp), pin_x.size))
    capi.check(lib.otfem_get_nodes(h_head, capi.VELOCITY, pin_v.ctypes.data_as(_dp), pin_v.size))
    pin_f[:] = r_head["fext"]
    x_start, v_start = pin_x.copy(), pin_v.copy()
    e2e_ms, staged_ms = [], []
    dist_barrier(world)
    for k in range(args.steps):
        flush_l2()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        capi.check(lib.otfem_simulate_host(h_head, w["dt"], 1, ctypes.byref(head), None,
                                           pin_x.ctypes.data_as(_dp), pin_v.ctypes.data_as(_dp),
                                           pin_f.ctypes.data_as(_dp)))
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    pin_x[:] = x_start
    pin_v[:] = v_start
    for k in range(args.steps):
        flush_l2()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        capi.check(lib.otfem_set_nodes(h_head, capi.COORD, pin_x.ctypes.data_as(_dp), pin_x.size))
        capi.check(lib.otfem_set_nodes(h_head, capi.VELOCITY, pin_v.ctypes.data_as(_dp), pin_v.size))
        capi.check(lib.otfem_set_nodes(h_head, capi.F_EXTERNAL, pin_f.ctypes.data_as(_dp), pin_f.size))
        capi.check(lib.otfem_simulate_ex(h_head, w["dt"], 1, ctypes.byref(head), None))
        # both downloads queued back to back, one wait
        capi.check(lib.otfem_get_nodes_async(h_head, capi.COORD, pin_x.ctypes.data_as(_dp), pin_x.size))
        capi.check(lib.otfem_get_nodes_async(h_head, capi.VELOCITY, pin_v.ctypes.data_as(_dp), pin_v.size))
        capi.check(lib.otfem_synchronize(h_head))
        staged_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_s = dist_max(world, sum(e2e_ms) / 1e3)
    staged_s = dist_max(world, sum(staged_ms) / 1e3)
    dist_barrier(world)
    # the headline arm against the reference trajectory: a fresh handle, the
    # same steps from rest to the trajectory's last sampled step (untimed)
    if fix128 is not None:
        h_chk = make_handle(lib, capi, tets, coord, fixed, stream)
        fext_chk = gravity(get_mass(lib, capi, h_chk, N), fixed)
        capi.check(lib.otfem_set_nodes(h_chk, capi.F_EXTERNAL, fext_chk.ctypes.data_as(_dp), fext_chk.size))
        chk = OracleError(fix128)
        for step in range(1, max(chk.keep) + 1):
            capi.check(lib.otfem_simulate_ex(h_chk, w["dt"], 1, ctypes.byref(head), None))
            if chk.wants(step):
                chk.record(step, *get_xv(lib, capi, h_chk, N))
        capi.check(lib.otfem_destroy(h_chk))
        r_head["oracle_error"] = chk.result()

    # ---- the other measured configurations (outside the headline timing) ---
    extra = {}
    if not args.no_extra:
        extra["inference_ab_64x16x16"] = run_inference_ab(lib, capi, torch, stream, net, args, flush_l2)
        extra["batch"] = run_batch_workload(lib, capi, torch, stream, net, args, flush_l2)
        if "apply_sweep" in extra["batch"]:
            sw = extra["batch"]["apply_sweep"]
            sw["frac"] = sw["achieved_gbs"] / peak
            sw["peak_gbs"] = peak

    total_tet_steps = T * args.steps * world
    value = total_tet_steps / r_head["dev_s"]
    plain_value = total_tet_steps / r_plain["dev_s"]
    learned_value = total_tet_steps / r_learn["dev_s"]
    projected_value = total_tet_steps / r_proj["dev_s"]
    e2e_value = total_tet_steps / e2e_s
    e2e_staged_value = total_tet_steps / staged_s
    if rank != 0:
        return
    fix_note = ("the reference's fem::simulate pipeline in FP64, CG to rel. residual 1e-10 "
                "(tests/golden/traj_beam128.npz); x over the largest displacement, v over the largest velocity, "
                "at the sampled steps of 200 from rest; fp64_rtol1e-6: the same pipeline stopped at the GPU's "
                "tolerance, against the same run")
    line = {
        "metric": METRIC, "value": value, "unit": "tet-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * r_head["dev_s"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 element apply and CG vectors (velocity as f32 hi/lo pairs), f32-pair reductions and scalars",
        "data": "synthetic",
        "config": {"workload": WORKLOAD["name"],
                   "warm_start": "extrapolated: CG starts from v + the velocity change the polynomial of "
                                 f"degree {head.warm_history} through the last {head.warm_history + 1} velocities "
                                 "predicts (the sum of the newest change's backward differences), no extra "
                                 "element apply.  The projected start (the least-energy point on v + span{last "
                                 f"{projected.warm_history} velocity changes}}, one extra apply per direction) and "
                                 "the learned start (the trained network's correction added to that search "
                                 "space) are measured below (config.projected, config.learned) and are slower",
                   "solver": "matrix-free persistent CG (OTFEM_SOLVER_MIXED), CUDA graph per step",
                   "preconditioner": "node Jacobi (OTFEM_PRECONDITIONER_JACOBI, the default)",
                   "l2": "flushed (512 MiB write) before every timed step", "replicas": world,
                   "trajectory": f"timed steps {args.lead_in + args.warmup + 1}..{args.lead_in + args.warmup + args.steps} "
                                 f"of the beam's motion from rest (every arm), after {args.lead_in} untimed lead-in "
                                 f"and {args.warmup} warm-up steps",
                   "iterations_per_step": float(np.mean(r_head["its"])),
                   "max_rel_residual": float(np.max(r_head["res"])),
                   "plain": {"method": "CG, no preconditioner, previous-velocity start (the reference's)",
                             "value": plain_value, "unit": "tet-steps/s",
                             "ms_per_step": 1e3 * r_plain["dev_s"] / args.steps,
                             "iterations_per_step": float(np.mean(r_plain["its"])),
                             "max_rel_residual": float(np.max(r_plain["res"])),
                             "oracle_error": r_plain["oracle_error"]},
                   "projected": {"method": "CG from the least-energy point on v + span{last "
                                           f"{projected.warm_history} velocity changes}}, Jacobi PCG",
                                 "value": projected_value, "unit": "tet-steps/s",
                                 "ms_per_step": 1e3 * r_proj["dev_s"] / args.steps,
                                 "iterations_per_step": float(np.mean(r_proj["its"])),
                                 "max_rel_residual": float(np.max(r_proj["res"])),
                                 "oracle_error": r_proj["oracle_error"]},
                   "learned": {"method": "node MLP (v, dv_prev, f_ext, 1-ring mean of Re; 3x64 GELU, BF16 "
                                         "tensor cores) trained in this run on 2M (state, converged dv) pairs; its "
                                         "correction joins the last 4 velocity changes in the search space",
                               "value": learned_value, "unit": "tet-steps/s",
                               "ms_per_step": 1e3 * r_learn["dev_s"] / args.steps,
                               "iterations_per_step": float(np.mean(r_learn["its"])),
                               "learned_over_plain": learned_value / plain_value,
                               "learned_over_projected": learned_value / projected_value,
                               "oracle_error": r_learn["oracle_error"]},
                   "ablations": {k: {"value": total_tet_steps / r["dev_s"], "unit": "tet-steps/s",
                                     "ms_per_step": 1e3 * r["dev_s"] / args.steps,
                                     "iterations_per_step": float(np.mean(r["its"])),
                                     "max_rel_residual": float(np.max(r["res"])),
                                     "oracle_error": r["oracle_error"]} for k, r in ablations.items()
                                 if k not in ("learned", "projected")},
                   "extrapolated_over_plain": value / plain_value,
                   "extrapolated_over_projected": value / projected_value,
                   "projected_over_plain": projected_value / plain_value,
                   "learned_over_plain": learned_value / plain_value,
                   "learned_over_projected": learned_value / projected_value,
                   "position_difference_vs_plain": pos_diff,
                   "training": train_info,
                   "other_configurations": extra},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": "k_cg_mixed", "peak_source": peak_note,
                     "algorithmic_bytes_per_launch": float(np.mean(cg_bytes)),
                     "kernel_ms": float(np.mean(cg_ms)),
                     "apply_sweep": {"kernel": "k_apply_sweep<float>", "variant": int(variant.value),
                                     "ms": float(np.median(sweep_ms)), "algorithmic_bytes": sweep_bytes,
                                     "achieved": sweep_gbs, "frac": sweep_gbs / peak,
                                     "l2": "flushed before each sweep"}},
        "e2e": {"value": e2e_value, "unit": "tet-steps/s", "h2d_bytes_per_step": 3 * 24 * N,
                "d2h_bytes_per_step": 2 * 24 * N,
                "call": "otfem_simulate_host on page-locked host arrays: one graph per step, the velocity and "
                        "force uploads beside the orientation kernel, the two downloads at once",
                "staged": {"value": e2e_staged_value, "unit": "tet-steps/s",
                           "call": "otfem_set_nodes x3, otfem_simulate_ex, otfem_get_nodes_async x2, one wait"}},
        "oracle_error": dict(r_head["oracle_error"] or {}, reference=fix_note),
        "gpu_launches": r_head["launches"],
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        times, cits = oracle_sample(tets, coord, fixed, args.cpu_steps)
        line["cpu_baseline"] = {"value": T * len(times) / sum(times), "unit": "tet-steps/s", "cores": 1,
                                "kind": "port",
                                "sample": f"{args.cpu_steps} steps of the full workload from rest, converged CG "
                                          f"({float(np.mean(cits)):.0f} iterations/step), one host core"}
    print(json.dumps(line), flush=True)
    capi.check(lib.otfem_destroy(h_plain))
    capi.check(lib.otfem_destroy(h_head))
    net.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--lead-in", type=int, default=10,
                    help="untimed steps of the trajectory before the warm-up (the velocity history fills)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="beam128", choices=sorted(WORKLOADS))
    ap.add_argument("--train-samples", type=int, default=2_000_000)
    ap.add_argument("--train-steps", type=int, default=40)
    ap.add_argument("--train-epochs", type=int, default=60)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--ab-steps", type=int, default=500)
    ap.add_argument("--batch-meshes", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=20)
    ap.add_argument("--no-extra", action="store_true")
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
