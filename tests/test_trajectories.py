"""Every warm start of the matrix-free solver against the reference's FP64
trajectories: positions AND velocities, per configuration, over the whole
run.

The fixtures (tests/golden/traj_*.npz) come from the reference's own
fem::simulate pipeline (fem_simulate.h:94-111, position update
fem_position_update.h:25-39) built from its unmodified headers, with the CG
run to relative residual 1e-10 (tests/golden/make_trajectories.py).  The GPU
runs stop at relative residual 1e-6, as the benchmark does.  Errors at every
sampled step: |x - x_ref| over the step's largest displacement and
|v - v_ref| over its largest velocity (all nodes).  The FP64 reference
pipeline itself, stopped at the same 1e-6, is not within 1e-5 everywhere
(the fixtures store its run at 1e-6 too: on the 64x16x16 beam it is 1.3e-5
off in x and v at step 1 and 2.4e-3 in v at step 250; on the batch beams up
to 5.7e-5 in x and v at step 1): what a solver stopped at 1e-6 can promise.
The bound per step is therefore max(1e-5, F x the FP64 pipeline's own error
at 1e-6), F = 3 for x and 10 for v: the GPU solver stays within the band the
reference run in FP64 spans with the same stopping rule, and within 1e-5
wherever that band is narrower.  (The factor covers that the arms stop
elsewhere than the reference's plain CG: preconditioned and warm-started
solves leave their 1e-6 residual in other components, and the velocity
errors of solves stopped at 1e-6 -- the largest over the nodes, relative to
the largest velocity -- differ by a few times between methods and, for the
warm starts, from run to run (the apply's float reductions are unordered);
measured up to 1.9x in x and 5.1x in v.)

  * 128x32x32 jittered beam under gravity, 200 steps (steps 1, 50, 100, 200)
  * 64x16x16 jittered beam under gravity and the seeded sinusoidal tip load,
    500 steps (steps 1, 100, 250, 500)
  * eight beams of the 256-beam batch (the five stiffest, E 4.6e6..5e6 Pa,
    and three others) stepped as one batch, dt 0.005, under a constant and
    under a sinusoidal tip force, 40 steps (steps 1, 20, 40; 256 sampled
    nodes per beam)
Arms: plain CG (the reference's method: no preconditioner, previous-velocity
start), Jacobi PCG, the projected start, the extrapolated start (degree 4)
and the learned start (a network trained here on other beams of the same
family).
"""
import ctypes

import numpy as np
import pytest

from helpers import Batch, GpuMesh, golden
from opentissue_gb300 import capi
from opentissue_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

TOL = 1e-5
X_FACTOR = 3.0
V_FACTOR = 10.0
ARMS = {
    "plain_cg": dict(preconditioner=capi.PRECONDITIONER_NONE),
    "jacobi": dict(),
    "projected": dict(warm_start=capi.WARM_START_PROJECTED),
    "extrapolated": dict(warm_start=capi.WARM_START_EXTRAPOLATED, warm_history=4),
    "learned": dict(warm_start=capi.WARM_START_LEARNED),
}


def params(arm):
    return capi.default_params(solver=capi.SOLVER_MIXED, max_iterations=5000, rtol=1e-6, **ARMS[arm])


@pytest.fixture(scope="module")
def net(gpu):
    """The learned start's network, trained on the GPU on plain-solver steps
    of two 64x16x16 beams of the workload family (other jitter seeds; gravity
    alone, and gravity plus a sinusoidal tip load of another seed)."""
    from opentissue_gb300.warmstart import WarmStartNet
    n = WarmStartNet(capacity=1 << 20, seed=5)
    p = params("jacobi")
    for seed, load_seed in ((101, None), (102, 103)):
        tets, coord, fixed = wl.jittered_beam(64, 16, 16, seed)
        load = wl.SineTip(64, 16, 16, load_seed) if load_seed else None
        m = GpuMesh(tets, coord, fixed)
        m.init()
        WarmStartNet.collect(m.h)
        g = wl.gravity(m.get(capi.MASS), fixed)
        for k in range(40):
            m.set(capi.F_EXTERNAL, g + (load.force(k, 0.01) if load else 0.0))
            m.step(0.01, True, p)
            n.add_samples(m.h, fraction=0.5, seed=k)
        m.close()
    n.fit_normalization()
    n.train(30, batch=8192, lr=1e-3, seed=7)
    yield n
    n.close()


def step_errors(fix, s, x, v, sample):
    """(x error, v error, the FP64 pipeline's x and v errors at 1e-6)."""
    xr, vr = fix[f"x_{s}"], fix[f"v_{s}"]
    ex = np.abs(x[sample] - xr).max() / float(fix[f"disp_{s}"])
    ev = np.abs(v[sample] - vr).max() / float(fix[f"vmax_{s}"])
    return ex, ev, float(fix[f"rtol6_x_err_{s}"]), float(fix[f"rtol6_v_err_{s}"])


def check(errs, tag):
    """errs: {step: (x error, v error, FP64@1e-6 x error, FP64@1e-6 v error)}."""
    print(tag, " ".join(f"s{s}: x {e[0]:.2e} (fp64@1e-6 {e[2]:.1e}) v {e[1]:.2e} (fp64@1e-6 {e[3]:.1e})"
                        for s, e in sorted(errs.items())))
    bad = {s: e for s, e in errs.items()
           if not (e[0] <= max(TOL, X_FACTOR * e[2]) and e[1] <= max(TOL, V_FACTOR * e[3]))}
    assert not bad, (tag, bad)


def run_single(name, cfg, forces, arm, net):
    fix = golden(name)
    tets, coord, fixed = wl.jittered_beam(cfg["I"], cfg["J"], cfg["K"], cfg["seed"])
    m = GpuMesh(tets, coord, fixed)
    m.init()
    if arm == "learned":
        net.attach(m.h)
    mass = m.get(capi.MASS)
    keep = set(int(s) for s in fix["keep"])
    p = params(arm)
    errs, its = {}, []
    for k in range(int(fix["steps"])):
        m.set(capi.F_EXTERNAL, forces(k, mass, fixed))
        _, st = m.step(cfg["dt"], True, p)
        assert st.status == capi.OK and st.rel_residual <= 1e-6, (arm, k, st.status, st.rel_residual)
        its.append(st.iterations)
        if k + 1 in keep:
            errs[k + 1] = step_errors(fix, k + 1, m.get(capi.COORD), m.get(capi.VELOCITY), fix["sample"])
    if arm == "learned":
        net.detach(m.h)
    m.close()
    check(errs, f"{name} {arm} ({np.mean(its):.1f} it/step)")


@pytest.mark.parametrize("arm", list(ARMS))
def test_beam128_200_steps_against_the_reference(arm, net):
    cfg = wl.BEAM128
    run_single("traj_beam128", cfg, lambda k, mass, fixed: wl.gravity(mass, fixed), arm, net)


@pytest.mark.parametrize("arm", list(ARMS))
def test_beam64_sine_500_steps_against_the_reference(arm, net):
    cfg = wl.BEAM64_SINE
    load = wl.SineTip(cfg["I"], cfg["J"], cfg["K"], cfg["load_seed"])
    run_single("traj_beam64_sine", cfg, lambda k, mass, fixed: wl.gravity(mass, fixed) + load.force(k, cfg["dt"]),
               arm, net)


@pytest.mark.parametrize("sine", [False, True], ids=["const", "sine"])
@pytest.mark.parametrize("arm", list(ARMS))
def test_batch_beams_against_the_reference(arm, sine, net):
    fix = golden("traj_batch")
    cfg = wl.BATCH
    pick = [int(i) for i in fix["beams"]]
    all_beams = wl.random_beams(cfg["count"], seed=cfg["seed"])
    beams = [all_beams[i] for i in pick]
    freqs = wl.batch_tip_frequencies(cfg["count"])[pick]
    b = Batch(beams)
    if arm == "learned":
        net.attach(b.h)
    mass = b.get(capi.MASS)
    keep = [int(s) for s in fix["keep"]]
    p = params(arm)
    tag = "sine" if sine else "const"
    errs = {}
    for k in range(max(keep)):
        b.set(capi.F_EXTERNAL, wl.batch_forces(beams, mass, k, cfg["dt"], sine, freqs))
        st = capi.StepStats()
        capi.check(b.lib.otfem_simulate_ex(b.h, cfg["dt"], 1, ctypes.byref(p), ctypes.byref(st)))
        its, status, rel, _ = b.stats()
        assert np.all(status == capi.OK) and np.all(rel <= 1e-6), (arm, k, status, rel)
        if k + 1 in keep:
            xs, vs = b.per_mesh(b.get(capi.COORD)), b.per_mesh(b.get(capi.VELOCITY))
            for j, i in enumerate(pick):
                pre, smp = f"b{i}_{tag}_", fix[f"b{i}_sample"]
                xr, vr = fix[f"{pre}x_{k + 1}"], fix[f"{pre}v_{k + 1}"]
                disp, vmax = float(fix[f"{pre}disp_{k + 1}"]), float(fix[f"{pre}vmax_{k + 1}"])
                errs[(k + 1, i)] = (np.abs(xs[j][smp] - xr).max() / disp, np.abs(vs[j][smp] - vr).max() / vmax,
                                    float(fix[f"{pre}rtol6_x_err_{k + 1}"]), float(fix[f"{pre}rtol6_v_err_{k + 1}"]))
    if arm == "learned":
        net.detach(b.h)
    b.close()
    check(errs, f"batch {tag} {arm}")
