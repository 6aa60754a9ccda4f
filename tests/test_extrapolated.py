"""Extrapolated start (OTFEM_WARM_START_EXTRAPOLATED): CG starts from v plus
the velocity change the polynomial of degree warm_history through the last
velocities predicts (the sum of the newest change's backward differences).
It changes where CG starts, not where it stops: every step still ends at rel.
residual 1e-6, so the positions match the plain start's to that tolerance.
The degree is lowered while the history holds fewer recorded steps: after
otfem_init, and after a step that records no velocity change (an FP64-solver
step), the start is the previous velocity's and then rises again."""
import numpy as np
import pytest

from helpers import GpuMesh, beam, gravity_force, run_loaded
from opentissue_gb300 import capi

pytestmark = pytest.mark.gpu

DIMS = (24, 6, 6)
LOAD = (75.0, 2.2, (0.0, -0.8, -0.6))
EXTRAP = capi.WARM_START_EXTRAPOLATED


def params(**kw):
    base = dict(solver=capi.SOLVER_MIXED, max_iterations=5000, rtol=1e-6)
    base.update(kw)
    return capi.default_params(**base)


def run(p, steps=40):
    tets, coord, fixed = beam(*DIMS, jitter_seed=11)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    its, xs = run_loaded(m, DIMS, steps, p, *LOAD)
    m.close()
    return its, xs, coord


def test_extrapolated_start_same_answer_fewer_iterations(gpu):
    its0, x0, coord = run(params())
    its4, x4, _ = run(params(warm_start=EXTRAP, warm_history=4))
    itsp, _, _ = run(params(warm_start=capi.WARM_START_PROJECTED, warm_history=4))
    for s, (a, b) in enumerate(zip(x4, x0)):
        assert np.abs(a - b).max() <= 1e-5 * np.abs(b - coord).max(), s
    # the first step has no history: both start from the previous velocity
    assert abs(int(its4[0]) - int(its0[0])) <= 1, (its4[0], its0[0])
    plain, ext, proj = its0[10:].mean(), its4[10:].mean(), itsp[10:].mean()
    print(f"iterations per step, steps 11-40: previous {plain:.2f}, extrapolated {ext:.2f}, projected {proj:.2f}")
    assert ext < 0.6 * plain, (plain, ext)


def _probe(m, f, p):
    """One step from the mesh's current state with params p, and the same
    step from the same state with the previous-velocity start: their initial
    relative residuals (the state is put back between them)."""
    x, v = m.get(capi.COORD), m.get(capi.VELOCITY)
    m.set(capi.F_EXTERNAL, f)
    _, st = m.step(0.01, True, p)
    m.set(capi.COORD, x)
    m.set(capi.VELOCITY, v)
    _, st0 = m.step(0.01, True, params())
    return st.initial_rel_residual, st0.initial_rel_residual


def test_extrapolated_start_degree_follows_the_history(gpu):
    tets, coord, fixed = beam(*DIMS, jitter_seed=11)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    p4 = params(warm_start=EXTRAP, warm_history=4)
    f = gravity_force(m.get(capi.MASS), fixed)
    for _ in range(12):
        m.set(capi.F_EXTERNAL, f)
        m.step(0.01, True, p4)
    ext, prev = _probe(m, f, p4)
    assert ext < 0.1 * prev, (ext, prev)
    # an FP64-solver step records no velocity change: the next extrapolated
    # step starts from the previous velocity
    m.set(capi.F_EXTERNAL, f)
    m.step(0.01, True, params(solver=capi.SOLVER_FP64))
    ext, prev = _probe(m, f, p4)
    assert abs(ext - prev) <= 1e-3 * prev, (ext, prev)
    # and the degree rises with the steps recorded since (five steps: the
    # four levels then hold differences of steps recorded after the probe,
    # whose two steps from one state are no trajectory)
    for _ in range(5):
        m.set(capi.F_EXTERNAL, f)
        m.step(0.01, True, p4)
    ext, prev = _probe(m, f, p4)
    assert ext < 0.3 * prev, (ext, prev)
    m.close()


def test_extrapolated_start_parameter_checks(gpu):
    tets, coord, fixed = beam(3, 2, 2)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    rc, _ = m.step(0.01, True, params(warm_start=EXTRAP, warm_history=0), check=False)
    assert rc == capi.ERR_INVALID_ARGUMENT
    rc, _ = m.step(0.01, True, params(warm_start=EXTRAP, warm_history=9), check=False)
    assert rc == capi.ERR_INVALID_ARGUMENT
    rc, _ = m.step(0.01, True, params(solver=capi.SOLVER_FP64, warm_start=EXTRAP), check=False)
    assert rc == capi.ERR_UNSUPPORTED
    m.close()


def test_extrapolated_start_after_a_velocity_reset(gpu):
    """An abrupt change of the motion (the velocities set to zero by hand)
    leaves the history predicting the old motion: the start is poor, and the
    step still ends at the answer a mesh without history gives from the
    same state."""
    tets, coord, fixed = beam(*DIMS, jitter_seed=11)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    p4 = params(warm_start=EXTRAP, warm_history=4)
    f = gravity_force(m.get(capi.MASS), fixed)
    for _ in range(10):
        m.set(capi.F_EXTERNAL, f)
        m.step(0.01, True, p4)
    x = m.get(capi.COORD)
    zero = np.zeros_like(x)
    m.set(capi.VELOCITY, zero)
    _, st = m.step(0.01, True, p4)
    assert st.status == capi.OK and st.rel_residual <= 1e-6
    fresh = GpuMesh(tets, coord, fixed)
    fresh.init()
    fresh.set(capi.COORD, x)
    fresh.set(capi.VELOCITY, zero)
    fresh.set(capi.F_EXTERNAL, f)
    _, st0 = fresh.step(0.01, True, params())
    v, v0 = m.get(capi.VELOCITY), fresh.get(capi.VELOCITY)
    assert np.abs(v - v0).max() <= 1e-5 * np.abs(v0).max(), np.abs(v - v0).max() / np.abs(v0).max()
    print(f"after the reset: extrapolated start {st.iterations} iterations "
          f"(start rel. residual {st.initial_rel_residual:.2e}), previous velocity {st0.iterations} "
          f"({st0.initial_rel_residual:.2e})")
    m.close()
    fresh.close()
