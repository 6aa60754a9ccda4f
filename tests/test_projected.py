"""Projected start (OTFEM_WARM_START_PROJECTED): CG starts from the least-energy
point of v + span{the last warm_history velocity changes}.  It changes where
CG starts, not where it stops: every step still ends at rel. residual 1e-6,
so the positions match the plain start's to that tolerance."""
import ctypes

import numpy as np
import pytest

from helpers import GpuMesh, beam, run_loaded
from opentissue_gb300 import capi

pytestmark = pytest.mark.gpu

DIMS = (24, 6, 6)
LOAD = (75.0, 2.2, (0.0, -0.8, -0.6))


def params(**kw):
    base = dict(solver=capi.SOLVER_MIXED, max_iterations=5000, rtol=1e-6)
    base.update(kw)
    return capi.default_params(**base)


def run(p, steps=40, variant=None):
    tets, coord, fixed = beam(*DIMS, jitter_seed=11)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    if variant is not None:
        capi.check(m.lib.otfem_set_apply_variant(m.h, variant))
    its, xs = run_loaded(m, DIMS, steps, p, *LOAD)
    m.close()
    return its, xs, coord


def same_positions(xs, ref, coord, tol=1e-5):
    for s, (a, b) in enumerate(zip(xs, ref)):
        disp = np.abs(b - coord).max()
        assert np.abs(a - b).max() <= tol * disp, s


def test_projected_start_same_answer_fewer_iterations(gpu):
    its0, x0, coord = run(params())
    its2, x2, _ = run(params(warm_start=capi.WARM_START_PROJECTED, warm_history=2))
    its8, x8, _ = run(params(warm_start=capi.WARM_START_PROJECTED, warm_history=8))
    same_positions(x2, x0, coord)
    same_positions(x8, x0, coord)
    # once the history has filled, each further vector cuts iterations
    plain, two, eight = its0[10:].mean(), its2[10:].mean(), its8[10:].mean()
    assert two < 0.85 * plain, (plain, two)
    assert eight < 0.5 * plain, (plain, eight)
    assert eight < two


@pytest.mark.parametrize("variant", range(capi.NUM_APPLY_VARIANTS))
def test_projected_start_every_apply_variant(gpu, variant):
    """The tets and staged variants apply A to all directions in one pass,
    the patch variants once per direction: all give the same start."""
    its0, x0, coord = run(params(), steps=16, variant=variant)
    its, x, _ = run(params(warm_start=capi.WARM_START_PROJECTED), steps=16, variant=variant)
    same_positions(x, x0, coord)
    assert its[10:].mean() < 0.7 * its0[10:].mean(), (variant, its0, its)


def test_projected_start_with_ordered_sums(gpu):
    """sequential_dots = 1: the Gram system is summed in CTA order."""
    its0, x0, coord = run(params(sequential_dots=1), steps=16)
    its, x, _ = run(params(sequential_dots=1, warm_start=capi.WARM_START_PROJECTED), steps=16)
    same_positions(x, x0, coord)
    assert its[10:].mean() < 0.7 * its0[10:].mean()


def test_history_restarts_at_init(gpu):
    """otfem_init clears the history: the first projected step after it
    starts from v, like the plain start."""
    tets, coord, fixed = beam(*DIMS, jitter_seed=11)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    p = params(warm_start=capi.WARM_START_PROJECTED)
    run_loaded(m, DIMS, 12, p, *LOAD)
    m.init()
    m.set(capi.COORD, coord)
    m.set(capi.VELOCITY, np.zeros_like(coord))
    its_a, _ = run_loaded(m, DIMS, 1, p, *LOAD)
    m.close()
    its_b, _, _ = run(params(), steps=1)
    assert abs(int(its_a[0]) - int(its_b[0])) <= 1, (its_a, its_b)


def test_projected_start_is_the_least_energy_point(gpu):
    """The kernel's start (its reported initial residual) is the FP64
    least-energy point of v + span{the last 4 velocity changes}, rebuilt on
    the host from the step's velocities, b and the library's own operator."""
    from helpers import gravity_force, tip_load
    tets, coord, fixed = beam(*DIMS, jitter_seed=11)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    mass = m.get(capi.MASS)
    free = np.repeat(fixed == 0, 3)
    p = params(warm_start=capi.WARM_START_PROJECTED, warm_history=4)
    _dp = ctypes.POINTER(ctypes.c_double)

    def apply(x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros_like(x)
        capi.check(m.lib.otfem_apply_operator(m.h, capi.SOLVER_MIXED, 0.01, 2.0, x.ctypes.data_as(_dp),
                                              y.ctypes.data_as(_dp)))
        return y.reshape(-1)[free]

    vs = [m.get(capi.VELOCITY)]
    checked = 0
    for s in range(12):
        f = gravity_force(mass, fixed) + tip_load(coord, *DIMS, LOAD[0], LOAD[1], LOAD[2], s * 0.01)
        m.set(capi.F_EXTERNAL, f)
        _, st = m.step(0.01, True, p)
        vs.append(m.get(capi.VELOCITY))
        if s < 6:
            continue
        v = vs[-2]
        W = [vs[-2 - j] - vs[-3 - j] for j in range(4)]  # the changes of the four steps before
        b = m.get(capi.B).reshape(-1)[free]
        r_v = b - apply(v)
        AW = np.stack([apply(w) for w in W], 1)
        Wf = np.stack([w.reshape(-1)[free] for w in W], 1)
        g = np.linalg.lstsq(Wf.T @ AW, Wf.T @ r_v, rcond=None)[0]
        rel = np.linalg.norm(r_v - AW @ g) / np.linalg.norm(b)
        assert np.linalg.norm(r_v) / np.linalg.norm(b) > 3 * rel  # the projection matters here
        assert abs(st.initial_rel_residual - rel) <= 0.02 * rel, (s, st.initial_rel_residual, rel)
        checked += 1
    assert checked == 6
    m.close()


def test_projected_start_with_plasticity_no_warping_and_dt_changes(gpu, oracle):
    """The projected start stops where the converged FP64 oracle does with
    plasticity active, with stiffness warping off, and when dt changes
    between steps (the history then spans changes of other step sizes)."""
    from helpers import gravity_force
    tets, coord, fixed = beam(10, 4, 4, jitter_seed=4)
    mat = (5e5, 0.33, 1000.0, 1e-4, 50.0, 1e-2)
    m = GpuMesh(tets, coord, fixed)
    m.init(mat)
    o = oracle.OracleMesh(tets, coord, coord, fixed)
    o.init(*mat)
    mass = o.get(oracle.MASS)
    p = params(warm_start=capi.WARM_START_PROJECTED)
    schedule = [(0.01, True)] * 6 + [(0.005, True)] * 3 + [(0.01, False)] * 4 + [(0.02, True)] * 3
    for dt, warp in schedule:
        f = gravity_force(mass, fixed) * 3.0
        m.set(capi.F_EXTERNAL, f)
        o.set(oracle.F_EXTERNAL, f)
        _, st = m.step(dt, warp, p)
        o.simulate_converged(dt, warp, 2.0, 1e-11, 100000)
        assert st.status == capi.OK and st.rel_residual <= 1e-6
        x, xo = m.get(capi.COORD), o.get(oracle.COORD)
        assert np.abs(x - xo).max() <= 1e-5 * np.abs(xo - coord).max(), (dt, warp)
    assert np.abs(m.plastic()).max() > 0
    o.close()
    m.close()


def test_projected_start_parameter_checks(gpu):
    tets, coord, fixed = beam(3, 2, 2)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    rc, _ = m.step(0.01, True, params(warm_start=capi.WARM_START_PROJECTED, warm_history=0), check=False)
    assert rc == capi.ERR_INVALID_ARGUMENT
    rc, _ = m.step(0.01, True, params(warm_start=capi.WARM_START_PROJECTED, warm_history=9), check=False)
    assert rc == capi.ERR_INVALID_ARGUMENT
    rc, _ = m.step(0.01, True, params(solver=capi.SOLVER_FP64, warm_start=capi.WARM_START_PROJECTED), check=False)
    assert rc == capi.ERR_UNSUPPORTED
    rc, _ = m.step(0.01, True, params(warm_start=4), check=False)
    assert rc == capi.ERR_INVALID_ARGUMENT
    m.close()


def test_solver_phases_record_the_start(gpu):
    """otfem_solver_phases: five ordered stamps for every mixed solve, and for
    the projected start three more (Gram sums begun, totals in, coefficients
    solved) between the start sweeps and the start; zeros otherwise."""
    tets, coord, fixed = beam(*DIMS, jitter_seed=11)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    dp = ctypes.POINTER(ctypes.c_double)
    ph = np.zeros(8)
    for warm in (capi.WARM_START_PREVIOUS, capi.WARM_START_PROJECTED, capi.WARM_START_PREVIOUS):
        run_loaded(m, DIMS, 3, params(warm_start=warm), *LOAD)
        capi.check(m.lib.otfem_solver_phases(m.h, ph.ctypes.data_as(dp)))
        assert np.all(np.diff(ph[:5]) > 0) and ph[0] > 0, ph
        if warm == capi.WARM_START_PROJECTED:
            assert ph[1] < ph[5] < ph[6] < ph[7] < ph[2], ph
        else:
            assert np.all(ph[5:] == 0), ph
    m.close()
