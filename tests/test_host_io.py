"""otfem_simulate_host: one step on host arrays against the C ABI sequence it
stands for (set coord, velocity and external forces, step, get coord and
velocity), on page-locked arrays (one graph with the copies overlapped) and on
ordinary pageable arrays (the same copies, no graph); the handle's device
fields must end as after the sequence."""
import ctypes

import numpy as np
import pytest

from helpers import GpuMesh, beam, gravity_force
from opentissue_gb300 import capi

pytestmark = pytest.mark.gpu

_dp = ctypes.POINTER(ctypes.c_double)
POS_TOL = 1e-5


def _arrays(n, pinned):
    if not pinned:
        return [np.zeros((n, 3)) for _ in range(3)]
    import torch
    return [torch.zeros((n, 3), dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]


def _run(params, pinned, steps=6, dims=(12, 5, 4)):
    tets, coord, fixed = beam(*dims, jitter_seed=8)
    seq, host = GpuMesh(tets, coord, fixed), GpuMesh(tets, coord, fixed)
    seq.init()
    host.init()
    mass = seq.get(capi.MASS)
    x, v, f = _arrays(coord.shape[0], pinned)
    x[:] = coord
    v[:] = 0.0
    out = []
    for s in range(steps):
        # a load that changes every step, so the forces are really re-read
        f[:] = gravity_force(mass, fixed) * (1.0 + 0.5 * np.sin(s))
        seq.set(capi.F_EXTERNAL, f)
        seq.step(0.01, True, params)
        st = capi.StepStats()
        capi.check(host.lib.otfem_simulate_host(host.h, 0.01, 1, ctypes.byref(params), ctypes.byref(st),
                                                x.ctypes.data_as(_dp), v.ctypes.data_as(_dp), f.ctypes.data_as(_dp)))
        assert st.status == capi.OK
        # the device fields end as after the copy sequence
        assert np.array_equal(host.get(capi.COORD), x)
        assert np.array_equal(host.get(capi.VELOCITY), v)
        assert np.array_equal(host.get(capi.F_EXTERNAL), f)
        out.append((seq.get(capi.COORD), seq.get(capi.VELOCITY), x.copy(), v.copy()))
    seq.close()
    host.close()
    return coord, out


@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("warm", [capi.WARM_START_PREVIOUS, capi.WARM_START_PROJECTED,
                                  capi.WARM_START_EXTRAPOLATED])
def test_host_step_matches_the_copy_sequence(gpu, pinned, warm):
    """The matrix-free solver: positions and velocities as the copy sequence's
    (the apply's unordered float reductions make two runs differ in the last
    bits, so within the solver's accuracy bound)."""
    params = capi.default_params(solver=capi.SOLVER_MIXED, max_iterations=2000, rtol=1e-6, warm_start=warm)
    coord, out = _run(params, pinned)
    for xs, vs, xh, vh in out:
        disp = np.abs(xs - coord).max()
        assert np.abs(xh - xs).max() <= POS_TOL * disp
        assert np.abs(vh - vs).max() <= POS_TOL * np.abs(vs).max()


def test_host_step_reference_solver_is_bit_identical(gpu):
    """The reference solver (copied around the step) with ordered sums: the
    same bits as the copy sequence."""
    params = capi.default_params(sequential_dots=1)
    _, out = _run(params, True, steps=3, dims=(6, 3, 3))
    for xs, vs, xh, vh in out:
        assert np.array_equal(xs, xh) and np.array_equal(vs, vh)


def test_host_step_rejects_null_arrays(gpu):
    tets, coord, fixed = beam(4, 2, 2)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    x = coord.copy()
    rc = m.lib.otfem_simulate_host(m.h, 0.01, 1, None, None, x.ctypes.data_as(_dp), None, None)
    assert rc == capi.ERR_INVALID_ARGUMENT
    m.close()


def _pair_host_steps(seq, host, coord, fixed, params, steps, pinned, load):
    """Steps `seq` by the copy sequence and `host` by otfem_simulate_host from
    the same state; returns per step (seq x, seq v, host x, host v)."""
    x, v, f = _arrays(coord.shape[0], pinned)
    x[:] = coord
    v[:] = 0.0
    out = []
    for s in range(steps):
        f[:] = load(s)
        seq.set(capi.F_EXTERNAL, f)
        capi.check(seq.lib.otfem_simulate_ex(seq.h, 0.01, 1, ctypes.byref(params), None))
        st = capi.StepStats()
        capi.check(host.lib.otfem_simulate_host(host.h, 0.01, 1, ctypes.byref(params), ctypes.byref(st),
                                                x.ctypes.data_as(_dp), v.ctypes.data_as(_dp), f.ctypes.data_as(_dp)))
        assert np.array_equal(host.get(capi.COORD), x) and np.array_equal(host.get(capi.VELOCITY), v)
        out.append((seq.get(capi.COORD), seq.get(capi.VELOCITY), x.copy(), v.copy()))
    return out


def test_host_step_on_a_batch(gpu):
    """A batch handle (every mesh's nodes in one array), projected start."""
    from helpers import Batch
    from opentissue_gb300.workloads import random_beams
    beams = random_beams(4, seed=7, nx=(8, 12), nyz=(3, 4))
    seq, host = Batch(beams), Batch(beams)
    coord = np.concatenate([b["coord"] for b in beams])
    fixed = np.concatenate([b["fixed"] for b in beams])
    mass = seq.get(capi.MASS)
    params = capi.default_params(solver=capi.SOLVER_MIXED, max_iterations=2000, rtol=1e-6,
                                 warm_start=capi.WARM_START_PROJECTED)
    out = _pair_host_steps(seq, host, coord, fixed, params, 5, True,
                           lambda s: gravity_force(mass, fixed) * (1.0 + 0.3 * s))
    for xs, vs, xh, vh in out:
        assert np.abs(xh - xs).max() <= POS_TOL * np.abs(xs - coord).max()
        assert np.abs(vh - vs).max() <= POS_TOL * np.abs(vs).max()
    seq.close()
    host.close()


def test_host_step_with_plasticity(gpu):
    """Plasticity adds to the external forces in the orientation phase, so the
    host step copies the inputs before it: the same states as the sequence,
    and the device forces as the step left them."""
    tets, coord, fixed = beam(10, 4, 4, jitter_seed=4)
    mat = (5e5, 0.33, 1000.0, 1e-4, 50.0, 1e-2)
    seq, host = GpuMesh(tets, coord, fixed), GpuMesh(tets, coord, fixed)
    seq.init(mat)
    host.init(mat)
    mass = seq.get(capi.MASS)
    params = capi.default_params(solver=capi.SOLVER_MIXED, max_iterations=2000, rtol=1e-6)
    out = _pair_host_steps(seq, host, coord, fixed, params, 6, False, lambda s: gravity_force(mass, fixed))
    for xs, vs, xh, vh in out:
        assert np.abs(xh - xs).max() <= POS_TOL * np.abs(xs - coord).max()
        assert np.abs(vh - vs).max() <= POS_TOL * np.abs(vs).max()
    assert np.abs(host.plastic()).max() > 0
    assert np.abs(host.get(capi.F_EXTERNAL) - seq.get(capi.F_EXTERNAL)).max() <= \
        POS_TOL * np.abs(seq.get(capi.F_EXTERNAL)).max()
    seq.close()
    host.close()
