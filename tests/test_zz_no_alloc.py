"""otfem_apply_operator_noalloc: the operator apply with its scratch in the
library's static device array, checked against otfem_apply_operator (which
allocates) on two calls in a row, through the C ABI, for every element-apply
variant and for a batch handle; and its argument checks (node limit, host
pointers, the set-up-only call)."""
import ctypes

import numpy as np
import pytest

from helpers import GpuMesh, MATERIAL, beam, gravity_force
from opentissue_gb300 import capi
from opentissue_gb300.fem import generate_blocks

pytestmark = pytest.mark.gpu

_dp = ctypes.POINTER(ctypes.c_double)
MAX_NODES = 1 << 18


def _noalloc(m, solver, dt, damping, x):
    import torch
    xd = torch.from_numpy(np.ascontiguousarray(x)).to("cuda:0")
    yd = torch.full_like(xd, float("nan"))
    torch.cuda.synchronize()  # x is written on torch's stream; the library uses the handle's
    capi.check(m.lib.otfem_apply_operator_noalloc(m.h, solver, dt, damping, ctypes.c_void_p(xd.data_ptr()),
                                                  ctypes.c_void_p(yd.data_ptr())))
    capi.check(m.lib.otfem_synchronize(m.h))
    return yd.cpu().numpy()


def _allocating(m, solver, dt, damping, x):
    y = np.zeros_like(x)
    capi.check(m.lib.otfem_apply_operator(m.h, solver, dt, damping, x.ctypes.data_as(_dp), y.ctypes.data_as(_dp)))
    return y


def _compare(m, fixed, solver, tol):
    dt, damping = 0.01, 2.0
    p = capi.default_params(solver=solver, max_iterations=2000, rtol=1e-6)
    capi.check(m.lib.otfem_simulate_phase(m.h, dt, 1, ctypes.byref(p), capi.PHASE_ORIENT))
    rng = np.random.default_rng(11)
    # two calls in a row: the second must not see the first call's scratch
    for scale in (1.0, 1e-3):
        x = scale * rng.normal(size=(m.N, 3))
        want = _allocating(m, solver, dt, damping, x)
        got = _noalloc(m, solver, dt, damping, x)
        assert np.isfinite(got).all()
        assert np.abs(got - want).max() <= tol * np.abs(want).max()
        assert (got[fixed == 1] == 0).all()


# every element-apply variant (0, 1: patches; 2: one tet per thread; 3: tiles
# staged by bulk copies, which the FP64 solver runs as 2), forced as the
# autotuner would pick it
@pytest.mark.parametrize("variant", [0, 1, 2, 3])
@pytest.mark.parametrize("solver,tol", [(capi.SOLVER_MIXED, 2e-6), (capi.SOLVER_FP64, 1e-13)])
def test_noalloc_matches_apply_operator(gpu, solver, tol, variant):
    tets, coord, fixed = beam(12, 5, 4, jitter_seed=6)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    capi.check(m.lib.otfem_set_apply_variant(m.h, variant))
    m.set(capi.F_EXTERNAL, gravity_force(m.get(capi.MASS), fixed))
    _compare(m, fixed, solver, tol)
    m.close()


def test_noalloc_matches_apply_operator_on_a_batch(gpu):
    """A batch handle (its node count is every mesh's nodes)."""
    from helpers import Batch
    from opentissue_gb300.workloads import random_beams
    beams = random_beams(3, seed=41, nx=(8, 12), nyz=(3, 4))
    b = Batch(beams)
    b.set(capi.F_EXTERNAL, np.zeros((b.N, 3)))
    fixed = np.concatenate([bm["fixed"] for bm in beams])
    _compare(b, fixed, capi.SOLVER_MIXED, 2e-6)
    b.close()


def test_noalloc_setup_call_and_pointer_checks(gpu):
    """x = y = NULL runs only the per-device set-up; host pointers are refused
    before any kernel runs."""
    tets, coord, fixed = beam(6, 3, 3, jitter_seed=2)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    capi.check(m.lib.otfem_apply_operator_noalloc(m.h, capi.SOLVER_MIXED, 0.01, 2.0, None, None))
    x = np.ones((m.N, 3))
    y = np.zeros((m.N, 3))
    rc = m.lib.otfem_apply_operator_noalloc(m.h, capi.SOLVER_MIXED, 0.01, 2.0, ctypes.c_void_p(x.ctypes.data),
                                            ctypes.c_void_p(y.ctypes.data))
    assert rc == capi.ERR_INVALID_ARGUMENT
    assert (y == 0).all()
    m.close()


def test_noalloc_rejects_meshes_above_its_limit(gpu):
    tets, coord = generate_blocks(64, 64, 64, 0.1, 0.1, 0.1)  # 65^3 = 274,625 nodes
    assert coord.shape[0] > MAX_NODES
    m = GpuMesh(tets, coord)
    m.init(MATERIAL)
    import torch
    # real buffers of the mesh's size; FP32 scratch for this mesh (48 B/node)
    # would still fit the array, so even a missing check stays in bounds
    xd = torch.zeros((m.N, 3), dtype=torch.float64, device="cuda:0")
    yd = torch.zeros_like(xd)
    torch.cuda.synchronize()
    rc = m.lib.otfem_apply_operator_noalloc(m.h, capi.SOLVER_MIXED, 0.01, 0.0, ctypes.c_void_p(xd.data_ptr()),
                                            ctypes.c_void_p(yd.data_ptr()))
    capi.check(m.lib.otfem_synchronize(m.h))
    assert rc == capi.ERR_INVALID_ARGUMENT
    assert b"262144" in m.lib.otfem_last_error()
    m.close()
