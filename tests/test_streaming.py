"""Sweeps of a mesh whose tiles do not fit in L2: the tile words stream past
L1 with an L2 evict-first policy and the warps claim 32-tet chunks from a
per-CTA counter.  The operator they apply, y = A x, must equal the FP64
operator's (which reads no tiles) to FP32 accuracy, for two operands in a
row, and a solve on the mesh must reach the tolerance."""
import ctypes

import numpy as np
import pytest

from helpers import GpuMesh, beam, gravity_force
from opentissue_gb300 import capi

pytestmark = pytest.mark.gpu

_dp = ctypes.POINTER(ctypes.c_double)
TILE_BYTES_PER_TET = 80


def _apply(m, solver, x):
    y = np.zeros_like(x)
    capi.check(m.lib.otfem_apply_operator(m.h, solver, 0.01, 2.0, x.ctypes.data_as(_dp), y.ctypes.data_as(_dp)))
    return y


def test_streamed_sweeps_apply_the_operator(gpu):
    import torch
    tets, coord, fixed = beam(160, 48, 48, jitter_seed=12)
    l2 = torch.cuda.get_device_properties(0).L2_cache_size
    assert tets.shape[0] * TILE_BYTES_PER_TET > l2, "the mesh's tiles must exceed L2"
    m = GpuMesh(tets, coord, fixed)
    m.init()
    capi.check(m.lib.otfem_set_apply_variant(m.h, 2))
    # rotated elements: a smooth displacement field, then the FP64
    # orientation phase, which sets the rotations every apply reads (the FP64
    # and FP32 copies and the tiles' quaternions)
    rng = np.random.default_rng(5)
    moved = coord + 0.02 * np.sin(coord[:, [1, 2, 0]] * 7.0) * (fixed == 0)[:, None]
    m.set(capi.COORD, moved)
    p64 = capi.default_params(solver=capi.SOLVER_FP64, max_iterations=2000, rtol=1e-6)
    capi.check(m.lib.otfem_simulate_phase(m.h, 0.01, 1, ctypes.byref(p64), capi.PHASE_ORIENT))
    for scale in (1.0, 1e-3):
        x = scale * rng.normal(size=(m.N, 3))
        y32 = _apply(m, capi.SOLVER_MIXED, x)
        y64 = _apply(m, capi.SOLVER_FP64, x)
        assert np.isfinite(y32).all()
        assert np.abs(y32 - y64).max() <= 2e-6 * np.abs(y64).max()
    # one matrix-free step on the streamed mesh reaches the tolerance
    p = capi.default_params(solver=capi.SOLVER_MIXED, max_iterations=2000, rtol=1e-6)
    m.set(capi.COORD, coord)
    m.set(capi.F_EXTERNAL, gravity_force(m.get(capi.MASS), fixed))
    _, st = m.step(0.01, True, p)
    assert st.status == capi.OK and st.rel_residual <= 1e-6
    m.close()
