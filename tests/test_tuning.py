"""The element-apply autotuner: a search over the apply variants and the
tile sizes at otfem_init (otfem_tuning_search), on a small beam and on the
128x32x32 workload beam.  Every measured shape computes the same operator
(against the FP64 element apply), the kept shape is the fastest measured,
and the steps with it still meet the oracle's positions."""
import ctypes

import numpy as np
import pytest

from helpers import GpuMesh, beam, golden, gravity_force, run_gpu
from opentissue_gb300 import capi

pytestmark = pytest.mark.gpu

_dp = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int32)


def search(m):
    rows = ctypes.c_int32()
    v = np.zeros(16, np.int32)
    tt = np.zeros(16, np.int32)
    ms = np.zeros(16)
    chosen = ctypes.c_int32()
    capi.check(m.lib.otfem_tuning_search(m.h, 16, ctypes.byref(rows), v.ctypes.data_as(_i32p),
                                         tt.ctypes.data_as(_i32p), ms.ctypes.data_as(_dp), ctypes.byref(chosen)))
    n = rows.value
    variant = ctypes.c_int32()
    capi.check(m.lib.otfem_tuning(m.h, ctypes.byref(variant), None))
    return v[:n], tt[:n], ms[:n], variant.value, chosen.value


def apply(m, solver, x):
    y = np.zeros_like(x)
    capi.check(m.lib.otfem_apply_operator(m.h, solver, 0.01, 2.0, x.ctypes.data_as(_dp), y.ctypes.data_as(_dp)))
    return y


@pytest.mark.parametrize("dims", [(12, 5, 4), (128, 32, 32)], ids=["beam12x5x4", "beam128x32x32"])
def test_search_covers_the_shapes_and_keeps_the_fastest(gpu, dims):
    tets, coord, fixed = beam(*dims, jitter_seed=20261203)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    v, tt, ms, variant, chosen = search(m)
    # patch variants once, the tiled variants at each candidate tile size
    assert list(v[:2]) == [0, 1] and list(tt[:2]) == [0, 0]
    cands = sorted(set(tt[2:].tolist()))
    assert {128, 256, 512, 1024} <= set(cands) and all(t % 16 == 0 and 16 <= t <= 1024 for t in cands)
    assert len(v) == 2 + 2 * len(cands) and np.all(ms > 0)
    k = int(np.argmin(ms))
    assert variant == v[k] and (v[k] < 2 or chosen == tt[k]), (v, tt, ms, variant, chosen)
    print(dims, "kept variant", variant, "tile", chosen, dict(zip(zip(v.tolist(), tt.tolist()), ms.round(4))))
    # every shape computes the same operator: after one step, the FP64
    # orientation phase sets the rotations every apply reads (FP64 and FP32
    # copies and the tiles' quaternions), and the FP64 element apply is the
    # reference
    m.set(capi.F_EXTERNAL, gravity_force(m.get(capi.MASS), fixed))
    p = capi.default_params(solver=capi.SOLVER_MIXED, max_iterations=2000, rtol=1e-6)
    m.step(0.01, True, p)
    p64 = capi.default_params(solver=capi.SOLVER_FP64, max_iterations=2000, rtol=1e-6)
    capi.check(m.lib.otfem_simulate_phase(m.h, 0.01, 1, ctypes.byref(p64), capi.PHASE_ORIENT))
    x = np.random.default_rng(4).normal(size=(m.N, 3))
    ref = apply(m, capi.SOLVER_FP64, x)
    for vv, t in zip(v, tt):
        capi.check(m.lib.otfem_set_apply_shape(m.h, int(vv), int(t)))
        y = apply(m, capi.SOLVER_MIXED, x)
        assert np.abs(y - ref).max() <= 2e-6 * np.abs(ref).max(), (vv, t)
    m.close()


def test_kept_shapes_meet_the_oracle(gpu):
    """Both meshes step with their kept shapes within 1e-5 of the reference's
    converged trajectories (the 16x6x6 golden run; the 128x32x32 run of
    tests/golden/large.npz)."""
    g = golden("converged")
    _, out = run_gpu(g["tets"], g["coord"], g["fixed"], 5,
                     params=capi.default_params(solver=capi.SOLVER_MIXED, max_iterations=2000, rtol=1e-6))
    x = out[4][0]
    assert np.abs(x - g["x_5"]).max() <= 1e-5 * np.abs(g["x_5"] - g["coord"]).max()
    lg = golden("large")
    tets, coord, fixed = beam(128, 32, 32, jitter_seed=20261203)
    _, out = run_gpu(tets, coord, fixed, 3, record=(3,),
                     params=capi.default_params(solver=capi.SOLVER_MIXED, max_iterations=2000, rtol=1e-6))
    x = out[2][0][lg["sample"]]
    assert np.abs(x - lg["x_3"]).max() <= 1e-5 * np.abs(lg["x_3"] - coord[lg["sample"]]).max()


def test_set_apply_shape_rejects_other_tile_sizes(gpu):
    tets, coord, fixed = beam(6, 3, 3)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    assert m.lib.otfem_set_apply_shape(m.h, 2, 100) == capi.ERR_INVALID_ARGUMENT
    capi.check(m.lib.otfem_set_apply_shape(m.h, 2, 128))
    m.close()
