"""The matrix-free solver (FP32 element apply, float-pair CG) against the
reference's relative-residual runs.  Tolerance from the target: position
error below 1e-5 relative to the FP64 oracle, measured here against the
largest displacement of the step (stricter than relative to the positions),
true relative residual <= rtol = 1e-6."""
import ctypes

import numpy as np
import pytest

from helpers import MATERIAL, GpuMesh, beam, golden, gravity_force, run_gpu, run_oracle
from opentissue_gb300 import capi

pytestmark = pytest.mark.gpu

POS_TOL = 1e-5


def mixed(**kw):
    base = dict(solver=capi.SOLVER_MIXED, max_iterations=2000, rtol=1e-6)
    base.update(kw)
    return capi.default_params(**base)


def rel_pos_err(x, x_ref, x_init):
    disp = np.abs(x_ref - x_init).max()
    return np.abs(x - x_ref).max() / max(disp, 1e-300)


def test_mixed_vs_reference_converged_golden(gpu):
    """Plain CG (the reference's method) takes the reference's iteration
    counts; the Jacobi-preconditioned default reaches the same positions."""
    g = golden("converged")
    _, out = run_gpu(g["tets"], g["coord"], g["fixed"], 20, params=mixed(preconditioner=capi.PRECONDITIONER_NONE))
    for s in (1, 5, 20):
        x, v, st = out[s - 1]
        err = rel_pos_err(x, g[f"x_{s}"], g["coord"])
        assert err < POS_TOL, (s, err)
    for (_, _, st), it_ref in zip(out, g["iterations"]):
        assert st.status == capi.OK
        assert st.rel_residual <= 1e-6
        assert abs(st.iterations - int(it_ref)) <= max(6, 0.2 * it_ref)
    _, outp = run_gpu(g["tets"], g["coord"], g["fixed"], 20, params=mixed())
    for s in (1, 5, 20):
        assert rel_pos_err(outp[s - 1][0], g[f"x_{s}"], g["coord"]) < POS_TOL, s
    for _, _, st in outp:
        assert st.status == capi.OK and st.rel_residual <= 1e-6


def test_node_stiffness_is_the_trace_of_the_assembled_diagonal(gpu, oracle):
    """OTFEM_NODE_STIFFNESS = tr(K_ii) / 3 of the oracle's assembled
    (rotated) stiffness matrix, for every node."""
    tets, coord, fixed = beam(6, 3, 4, jitter_seed=5)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    k = m.get(capi.NODE_STIFFNESS)
    o = oracle.OracleMesh(tets, coord, coord, fixed)
    o.init(*MATERIAL)
    mass = o.get(oracle.MASS)
    for _ in range(2):  # non-identity orientations in the assembled K
        o.set(oracle.F_EXTERNAL, gravity_force(mass, fixed) * 50.0)
        o.simulate(0.01, True)
    rp, cols = o.k_pattern()
    K = o.k_values()
    diag = np.array([K[q] for i in range(len(rp) - 1) for q in range(rp[i], rp[i + 1]) if cols[q] == i])
    ref = np.trace(diag, axis1=1, axis2=2) / 3.0
    assert np.allclose(k, ref, rtol=1e-10, atol=0.0)
    o.close()
    m.close()


@pytest.mark.parametrize("solver", [capi.SOLVER_MIXED, capi.SOLVER_FP64])
def test_jacobi_preconditioner_same_answer_fewer_iterations(gpu, oracle, solver):
    tets, coord, fixed = beam(24, 6, 6, jitter_seed=9)
    _, ref = run_oracle(oracle, tets, coord, fixed, 4, converged=True, rtol=1e-11)
    its = {}
    for pre in (capi.PRECONDITIONER_NONE, capi.PRECONDITIONER_JACOBI):
        _, out = run_gpu(tets, coord, fixed, 4, params=mixed(solver=solver, preconditioner=pre))
        for s in range(4):
            x, _, st = out[s]
            assert st.status == capi.OK and st.rel_residual <= 1e-6
            assert rel_pos_err(x, ref[s][0], coord) < POS_TOL, (pre, s)
        its[pre] = np.mean([st.iterations for _, _, st in out])
    assert its[capi.PRECONDITIONER_JACOBI] < 0.85 * its[capi.PRECONDITIONER_NONE], its


def test_unknown_preconditioner_is_rejected(gpu):
    tets, coord, fixed = beam(3, 2, 2)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    rc, _ = m.step(0.01, True, mixed(preconditioner=7), check=False)
    assert rc == capi.ERR_INVALID_ARGUMENT
    m.close()


def test_fp64_matrix_free_vs_reference(gpu):
    """Plain CG in FP64 follows the reference's CG iterates: both stop at
    rel. residual 1e-6 on nearly the same iterate."""
    g = golden("converged")
    _, out = run_gpu(g["tets"], g["coord"], g["fixed"], 5,
                     params=mixed(solver=capi.SOLVER_FP64, preconditioner=capi.PRECONDITIONER_NONE))
    x, v, st = out[4]
    assert rel_pos_err(x, g["x_5"], g["coord"]) < 1e-7
    assert st.rel_residual <= 1e-6


def test_mixed_large_mesh_golden(gpu):
    g = golden("large")
    tets, coord, fixed = beam(int(g["I"]), int(g["J"]), int(g["K"]), jitter_seed=int(g["seed"]))
    m, out = run_gpu(tets, coord, fixed, 3, params=mixed())
    sample = g["sample"]
    for s in (1, 2, 3):
        x, v, st = out[s - 1]
        err = rel_pos_err(x[sample], g[f"x_{s}"], coord[sample])
        assert err < POS_TOL, (s, err)
        assert st.rel_residual <= 1e-6 and st.status == capi.OK


def test_mixed_plasticity_vs_oracle(gpu, oracle):
    tets, coord, fixed = beam(10, 4, 4, jitter_seed=4)
    mat = (5e5, 0.33, 1000.0, 1e-4, 50.0, 1e-2)
    m, out = run_gpu(tets, coord, fixed, 15, params=mixed(), material=mat)
    _, ref = run_oracle(oracle, tets, coord, fixed, 15, material=mat, converged=True, rtol=1e-6)
    for s in (1, 15):
        assert rel_pos_err(out[s - 1][0], ref[s - 1][0], coord) < POS_TOL
    assert np.abs(m.plastic()).max() > 0
    # the FP64 matrix-free solver reaches the tight tolerance as well
    _, out64 = run_gpu(tets, coord, fixed, 15, params=mixed(solver=capi.SOLVER_FP64, rtol=1e-10), material=mat)
    _, ref64 = run_oracle(oracle, tets, coord, fixed, 15, material=mat, converged=True, rtol=1e-10)
    assert rel_pos_err(out64[-1][0], ref64[-1][0], coord) < 1e-8


def test_rigid_translation_is_force_free(gpu):
    tets, coord, _ = beam(6, 3, 3, jitter_seed=2)
    fixed = np.zeros(coord.shape[0], np.uint8)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    v0 = np.tile([0.3, -0.2, 0.1], (coord.shape[0], 1))
    m.set(capi.VELOCITY, v0)
    m.set(capi.F_EXTERNAL, np.zeros_like(v0))
    _, st = m.step(0.01, True, mixed())
    v = m.get(capi.VELOCITY)
    # mass damping alone acts: (1 + dt*alpha) M v = M v0 (fem_dynamics_assembly.h:84-85)
    assert np.abs(v - v0 / (1.0 + 0.01 * 2.0)).max() < 1e-6
    assert np.abs(m.get(capi.COORD) - (coord + 0.01 * v)).max() < 1e-12


def test_nonfinite_force_reports_error_and_context_recovers(gpu):
    tets, coord, fixed = beam(4, 2, 2)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    f = gravity_force(m.get(capi.MASS), fixed)
    bad = f.copy()
    bad[-1, 0] = np.nan
    m.set(capi.F_EXTERNAL, bad)
    rc, st = m.step(0.01, True, mixed(), check=False)
    assert rc == capi.ERR_NONFINITE
    # the context stays usable: reset the state and step again
    m.set(capi.COORD, coord)
    m.set(capi.VELOCITY, np.zeros_like(coord))
    m.set(capi.F_EXTERNAL, f)
    rc, st = m.step(0.01, True, mixed())
    assert rc == capi.OK and st.rel_residual <= 1e-6


def test_device_wait_times_out_and_context_recovers(gpu):
    """The grid barrier's bounded wait, with nothing to release it (one CTA
    waits for a second arrival), gives up after its limit and records
    OTFEM_ERR_TIMEOUT; the kernel returns and the handle keeps working."""
    tets, coord, fixed = beam(4, 2, 2)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    st = ctypes.c_int32(0)
    capi.check(m.lib.otfem_check_wait_timeout(m.h, 4_000_000, ctypes.byref(st)))  # ~2 ms of SM cycles
    assert st.value == capi.ERR_TIMEOUT
    assert m.lib.otfem_check_wait_timeout(m.h, 0, ctypes.byref(st)) == capi.ERR_INVALID_ARGUMENT
    m.set(capi.F_EXTERNAL, gravity_force(m.get(capi.MASS), fixed))
    rc, stats = m.step(0.01, True, mixed())
    assert rc == capi.OK and stats.rel_residual <= 1e-6


def test_model_coordinate_changes_follow_the_oracle(gpu, oracle):
    """The mixed solver's rest edges (a per-tet FP32 table) follow the model
    coordinates: update_original_coord after step 3 and model coordinates set
    to a stretched shape after step 6, against the converged FP64 oracle."""
    tets, coord, fixed = beam(8, 3, 3, jitter_seed=5)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    o = oracle.OracleMesh(tets, coord, coord, fixed)
    o.init(*MATERIAL)
    mass = o.get(oracle.MASS)
    stretched = coord * np.array([1.01, 1.0, 0.995])
    for s in range(10):
        f = gravity_force(mass, fixed)
        m.set(capi.F_EXTERNAL, f)
        o.set(oracle.F_EXTERNAL, f)
        m.step(0.01, True, mixed())
        o.simulate_converged(0.01, True, 2.0, 1e-11, 100000)
        if s == 2:
            capi.check(m.lib.otfem_update_original_coord(m.h))
            o.update_original_coord()
        if s == 5:
            m.set(capi.MODEL_COORD, stretched)
            o.set(oracle.MODEL_COORD, stretched)
        x, xo = m.get(capi.COORD), o.get(oracle.COORD)
        assert np.abs(x - xo).max() <= 1e-5 * np.abs(xo - coord).max(), s
    o.close()
    m.close()


def test_async_download_matches_blocking_one(gpu):
    """otfem_get_nodes_async queues the copy behind the step; after
    otfem_synchronize the values equal a blocking download's."""
    import torch
    tets, coord, fixed = beam(6, 3, 3, jitter_seed=2)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    m.set(capi.F_EXTERNAL, gravity_force(m.get(capi.MASS), fixed))
    pinned = torch.empty((2, m.N, 3), dtype=torch.float64, pin_memory=True).numpy()
    pageable = np.zeros((m.N, 3))
    for _ in range(3):
        m.step(0.01, True, mixed(), check=False)
        dp = ctypes.POINTER(ctypes.c_double)
        capi.check(m.lib.otfem_get_nodes_async(m.h, capi.COORD, pinned[0].ctypes.data_as(dp), pinned[0].size))
        capi.check(m.lib.otfem_get_nodes_async(m.h, capi.VELOCITY, pinned[1].ctypes.data_as(dp), pinned[1].size))
        capi.check(m.lib.otfem_get_nodes_async(m.h, capi.COORD, pageable.ctypes.data_as(dp), pageable.size))
        capi.check(m.lib.otfem_synchronize(m.h))
        assert np.array_equal(pinned[0], m.get(capi.COORD))
        assert np.array_equal(pinned[1], m.get(capi.VELOCITY))
        assert np.array_equal(pageable, pinned[0])
    assert m.lib.otfem_get_nodes_async(m.h, capi.COORD, pageable.ctypes.data_as(dp), 5) == capi.ERR_INVALID_ARGUMENT
    m.close()


def test_iteration_cap_is_a_warning(gpu):
    tets, coord, fixed = beam(8, 3, 3, jitter_seed=1)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    m.set(capi.F_EXTERNAL, gravity_force(m.get(capi.MASS), fixed))
    rc, st = m.step(0.01, True, mixed(max_iterations=3), check=False)
    assert rc == capi.WARN_NOT_CONVERGED and st.iterations == 3


def test_orientations_follow_reference_gram_schmidt(gpu):
    # the FP64 matrix-free path reproduces the reference orientations to FP64
    # rounding; the mixed path's FP32 Gram-Schmidt to FP32 rounding
    tets, coord, fixed = beam(5, 3, 3, jitter_seed=8)
    meshes = [GpuMesh(tets, coord, fixed) for _ in range(3)]
    f = None
    for m in meshes:
        m.init()
        f = gravity_force(m.get(capi.MASS), fixed) if f is None else f
        m.set(capi.F_EXTERNAL, f)
        m.set(capi.COORD, coord + np.random.default_rng(1).normal(0, 0.002, coord.shape))
    meshes[0].step(0.01, True, capi.default_params(sequential_dots=1))
    meshes[1].step(0.01, True, mixed(solver=capi.SOLVER_FP64))
    meshes[2].step(0.01, True, mixed())
    ref = meshes[0].re()
    assert np.abs(meshes[1].re() - ref).max() < 1e-13
    assert np.abs(meshes[2].re() - ref).max() < 2e-6


@pytest.mark.parametrize("dims,seed", [((4, 2, 2), 3), ((12, 5, 4), 6)])
def test_apply_operator_vs_assembled_reference(gpu, oracle, dims, seed):
    """The matrix-free A x (FP32 and FP64 element apply) against the
    reference's assembled A = K dt^2 + M (1 + dt alpha) (fem_dynamics_assembly.h)."""
    import ctypes
    tets, coord, fixed = beam(*dims, jitter_seed=seed)
    n = coord.shape[0]
    o = oracle.OracleMesh(tets, coord, coord, fixed)
    o.init(*MATERIAL)
    mass = o.get(oracle.MASS)
    f = gravity_force(mass, fixed)
    o.set(oracle.F_EXTERNAL, f)
    o.simulate(0.01, True)  # assembles K from the orientations at the initial coordinates
    rp, cols = o.k_pattern()
    K = o.k_values()
    dt = 0.01
    x = np.random.default_rng(seed).normal(size=(n, 3))
    ref = np.zeros_like(x)
    for i in range(n):
        if fixed[i]:
            continue
        for q in range(rp[i], rp[i + 1]):
            ref[i] += K[q] @ x[cols[q]]
        ref[i] = ref[i] * dt * dt + mass[i] * (1 + dt * 2.0) * x[i]
    m = GpuMesh(tets, coord, fixed)
    m.init()
    m.set(capi.F_EXTERNAL, f)
    _dp = ctypes.POINTER(ctypes.c_double)
    for solver, tol in ((capi.SOLVER_MIXED, 2e-6), (capi.SOLVER_FP64, 1e-13)):
        # the orientations of the solver's own first phase
        p = mixed(solver=solver)
        capi.check(m.lib.otfem_simulate_phase(m.h, dt, 1, ctypes.byref(p), capi.PHASE_ORIENT))
        for variant in range(capi.NUM_APPLY_VARIANTS):
            capi.check(m.lib.otfem_set_apply_variant(m.h, variant))
            y = np.zeros_like(x)
            capi.check(m.lib.otfem_apply_operator(m.h, solver, dt, 2.0, x.ctypes.data_as(_dp),
                                                  y.ctypes.data_as(_dp)))
            assert np.abs(y - ref).max() <= tol * np.abs(ref).max(), (solver, variant)


def test_every_apply_variant_solves_alike(gpu):
    """Every element-apply variant the autotuner chooses from gives the
    same solution to FP32-apply accuracy."""
    import ctypes
    g = golden("converged")
    results = []
    for variant in range(capi.NUM_APPLY_VARIANTS):
        m = GpuMesh(g["tets"], g["coord"], g["fixed"])
        m.init()
        capi.check(m.lib.otfem_set_apply_variant(m.h, variant))
        mass = m.get(capi.MASS)
        for _ in range(5):
            m.set(capi.F_EXTERNAL, gravity_force(mass, g["fixed"]))
            _, st = m.step(0.01, True, mixed())
            assert st.rel_residual <= 1e-6
        results.append(m.get(capi.COORD))
        v = ctypes.c_int32()
        ms = np.zeros(capi.NUM_APPLY_VARIANTS)
        capi.check(m.lib.otfem_tuning(m.h, ctypes.byref(v), ms.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        assert v.value == variant and (ms > 0).all()
    for x in results:
        assert rel_pos_err(x, g["x_5"], g["coord"]) < POS_TOL


def test_tolerance_below_the_precision_floor_ends_unconverged(gpu):
    """A tolerance the FP32 apply cannot reach: the solve stops at the floor
    with OTFEM_WARN_NOT_CONVERGED and a finite, small true residual (the
    recurrence check restarts the direction instead of letting it grow)."""
    tets, coord, fixed = beam(8, 3, 4, jitter_seed=8)
    m = GpuMesh(tets, coord, fixed)
    m.init()
    mass = m.get(capi.MASS)
    for variant in range(capi.NUM_APPLY_VARIANTS):
        capi.check(m.lib.otfem_set_apply_variant(m.h, variant))
        m.set(capi.F_EXTERNAL, gravity_force(mass, fixed))
        rc, st = m.step(0.01, True, mixed(rtol=1e-10, max_iterations=3000), check=False)
        assert rc in (capi.OK, capi.WARN_NOT_CONVERGED), (variant, rc)
        # the floor of the FP32 accumulation of node forces, far below the
        # divergence (1e18) the unchecked recurrence reached
        assert np.isfinite(st.rel_residual) and st.rel_residual < 1e-4, (variant, st.rel_residual)
        assert st.iterations < 3000
    m.close()
