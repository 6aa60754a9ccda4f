"""Batched solve (otfem_batch_*): uneven meshes stepped together by one
persistent launch per step, each with its own CG, against the same meshes
solved one by one (and one of them against the FP64 oracle)."""
import ctypes

import numpy as np
import pytest

from helpers import Batch, GpuMesh
from opentissue_gb300 import capi
from opentissue_gb300.workloads import random_beams

pytestmark = pytest.mark.gpu

_dp = ctypes.POINTER(ctypes.c_double)
DT = 0.005


def loads(mass, fixed, tip_force):
    f = tip_force.copy()
    free = fixed == 0
    f[free, 1] += -9.81 * mass[free]
    f[~free] = 0.0
    return f


def params(**kw):
    base = dict(solver=capi.SOLVER_MIXED, max_iterations=3000, rtol=1e-6)
    base.update(kw)
    return capi.default_params(**base)


def run_batch(beams, steps, variant=None, net=None, **kw):
    b = Batch(beams)
    if variant is not None:
        capi.check(b.lib.otfem_set_apply_variant(b.h, variant))
    if net is not None:
        net.attach(b.h)
    mass = b.get(capi.MASS)
    f = np.concatenate([loads(m, bm["fixed"], bm["tip_force"]) for m, bm in zip(b.per_mesh(mass), beams)])
    out = []
    for _ in range(steps):
        b.set(capi.F_EXTERNAL, f)
        st = capi.StepStats()
        capi.check(b.lib.otfem_simulate_ex(b.h, DT, 1, ctypes.byref(params(**kw)), ctypes.byref(st)))
        out.append((b.per_mesh(b.get(capi.COORD)), b.stats(), st))
    return b, out


def run_single(bm, steps):
    m = GpuMesh(bm["tets"], bm["coord"], bm["fixed"])
    m.init((bm["young"], bm["poisson"], bm["density"], 1e30, 0.0, 0.0))
    f = loads(m.get(capi.MASS), bm["fixed"], bm["tip_force"])
    xs = []
    for _ in range(steps):
        m.set(capi.F_EXTERNAL, f)
        m.step(DT, True, params())
        xs.append(m.get(capi.COORD))
    m.close()
    return xs


def test_batch_matches_meshes_solved_one_by_one(gpu):
    beams = random_beams(6, seed=31, nx=(8, 16), nyz=(3, 5))
    b, out = run_batch(beams, 4)
    singles = [run_single(bm, 4) for bm in beams]
    for s in range(4):
        xs, (its, st, rel, rel0), agg = out[s]
        assert np.all(st == capi.OK) and np.all(rel <= 1e-6), (st, rel)
        assert agg.iterations == its.max()
        for k, bm in enumerate(beams):
            # both stop at rel. residual 1e-6
            ref = singles[k][s]
            disp = np.abs(ref - bm["coord"]).max()
            assert np.abs(xs[k] - ref).max() <= 1e-5 * disp, (s, k)
    # meshes of different size and stiffness converge in different counts
    assert len(set(out[-1][1][0].tolist())) > 1
    b.close()


def oracle_state(oracle, bm, steps, rtol):
    o = oracle.OracleMesh(bm["tets"], bm["coord"], bm["coord"], bm["fixed"])
    o.init(bm["young"], bm["poisson"], bm["density"], 1e30, 0.0, 0.0)
    f = loads(o.get(oracle.MASS), bm["fixed"], bm["tip_force"])
    for _ in range(steps):
        o.set(oracle.F_EXTERNAL, f)
        o.simulate_converged(DT, True, 2.0, rtol, 100000)
    x, v = o.get(oracle.COORD), o.get(oracle.VELOCITY)
    o.close()
    return x, v


def test_batch_against_the_fp64_oracle(gpu, oracle):
    """Every mesh of the batch against the tightly converged FP64 oracle,
    positions and velocities, on the stiffest beams of the batch's family
    (E = 5e6 Pa: displacements of ~1e-4 m after a few steps, strains of
    1e-5, where FP32 edge differences alone would leave errors of a few 1e-5
    of the displacement) and on softer ones: within 1e-5 of the largest
    displacement and of the largest velocity."""
    beams = random_beams(4, seed=32, nx=(8, 16), nyz=(3, 5))
    beams[0]["young"] = beams[1]["young"] = 5e6
    steps = 4
    b = Batch(beams)
    mass = b.get(capi.MASS)
    f = np.concatenate([loads(m, bm["fixed"], bm["tip_force"]) for m, bm in zip(b.per_mesh(mass), beams)])
    for _ in range(steps):
        b.set(capi.F_EXTERNAL, f)
        capi.check(b.lib.otfem_simulate_ex(b.h, DT, 1, ctypes.byref(params()), None))
    xs, vs = b.per_mesh(b.get(capi.COORD)), b.per_mesh(b.get(capi.VELOCITY))
    for k, bm in enumerate(beams):
        x_ref, v_ref = oracle_state(oracle, bm, steps, 1e-11)
        err_x = np.abs(xs[k] - x_ref).max() / np.abs(x_ref - bm["coord"]).max()
        err_v = np.abs(vs[k] - v_ref).max() / np.abs(v_ref).max()
        print(f"batch mesh {k} E {bm['young']:.3g}: x {err_x:.2e} v {err_v:.2e}")
        assert err_x <= 1e-5 and err_v <= 1e-5, (k, bm["young"], err_x, err_v)
    b.close()


@pytest.mark.parametrize("warm", [capi.WARM_START_PREVIOUS, capi.WARM_START_EXTRAPOLATED])
def test_batch_beyond_the_local_mesh_limit(gpu, warm):
    """Up to 512 meshes every CTA runs the iterations' scalar steps on its own
    copy of the meshes' state; beyond that the last CTA of each reduction runs
    them for all.  520 copies of six beams step as the six beams do alone.
    The iteration counts may differ by one refresh period (4): a mesh near
    the tolerance at a refresh point converges there or 4 iterations later,
    depending on the last bits of its sums (FP64 atomics in no fixed order
    already flip it from run to run).  With the extrapolated start the large
    batch projects every mesh (the per-mesh choice needs the shared copy), so
    only the answers are compared."""
    beams = random_beams(6, seed=35, nx=(4, 7), nyz=(2, 3))
    many = [beams[k % len(beams)] for k in range(520)]
    small_b, small = run_batch(beams, 3, warm_start=warm)
    big_b, big = run_batch(many, 3, warm_start=warm)
    for s in range(3):
        xs_small, (its_small, _, _, _), _ = small[s]
        xs_big, (its_big, st_big, rel_big, _), agg = big[s]
        assert np.all(st_big == capi.OK) and np.all(rel_big <= 1e-6), (s, st_big, rel_big)
        assert agg.iterations == its_big.max()
        for k in range(len(many)):
            j = k % len(beams)
            disp = np.abs(xs_small[j] - beams[j]["coord"]).max()
            assert np.abs(xs_big[k] - xs_small[j]).max() <= 1e-5 * disp, (s, k)
            if warm == capi.WARM_START_PREVIOUS:
                assert abs(int(its_big[k]) - int(its_small[j])) <= 4, (s, k)
    small_b.close()
    big_b.close()


def test_batch_apply_variants_agree(gpu):
    beams = random_beams(5, seed=33, nx=(8, 14), nyz=(3, 5))
    res = []
    for v in (2, 3):
        b, out = run_batch(beams, 3, variant=v)
        res.append(out[-1][0])
        b.close()
    for k, bm in enumerate(beams):
        disp = np.abs(res[0][k] - bm["coord"]).max()
        assert np.abs(res[0][k] - res[1][k]).max() <= 1e-5 * disp


def test_batch_preconditioner_same_answer_fewer_iterations(gpu):
    beams = random_beams(4, seed=35, nx=(10, 16), nyz=(3, 5))
    res, its = {}, {}
    for pre in (capi.PRECONDITIONER_NONE, capi.PRECONDITIONER_JACOBI):
        b, out = run_batch(beams, 3, preconditioner=pre)
        res[pre] = out[-1][0]
        its[pre] = np.sum([o[1][0] for o in out])
        for _, (it, st, rel, _), _ in out:
            assert np.all(st == capi.OK) and np.all(rel <= 1e-6)
        b.close()
    for k, bm in enumerate(beams):
        disp = np.abs(res[0][k] - bm["coord"]).max()
        assert np.abs(res[0][k] - res[1][k]).max() <= 1e-5 * disp
    assert its[capi.PRECONDITIONER_JACOBI] < 0.9 * its[capi.PRECONDITIONER_NONE], its


def test_batch_projected_start_per_mesh(gpu):
    """Each mesh of a batch starts from its own least-energy point over its
    own velocity history: the same answer as the plain start, fewer
    iterations once the history has filled."""
    beams = random_beams(5, seed=36, nx=(10, 16), nyz=(3, 5))
    steps = 12
    b0, out0 = run_batch(beams, steps)
    b1, out1 = run_batch(beams, steps, warm_start=capi.WARM_START_PROJECTED)
    for s in range(steps):
        for k, bm in enumerate(beams):
            disp = np.abs(out0[s][0][k] - bm["coord"]).max()
            assert np.abs(out1[s][0][k] - out0[s][0][k]).max() <= 1e-5 * disp, (s, k)
        its, st, rel, _ = out1[s][1]
        assert np.all(st == capi.OK) and np.all(rel <= 1e-6)
    late0 = np.sum([o[1][0] for o in out0[6:]])
    late1 = np.sum([o[1][0] for o in out1[6:]])
    assert late1 < 0.75 * late0, (late0, late1)
    b0.close()
    b1.close()


def test_batch_extrapolated_start_per_mesh(gpu):
    """Each mesh of a batch starts from its own extrapolated velocity: the
    same answer as the plain start, fewer iterations once the history has
    filled."""
    beams = random_beams(5, seed=36, nx=(10, 16), nyz=(3, 5))
    steps = 12
    b0, out0 = run_batch(beams, steps)
    b1, out1 = run_batch(beams, steps, warm_start=capi.WARM_START_EXTRAPOLATED, warm_history=4)
    for s in range(steps):
        for k, bm in enumerate(beams):
            disp = np.abs(out0[s][0][k] - bm["coord"]).max()
            assert np.abs(out1[s][0][k] - out0[s][0][k]).max() <= 1e-5 * disp, (s, k)
        its, st, rel, _ = out1[s][1]
        assert np.all(st == capi.OK) and np.all(rel <= 1e-6)
    late0 = np.sum([o[1][0] for o in out0[6:]])
    late1 = np.sum([o[1][0] for o in out1[6:]])
    print("batch iterations, steps 7-12: plain start", late0, "extrapolated", late1)
    assert late1 < 0.75 * late0, (late0, late1)
    b0.close()
    b1.close()


def test_batch_learned_start_per_mesh(gpu):
    """A network attached to a batch: each mesh starts from its least-energy
    point over the network's correction and its own history.  The network is
    untrained (random weights), so its correction is arbitrary; the search
    space still holds the projected start's directions, and every mesh ends
    at the plain start's answer."""
    from oracle import mlp_oracle as mo
    from opentissue_gb300.warmstart import WarmStartNet
    rng = np.random.default_rng(8)
    w = {name: rng.uniform(-1, 1, shape) / np.sqrt(shape[1] if len(shape) == 2 else 64) for name, shape in mo.SHAPES}
    norm = {"mu_x": np.zeros(18), "sd_x": np.ones(18), "mu_y": np.zeros(3), "sd_y": np.full(3, 1e-3)}
    net = WarmStartNet(capacity=1 << 10, seed=3)
    net.set_state(mo.pack(w, norm))
    beams = random_beams(5, seed=36, nx=(10, 16), nyz=(3, 5))
    steps = 10
    b0, out0 = run_batch(beams, steps)
    b1, out1 = run_batch(beams, steps, net=net, warm_start=capi.WARM_START_LEARNED)
    for s in range(steps):
        for k, bm in enumerate(beams):
            disp = np.abs(out0[s][0][k] - bm["coord"]).max()
            assert np.abs(out1[s][0][k] - out0[s][0][k]).max() <= 1e-5 * disp, (s, k)
        its, st, rel, _ = out1[s][1]
        assert np.all(st == capi.OK) and np.all(rel <= 1e-6)
    WarmStartNet.detach(b1.h)
    b0.close()
    b1.close()
    net.close()


def test_batch_rejects_other_solvers_and_variants(gpu):
    beams = random_beams(2, seed=34, nx=(8, 8), nyz=(3, 3))
    b = Batch(beams)
    rc = b.lib.otfem_simulate_ex(b.h, DT, 1, ctypes.byref(capi.default_params()), None)
    assert rc == capi.ERR_UNSUPPORTED
    assert b.lib.otfem_set_apply_variant(b.h, 0) == capi.ERR_UNSUPPORTED
    b.close()
