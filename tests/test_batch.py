"""Batched solve (otfem_batch_*): uneven meshes stepped together by one
persistent launch per step, each with its own CG, against the same meshes
solved one by one (and one of them against the FP64 oracle)."""
import ctypes

import numpy as np
import pytest

from helpers import GpuMesh
from opentissue_gb300 import capi
from opentissue_gb300.workloads import random_beams

pytestmark = pytest.mark.gpu

_dp = ctypes.POINTER(ctypes.c_double)
DT = 0.005


class Batch:
    def __init__(self, beams):
        self.lib = capi.lib()
        self.beams = beams
        self.keep = []
        descs = (capi.MeshDesc * len(beams))()
        for k, b in enumerate(beams):
            tets = np.ascontiguousarray(b["tets"], np.int32)
            coord = np.ascontiguousarray(b["coord"], np.float64)
            fixed = np.ascontiguousarray(b["fixed"], np.uint8)
            self.keep += [tets, coord, fixed]
            descs[k] = capi.MeshDesc(coord.shape[0], tets.shape[0], tets.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                     coord.ctypes.data_as(_dp), coord.ctypes.data_as(_dp),
                                     fixed.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
        self.h = ctypes.c_void_p()
        capi.check(self.lib.otfem_batch_create(descs, len(beams), None, ctypes.byref(self.h)))
        e = np.array([b["young"] for b in beams])
        nu = np.array([b["poisson"] for b in beams])
        rho = np.array([b["density"] for b in beams])
        capi.check(self.lib.otfem_batch_init(self.h, e.ctypes.data_as(_dp), nu.ctypes.data_as(_dp),
                                             rho.ctypes.data_as(_dp), 1e30, 0.0, 0.0))
        cnt = ctypes.c_int32()
        self.noff = np.zeros(len(beams) + 1, np.int32)
        self.toff = np.zeros(len(beams) + 1, np.int32)
        capi.check(self.lib.otfem_batch_layout(self.h, ctypes.byref(cnt),
                                               self.noff.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                               self.toff.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))))
        assert cnt.value == len(beams)
        self.N = int(self.noff[-1])

    def get(self, field):
        out = np.zeros(self.N if field == capi.MASS else (self.N, 3))
        capi.check(self.lib.otfem_get_nodes(self.h, field, out.ctypes.data_as(_dp), out.size))
        return out

    def set(self, field, arr):
        a = np.ascontiguousarray(arr, np.float64).reshape(-1)
        capi.check(self.lib.otfem_set_nodes(self.h, field, a.ctypes.data_as(_dp), a.size))

    def per_mesh(self, arr):
        return [arr[self.noff[m]:self.noff[m + 1]] for m in range(len(self.beams))]

    def stats(self):
        M = len(self.beams)
        its = np.zeros(M, np.int32)
        st = np.zeros(M, np.int32)
        rel = np.zeros(M)
        rel0 = np.zeros(M)
        capi.check(self.lib.otfem_batch_stats(self.h, its.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                              st.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                              rel.ctypes.data_as(_dp), rel0.ctypes.data_as(_dp)))
        return its, st, rel, rel0

    def close(self):
        if self.h:
            self.lib.otfem_destroy(self.h)
            self.h = None


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
            # both stop at rel. residual 1e-6; on stiff beams with small
            # displacements that leaves position differences of a few 1e-5
            # of the displacement (the FP64 oracle's own error at this
            # tolerance is as large: test_batch_against_the_fp64_oracle)
            ref = singles[k][s]
            disp = np.abs(ref - bm["coord"]).max()
            assert np.abs(xs[k] - ref).max() <= 1e-4 * disp, (s, k)
    # meshes of different size and stiffness converge in different counts
    assert len(set(out[-1][1][0].tolist())) > 1
    b.close()


def oracle_positions(oracle, bm, steps, rtol):
    o = oracle.OracleMesh(bm["tets"], bm["coord"], bm["coord"], bm["fixed"])
    o.init(bm["young"], bm["poisson"], bm["density"], 1e30, 0.0, 0.0)
    f = loads(o.get(oracle.MASS), bm["fixed"], bm["tip_force"])
    for _ in range(steps):
        o.set(oracle.F_EXTERNAL, f)
        o.simulate_converged(DT, True, 2.0, rtol, 100000)
    x = o.get(oracle.COORD)
    o.close()
    return x


def test_batch_against_the_fp64_oracle(gpu, oracle):
    """Every mesh of the batch against the tightly converged FP64 oracle.
    The batch converges to the FP32 operator's solution: on these small stiff
    beams (displacements ~1e-4 m) the FP32 element forces, which cancel at the
    nodes, leave a few 1e-5 of the displacement, where the FP64 oracle stopped
    at the same tolerance is ~1e-7 away; the bound states that accuracy."""
    beams = random_beams(3, seed=32, nx=(8, 12), nyz=(3, 4))
    b, out = run_batch(beams, 3)
    for k, bm in enumerate(beams):
        exact = oracle_positions(oracle, bm, 3, 1e-11)
        disp = np.abs(exact - bm["coord"]).max()
        err_batch = np.abs(out[-1][0][k] - exact).max() / disp
        assert err_batch <= 1e-4, (k, err_batch)
    b.close()


def test_batch_apply_variants_agree(gpu):
    beams = random_beams(5, seed=33, nx=(8, 14), nyz=(3, 5))
    res = []
    for v in (2, 3):
        b, out = run_batch(beams, 3, variant=v)
        res.append(out[-1][0])
        b.close()
    for k, bm in enumerate(beams):
        disp = np.abs(res[0][k] - bm["coord"]).max()
        assert np.abs(res[0][k] - res[1][k]).max() <= 1e-4 * disp


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
        assert np.abs(res[0][k] - res[1][k]).max() <= 1e-4 * disp
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
            assert np.abs(out1[s][0][k] - out0[s][0][k]).max() <= 1e-4 * disp, (s, k)
        its, st, rel, _ = out1[s][1]
        assert np.all(st == capi.OK) and np.all(rel <= 1e-6)
    late0 = np.sum([o[1][0] for o in out0[6:]])
    late1 = np.sum([o[1][0] for o in out1[6:]])
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
            assert np.abs(out1[s][0][k] - out0[s][0][k]).max() <= 1e-4 * disp, (s, k)
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
