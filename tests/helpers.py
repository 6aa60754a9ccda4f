"""Shared test helpers: beam meshes, loads, and a thin C-ABI mesh wrapper."""
import ctypes
import hashlib
import os

import numpy as np

from opentissue_gb300 import capi
from opentissue_gb300.fem import generate_blocks

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GRAVITY = -9.81
MATERIAL = (5e5, 0.33, 1000.0, 1e30, 0.0, 0.0)

_dp = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u8p = ctypes.POINTER(ctypes.c_uint8)


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def beam(I, J, K, jitter_seed=None, jitter=0.01, edge=0.1):
    """Block beam with the x = 0 face (grid index i == 0) fixed."""
    tets, coord = generate_blocks(I, J, K, edge, edge, edge)
    if jitter_seed is not None:
        rng = np.random.default_rng(jitter_seed)
        coord = coord + rng.uniform(-jitter, jitter, coord.shape)
    fixed = (np.arange(coord.shape[0]) < (J + 1) * (K + 1)).astype(np.uint8)
    return tets, coord, fixed


def gravity_force(mass, fixed):
    f = np.zeros((mass.shape[0], 3))
    free = fixed == 0
    f[free, 1] = GRAVITY * mass[free]
    return f


def step_hash(x, v):
    return hashlib.sha256(np.ascontiguousarray(x).tobytes() + np.ascontiguousarray(v).tobytes()).hexdigest()


class GpuMesh:
    """A mesh on the GPU driven directly through the C ABI."""

    def __init__(self, tets, coord, fixed=None, model_coord=None, stream=None):
        self.lib = capi.lib()
        self.tets = np.ascontiguousarray(tets, np.int32)
        self.coord = np.ascontiguousarray(coord, np.float64)
        self.model = self.coord if model_coord is None else np.ascontiguousarray(model_coord, np.float64)
        self.N, self.T = self.coord.shape[0], self.tets.shape[0]
        self.fixed = np.zeros(self.N, np.uint8) if fixed is None else np.ascontiguousarray(fixed, np.uint8)
        desc = capi.MeshDesc(self.N, self.T, self.tets.ctypes.data_as(_i32p), self.coord.ctypes.data_as(_dp),
                             self.model.ctypes.data_as(_dp), self.fixed.ctypes.data_as(_u8p))
        self.h = ctypes.c_void_p()
        capi.check(self.lib.otfem_create(ctypes.byref(desc), stream, ctypes.byref(self.h)))

    def close(self):
        if self.h:
            self.lib.otfem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init(self, material=MATERIAL):
        capi.check(self.lib.otfem_init(self.h, *material))

    def set(self, field, arr):
        a = np.ascontiguousarray(arr, np.float64).reshape(-1)
        capi.check(self.lib.otfem_set_nodes(self.h, field, a.ctypes.data_as(_dp), a.size))

    def get(self, field):
        out = np.zeros(self.N if field in (capi.MASS, capi.NODE_STIFFNESS) else (self.N, 3))
        capi.check(self.lib.otfem_get_nodes(self.h, field, out.ctypes.data_as(_dp), out.size))
        return out

    def step(self, dt=0.01, warp=True, params=None, check=True):
        st = capi.StepStats()
        p = params if params is not None else capi.default_params()
        rc = self.lib.otfem_simulate_ex(self.h, dt, int(warp), ctypes.byref(p), ctypes.byref(st))
        if check:
            capi.check(rc)
        return rc, st

    def re(self):
        out = np.zeros((self.T, 3, 3))
        capi.check(self.lib.otfem_get_orientations(self.h, out.ctypes.data_as(_dp)))
        return out

    def plastic(self):
        out = np.zeros((self.T, 6))
        capi.check(self.lib.otfem_get_plastic(self.h, out.ctypes.data_as(_dp)))
        return out

    def k_pattern(self):
        nnz = ctypes.c_int64()
        capi.check(self.lib.otfem_k_pattern(self.h, ctypes.byref(nnz), None, None))
        rp = np.zeros(self.N + 1, np.int32)
        cols = np.zeros(max(nnz.value, 1), np.int32)
        capi.check(self.lib.otfem_k_pattern(self.h, ctypes.byref(nnz), rp.ctypes.data_as(_i32p),
                                            cols.ctypes.data_as(_i32p)))
        return rp, cols[:nnz.value]

    def k_values(self):
        nnz = ctypes.c_int64()
        capi.check(self.lib.otfem_k_pattern(self.h, ctypes.byref(nnz), None, None))
        v = np.zeros((max(nnz.value, 1), 3, 3))
        capi.check(self.lib.otfem_k_values(self.h, v.ctypes.data_as(_dp)))
        return v[:nnz.value]

    def export_k(self):
        """export_K triplets in the reference's push order."""
        nnz = ctypes.c_int64()
        capi.check(self.lib.otfem_export_k_csr(self.h, ctypes.byref(nnz), None, None, None))
        rp = np.zeros(self.N + 1, np.int32)
        cols = np.zeros(max(nnz.value, 1), np.int32)
        vals = np.zeros((max(nnz.value, 1), 3, 3))
        capi.check(self.lib.otfem_export_k_csr(self.h, ctypes.byref(nnz), rp.ctypes.data_as(_i32p),
                                               cols.ctypes.data_as(_i32p), vals.ctypes.data_as(_dp)))
        rows, cs, vs = [], [], []
        for i in range(self.N):
            for r in range(3):
                if self.fixed[i]:
                    rows.append(3 * i + r)
                    cs.append(3 * i + r)
                    vs.append(1.0)
                    continue
                for q in range(rp[i], rp[i + 1]):
                    for c in range(3):
                        rows.append(3 * i + r)
                        cs.append(3 * cols[q] + c)
                        vs.append(vals[q, r, c])
        return np.array(rows, np.int32), np.array(cs, np.int32), np.array(vs)


def run_gpu(tets, coord, fixed, steps, params=None, material=MATERIAL, dt=0.01, warp=True, record=None):
    """Runs `steps` gravity steps; returns (mesh, per-step list of (x, v, stats))."""
    m = GpuMesh(tets, coord, fixed)
    m.init(material)
    mass = m.get(capi.MASS)
    out = []
    for s in range(1, steps + 1):
        m.set(capi.F_EXTERNAL, gravity_force(mass, fixed))
        _, st = m.step(dt, warp, params)
        if record is None or s in record:
            out.append((m.get(capi.COORD), m.get(capi.VELOCITY), st))
        else:
            out.append((None, None, st))
    return m, out


def run_oracle(po, tets, coord, fixed, steps, material=MATERIAL, dt=0.01, warp=True, converged=False,
               rtol=1e-6):
    m = po.OracleMesh(tets, coord, coord, fixed)
    m.init(*material)
    mass = m.get(po.MASS)
    out = []
    for _ in range(steps):
        m.set(po.F_EXTERNAL, gravity_force(mass, fixed))
        if converged:
            it, rr = m.simulate_converged(dt, warp, 2.0, rtol, 100000)
        else:
            m.simulate(dt, warp)
            it, rr = 20, None
        out.append((m.get(po.COORD), m.get(po.VELOCITY), it, rr))
    return m, out


def tip_load(coord, I, J, K, amp, freq, direction, t):
    """A sinusoidal load spread over the free end face of an I x J x K beam."""
    n = coord.shape[0]
    tip = np.arange(n) >= I * (J + 1) * (K + 1)
    f = np.zeros((n, 3))
    f[tip] = amp * np.sin(2 * np.pi * freq * t) * np.asarray(direction) / tip.sum()
    return f


def run_loaded(m, dims, steps, params, amp, freq, direction, net=None, dt=0.01):
    """Gravity plus a tip load; returns the iteration counts and positions per step."""
    I, J, K = dims
    mass = m.get(capi.MASS)
    its, xs = [], []
    for s in range(steps):
        f = gravity_force(mass, m.fixed) + tip_load(m.coord, I, J, K, amp, freq, direction, s * dt)
        m.set(capi.F_EXTERNAL, f)
        _, st = m.step(dt, True, params)
        assert st.rel_residual <= 1e-6
        its.append(st.iterations)
        xs.append(m.get(capi.COORD))
        if net is not None:
            net.add_samples(m.h)
    return np.array(its), xs


def irregular_mesh(shape=(8, 4, 4), h=0.1, jitter=0.35, seed=0):
    """An unstructured tetrahedral mesh: the Delaunay tetrahedralization of a
    jittered lattice of (shape + 1) points (spacing h, jitter in units of h),
    flat tets (volume below 5% of the median) dropped, every tet oriented to
    a positive volume and unused points removed; the x = min face fixed.
    Node order and tet order come from the triangulation, so the
    connectivity has none of the block mesh's regularity."""
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    I, J, K = shape
    g = np.stack(np.meshgrid(np.arange(I + 1), np.arange(J + 1), np.arange(K + 1), indexing="ij"), -1).reshape(-1, 3)
    pts = g.astype(np.float64) * h
    interior = np.all((g > 0) & (g < np.array([I, J, K])), axis=1)
    pts[interior] += rng.uniform(-jitter * h, jitter * h, (int(interior.sum()), 3))
    perm = rng.permutation(len(pts))  # scramble the node numbering
    pts = pts[perm]
    tri = Delaunay(pts)
    tets = tri.simplices.astype(np.int64)
    e = pts[tets[:, 1:]] - pts[tets[:, :1]]
    vol = np.einsum("ij,ij->i", e[:, 0], np.cross(e[:, 1], e[:, 2])) / 6.0
    keep = np.abs(vol) > 0.05 * np.median(np.abs(vol))
    tets, vol = tets[keep], vol[keep]
    neg = vol < 0
    tets[neg, 0], tets[neg, 1] = tets[neg, 1].copy(), tets[neg, 0].copy()
    used = np.unique(tets)
    remap = np.full(len(pts), -1, np.int64)
    remap[used] = np.arange(len(used))
    tets = remap[tets].astype(np.int32)
    coord = np.ascontiguousarray(pts[used])
    fixed = (coord[:, 0] < 1e-9).astype(np.uint8)
    return tets, coord, fixed


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
