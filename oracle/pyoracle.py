"""ctypes wrapper around the CPU oracle (oracle/otfem_oracle.h).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference legs of bench.py.  It wraps either the C restatement
(oracle/_build/liboracle.so, built by oracle/build.py) or the reference-backed
build (oracle/_ref/libotfem_ref.so), which export the same C interface.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libotfem_ref.so")

COORD, MODEL_COORD, VELOCITY, F_EXTERNAL, MASS, F0, B = range(7)

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_up = ctypes.POINTER(ctypes.c_ubyte)
_libs = {}


def _ptr(a, t):
    return a.ctypes.data_as(t)


def load(kind="port"):
    """Loads the oracle library: kind 'port' (C restatement) or 'reference'."""
    path = PORT_LIB if kind == "port" else REF_LIB
    if path in _libs:
        return _libs[path]
    if not os.path.exists(path):
        raise FileNotFoundError(f"oracle library not built: {path}")
    lib = ctypes.CDLL(path)
    v = ctypes.c_void_p
    lib.orc_create.restype = v
    lib.orc_create.argtypes = [ctypes.c_int, ctypes.c_int, _ip, _dp, _dp, _up]
    lib.orc_destroy.argtypes = [v]
    lib.orc_set_fixed.argtypes = [v, _up]
    lib.orc_set_field.argtypes = [v, ctypes.c_int, _dp]
    lib.orc_get_field.argtypes = [v, ctypes.c_int, _dp]
    lib.orc_init.argtypes = [v] + [ctypes.c_double] * 6
    lib.orc_simulate.argtypes = [v, ctypes.c_double, ctypes.c_int]
    lib.orc_simulate_converged.argtypes = [v, ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_int, _ip, _dp]
    lib.orc_update_original_coord.argtypes = [v]
    lib.orc_export_k_count.restype = ctypes.c_long
    lib.orc_export_k_count.argtypes = [v]
    lib.orc_export_k.argtypes = [v, _ip, _ip, _dp]
    lib.orc_k_nnz.restype = ctypes.c_long
    lib.orc_k_nnz.argtypes = [v]
    lib.orc_k_pattern.argtypes = [v, _ip, _ip]
    lib.orc_k_values.argtypes = [v, _dp]
    lib.orc_get_re.argtypes = [v, _dp]
    lib.orc_get_plastic.argtypes = [v, _dp]
    lib.orc_get_volume.argtypes = [v, _dp]
    lib.orc_generate_blocks.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 3 + [_ip, _dp]
    if kind == "reference":
        lib.orc_coupling_bind.restype = ctypes.c_int
        lib.orc_coupling_bind.argtypes = [ctypes.c_int, ctypes.c_int, _ip, _dp, ctypes.c_int, _dp, _ip, _dp]
        lib.orc_coupling_update.restype = ctypes.c_int
        lib.orc_coupling_update.argtypes = [ctypes.c_int, ctypes.c_int, _ip, _dp, ctypes.c_int, _ip, _dp, _dp]
    _libs[path] = lib
    return lib


def coupling_bind(tets, coord, points):
    """t4mesh::mesh_coupling::bind_surface of the reference build: per point
    the tet index (-1: unbound) and (w1, w2, w3)."""
    lib = load("reference")
    tets = np.ascontiguousarray(tets, np.int32)
    coord = np.ascontiguousarray(coord, np.float64)
    pts = np.ascontiguousarray(points, np.float64)
    tet = np.full(pts.shape[0], -1, np.int32)
    bary = np.zeros((pts.shape[0], 3))
    lib.orc_coupling_bind(coord.shape[0], tets.shape[0], _ptr(tets, _ip), _ptr(coord, _dp), pts.shape[0],
                          _ptr(pts, _dp), _ptr(tet, _ip), _ptr(bary, _dp))
    return tet, bary


def coupling_update(tets, coord, tet, bary):
    """t4mesh::mesh_coupling::update_surface of the reference build for bound
    points (every tet index >= 0)."""
    lib = load("reference")
    tets = np.ascontiguousarray(tets, np.int32)
    coord = np.ascontiguousarray(coord, np.float64)
    tet = np.ascontiguousarray(tet, np.int32)
    bary = np.ascontiguousarray(bary, np.float64)
    out = np.zeros((tet.shape[0], 3))
    rc = lib.orc_coupling_update(coord.shape[0], tets.shape[0], _ptr(tets, _ip), _ptr(coord, _dp), tet.shape[0],
                                 _ptr(tet, _ip), _ptr(bary, _dp), _ptr(out, _dp))
    if rc != 0:
        raise ValueError("update_surface needs a tet for every point")
    return out


def generate_blocks(I, J, K, w, h, d, kind="port"):
    """t4mesh::generate_blocks through the oracle: returns (tets int32 [T,4], coord f64 [N,3])."""
    lib = load(kind)
    tets = np.zeros((5 * I * J * K, 4), np.int32)
    coord = np.zeros(((I + 1) * (J + 1) * (K + 1), 3), np.float64)
    lib.orc_generate_blocks(I, J, K, w, h, d, _ptr(tets, _ip), _ptr(coord, _dp))
    return tets, coord


class OracleMesh:
    """One oracle FEM mesh (fem::Mesh + fem::init/simulate on the CPU)."""

    def __init__(self, tets, coord, model_coord=None, fixed=None, kind="port"):
        self.lib = load(kind)
        self.kind = kind
        tets = np.ascontiguousarray(tets, np.int32)
        coord = np.ascontiguousarray(coord, np.float64)
        model = coord if model_coord is None else np.ascontiguousarray(model_coord, np.float64)
        self.N, self.T = coord.shape[0], tets.shape[0]
        fx = np.zeros(self.N, np.uint8) if fixed is None else np.ascontiguousarray(fixed, np.uint8)
        self.h = self.lib.orc_create(self.N, self.T, _ptr(tets, _ip), _ptr(coord, _dp),
                                     _ptr(model, _dp), _ptr(fx, _up))

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def init(self, young, poisson, density, c_yield=1e30, c_creep=0.0, c_max=0.0):
        self.lib.orc_init(self.h, young, poisson, density, c_yield, c_creep, c_max)

    def set(self, field, arr):
        a = np.ascontiguousarray(arr, np.float64).reshape(-1)
        assert a.size == 3 * self.N
        self.lib.orc_set_field(self.h, field, _ptr(a, _dp))

    def get(self, field):
        out = np.zeros(self.N if field == MASS else (self.N, 3), np.float64)
        self.lib.orc_get_field(self.h, field, _ptr(out, _dp))
        return out

    def set_fixed(self, fixed):
        fx = np.ascontiguousarray(fixed, np.uint8)
        self.lib.orc_set_fixed(self.h, _ptr(fx, _up))

    def simulate(self, dt, warp=True):
        self.lib.orc_simulate(self.h, dt, int(bool(warp)))

    def simulate_converged(self, dt, warp=True, mass_damping=2.0, rtol=1e-6, max_it=10000):
        it = ctypes.c_int(0)
        rr = ctypes.c_double(0.0)
        self.lib.orc_simulate_converged(self.h, dt, int(bool(warp)), mass_damping, rtol, max_it,
                                        ctypes.byref(it), ctypes.byref(rr))
        return it.value, rr.value

    def update_original_coord(self):
        self.lib.orc_update_original_coord(self.h)

    def export_k(self):
        n = self.lib.orc_export_k_count(self.h)
        r = np.zeros(n, np.int32)
        c = np.zeros(n, np.int32)
        v = np.zeros(n, np.float64)
        self.lib.orc_export_k(self.h, _ptr(r, _ip), _ptr(c, _ip), _ptr(v, _dp))
        return r, c, v

    def k_pattern(self):
        nnz = self.lib.orc_k_nnz(self.h)
        rp = np.zeros(self.N + 1, np.int32)
        cols = np.zeros(max(nnz, 1), np.int32)
        self.lib.orc_k_pattern(self.h, _ptr(rp, _ip), _ptr(cols, _ip))
        return rp, cols[:nnz]

    def k_values(self):
        nnz = self.lib.orc_k_nnz(self.h)
        v = np.zeros((max(nnz, 1), 3, 3), np.float64)
        self.lib.orc_k_values(self.h, _ptr(v, _dp))
        return v[:nnz]

    def re(self):
        out = np.zeros((self.T, 3, 3), np.float64)
        self.lib.orc_get_re(self.h, _ptr(out, _dp))
        return out

    def plastic(self):
        out = np.zeros((self.T, 6), np.float64)
        self.lib.orc_get_plastic(self.h, _ptr(out, _dp))
        return out

    def volume(self):
        out = np.zeros(self.T, np.float64)
        self.lib.orc_get_volume(self.h, _ptr(out, _dp))
        return out
