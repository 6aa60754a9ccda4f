"""Python mirror of OpenTissue's fem namespace (OpenTissue/dynamics/fem/fem.h),
running on the GB300 through libotfem_gpu.so.

    mesh = Mesh(tets, coord)                  # fem::Mesh (fem_mesh.h:21-34)
    mesh.fixed[...] = True                    # node m_fixed, before init
    init(mesh, 5e5, 0.33, 1000, 1e30, 0, 0)   # fem::init (fem_init.h:45-65)
    mesh.f_external[:] = ...                  # node m_f_external, every step
    simulate(mesh, 0.01, True)                # fem::simulate (fem_simulate.h:49-113)
    mesh.coord, mesh.velocity                 # node m_coord / m_velocity

Node fields live in host numpy arrays, as the reference's nodes do; simulate()
uploads coord, velocity and f_external, runs the step on the device and
downloads coord and velocity.  Errors raise capi.OtfemError, like the
reference's std::out_of_range / std::invalid_argument (t4mesh_t4mesh.h:139-164).
"""
import ctypes

import numpy as np

from . import capi

_dp = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int32)
_u8p = ctypes.POINTER(ctypes.c_uint8)


def _p(a, t):
    return a.ctypes.data_as(t)


def generate_blocks(I, J, K, block_width, block_height, block_depth):
    """t4mesh::generate_blocks (t4mesh_block_generator.h:32-110).

    Returns (tets int32 [5*I*J*K, 4], coord float64 [(I+1)(J+1)(K+1), 3]).
    Node (x, y, z) has index (x*(J+1)+y)*(K+1)+z and coordinate
    (w*x, h*z, d*y); each block splits into 5 tets with the split alternating
    on (i+j+k) parity so neighbouring blocks share faces.
    """
    x, y, z = np.meshgrid(np.arange(I + 1), np.arange(J + 1), np.arange(K + 1), indexing="ij")
    coord = np.stack([block_width * x.ravel().astype(np.float64), block_height * z.ravel().astype(np.float64),
                      block_depth * y.ravel().astype(np.float64)], axis=1)
    i, j, k = np.meshgrid(np.arange(I), np.arange(J), np.arange(K), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    p0 = (i * (J + 1) + j) * (K + 1) + k
    p1 = p0 + 1
    p3 = ((i + 1) * (J + 1) + j) * (K + 1) + k
    p2 = p3 + 1
    p7 = ((i + 1) * (J + 1) + (j + 1)) * (K + 1) + k
    p6 = p7 + 1
    p4 = (i * (J + 1) + (j + 1)) * (K + 1) + k
    p5 = p4 + 1
    odd = np.stack([p1, p2, p6, p3, p3, p6, p4, p7, p1, p4, p6, p5, p1, p3, p4, p0, p1, p6, p4, p3], 1)
    even = np.stack([p2, p0, p5, p1, p2, p7, p0, p3, p2, p5, p7, p6, p0, p7, p5, p4, p2, p0, p7, p5], 1)
    tets = np.where(((i + j + k) % 2 == 1)[:, None], odd, even).reshape(-1, 4).astype(np.int32)
    return tets, coord


def tetgen_read(basename):
    """t4mesh::tetgen_read (t4mesh_tetgen_read.h:30-136): a TetGen mesh from
    `basename`.node and `basename`.ele.

    .node: first line `<#points> <dimension 3> <#attributes> <boundary markers 0/1>`,
    then `<point id> <x> <y> <z> [attributes] [marker]`.  .ele: first line
    `<#tets> <points per tet 4> <#attributes (at most 1, the region)>`, then
    `<tet id> <p0> <p1> <p2> <p3> [attribute]`, the points given by their ids
    in the .node file (any base).  '#' starts a comment, as in TetGen's
    files.  Returns (tets int32 [T, 4], coord float64 [N, 3]), nodes in file
    order; raises ValueError where the reference returns false.
    """
    def numbers(path):
        try:
            with open(path) as f:
                return [tok for line in f for tok in line.split('#', 1)[0].split()]
        except OSError as e:
            raise ValueError(f"unable to open file '{path}'") from e

    tok = numbers(basename + ".node")
    n, dim, nattr, has_marker = int(tok[0]), int(tok[1]), int(tok[2]), int(tok[3])
    if dim != 3:
        raise ValueError("TetGen .node files of dimension 3 only")
    width = 4 + nattr + (1 if has_marker else 0)
    rows = np.array(tok[4:4 + n * width], dtype=np.float64).reshape(n, width)
    ids = rows[:, 0].astype(np.int64)
    coord = np.ascontiguousarray(rows[:, 1:4])
    index = {int(k): i for i, k in enumerate(ids)}
    tok = numbers(basename + ".ele")
    t, per, nattr = int(tok[0]), int(tok[1]), int(tok[2])
    if per != 4:
        raise ValueError("We only support tetrahedra with 4 points")
    if nattr > 1:
        raise ValueError("We only support tetrahedra with 1 region")
    rows = np.array(tok[3:3 + t * (5 + nattr)], dtype=np.float64).reshape(t, 5 + nattr)
    try:
        tets = np.array([[index[int(k)] for k in r[1:5]] for r in rows], dtype=np.int32).reshape(-1, 4)
    except KeyError as e:
        raise ValueError(f"tetrahedron refers to an unknown point {e}") from e
    return tets, coord


def tetgen_write(basename, tets, coord):
    """Writes a mesh as TetGen .node/.ele files (1-based ids), the format
    tetgen_read reads."""
    with open(basename + ".node", "w") as f:
        f.write(f"{len(coord)} 3 0 0\n")
        for i, (x, y, z) in enumerate(coord):
            f.write(f"{i + 1} {float(x)!r} {float(y)!r} {float(z)!r}\n")
    with open(basename + ".ele", "w") as f:
        f.write(f"{len(tets)} 4 0\n")
        for i, t in enumerate(tets):
            f.write(f"{i + 1} {t[0] + 1} {t[1] + 1} {t[2] + 1} {t[3] + 1}\n")


class Mesh:
    """fem::Mesh: host node fields plus the device-resident mesh handle."""

    def __init__(self, tets, coord, model_coord=None, fixed=None, stream=None):
        self._lib = capi.lib()
        self.tets = np.ascontiguousarray(tets, np.int32).reshape(-1, 4)
        self.coord = np.ascontiguousarray(coord, np.float64).reshape(-1, 3).copy()
        n = self.coord.shape[0]
        self.model_coord = (self.coord.copy() if model_coord is None
                            else np.ascontiguousarray(model_coord, np.float64).reshape(-1, 3).copy())
        self.fixed = np.zeros(n, bool) if fixed is None else np.asarray(fixed, bool).copy()
        self.velocity = np.zeros((n, 3))
        self.f_external = np.zeros((n, 3))
        self.mass = np.zeros(n)
        self._stream = stream
        self.handle = None
        self._created_fixed = None

    @property
    def num_nodes(self):
        return self.coord.shape[0]

    @property
    def num_tets(self):
        return self.tets.shape[0]

    def _ensure_handle(self):
        if self.handle is not None:
            return
        fx = self.fixed.astype(np.uint8)
        desc = capi.MeshDesc(self.num_nodes, self.num_tets, _p(self.tets, _i32p), _p(self.coord, _dp),
                             _p(self.model_coord, _dp), _p(fx, _u8p))
        h = ctypes.c_void_p()
        stream = ctypes.c_void_p(self._stream) if self._stream is not None else None
        capi.check(self._lib.otfem_create(ctypes.byref(desc), stream, ctypes.byref(h)))
        self.handle = h

    def close(self):
        if self.handle is not None:
            self._lib.otfem_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- transfers ------------------------------------------------------
    def upload(self, *fields):
        names = {capi.COORD: "coord", capi.MODEL_COORD: "model_coord", capi.VELOCITY: "velocity",
                 capi.F_EXTERNAL: "f_external"}
        for f in fields:
            a = np.ascontiguousarray(getattr(self, names[f]), np.float64)
            capi.check(self._lib.otfem_set_nodes(self.handle, f, _p(a, _dp), a.size))

    def download(self, field):
        out = np.zeros(self.num_nodes if field == capi.MASS else (self.num_nodes, 3))
        capi.check(self._lib.otfem_get_nodes(self.handle, field, _p(out, _dp), out.size))
        return out

    def orientations(self):
        out = np.zeros((self.num_tets, 3, 3))
        capi.check(self._lib.otfem_get_orientations(self.handle, _p(out, _dp)))
        return out

    def plastic(self):
        out = np.zeros((self.num_tets, 6))
        capi.check(self._lib.otfem_get_plastic(self.handle, _p(out, _dp)))
        return out

    def k_pattern(self):
        nnz = ctypes.c_int64()
        capi.check(self._lib.otfem_k_pattern(self.handle, ctypes.byref(nnz), None, None))
        rp = np.zeros(self.num_nodes + 1, np.int32)
        cols = np.zeros(max(nnz.value, 1), np.int32)
        capi.check(self._lib.otfem_k_pattern(self.handle, ctypes.byref(nnz), _p(rp, _i32p), _p(cols, _i32p)))
        return rp, cols[:nnz.value]

    def k_values(self):
        nnz = ctypes.c_int64()
        capi.check(self._lib.otfem_k_pattern(self.handle, ctypes.byref(nnz), None, None))
        v = np.zeros((max(nnz.value, 1), 3, 3))
        capi.check(self._lib.otfem_k_values(self.handle, _p(v, _dp)))
        return v[:nnz.value]


def init(mesh, young, poisson, density, c_yield, c_creep, c_max):
    """fem::init (fem_init.h:45-65).  Fixed flags must be set before this call."""
    mesh._ensure_handle()
    fx = mesh.fixed.astype(np.uint8)
    capi.check(mesh._lib.otfem_set_fixed(mesh.handle, _p(fx, _u8p), fx.size))
    mesh.upload(capi.COORD, capi.MODEL_COORD)
    capi.check(mesh._lib.otfem_init(mesh.handle, young, poisson, density, c_yield, c_creep, c_max))
    mesh.mass = mesh.download(capi.MASS)


def simulate(mesh, time_step, use_stiffness_warping, params=None):
    """fem::simulate (fem_simulate.h:49-113).  Returns the step's StepStats.

    With params None the reference's fixed settings are used (20-iteration CG,
    mass damping 2.0); pass capi.default_params(solver=capi.SOLVER_MIXED, ...)
    for the matrix-free relative-residual solver.
    """
    if mesh.handle is None:
        raise capi.OtfemError(capi.ERR_NOT_INITIALIZED, "fem.init has not been called")
    fx = mesh.fixed.astype(np.uint8)
    capi.check(mesh._lib.otfem_set_fixed(mesh.handle, _p(fx, _u8p), fx.size))
    mesh.upload(capi.COORD, capi.VELOCITY, capi.F_EXTERNAL)
    st = capi.StepStats()
    p = params if params is not None else capi.default_params()
    capi.check(mesh._lib.otfem_simulate_ex(mesh.handle, time_step, int(bool(use_stiffness_warping)),
                                           ctypes.byref(p), ctypes.byref(st)))
    mesh.coord = mesh.download(capi.COORD)
    mesh.velocity = mesh.download(capi.VELOCITY)
    mesh.f_external = mesh.download(capi.F_EXTERNAL)
    return st


def update_original_coord(mesh):
    """fem::update_original_coord (fem_update_original_coord.h:28-33)."""
    mesh.model_coord = mesh.coord.copy()
    if mesh.handle is not None:
        mesh.upload(capi.COORD)
        capi.check(mesh._lib.otfem_update_original_coord(mesh.handle))


def export_K(mesh):
    """fem::export_K (fem_export_k.h:23-68) as (rows, cols, values) triplets in
    the reference's push_back order: row by row, fixed rows as 1.0 on the
    diagonal, free rows over the non-fixed columns of K_row in key order."""
    nnz = ctypes.c_int64()
    capi.check(mesh._lib.otfem_export_k_csr(mesh.handle, ctypes.byref(nnz), None, None, None))
    n = nnz.value
    rp = np.zeros(mesh.num_nodes + 1, np.int32)
    cols = np.zeros(max(n, 1), np.int32)
    vals = np.zeros((max(n, 1), 3, 3))
    capi.check(mesh._lib.otfem_export_k_csr(mesh.handle, ctypes.byref(nnz), _p(rp, _i32p), _p(cols, _i32p),
                                            _p(vals, _dp)))
    rows, cs, vs = [], [], []
    for i in range(mesh.num_nodes):
        for r in range(3):
            row = 3 * i + r
            if mesh.fixed[i]:
                rows.append(row)
                cs.append(row)
                vs.append(1.0)
                continue
            for q in range(rp[i], rp[i + 1]):
                j = cols[q]
                for c in range(3):
                    rows.append(row)
                    cs.append(3 * j + c)
                    vs.append(vals[q, r, c])
    return np.array(rows, np.int32), np.array(cs, np.int32), np.array(vs)


class SurfaceBinding:
    """t4mesh::mesh_coupling (t4mesh_mesh_coupling.h): points bound to the
    tets of a mesh that embed them, moved with the deformed tets.  The
    binding keeps a reference to the mesh, whose handle must outlive it."""

    def __init__(self, mesh, points):
        self.lib = capi.lib()
        self.mesh = mesh
        pts = np.ascontiguousarray(points, np.float64).reshape(-1, 3)
        self.count = pts.shape[0]
        self.s = ctypes.c_void_p()
        bound = ctypes.c_int64()
        capi.check(self.lib.otfem_surface_bind(mesh.handle, _p(pts, _dp), self.count, ctypes.byref(self.s),
                                               ctypes.byref(bound)))
        self.bound = bound.value

    def update(self):
        """update_surface: the points at their tets' current coordinates."""
        out = np.zeros((self.count, 3))
        capi.check(self.lib.otfem_surface_update(self.s, _p(out, _dp), self.count))
        return out

    def binding(self):
        """(tet per point, -1 if unbound; barycentric (w1, w2, w3) per point)."""
        tet = np.zeros(self.count, np.int32)
        bary = np.zeros((self.count, 3))
        capi.check(self.lib.otfem_surface_binding(self.s, _p(tet, _i32p), _p(bary, _dp), self.count))
        return tet, bary

    def close(self):
        if self.s:
            self.lib.otfem_surface_destroy(self.s)
            self.s = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def bind_surface(mesh, points):
    """t4mesh::mesh_coupling::bind_surface (t4mesh_mesh_coupling.h:129-236)
    against the mesh's current coordinates."""
    return SurfaceBinding(mesh, points)


def update_surface(binding):
    """t4mesh::mesh_coupling::update_surface (t4mesh_mesh_coupling.h:238-275)."""
    return binding.update()
