"""ctypes declarations of the C ABI in include/otfem_gpu.h.

Loads the in-tree libotfem_gpu.so (opentissue_gb300/_build/).  There is no
fallback: if the library is missing or cannot be loaded, ``lib()`` raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libotfem_gpu.so")

# status codes
OK = 0
WARN_NOT_CONVERGED = 1
ERR_INVALID_ARGUMENT = -1
ERR_BAD_MESH = -2
ERR_NOT_INITIALIZED = -3
ERR_CUDA = -4
ERR_NONFINITE = -5
ERR_TIMEOUT = -6
ERR_OUT_OF_MEMORY = -7
ERR_UNSUPPORTED = -8

# node fields
COORD, MODEL_COORD, VELOCITY, F_EXTERNAL, MASS, F0, B, NODE_STIFFNESS = range(8)
# solvers
SOLVER_REFERENCE, SOLVER_MIXED, SOLVER_FP64 = 0, 1, 2
WARM_START_PREVIOUS, WARM_START_LEARNED, WARM_START_PROJECTED, WARM_START_EXTRAPOLATED = 0, 1, 2, 3
MAX_WARM_HISTORY = 8
PRECONDITIONER_NONE, PRECONDITIONER_JACOBI = 0, 1
PHASE_ORIENT, PHASE_SOLVE = 1, 2
# the steps of fem::simulate one at a time (otfem_reference_stage)
(STAGE_CLEAR_STIFFNESS_ASSEMBLY, STAGE_UPDATE_ORIENTATION, STAGE_RESET_ORIENTATION, STAGE_STIFFNESS_ASSEMBLY,
 STAGE_ADD_PLASTICITY_FORCE, STAGE_DYNAMICS_ASSEMBLY, STAGE_CONJUGATE_GRADIENTS, STAGE_POSITION_UPDATE) = range(1, 9)
NUM_APPLY_VARIANTS = 4
# learned warm start: network state = 9731 weights + 42 normalisation values
MLP_STATE_SIZE = 9773
MLP_NUM_WEIGHTS = 9731


class SolverParams(ctypes.Structure):
    _fields_ = [
        ("solver", ctypes.c_int),
        ("mass_damping", ctypes.c_double),
        ("min_iterations", ctypes.c_int),
        ("max_iterations", ctypes.c_int),
        ("rtol", ctypes.c_double),
        ("refresh_period", ctypes.c_int),
        ("sequential_dots", ctypes.c_int),
        ("warm_start", ctypes.c_int),
        ("graph", ctypes.c_int),
        ("preconditioner", ctypes.c_int),
        ("warm_history", ctypes.c_int),
    ]


class StepStats(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int),
        ("status", ctypes.c_int),
        ("rel_residual", ctypes.c_double),
        ("initial_rel_residual", ctypes.c_double),
        ("bnorm", ctypes.c_double),
        ("applies", ctypes.c_int),
    ]


class MeshDesc(ctypes.Structure):
    _fields_ = [
        ("num_nodes", ctypes.c_int32),
        ("num_tets", ctypes.c_int32),
        ("tets", ctypes.POINTER(ctypes.c_int32)),
        ("coord", ctypes.POINTER(ctypes.c_double)),
        ("model_coord", ctypes.POINTER(ctypes.c_double)),
        ("fixed", ctypes.POINTER(ctypes.c_uint8)),
    ]


class OtfemError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"otfem error {code}: {msg}")
        self.code = code


_lib = None
_dp = ctypes.POINTER(ctypes.c_double)
_i32p = ctypes.POINTER(ctypes.c_int32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_fp = ctypes.POINTER(ctypes.c_float)
_h = ctypes.c_void_p

# every exported symbol with (restype, argtypes); test_abi checks this list
# against include/otfem_gpu.h
SIGNATURES = {
    "otfem_default_params": (None, [ctypes.POINTER(SolverParams)]),
    "otfem_last_error": (ctypes.c_char_p, []),
    "otfem_abi_version": (ctypes.c_int, []),
    "otfem_create": (ctypes.c_int, [ctypes.POINTER(MeshDesc), ctypes.c_void_p, ctypes.POINTER(_h)]),
    "otfem_destroy": (ctypes.c_int, [_h]),
    "otfem_num_nodes": (ctypes.c_int, [_h, _i32p]),
    "otfem_num_tets": (ctypes.c_int, [_h, _i32p]),
    "otfem_init": (ctypes.c_int, [_h] + [ctypes.c_double] * 6),
    "otfem_set_nodes": (ctypes.c_int, [_h, ctypes.c_int, _dp, ctypes.c_int64]),
    "otfem_get_nodes": (ctypes.c_int, [_h, ctypes.c_int, _dp, ctypes.c_int64]),
    "otfem_get_nodes_async": (ctypes.c_int, [_h, ctypes.c_int, _dp, ctypes.c_int64]),
    "otfem_set_nodes_device": (ctypes.c_int, [_h, ctypes.c_int, ctypes.c_void_p, ctypes.c_int64]),
    "otfem_get_nodes_device": (ctypes.c_int, [_h, ctypes.c_int, ctypes.c_void_p, ctypes.c_int64]),
    "otfem_set_fixed": (ctypes.c_int, [_h, _u8p, ctypes.c_int64]),
    "otfem_simulate": (ctypes.c_int, [_h, ctypes.c_double, ctypes.c_int]),
    "otfem_simulate_ex": (ctypes.c_int, [_h, ctypes.c_double, ctypes.c_int, ctypes.POINTER(SolverParams),
                                         ctypes.POINTER(StepStats)]),
    "otfem_simulate_phase": (ctypes.c_int, [_h, ctypes.c_double, ctypes.c_int, ctypes.POINTER(SolverParams),
                                            ctypes.c_int]),
    "otfem_simulate_host": (ctypes.c_int, [_h, ctypes.c_double, ctypes.c_int, ctypes.POINTER(SolverParams),
                                           ctypes.POINTER(StepStats), _dp, _dp, _dp]),
    "otfem_last_stats": (ctypes.c_int, [_h, ctypes.POINTER(StepStats)]),
    "otfem_synchronize": (ctypes.c_int, [_h]),
    "otfem_update_original_coord": (ctypes.c_int, [_h]),
    "otfem_export_k_csr": (ctypes.c_int, [_h, _i64p, _i32p, _i32p, _dp]),
    "otfem_k_pattern": (ctypes.c_int, [_h, _i64p, _i32p, _i32p]),
    "otfem_k_values": (ctypes.c_int, [_h, _dp]),
    "otfem_get_orientations": (ctypes.c_int, [_h, _dp]),
    "otfem_get_plastic": (ctypes.c_int, [_h, _dp]),
    "otfem_get_volumes": (ctypes.c_int, [_h, _dp]),
    "otfem_apply_operator": (ctypes.c_int, [_h, ctypes.c_int, ctypes.c_double, ctypes.c_double, _dp, _dp]),
    "otfem_apply_operator_noalloc": (ctypes.c_int, [_h, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                                    ctypes.c_void_p, ctypes.c_void_p]),
    "otfem_apply_sweeps": (ctypes.c_int, [_h, ctypes.c_int, ctypes.c_double, ctypes.c_int32]),
    "otfem_solver_trace": (ctypes.c_int, [_h, _dp, ctypes.c_int32, _i32p]),
    "otfem_solver_phases": (ctypes.c_int, [_h, _dp]),
    "otfem_check_wait_timeout": (ctypes.c_int, [_h, ctypes.c_int64, ctypes.POINTER(ctypes.c_int32)]),
    "otfem_surface_bind": (ctypes.c_int, [_h, _dp, ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p), _i64p]),
    "otfem_surface_update": (ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.c_int64]),
    "otfem_surface_update_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]),
    "otfem_surface_binding": (ctypes.c_int, [ctypes.c_void_p, _i32p, _dp, ctypes.c_int64]),
    "otfem_surface_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "otfem_tuning": (ctypes.c_int, [_h, _i32p, _dp]),
    "otfem_set_apply_variant": (ctypes.c_int, [_h, ctypes.c_int32]),
    "otfem_tuning_search": (ctypes.c_int, [_h, ctypes.c_int32, _i32p, _i32p, _i32p, _dp, _i32p]),
    "otfem_set_apply_shape": (ctypes.c_int, [_h, ctypes.c_int32, ctypes.c_int32]),
    "otfem_a_values": (ctypes.c_int, [_h, _dp]),
    "otfem_reference_stage": (ctypes.c_int, [_h, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                             ctypes.c_int32]),
    "otfem_host_alloc": (ctypes.c_int, [ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]),
    "otfem_host_free": (ctypes.c_int, [ctypes.c_void_p]),
    "otfem_launch_count": (ctypes.c_int, [_h, _i64p]),
    "otfem_solver_shape": (ctypes.c_int, [_h, _i32p, _i32p]),
    "otfem_batch_create": (ctypes.c_int, [ctypes.POINTER(MeshDesc), ctypes.c_int32, ctypes.c_void_p,
                                          ctypes.POINTER(_h)]),
    "otfem_batch_init": (ctypes.c_int, [_h, _dp, _dp, _dp, ctypes.c_double, ctypes.c_double, ctypes.c_double]),
    "otfem_batch_layout": (ctypes.c_int, [_h, _i32p, _i32p, _i32p]),
    "otfem_batch_stats": (ctypes.c_int, [_h, _i32p, _i32p, _dp, _dp]),
    "otfem_mlp_create": (ctypes.c_int, [ctypes.c_int64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_void_p)]),
    "otfem_mlp_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "otfem_mlp_get_state": (ctypes.c_int, [ctypes.c_void_p, _fp, ctypes.c_int64]),
    "otfem_mlp_set_state": (ctypes.c_int, [ctypes.c_void_p, _fp, ctypes.c_int64]),
    "otfem_set_collect": (ctypes.c_int, [_h, ctypes.c_int32]),
    "otfem_get_features": (ctypes.c_int, [_h, _fp, ctypes.c_int64]),
    "otfem_mlp_add_samples": (ctypes.c_int, [ctypes.c_void_p, _h, ctypes.c_double, ctypes.c_uint64, _i64p]),
    "otfem_mlp_num_samples": (ctypes.c_int, [ctypes.c_void_p, _i64p]),
    "otfem_mlp_clear_samples": (ctypes.c_int, [ctypes.c_void_p]),
    "otfem_mlp_fit_normalization": (ctypes.c_int, [ctypes.c_void_p]),
    "otfem_mlp_train": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                       ctypes.c_uint64, _dp]),
    "otfem_mlp_evaluate": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "otfem_mlp_gradient": (ctypes.c_int, [ctypes.c_void_p, _fp, _fp, ctypes.c_int64, _dp, _fp]),
    "otfem_mlp_predict": (ctypes.c_int, [ctypes.c_void_p, _fp, ctypes.c_int64, _fp]),
    "otfem_set_mlp": (ctypes.c_int, [_h, ctypes.c_void_p]),
    "otfem_set_warm_start_smoothing": (ctypes.c_int, [_h, ctypes.c_int32]),
}


def lib(path=None):
    """Loads libotfem_gpu.so and declares every exported function."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"libotfem_gpu.so is not built ({p}); run __graft_entry__.build()")
    handle = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(handle, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = handle
    return handle


def last_error():
    return lib().otfem_last_error().decode(errors="replace")


def check(rc, allow_warning=True):
    if rc < 0 or (rc > 0 and not allow_warning):
        raise OtfemError(rc, last_error())
    return rc


def default_params(**overrides):
    p = SolverParams()
    lib().otfem_default_params(ctypes.byref(p))
    for k, v in overrides.items():
        setattr(p, k, v)
    return p
