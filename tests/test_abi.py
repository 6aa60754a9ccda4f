"""The C-ABI library: it loads, exports every function declared in
include/otfem_gpu.h, and rejects bad arguments before touching a GPU."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from opentissue_gb300 import build, capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "otfem_gpu.h")


@pytest.fixture(scope="module")
def lib():
    build.build()
    return capi.lib()


def declared_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^OTFEM_API\s+[\w\s\*]+?\b(otfem_\w+)\(", src, re.M)))


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 20
    out = subprocess.check_output(["nm", "-D", "--defined-only", build.LIB], text=True)
    exported = set(re.findall(r"\bT (otfem_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        getattr(lib, n)
    # the ctypes declarations cover the same set
    assert sorted(capi.SIGNATURES) == names


def test_abi_version_and_defaults(lib):
    assert lib.otfem_abi_version() == 8
    p = capi.default_params()
    assert p.solver == capi.SOLVER_REFERENCE
    assert p.mass_damping == 2.0 and p.min_iterations == 20 and p.max_iterations == 20
    assert p.rtol == 1e-6 and p.refresh_period == 16 and p.graph == 1
    assert p.preconditioner == capi.PRECONDITIONER_JACOBI
    assert p.warm_history == 4 and capi.MAX_WARM_HISTORY == 8


def _create(lib, tets, coord):
    tets = np.ascontiguousarray(tets, np.int32)
    coord = np.ascontiguousarray(coord, np.float64)
    desc = capi.MeshDesc(coord.shape[0], tets.shape[0], tets.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                         coord.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None, None)
    h = ctypes.c_void_p()
    rc = lib.otfem_create(ctypes.byref(desc), None, ctypes.byref(h))
    return rc, h


def test_create_rejects_bad_meshes_on_host(lib):
    coord = np.zeros((4, 3))
    rc, h = _create(lib, [[0, 1, 2, 4]], coord)  # index out of range (t4mesh_t4mesh.h:139-144)
    assert rc == capi.ERR_BAD_MESH and not h.value
    assert "out of range" in capi.last_error()
    rc, h = _create(lib, [[0, 1, 1, 3]], coord)  # repeated node
    assert rc == capi.ERR_BAD_MESH and "repeats" in capi.last_error()
    rc, h = _create(lib, [[0, -1, 2, 3]], coord)
    assert rc == capi.ERR_BAD_MESH
    assert lib.otfem_create(None, None, None) == capi.ERR_INVALID_ARGUMENT


def test_null_handles_are_rejected(lib):
    assert lib.otfem_init(None, 1.0, 0.3, 1.0, 0.0, 0.0, 0.0) == capi.ERR_INVALID_ARGUMENT
    assert lib.otfem_simulate(None, 0.01, 1) == capi.ERR_INVALID_ARGUMENT
    assert lib.otfem_update_original_coord(None) == capi.ERR_INVALID_ARGUMENT
    assert lib.otfem_destroy(None) == capi.OK
    with pytest.raises(capi.OtfemError):
        capi.check(lib.otfem_simulate(None, 0.01, 1))


def test_product_has_no_oracle_dependency():
    # the shipped library and package never reference the oracle
    out = subprocess.check_output(["nm", "-D", build.LIB], text=True)
    assert "orc_" not in out
    for root, _, files in os.walk(os.path.join(ROOT, "opentissue_gb300")):
        for f in files:
            if f.endswith((".py", ".cu", ".h", ".cuh")):
                txt = open(os.path.join(root, f)).read()
                assert "import oracle" not in txt and "from oracle" not in txt and "pyoracle" not in txt
