"""The drop-in C++ headers (include/OpenTissue/dynamics/fem) and the plain-C
ABI, compiled as a user of the reference would compile them."""
import hashlib
import os
import subprocess

import numpy as np
import pytest

from helpers import golden, step_hash
from opentissue_gb300 import build as ext_build
from oracle.build import REFERENCE_ROOT as REF_ROOT

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CPP = os.path.join(ROOT, "tests", "cpp")
HAVE_REF = os.path.exists(os.path.join(REF_ROOT, "OpenTissue", "dynamics", "fem", "fem.h"))
LIBDIR = os.path.dirname(ext_build.LIB)


def _link_flags():
    return ["-L", LIBDIR, "-lotfem_gpu", f"-Wl,-rpath,{LIBDIR}"]


def compile_demo(out_dir, core="stub"):
    ext_build.build()
    exe = os.path.join(out_dir, f"fem_dropin_demo_{core}")
    inc = ["-I", os.path.join(ROOT, "include")]
    if core == "stub":
        inc += ["-I", os.path.join(CPP, "ot_core")]
    else:
        from oracle import build as obuild
        obuild.build_reference()
        inc += ["-I", os.path.join(ROOT, "oracle", "_ref", "include"), "-I", REF_ROOT,
                "-I", os.path.join(ROOT, "oracle", "ref", "boost_shim")]
    cmd = ["g++", "-std=c++11", "-O2", "-w", *inc, os.path.join(CPP, "fem_dropin_demo.cpp"), "-o", exe,
           *_link_flags()]
    subprocess.check_call(cmd)
    return exe


def compile_c_consumer(out_dir):
    ext_build.build()
    exe = os.path.join(out_dir, "capi_consumer")
    subprocess.check_call(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                           os.path.join(CPP, "capi_consumer.c"), "-o", exe, *_link_flags()])
    return exe


def test_c_consumer_compiles_and_links(tmp_path):
    assert os.path.exists(compile_c_consumer(str(tmp_path)))


def test_dropin_compiles_against_stub_core(tmp_path):
    assert os.path.exists(compile_demo(str(tmp_path), "stub"))


@pytest.mark.skipif(not HAVE_REF, reason="OpenTissue source tree not present on this machine")
def test_dropin_compiles_against_real_opentissue_core(tmp_path):
    # the drop-in fem headers with the reference's own t4mesh, math types and
    # Boost-dependent utilities (through the oracle's Boost shim)
    assert os.path.exists(compile_demo(str(tmp_path), "real"))


def _run_demo(exe, tmp, dims, steps, solver, export=False):
    out = os.path.join(tmp, f"traj_{solver}.bin")
    args = [exe, *map(str, dims), str(steps), solver, out]
    if export:
        args.append(os.path.join(tmp, "export.bin"))
    subprocess.check_call(args)
    I, J, K = dims
    n = (I + 1) * (J + 1) * (K + 1)
    data = np.fromfile(out, np.float64).reshape(steps, 2, n, 3)
    return data


@pytest.mark.gpu
def test_dropin_cpp_bitwise_vs_reference(gpu, tmp_path):
    g = golden("config1")
    exe = compile_demo(str(tmp_path), "stub")
    data = _run_demo(exe, str(tmp_path), (10, 4, 4), 100, "sequential", export=True)
    assert [step_hash(d[0], d[1]) for d in data] == list(g["hashes"])
    raw = np.fromfile(os.path.join(str(tmp_path), "export.bin"),
                      dtype=np.dtype([("r", "<i4"), ("c", "<i4"), ("v", "<f8")]))
    assert np.array_equal(raw["r"], g["export_rows_1"]) and np.array_equal(raw["c"], g["export_cols_1"])
    assert np.array_equal(raw["v"], g["export_vals_1"])


@pytest.mark.gpu
@pytest.mark.parametrize("core", ["stub", "real"])
def test_dropin_detail_steps_bitwise_vs_reference(gpu, tmp_path, core):
    """The reference's own step sequence written as host code against the
    drop-in fem::detail functions (fem_simulate.h:94-111): every step's
    positions and velocities bit-identical to the reference's fem::simulate
    over 100 steps, and after step 1 the host m_K_row maps filled with the
    reference's keys and values."""
    if core == "real" and not HAVE_REF:
        pytest.skip("OpenTissue source tree not present on this machine")
    g = golden("config1")
    exe = compile_demo(str(tmp_path), core)
    data = _run_demo(exe, str(tmp_path), (10, 4, 4), 100, "detail", export=True)
    assert [step_hash(d[0], d[1]) for d in data] == list(g["hashes"])
    raw = np.fromfile(os.path.join(str(tmp_path), "export.bin"),
                      dtype=np.dtype([("r", "<i4"), ("c", "<i4"), ("v", "<f8", (3, 3))]))
    rp, cols = g["k_row_ptr"], g["k_cols"]
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    assert np.array_equal(raw["r"], rows) and np.array_equal(raw["c"], cols)
    assert np.array_equal(raw["v"], g["k_values_1"])


@pytest.mark.gpu
def test_dropin_cpp_default_and_mixed_solvers(gpu, oracle, tmp_path):
    g = golden("config1")
    exe = compile_demo(str(tmp_path), "stub")
    data = _run_demo(exe, str(tmp_path), (10, 4, 4), 20, "reference")
    disp = np.abs(g["x_10"] - g["coord"]).max()
    assert np.abs(data[9, 0] - g["x_10"]).max() <= 2e-5 * disp
    from helpers import run_oracle
    _, ref = run_oracle(oracle, g["tets"], g["coord"], g["fixed"], 10, converged=True)
    x_ref = ref[-1][0]
    for solver in ("mixed", "projected", "extrapolated"):
        data = _run_demo(exe, str(tmp_path), (10, 4, 4), 10, solver)
        assert np.abs(data[-1, 0] - x_ref).max() <= 1e-5 * np.abs(x_ref - g["coord"]).max(), solver


@pytest.mark.gpu
def test_c_consumer_runs(gpu, oracle, tmp_path):
    exe = compile_c_consumer(str(tmp_path))
    out = subprocess.check_output([exe], text=True).split()
    tets = np.array([[0, 1, 2, 3]], np.int32)
    coord = np.array([[0, 0, 0], [0.1, 0, 0], [0, 0.1, 0], [0, 0, 0.1]], float)
    o = oracle.OracleMesh(tets, coord, coord, np.array([1, 0, 0, 0], np.uint8))
    o.init(5e5, 0.33, 1000.0, 1e30, 0.0, 0.0)
    f = np.zeros((4, 3))
    f[1, 1] = -9.81
    o.set(oracle.F_EXTERNAL, f)
    o.simulate(0.01, True)
    x = o.get(oracle.COORD)[1]
    assert np.allclose([float(v) for v in out], x, rtol=0, atol=1e-15)
