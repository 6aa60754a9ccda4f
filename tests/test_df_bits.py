"""The FP64 <-> (hi, lo) pair conversions the mixed solver does with integer
instructions (otfem_df.h), compiled for the host and checked against long
double arithmetic (tests/cpp/df_bits_test.cpp)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "opentissue_gb300", "csrc")


def test_df_bits(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "df_bits_test")
    subprocess.check_call([cxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "cpp", "df_bits_test.cpp"),
                           "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
