"""The constant-divisor division used by the heat3D functor (x / 6) is
checked against IEEE division for all 2^32 float inputs."""
import ctypes
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_div6_matches_ieee_division_for_every_float(gpu):
    src = os.path.join(HERE, "frontend", "div_check.cu")
    out = os.path.join(HERE, "_build", "libdiv_check.so")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    r = subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-Xcompiler",
                        "-fPIC", "-shared", "-I", os.path.join(ROOT, "muesli4_gb300", "include"), "-o", out, src],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    L = ctypes.CDLL(out)
    mism, first = ctypes.c_ulonglong(), ctypes.c_uint()
    assert L.div6_exhaustive(ctypes.byref(mism), ctypes.byref(first)) == 0
    assert mism.value == 0, f"{mism.value} mismatches, first at bits 0x{first.value:08x}"
