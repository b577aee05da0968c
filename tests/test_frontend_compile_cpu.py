"""The integration path needs no GPU to build: the reference-style example
program compiles for sm_103a against the front end and links against
libmsl_gb300.so with the command the integration guide gives."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.mark.timeout(600)
def test_integration_example_builds(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    lib = os.path.join(ROOT, "muesli4_gb300", "libmsl_gb300.so")
    if not os.path.exists(lib):
        from muesli4_gb300 import build as B
        B.build()
    out = tmp_path / "prog"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "--extended-lambda",
           "-I", os.path.join(ROOT, "muesli4_gb300", "include"), "-I", os.path.join(ROOT, "include"),
           os.path.join(HERE, "frontend", "integration_example.cu"),
           "-L", os.path.join(ROOT, "muesli4_gb300"), "-lmsl_gb300",
           "-Xlinker", "-rpath," + os.path.join(ROOT, "muesli4_gb300"), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    assert out.exists()
