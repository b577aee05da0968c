"""The reference's own hot-path example programs compile unchanged against the
front end.

Each program of the reference checkout's examples/ directory that uses the
skeleton path (the Jacobi solver, Game of Life, heat diffusion, the mean-blur
radius sweep, the pi estimate, and the DA / DM / DC known-answer tests) is
compiled for sm_103a with nvcc, the front end's include directory placed
before the reference's (which still supplies the test helper
include/test_hepers/basic.cpp and the example struct vec3.h), and linked
against libmsl_gb300.so. No source line is changed.

examples/dm_test.cpp does not compile against the reference's own headers
either: it passes four arguments to print_and_doc_runtimes, which takes six
(include/test_hepers/basic.cpp:117). The test checks that this is its only
error with the front end as well.

Skipped when the reference checkout or nvcc is absent (the checkout is not
shipped with this repository). The binaries need a GPU to run; the known
answers these programs check are ported to tests/frontend/frontend_checks.cu
and run by the GPU tests.
"""
import concurrent.futures as cf
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REFERENCE = os.environ.get("MUESLI4_REFERENCE_DIR") or os.path.join(os.path.dirname(ROOT), "reference")
EXAMPLES = os.path.join(REFERENCE, "examples")

PROGRAMS = ["jacobisolver", "gameoflife", "heatdiffusion", "piDA", "da_test", "dc_test", "dc_test_comp",
            "dc_map_stencil_test", "ds_test"] + [f"meanblur{r}" for r in (2, 4, 6, 8, 10, 12, 14, 16, 18, 20)]
BROKEN_IN_REFERENCE = {"dm_test": r"print_and_doc_runtimes"}

nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
pytestmark = [
    pytest.mark.skipif(not os.path.isdir(EXAMPLES), reason="reference checkout not present"),
    pytest.mark.skipif(not os.path.exists(nvcc), reason="nvcc not available"),
]


def build_example(name, out_dir):
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O1", "-std=c++17", "--extended-lambda", "-x", "cu",
           "-w", "-I", os.path.join(ROOT, "muesli4_gb300", "include"), "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(REFERENCE, "include"), os.path.join(EXAMPLES, name + ".cpp"),
           "-L", os.path.join(ROOT, "muesli4_gb300"), "-lmsl_gb300",
           "-Xlinker", "-rpath," + os.path.join(ROOT, "muesli4_gb300"), "-o", os.path.join(out_dir, name)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    return name, r.returncode, r.stdout + r.stderr


@pytest.fixture(scope="module")
def built(tmp_path_factory):
    lib = os.path.join(ROOT, "muesli4_gb300", "libmsl_gb300.so")
    if not os.path.exists(lib):
        from muesli4_gb300 import build as B
        B.build()
    out = str(tmp_path_factory.mktemp("examples"))
    names = PROGRAMS + sorted(BROKEN_IN_REFERENCE)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        results = {n: (rc, log) for n, rc, log in ex.map(lambda n: build_example(n, out), names)}
    return out, results


@pytest.mark.timeout(900)
@pytest.mark.parametrize("name", PROGRAMS)
def test_reference_example_compiles_unchanged(built, name):
    out, results = built
    rc, log = results[name]
    assert rc == 0, log[-3000:]
    assert os.path.exists(os.path.join(out, name))


@pytest.mark.timeout(900)
@pytest.mark.parametrize("name", sorted(BROKEN_IN_REFERENCE))
def test_example_broken_in_the_reference_fails_only_where_the_reference_does(built, name):
    _, results = built
    rc, log = results[name]
    assert rc != 0
    errors = [l for l in log.splitlines() if re.search(r"\berror\b", l) and not re.search(r"errors? detected", l)]
    assert errors and all(re.search(BROKEN_IN_REFERENCE[name], l) for l in errors), errors
