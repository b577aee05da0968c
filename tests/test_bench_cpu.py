"""bench.py's JSON contract where it runs without a GPU: the reference arm
(the CPU implementation of the path, timed on a bounded sample) and the
launch bookkeeping of the Life and heat3D parts."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_life_launch_count():
    # one cell-by-cell generation, then ceil((steps - 1) / depth) packed launches
    assert bench.life_launches(200, 32) == 8
    assert bench.life_launches(200, 1) == 200
    assert bench.life_launches(200, 8) == 26
    assert bench.life_launches(1, 32) == 1


def test_heat_launch_count():
    # two sweeps per launch on the z-marching kernel, an odd last sweep alone
    assert bench.heat_launches(100, 2) == 50
    assert bench.heat_launches(101, 2) == 51
    assert bench.heat_launches(100, 1) == 100
    assert bench.heat_launches(1, 2) == 1


@pytest.mark.timeout(300)
def test_reference_arm_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == "stencil GCUPS" and line["unit"] == "GCUPS"
    assert line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] == 3
    assert line["value"] > 0
    cpu = line["cpu_baseline"]
    assert cpu["kind"] in ("port", "reference") and cpu["cores"] >= 1 and cpu["sample"]
    assert cpu["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert line["config"]["workload"].startswith("stencil radius sweep")
