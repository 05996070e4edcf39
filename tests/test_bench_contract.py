"""bench.py on the CPU: the algorithmic byte counts the roofline divides by,
and the reference arm's JSON line (the reference's OpenMP step on the host,
run here at a small size)."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
import bench  # noqa: E402

KERNELS = ("time_increment", "elem_force", "node_update", "elem_kinematics", "elem_material", "finalize")


@pytest.mark.parametrize("precision,per_zone_cycle", [("fp64", 1636), ("split", 837)])
def test_algorithmic_bytes_per_zone_cycle(precision, per_zone_cycle):
    s = 192
    ne, nn = s ** 3, (s + 1) ** 3
    b = bench.algorithmic_bytes(ne, nn, precision)
    assert set(b) == set(KERNELS)
    assert all(v >= 0 for v in b.values())
    assert b["elem_force"] > 0 and b["node_update"] > 0 and b["elem_kinematics"] > 0 and b["elem_material"] > 0
    assert round(sum(b.values()) / ne) == per_zone_cycle


def test_fp64_geometry_cache_bytes_balance():
    """The kinematics kernel writes the 39-word geometry cache that the force
    kernel reads: both kernels' counts carry its 312 bytes per element."""
    ne, nn = 1000, 1331
    with_cache = bench.algorithmic_bytes(ne, nn, "fp64")
    assert with_cache["elem_kinematics"] - (48 * nn + (32 + 24 + 80) * ne) == 312 * ne
    assert with_cache["elem_force"] - (24 * nn + (32 + 48 + 192) * ne) == 312 * ne


def test_reference_arm_line():
    lib = ROOT / "oracle" / "_ref" / "lulesh_ref"
    if not lib.exists():
        pytest.skip("the reference build (oracle/_ref) is absent")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--size", "8",
                        "--steps", "2", "--warmup", "3"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["config"]["workload"] == "sedov_s8_fp64"
    cb = line["cpu_baseline"]
    assert cb["kind"] == "reference" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
