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


@pytest.mark.parametrize("precision,per_zone_cycle", [("fp64", 827.3), ("split", 635.3)])
def test_step_bytes_per_zone_cycle(precision, per_zone_cycle):
    """The step's own compulsory traffic (K1 + K2 + K3): 616 E + 208 N bytes
    per cycle in FP64, 424 E + 208 N with FP32 corner forces."""
    s = 192
    ne, nn = s ** 3, (s + 1) ** 3
    b = bench.step_bytes(ne, nn, precision)
    assert set(b) == {"K1", "K2", "K3"}
    assert b["K1"] == 48 * nn + (272 if precision == "fp64" else 176) * ne
    assert round(sum(b.values()) / ne, 1) == per_zone_cycle
    # every kernel of this library maps onto one of the three
    assert set(bench.SECTION8_KERNELS.values()) == set(b)


def test_design_adds_bytes_over_the_step():
    """The library's kernels move at least the step's compulsory bytes; the
    FP64 surplus includes the geometry cache's 624 bytes per zone-cycle."""
    ne, nn = 50 ** 3, 51 ** 3
    for prec in ("fp64", "split"):
        design = sum(bench.algorithmic_bytes(ne, nn, prec).values())
        step = sum(bench.step_bytes(ne, nn, prec).values())
        assert design >= step
    assert (sum(bench.algorithmic_bytes(ne, nn, "fp64").values()) -
            sum(bench.step_bytes(ne, nn, "fp64").values())) >= 624 * ne


@pytest.mark.parametrize("n", [1, 2, 3, 7, 16, 33])
def test_spread_order_is_a_permutation_that_starts_mid_range(n):
    order = bench.spread_order(n)
    assert sorted(order) == list(range(n))
    assert order[0] == n // 2
    if n >= 4:
        # the first three picks span the range
        first = sorted(order[:3])
        assert first[0] < n // 2 < first[-1]


def test_size_bands_cover_every_ensemble_size():
    fx = json.loads((ROOT / "tests" / "golden" / "ensembles.json").read_text())
    for name in ("c3", "c4"):
        for s in fx[name]["sizes"]:
            assert sum(1 for lo, hi in bench.SIZE_BANDS if lo <= s <= hi) == 1, s


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
    assert line["warmup"] == 3 and line["steps"] == 2
    cb = line["cpu_baseline"]
    assert cb["kind"] == "reference" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
