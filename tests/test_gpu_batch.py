"""Batched ensembles against single-instance runs and the oracle.

Every instance of a batch must evolve exactly as a single-instance context
started from the same state (bitwise: the same kernels and arithmetic, an
order-free constraint minimum), reach its own stop time at its own cycle
count, and match the oracle like any single run.
"""
from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

SIZES = [4, 9, 6, 12, 5, 17]
SCALE = [1.0, 0.7, 1.6, 1.0, 0.55, 1.9]


def _solo_like(pkg, batch, i, precision):
    """A single-instance context with batch instance i's initial state."""
    s = int(batch.sizes[i])
    sc, e0, _ = batch.instance(i)
    g = pkg.Lulesh(s, pkg.INIT_V2, precision)
    e = np.zeros(s ** 3)
    e[0] = e0
    g.set_field("e", e)
    cur = g.scalars
    cur.deltatime = sc.deltatime
    g.scalars = cur
    return g


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_batch_instances_equal_solo_runs(pkg, precision):
    prec = pkg.FP64 if precision == "fp64" else pkg.SPLIT
    with pkg.Batch(SIZES, SCALE, pkg.INIT_V2, prec) as b:
        solos = [_solo_like(pkg, b, i, prec) for i in range(len(SIZES))]
        most = b.run()
        counts = []
        for i, g in enumerate(solos):
            n = g.run()
            counts.append(n)
            sc, e0, status = b.instance(i)
            assert status == pkg.OK
            assert sc.cycle == n, (i, sc.cycle, n)
            assert sc.time == g.scalars.time
            for k in ("x", "y", "z", "xd", "yd", "zd", "e", "p", "q", "v", "ss"):
                assert np.array_equal(b.get_field(i, k), g.get_field(k)), (i, k)
            g.close()
        assert most == max(counts)
        assert len(set(counts)) > 1          # instances really ran to different cycle counts
        assert b.zone_cycles() == sum(s ** 3 * n for s, n in zip(SIZES, counts))


def test_batch_instance_matches_oracle(pkg, orc):
    """A scaled-energy instance against the oracle started from its state."""
    with pkg.Batch([10, 7], [0.7, 1.3], pkg.INIT_V2, pkg.FP64) as b:
        sc0, e00, _ = b.instance(0)
        b.run()
        sc, e0, _ = b.instance(0)
    o = orc.Oracle(10, orc.INIT_V2)
    o.field("e")[0] = e00
    o.set_scalar("deltatime", sc0.deltatime)
    rc, _ = o.run()
    assert rc == 0
    assert sc.cycle == o.cycle
    assert abs(e0 - o.field("e")[0]) <= 1e-10 * abs(o.field("e")[0])


def test_autotune_restores_state_and_caches(pkg, tmp_path):
    cache = tmp_path / "tuning.json"
    with pkg.Batch(SIZES, SCALE) as ref:
        ref.run()
        want = [ref.get_field(i, "e") for i in range(len(SIZES))]
    with pkg.Batch(SIZES, SCALE) as b:
        b.autotune(str(cache))
        tuned = b.tuning()
        b.run()
        for i in range(len(SIZES)):
            assert np.array_equal(b.get_field(i, "e"), want[i]), i
    entries = json.loads(cache.read_text())
    assert entries and all(v[0] in (64, 128, 256) for v in entries.values())
    with pkg.Batch(SIZES, SCALE) as c:
        c.autotune(str(cache))                 # served from the cache
        assert c.tuning() == tuned


def test_batch_of_tiny_and_single_instances(pkg):
    """Edge sizes: one-element instances beside larger ones, and a batch of
    one instance, each equal to its single-instance run."""
    for sizes, scale in (([1, 2, 3, 1, 7], [1.0, 1.3, 0.8, 0.6, 1.0]), ([5], [1.0])):
        with pkg.Batch(sizes, scale, pkg.INIT_V2, pkg.FP64) as b:
            solos = [_solo_like(pkg, b, i, pkg.FP64) for i in range(len(sizes))]
            b.run()
            for i, g in enumerate(solos):
                n = g.run()
                sc, _, status = b.instance(i)
                assert status == pkg.OK and sc.cycle == n, (sizes, i)
                for k in ("x", "e", "p", "v"):
                    assert np.array_equal(b.get_field(i, k), g.get_field(k)), (sizes, i, k)
                g.close()


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_retuned_run_equals_plain_run(pkg, precision):
    """Re-tuning the launch shapes as instances retire changes no element's
    arithmetic: the chunked, re-tuned run ends in the same bits and cycle
    counts as one run."""
    prec = pkg.FP64 if precision == "fp64" else pkg.SPLIT
    with pkg.Batch(SIZES, SCALE, pkg.INIT_V2, prec) as a, pkg.Batch(SIZES, SCALE, pkg.INIT_V2, prec) as b:
        most = a.run()
        most_b, retunes = b.run_retuned(chunk=60, fraction=0.95)
        assert most_b == most
        assert retunes >= 1
        assert b.zone_cycles() == a.zone_cycles()
        for i in range(len(SIZES)):
            assert a.instance(i)[0].cycle == b.instance(i)[0].cycle
            for k in ("x", "xd", "e", "p", "q", "v", "ss"):
                assert np.array_equal(a.get_field(i, k), b.get_field(i, k)), (i, k)



def test_staged_force_equals_gathered_in_batch(pkg):
    """The staging depth of the split force kernel (corners gathered, or
    tiles of 2 or 4 element rows staged in shared memory) changes no bit:
    a class of cubes with s >= 64, among them sizes that leave partial tiles
    (66: a partial row pair and column block, 70), run at each depth."""
    sizes, scale = [64, 66, 70], [1.0, 0.8, 1.3]
    results = {}
    for rows in (0, 2, 4):
        with pkg.Batch(sizes, scale, pkg.INIT_V2, pkg.SPLIT) as b:
            b.set_tuning(2, "elem_force", block=128, blocks_per_sm=4, rows=rows)
            assert b.tuning()["class2/elem_force"]["stage"] == rows
            b.run(40)
            results[rows] = [[b.get_field(i, k) for k in ("x", "xd", "e", "p", "q", "v", "ss")]
                             for i in range(len(sizes))]
            assert all(b.instance(i)[0].cycle == 40 for i in range(len(sizes)))
    for rows in (2, 4):
        for i in range(len(sizes)):
            for a, c in zip(results[0][i], results[rows][i]):
                assert np.array_equal(a, c), (rows, i)


def test_staging_needs_a_class_of_wide_cubes(pkg):
    """A class holding an instance narrower than a tile row (s < 64) cannot be
    staged; asking for it is an argument error, and so is staging another
    kernel or an FP64 batch."""
    with pkg.Batch([50, 64], [1.0, 1.0], pkg.INIT_V2, pkg.SPLIT) as b:
        with pytest.raises(pkg.LuleshError):
            b.set_tuning(2, "elem_force", rows=2)
        assert b.tuning()["class2/elem_force"]["stage"] == 0
    with pkg.Batch([64], [1.0], pkg.INIT_V2, pkg.SPLIT) as b:
        with pytest.raises(pkg.LuleshError):
            b.set_tuning(2, "elem_kinematics", rows=2)
        b.set_tuning(2, "elem_force", rows=4)
    with pkg.Batch([64], [1.0], pkg.INIT_V2, pkg.FP64) as b:
        with pytest.raises(pkg.LuleshError):
            b.set_tuning(0, "elem_force", rows=2)


def test_autotune_considers_staging(pkg, tmp_path):
    """The autotuner times the staged depths for a class of wide cubes and
    records the depth it chose with the shape; a cached choice is restored
    with its depth."""
    cache = tmp_path / "tuning.json"
    with pkg.Batch([64, 65], [1.0, 1.1], pkg.INIT_V2, pkg.SPLIT) as b:
        b.autotune(str(cache))
        t = b.tuning()["class2/elem_force"]
        assert t["stage"] in (0, 2, 4)
        if t["stage"]:
            assert t["block"] == 64 * t["stage"]
    entries = json.loads(cache.read_text())
    force = [v for k, v in entries.items() if k.endswith("class2|elem_force")]
    assert force and len(force[0]) == 3 and force[0][2] == t["stage"]
    with pkg.Batch([64, 65], [1.0, 1.1], pkg.INIT_V2, pkg.SPLIT) as c:
        c.autotune(str(cache))
        assert c.tuning()["class2/elem_force"] == t
