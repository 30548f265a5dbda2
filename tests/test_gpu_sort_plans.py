"""GPU tests of the digit-pass plans and the autotuner: every keys-only shape
at every digit width and every key/value shape sorts exactly like numpy's
stable sort; a tuned or loaded plan is the one the sorts take, and results
stay bit-exact under it."""
import json
import os

import numpy as np
import pytest

import dag_compression_fast_gb300 as D
from oracle import oracle as O
from tests.test_gpu_parity import assert_dag_equal

pytestmark = pytest.mark.gpu


def stable(k, lo, hi):
    mask = np.uint64((1 << (hi - lo)) - 1) if hi - lo < 64 else np.uint64(2**64 - 1)
    return np.argsort((k >> np.uint64(lo)) & mask, kind="stable")


@pytest.mark.parametrize("shape", range(D.NUM_KEY_SHAPES))
@pytest.mark.parametrize("bits", D.RADIX_BITS)
def test_every_key_plan_sorts_stably(shape, bits):
    with D.Context(0) as c:
        c.set_option(D.OPT_SORT_SHAPE_KEYS, shape)
        c.set_option(D.OPT_SORT_RADIX_BITS, bits)
        for n, lo, hi in [(1, 0, 64), (4097, 6, 39), (300_001, 6, 33), (1_000_003, 0, 64), (70_000, 61, 64)]:
            rng = np.random.default_rng(n + 7 * shape + bits)
            k = rng.integers(0, 2**64 - 1, n, dtype=np.uint64)
            if n > 10:
                k[: n // 3] = k[0]
            out = c.sort_keys(k, lo, hi).cpu().numpy().view(np.uint64)
            assert np.array_equal(out, k[stable(k, lo, hi)]), (n, lo, hi, c.sort_plan(n, lo, hi))


@pytest.mark.parametrize("shape", range(D.NUM_PAIR_SHAPES))
def test_every_pair_shape_sorts_stably(shape):
    with D.Context(0) as c:
        c.set_option(D.OPT_SORT_SHAPE_PAIRS, shape)
        for n in [5, 65_537, 400_000]:
            rng = np.random.default_rng(n + shape)
            k = rng.integers(0, 5000, n, dtype=np.uint64)  # many ties
            keys, vals = c.sort_pairs(k)
            order = stable(k, 0, 64)
            assert np.array_equal(keys.cpu().numpy().view(np.uint64), k[order])
            assert np.array_equal(vals.cpu().numpy().view(np.uint32), order.astype(np.uint32))


def test_tuned_plan_is_applied_and_bit_exact(tmp_path):
    """The autotuner times the plans of one class, keeps the fastest and the
    context's sorts of that class take it; a saved table loads into a fresh
    context with the same plan."""
    n, lo, hi = 3_000_000, 6, 39
    with D.Context(0) as c:
        c.tune_clear()
        assert c.sort_plan(n, lo, hi) == (0, 8)  # the default
        r = c.tune_sort(n, lo, hi, reps=2)
        assert r["ms"] > 0 and r["default_ms"] > 0 and r["ms"] <= r["default_ms"]
        assert c.sort_plan(n, lo, hi) == (r["shape"], r["radix_bits"])
        path = str(tmp_path / "plans.json")
        c.tune_save(path)
    entries = json.load(open(path))["entries"]
    assert any(e["bits"] == hi - lo and e["values"] == 0 for e in entries)
    with D.Context(0) as c2:
        c2.tune_load(path)
        assert c2.sort_plan(n, lo, hi) == (r["shape"], r["radix_bits"])


def test_loaded_wide_digit_plan_drives_create_dag(tmp_path):
    """A table that gives the fragment sort 11-bit digits (3 passes over 33
    bits instead of 5): the plan is taken (fewer kernel launches) and the DAG
    stays bit-exact with the oracle."""
    codes = D.gen_triangle_soup(13, 77, 60_000, threads=8)
    n = codes.size
    log2n = int(np.floor(np.log2(n)))
    table = {"format": "dagc digit-pass plans", "version": 1,
             "entries": [{"values": 0, "bits": 33, "log2n": log2n, "shape": 1, "radix_bits": 11}]}
    path = tmp_path / "wide.json"
    path.write_text(json.dumps(table))
    ref = O.create_dag(codes, 13, threads=8)
    launches = {}
    for name in ["default", "wide"]:
        with D.Context(0) as c:
            c.tune_clear()
            c.set_option(D.OPT_GROUP, 0)
            if name == "wide":
                c.tune_load(str(path))
                assert c.sort_plan(n, 6, 39) == (1, 11)
            l0 = c.kernel_launches()
            dag = c.create_dag(codes, 13)
            launches[name] = c.kernel_launches() - l0
            assert_dag_equal(dag.to_host(), ref)
    assert launches["default"] - launches["wide"] == 2  # 5 digit passes -> 3
