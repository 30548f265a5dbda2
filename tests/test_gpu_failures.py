"""GPU tests of the failure paths that can be exercised without faulting a
GPU: a bounded device wait that runs out (a look-back predecessor that never
publishes, with a lowered wait limit) returns DAGC_ERR_DEVICE_TIMEOUT and
leaves the context usable; injected allocation failures take the pool's
release-and-retry path (src/Memory.cpp:56-70) or report OUT_OF_MEMORY, also
through the serving loop with the other jobs intact; and the memory
statistics follow the context's allocations."""
import numpy as np
import pytest

import dag_compression_fast_gb300 as D
from oracle import oracle as O
from tests.inputs import random_codes
from tests.test_gpu_parity import assert_dag_equal

pytestmark = pytest.mark.gpu


def stable(k, lo, hi):
    mask = np.uint64((1 << (hi - lo)) - 1)
    return k[np.argsort((k >> np.uint64(lo)) & mask, kind="stable")]


def test_lookback_wait_runs_out_and_context_recovers():
    keys = np.random.default_rng(3).integers(0, 1 << 40, 10_000, dtype=np.uint64)  # three 4096-key tiles
    with D.Context(0) as c:
        c.set_option(D.OPT_TEST_SPIN_LIMIT, 2048)
        c.set_option(D.OPT_TEST_STALL_LOOKBACK, 1)
        with pytest.raises(D.DagcError) as e:
            c.sort_keys(keys, 0, 40)
        assert e.value.status == D.ERR_DEVICE_TIMEOUT
        c.set_option(D.OPT_TEST_STALL_LOOKBACK, 0)
        c.set_option(D.OPT_TEST_SPIN_LIMIT, 0)
        out = c.sort_keys(keys, 0, 40).cpu().numpy().view(np.uint64)
        assert np.array_equal(out, stable(keys, 0, 40))


def test_create_dag_times_out_then_runs_bit_exact():
    codes = random_codes(8, 12_000, 9)
    ref = O.create_dag(codes, 8)
    with D.Context(0) as c:
        c.set_option(D.OPT_GROUP, 0)  # the sort path: its digit passes wait on each other
        c.set_option(D.OPT_TEST_SPIN_LIMIT, 2048)
        c.set_option(D.OPT_TEST_STALL_LOOKBACK, 1)
        with pytest.raises(D.DagcError) as e:
            c.create_dag(codes, 8)
        assert e.value.status == D.ERR_DEVICE_TIMEOUT
        c.set_option(D.OPT_TEST_STALL_LOOKBACK, 0)
        c.set_option(D.OPT_TEST_SPIN_LIMIT, 0)
        for _ in range(3):  # direct launches, then the recorded graph
            assert_dag_equal(c.create_dag(codes, 8).to_host(), ref)


def test_allocation_failure_is_retried_after_release():
    small, big = random_codes(9, 20_000, 1), random_codes(9, 400_000, 2)
    with D.Context(0) as c:
        c.compress(small, 9).free()
        before = c.memory_events()
        c.set_option(D.OPT_TEST_FAIL_ALLOCS, 1)  # the next allocation fails once
        dag = c.create_dag(big, 9)  # the arena grows: first attempt fails, the retry succeeds
        after = c.memory_events()
        assert after["alloc_failures"] == before["alloc_failures"] + 1
        assert after["retries_ok"] == before["retries_ok"] + 1
        assert_dag_equal(dag.to_host(), O.create_dag(big, 9))


def test_allocation_failure_reports_out_of_memory_and_recovers():
    small, big = random_codes(9, 20_000, 3), random_codes(9, 400_000, 4)
    with D.Context(0) as c:
        c.compress(small, 9).free()
        c.set_option(D.OPT_TEST_FAIL_ALLOCS, 2)  # the allocation and its retry fail
        with pytest.raises(D.DagcError) as e:
            c.create_dag(big, 9)
        assert e.value.status == D.ERR_OUT_OF_MEMORY
        assert c.memory_events()["alloc_failures"] >= 2
        c.set_option(D.OPT_TEST_FAIL_ALLOCS, 0)
        assert_dag_equal(c.create_dag(big, 9).to_host(), O.create_dag(big, 9))


def test_server_job_out_of_memory_leaves_other_jobs_intact(ctx):
    a, b, c3 = random_codes(9, 30_000, 5), random_codes(10, 600_000, 6), random_codes(9, 50_000, 7)
    alone = {k: ctx.compress_host(x, d) for k, (x, d) in {"a": (a, 9), "c": (c3, 9)}.items()}
    srv = D.Server(0, slots=1, hbm_budget_bytes=64 << 30)  # one slot: jobs run in submission order
    try:
        words, _ = srv.wait(srv.submit(a, 9))
        assert np.array_equal(words, alone["a"])
        srv.set_option(D.OPT_TEST_FAIL_ALLOCS, 2)
        with pytest.raises(D.DagcError) as e:
            srv.wait(srv.submit(b, 10))  # larger than anything cached: its allocations fail
        assert e.value.status == D.ERR_OUT_OF_MEMORY
        srv.set_option(D.OPT_TEST_FAIL_ALLOCS, 0)
        words, _ = srv.wait(srv.submit(c3, 9))
        assert np.array_equal(words, alone["c"])
        assert srv.stats()["completed"] == 3
    finally:
        srv.close()


def test_memory_stats_follow_allocations():
    codes = random_codes(10, 300_000, 8)
    with D.Context(0) as c:
        s0 = c.memory_stats()
        assert s0["in_use"] == 0 and s0["arena"] == 0
        dag = c.create_dag(codes, 10)
        s1 = c.memory_stats()
        assert s1["in_use"] > 0 and 0 < s1["arena"] <= 2 * D.create_footprint(codes.size, 10)
        assert s1["peak"] >= s1["in_use"]
        words = c.create_final_dag(dag)  # consumes the DAG
        s2 = c.memory_stats()
        assert s2["in_use"] >= words.n * 4 and s2["peak"] >= s1["in_use"]
        report = c.memory_report()
        assert "final DAG words" in report and "scratch arena" in report and "GPU memory" in report
        words.free()
        c.create_dag(codes, 10).free()  # the cached blocks are reused
        s3 = c.memory_stats()
        assert s3["in_use"] == 0 and s3["cached"] > 0 and s3["peak"] == max(s2["peak"], s3["peak"])
        c.free_all()
        s4 = c.memory_stats()
        assert s4["in_use"] == 0 and s4["cached"] == 0 and s4["arena"] == 0
