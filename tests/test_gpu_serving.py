"""GPU tests of the serving loop: jobs in a concurrent mix give the same words
as each job alone, work overlaps across slots, and chunk jobs merge into a
shared DAG equal to compressing the whole volume."""
import numpy as np
import pytest

import dag_compression_fast_gb300 as D
from oracle import oracle as O
from tests.inputs import chunks_of, random_codes
from tests.test_gpu_parity import assert_dag_equal

pytestmark = pytest.mark.gpu


def job_mix(seed):
    rng = np.random.default_rng(seed)
    jobs = []
    for i in range(12):
        depth = int(rng.integers(8, 12))
        kind = i % 3
        if kind == 0:
            codes = D.gen_sphere_shell(depth, seed + i, float(rng.integers(50_000, 600_000)))
        elif kind == 1:
            codes = D.gen_terrain(depth, seed + i, float(rng.uniform(0.02, 0.2)))
        else:
            codes = D.gen_triangle_soup(depth, seed + i, int(rng.integers(2_000, 20_000)), threads=4)
        jobs.append((codes, depth))
    return jobs


def test_results_same_alone_and_in_the_mix(ctx):
    jobs = job_mix(77)
    alone = [ctx.compress_host(codes, depth) for codes, depth in jobs]
    srv = D.Server(0, slots=4, hbm_budget_bytes=32 << 30)
    try:
        tickets = [srv.submit(codes, depth) for codes, depth in jobs]
        for t, ref in zip(tickets, alone):
            words, lat = srv.wait(t)
            assert lat > 0
            assert np.array_equal(words, ref)
        st = srv.stats()
        assert st["completed"] == len(jobs)
        assert st["max_concurrent"] >= 2  # admitted jobs overlapped
    finally:
        srv.close()


def test_budget_admits_one_at_a_time_when_tight(ctx):
    jobs = job_mix(5)[:4]
    srv = D.Server(0, slots=4, hbm_budget_bytes=1)  # every job exceeds it: runs alone
    try:
        tickets = [srv.submit(codes, depth) for codes, depth in jobs]
        for (codes, depth), t in zip(jobs, tickets):
            words, _ = srv.wait(t)
            assert np.array_equal(words, ctx.compress_host(codes, depth))
        assert srv.stats()["max_concurrent"] == 1
    finally:
        srv.close()


def test_shared_dag_of_chunk_jobs(ctx):
    codes = random_codes(9, 200_000, 31, cluster=True)
    chunks, sub = chunks_of(codes, 9, 1)
    srv = D.Server(0, slots=3)
    try:
        tickets = [srv.submit(c, sub, chunk_morton=i) for i, c in enumerate(chunks) if c.size]
        for t in tickets:
            srv.wait(t)
        shared = srv.shared_dag(1)
        assert_dag_equal(shared.to_host(), O.create_dag(codes, 9))
    finally:
        srv.close()


def test_shared_dag_grows_as_chunks_finish(ctx):
    """Each finished chunk is folded into the resident union; after every
    chunk the shared DAG equals the oracle's DAG of the chunks so far, and a
    chunk submitted again replaces its earlier version."""
    codes = random_codes(9, 150_000, 41, cluster=True)
    chunks, sub = chunks_of(codes, 9, 1)
    srv = D.Server(0, slots=2)
    try:
        so_far = []
        for i, c in enumerate(chunks):
            if not c.size:
                continue
            srv.wait(srv.submit(c, sub, chunk_morton=i))
            so_far.append((np.uint64(i) << np.uint64(3 * sub)) | c)
            shared = srv.shared_dag(1)
            assert_dag_equal(shared.to_host(), O.create_dag(np.concatenate(so_far), 9))
        assert srv.folds() >= 2
        # Chunk 0 again, with other fragments: the shared DAG follows.
        repl = random_codes(sub, 5_000, 42)
        srv.wait(srv.submit(repl, sub, chunk_morton=0))
        rest = [(np.uint64(i) << np.uint64(3 * sub)) | c for i, c in enumerate(chunks) if i and c.size]
        assert_dag_equal(srv.shared_dag(1).to_host(), O.create_dag(np.concatenate([repl] + rest), 9))
    finally:
        srv.close()


def test_union_and_lift_equal_merge(ctx):
    codes = random_codes(8, 80_000, 43)
    chunks, sub = chunks_of(codes, 8, 1)
    dags = [ctx.create_dag(c, sub) for c in chunks]
    body, roots = ctx.union_dags(dags)
    lifted = ctx.lift_dag(body, roots)
    assert_dag_equal(lifted.to_host(), O.create_dag(codes, 8))


def test_jobs_overlap_on_the_device(ctx):
    """Device-side evidence of overlap: each job's work is bracketed by CUDA
    events on its slot's stream; some pair of jobs has intersecting
    intervals."""
    jobs = job_mix(91)
    srv = D.Server(0, slots=4, hbm_budget_bytes=32 << 30)
    try:
        for _ in range(2):  # warm: arenas and graphs
            tickets = [srv.submit(codes, depth) for codes, depth in jobs]
            for t in tickets:
                srv.wait(t)
        iv = [srv.timeline(t) for t in tickets]
        assert all(0 <= a < b for a, b in iv)
        overlaps = sum(1 for i in range(len(iv)) for j in range(i + 1, len(iv))
                       if iv[i][0] < iv[j][1] and iv[j][0] < iv[i][1])
        assert overlaps >= 1
    finally:
        srv.close()


def test_submit_into_caller_buffers(ctx):
    """Words written straight into the caller's buffers equal the plain
    submit's; a buffer too small keeps the words inside the server."""
    jobs = job_mix(17)[:6]
    alone = [ctx.compress_host(codes, depth) for codes, depth in jobs]
    srv = D.Server(0, slots=3, hbm_budget_bytes=32 << 30)
    try:
        outs = [np.zeros(w.size + 7, np.uint32) for w in alone]
        outs[2] = np.zeros(max(alone[2].size - 1, 1), np.uint32)  # too small
        tickets = [srv.submit_into(codes, depth, out) for (codes, depth), out in zip(jobs, outs)]
        for t, ref in zip(tickets, alone):
            words, _ = srv.wait(t)
            assert np.array_equal(words, ref)
    finally:
        srv.close()
