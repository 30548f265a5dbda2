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
