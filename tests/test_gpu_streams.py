"""Stream ordering of CreateDAG's result. CreateDAG returns before the kernel
that copies the DAG out of the context's scratch has finished; every later
reader (CreateFinalDAG or MergeDAGs on any stream, host downloads, a copy)
and every later call that reuses the scratch is ordered after that copy.
These tests read DAGs on other streams and from the host right after
CreateDAG, reuse the scratch before an earlier DAG is read, and free DAGs
right after creating them."""
import numpy as np
import pytest
import torch

import dag_compression_fast_gb300 as D
from oracle import oracle as O
from tests.inputs import chunks_of, random_codes
from tests.test_gpu_parity import assert_dag_equal

pytestmark = pytest.mark.gpu


def _input(depth, seed):
    codes = D.gen_terrain(depth, seed)
    t = torch.from_numpy(codes.view(np.int64)).cuda()
    torch.cuda.synchronize()
    return codes, t


def test_final_on_another_stream(ctx):
    codes, t = _input(9, 11)
    ref = O.final_dag(O.create_dag(codes, 9))
    a, b = torch.cuda.Stream(), torch.cuda.Stream()
    dag = ctx.create_dag(t, 9, stream=a)
    words = ctx.create_final_dag(dag, stream=b)
    assert np.array_equal(words.to_numpy(), ref)


def test_host_download_right_after_create(ctx):
    codes, t = _input(10, 12)
    ref = O.create_dag(codes, 10)
    s = torch.cuda.Stream()
    dag = ctx.create_dag(t, 10, stream=s)
    assert_dag_equal(dag.to_host(), ref)
    dag.free()


def test_scratch_reused_before_first_dag_is_read(ctx):
    c1, t1 = _input(10, 13)
    c2, t2 = _input(8, 14)
    r1 = O.final_dag(O.create_dag(c1, 10))
    r2 = O.final_dag(O.create_dag(c2, 8))
    s1, s2, s3 = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
    d1 = ctx.create_dag(t1, 10, stream=s1)
    d2 = ctx.create_dag(t2, 8, stream=s2)  # overwrites the scratch d1 was copied from
    w1 = ctx.create_final_dag(d1, stream=s3)
    w2 = ctx.create_final_dag(d2, stream=s3)
    assert np.array_equal(w1.to_numpy(), r1)
    assert np.array_equal(w2.to_numpy(), r2)


def test_merge_of_dags_made_on_several_streams(ctx):
    codes = random_codes(8, 60_000, 15, cluster=True)
    chunks, sub = chunks_of(codes, 8, 1)
    ref = O.merge_dags([O.create_dag(c, sub) for c in chunks])
    streams = [torch.cuda.Stream() for _ in range(3)]
    dags = []
    for i, c in enumerate(chunks):
        t = torch.from_numpy(np.ascontiguousarray(c).view(np.int64)).cuda()
        torch.cuda.synchronize()
        dags.append(ctx.create_dag(t, sub, stream=streams[i % 3]))
    merged = ctx.merge_dags(dags, stream=streams[0])
    assert_dag_equal(merged.to_host(), ref)


def test_free_right_after_create(ctx):
    codes, t = _input(9, 16)
    ref = O.final_dag(O.create_dag(codes, 9))
    s = torch.cuda.Stream()
    for _ in range(3):
        ctx.create_dag(t, 9, stream=s).free()
    words = ctx.create_final_dag(ctx.create_dag(t, 9, stream=s), stream=s)
    assert np.array_equal(words.to_numpy(), ref)
