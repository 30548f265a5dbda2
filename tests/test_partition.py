"""CPU tests of the chunk-partitioned path (several ranks, one all-gather):
simulated in one process for 1..4 ranks, and as two gloo processes."""
import os

import numpy as np
import pytest

from dag_compression_fast_gb300 import partition as P
from oracle import oracle as O
from tests.inputs import chunks_of, random_codes


def oracle_local(chunks, morton, chunk_depth, top_levels):
    """A rank's compressor: the oracle on the global codes of its chunks."""
    parts = [(np.uint64(m) << np.uint64(3 * chunk_depth)) | c for c, m in zip(chunks, morton) if c.size]
    codes = np.concatenate(parts) if parts else np.zeros(0, np.uint64)
    return O.create_dag(codes, chunk_depth + top_levels)


def simulate(world, codes, depth, top_levels):
    chunks, sub = chunks_of(codes, depth, top_levels)
    morton = list(range(len(chunks)))
    payloads = []
    for rank in range(world):
        mine = P.assign_chunks(morton, world)[rank]
        local = oracle_local([chunks[i] for i in mine], [morton[i] for i in mine], sub, top_levels)
        payloads.append((P.to_records(local, top_levels), P.chunk_roots(local, top_levels)))
    return P.merge_payloads(payloads, sub, top_levels, O.hash_children)


@pytest.mark.parametrize("world", [1, 2, 3, 4])
@pytest.mark.parametrize("depth,top_levels,seed", [(7, 1, 1), (8, 2, 2)])
def test_partitioned_union_equals_single_device(world, depth, top_levels, seed):
    codes = random_codes(depth, 40_000, seed, cluster=True)
    got = simulate(world, codes, depth, top_levels)
    assert O.dags_equal(got, O.create_dag(codes, depth))


def test_partitioned_with_empty_ranks():
    codes = random_codes(7, 5_000, 9, cluster=True)
    codes = codes[(codes >> np.uint64(18)) < np.uint64(2)]  # only chunk slots 0 and 1 hold voxels
    got = simulate(4, codes, 7, 1)
    assert O.dags_equal(got, O.create_dag(codes, 7))


def _gloo_rank(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        codes = random_codes(8, 60_000, 5, cluster=True)
        chunks, sub = chunks_of(codes, 8, 1)
        dag = P.partitioned_create(chunks, list(range(len(chunks))), sub, 1, oracle_local, O.hash_children)
        ok = O.dags_equal(dag, O.create_dag(codes, 8))
        with open(os.path.join(out_dir, f"rank{rank}"), "w") as f:
            f.write("ok" if ok else "mismatch")
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    import socket

    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.spawn(_gloo_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        assert (tmp_path / f"rank{r}").read_text() == "ok"
