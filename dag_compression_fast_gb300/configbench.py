"""Per-configuration measurements besides bench.py's headline (config 2):

  1  sphere shell, 128^3 (depth 7)         -- L2-resident, latency-bound
  2  fBm terrain, 2048^3 (depth 11)        -- the headline workload
  3  triangle soup, 8192^3 (depth 13), 2M triangles, ~65M fragments; the
     fragments come from the GPU voxelizer's separating-axis rule (the same
     set as the host generator) and are shuffled on the GPU with a seeded
     permutation, as the workload prescribes

For each: CreateDAG + CreateFinalDAG from device fragments to device words,
replayed as a CUDA graph, CUDA events around K steps after W warm-up steps;
and the CPU oracle (the reference algorithm on all host cores) on the same
input, or on a bounded prefix of it for config 3. One JSON line per config.

  python -m dag_compression_fast_gb300.configbench [--configs 1 2 3] [--steps 10]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np


def fragments(cfg: int, ctx):
    import torch

    import dag_compression_fast_gb300 as D
    if cfg == 1:
        return torch.from_numpy(D.gen_sphere_shell(7, 0xDA6C0DE + 1).view(np.int64)).cuda(), 7
    if cfg == 2:
        return torch.from_numpy(D.gen_terrain(11, 0xDA6C0DE + 2).view(np.int64)).cuda(), 11
    depth = 13
    g = 1 << depth
    tris = D.gen_soup_triangles(depth, 0xDA6C0DE + 3, 2_000_000)
    codes = ctx.voxelize(tris, (0, 0, 0, g, g, g), depth, D.VOXELIZE_SAT)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(0xDA6C0DE + 3)
    return codes[torch.randperm(codes.numel(), device="cuda", generator=gen)].contiguous(), depth


def main(argv=None) -> int:
    p = argparse.ArgumentParser()
    p.add_argument("--configs", type=int, nargs="+", default=[1, 2, 3])
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--cpu-fragments", type=int, default=40_000_000, help="oracle sample cap (fragments)")
    a = p.parse_args(argv)
    import torch

    import dag_compression_fast_gb300 as D
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from oracle import oracle as O

    ctx = D.Context(0)
    threads = os.cpu_count() or 1
    for cfg in a.configs:
        frags, depth = fragments(cfg, ctx)
        n = frags.numel()
        stream = torch.cuda.current_stream()

        def step():
            dag = ctx.create_dag(frags, depth, stream=stream)
            words = ctx.create_final_dag(dag, stream=stream)
            return words

        for _ in range(a.warmup):
            w = step()
        nwords = w.n
        del w
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(a.steps):
            w = step()
            del w
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / a.steps
        counts = ctx.last_counts()
        # CPU oracle on the host cores (the whole input, or its first
        # cpu_fragments fragments: a bounded sample of the same workload).
        host = frags[: min(n, a.cpu_fragments)].cpu().numpy().view(np.uint64)
        t = time.perf_counter()
        O.final_dag(O.create_dag(host, depth, threads=threads))
        cpu_s = time.perf_counter() - t
        print(json.dumps({
            "config": cfg, "depth": depth, "fragments": n, "bricks": counts[1], "leaves": counts[2],
            "words": nwords, "ms_per_step": round(ms, 4), "voxels_per_s": n / (ms * 1e-3),
            "dedup_fallbacks": ctx.dedup_fallbacks(),
            "cpu_baseline": {"voxels_per_s": host.size / cpu_s, "threads": threads, "sample_fragments": host.size},
        }), flush=True)
        del frags
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
