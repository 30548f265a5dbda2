"""Runs the compression pipeline on one seeded workload, for profiling and
quick measurements (the profiler captures in profiles/ are made with it).

  python -m dag_compression_fast_gb300.workload --workload terrain --depth 11 \
      --fraction 0.6 --steps 2
Prints one line per step: fragments, device ms (CUDA events), words.
"""
from __future__ import annotations

import argparse
import sys

import numpy as np


def make(workload: str, depth: int, fraction: float, seed: int) -> np.ndarray:
    import dag_compression_fast_gb300 as D
    if workload == "terrain":
        return D.gen_terrain(depth, seed, fraction)
    if workload == "sphere":
        return D.gen_sphere_shell(depth, seed)
    if workload == "soup":
        return D.gen_triangle_soup(depth, seed, int(2_000_000 * fraction))
    raise ValueError(workload)


def main(argv=None) -> int:
    p = argparse.ArgumentParser()
    p.add_argument("--workload", default="terrain", choices=["terrain", "sphere", "soup"])
    p.add_argument("--depth", type=int, default=11)
    p.add_argument("--fraction", type=float, default=1.0, help="terrain column / soup triangle fraction")
    p.add_argument("--seed", type=int, default=0xDA6C0DE + 1)
    p.add_argument("--steps", type=int, default=2)
    p.add_argument("--group", choices=["auto", "sort", "group"], default="auto",
                   help="leaf path: the device's choice, always the fragment sort, always grouping (DAGC_OPT_GROUP)")
    a = p.parse_args(argv)
    import torch

    import dag_compression_fast_gb300 as D
    codes = make(a.workload, a.depth, a.fraction, a.seed)
    ctx = D.Context(0)
    ctx.set_option(D.OPT_GROUP, {"auto": 1, "sort": 0, "group": 2}[a.group])
    t = torch.from_numpy(codes.view(np.int64)).cuda()
    s = torch.cuda.current_stream()
    for i in range(a.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        w = ctx.compress(t, a.depth)
        e1.record(s)
        torch.cuda.synchronize()
        print(f"step {i}: {codes.size} fragments, {e0.elapsed_time(e1):.3f} ms, {w.n} words", flush=True)
        w.free()
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
