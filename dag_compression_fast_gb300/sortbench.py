"""Radix-sort throughput sweeps, the GB300 counterpart of the reference's
published CUB sort measurements (Python/constant64.csv, variable64.csv of
Phyronnaz/DAG_Compression_Fast: 64-bit keys, throughput in G keys/s against the
key count or the number of sorted bits).

  python -m dag_compression_fast_gb300.sortbench                 # one case
  python -m dag_compression_fast_gb300.sortbench --sweep bits    # 1..64 bits, 100M keys
  python -m dag_compression_fast_gb300.sortbench --sweep n       # 1M..200M keys, 64 bits

Each line: bits;keys;G keys/s;GB/s (algorithmic bytes: one key read for the
histogram plus a read and a write per digit pass).
"""
from __future__ import annotations

import argparse
import sys

import numpy as np


def run(ctx, n: int, lo: int, hi: int, reps: int, seed: int = 1, pairs: bool = False):
    import torch
    rng = np.random.default_rng(seed)
    keys = torch.from_numpy(rng.integers(0, 2**63, n, dtype=np.int64)).cuda()
    out = torch.empty_like(keys)
    vout = torch.empty(n, dtype=torch.int32, device=keys.device)
    import dag_compression_fast_gb300 as D
    lib = D.lib()
    s = torch.cuda.current_stream()

    def once():
        if pairs:
            ctx._check(lib.dagc_sort_pairs(ctx.handle, keys.data_ptr(), out.data_ptr(), None, vout.data_ptr(), n,
                                           lo, hi, s.cuda_stream))
        else:
            ctx._check(lib.dagc_sort_keys(ctx.handle, keys.data_ptr(), out.data_ptr(), n, lo, hi, s.cuda_stream))

    for _ in range(2):
        once()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        once()
    e1.record(s)
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3 / reps
    shape, bits = ctx.sort_plan(n, lo, hi, pairs)
    passes = (hi - lo + bits - 1) // bits
    kv = 12 if pairs else 8
    bytes_ = 8 * n + passes * 2 * kv * n
    return n / sec / 1e9, bytes_ / sec / 1e9


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--n", type=int, default=20_000_000)
    p.add_argument("--lo", type=int, default=6)
    p.add_argument("--hi", type=int, default=33)
    p.add_argument("--reps", type=int, default=5)
    p.add_argument("--sweep", choices=["none", "bits", "n", "shapes", "plans"], default="none")
    p.add_argument("--radix-bits", type=int, default=-1, help="widest digit of keys-only sorts (8..11)")
    p.add_argument("--pairs", action="store_true", help="key/value pairs (values = input positions)")
    p.add_argument("--shape", type=int, default=-1, help="digit-pass kernel shape (dagc_set_option)")
    a = p.parse_args(argv)
    import dag_compression_fast_gb300 as D
    ctx = D.Context(0)
    opt = D.OPT_SORT_SHAPE_PAIRS if a.pairs else D.OPT_SORT_SHAPE_KEYS
    if a.shape >= 0:
        ctx.set_option(opt, a.shape)
    if a.radix_bits >= 0:
        ctx.set_option(D.OPT_SORT_RADIX_BITS, a.radix_bits)
    if a.sweep == "plans":
        # every keys-only shape at every digit width: shape;bits;passes;keys;G keys/s;GB/s
        for sh in range(D.NUM_KEY_SHAPES):
            for rb in D.RADIX_BITS:
                ctx.set_option(D.OPT_SORT_SHAPE_KEYS, sh)
                ctx.set_option(D.OPT_SORT_RADIX_BITS, rb)
                if ctx.sort_plan(a.n, a.lo, a.hi) != (sh, rb):
                    continue  # not a valid plan for this range
                gk, gb = run(ctx, a.n, a.lo, a.hi, a.reps)
                print(f"plan shape={sh} bits={rb};passes={(a.hi - a.lo + rb - 1) // rb};{a.n};{gk:.3f};{gb:.1f}",
                      flush=True)
    elif a.sweep == "shapes":
        for sh in range(D.NUM_PAIR_SHAPES if a.pairs else D.NUM_KEY_SHAPES):
            ctx.set_option(opt, sh)
            gk, gb = run(ctx, a.n, a.lo, a.hi, a.reps, pairs=a.pairs)
            print(f"shape={sh};{'pairs' if a.pairs else 'keys'};{a.hi - a.lo};{a.n};{gk:.3f};{gb:.1f}", flush=True)
    elif a.sweep == "bits":
        for bits in range(1, 65):
            gk, gb = run(ctx, 100_000_000, 0, bits, a.reps)
            print(f"{bits};{100_000_000};{gk:.3f};{gb:.1f}", flush=True)
    elif a.sweep == "n":
        for n in [1_000_000, 2_000_000, 5_000_000, 10_000_000, 20_000_000, 50_000_000, 100_000_000, 200_000_000]:
            gk, gb = run(ctx, n, 0, 64, a.reps)
            print(f"64;{n};{gk:.3f};{gb:.1f}", flush=True)
    else:
        gk, gb = run(ctx, a.n, a.lo, a.hi, a.reps, pairs=a.pairs)
        print(f"{a.hi - a.lo};{a.n};{gk:.3f};{gb:.1f}", flush=True)
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
