"""Digit-pass autotuner: measures every valid plan (kernel shape x digit
width) of a grid of sort classes on this GPU and writes the winners to the
tuning file that every new context loads (sort_plans.json beside this
module, or --out).

A sort class is (keys-only or key/value, number of sorted bits, power of two
of the key count). The grid covers the sorts the compression path runs: the
fragment sort on the brick bits [6, 3*depth) for depths 7-13 and the batched
composite keys, the brick sort of the grouping path, the 64-bit hash
sorts of the radix dedup form and the sort of the distinct leaf masks.

  python -m dag_compression_fast_gb300.autotune [--reps 3] [--out FILE] [--quick]

Prints one JSON line per class (plan, its time, the default plan's time) and
a summary line.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_OUT = os.path.join(HERE, "sort_plans.json")

KEY_BITS = [15, 18, 21, 24, 27, 30, 32, 33, 36, 39, 64]
PAIR_BITS = [15, 21, 27, 32, 33, 64]


def classes(quick: bool):
    key_lg = range(12, 29, 4 if quick else 1)
    pair_lg = range(12, 25, 4 if quick else 1)
    for bits in KEY_BITS:
        for lg in key_lg:
            yield False, bits, lg
    for bits in PAIR_BITS:
        for lg in pair_lg:
            yield True, bits, lg


def main(argv=None) -> int:
    p = argparse.ArgumentParser()
    p.add_argument("--reps", type=int, default=3)
    p.add_argument("--out", default=DEFAULT_OUT)
    p.add_argument("--quick", action="store_true", help="every fourth key-count class only")
    a = p.parse_args(argv)
    import dag_compression_fast_gb300 as D
    ctx = D.Context(0)
    ctx.tune_clear()
    t0 = time.perf_counter()
    gain = []
    for values, bits, lg in classes(a.quick):
        n = int(1.41 * (1 << lg))
        lo = 6 if bits < 64 else 0
        r = ctx.tune_sort(n, lo, lo + bits, values, reps=a.reps)
        gain.append(r["default_ms"] / r["ms"] if r["ms"] > 0 else 1.0)
        print(json.dumps({"values": int(values), "bits": bits, "log2n": lg, "n": n, **r}), flush=True)
    ctx.tune_save(a.out)
    ctx.close()
    print(json.dumps({"classes": len(gain), "seconds": round(time.perf_counter() - t0, 1), "out": a.out,
                      "median_speedup_vs_default": sorted(gain)[len(gain) // 2] if gain else None}), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
