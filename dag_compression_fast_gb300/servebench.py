"""Serving workload: a Poisson stream of compression jobs through the serving
loop (dagc_server_*), at one or more arrival rates.

Jobs: generator uniform over {sphere shell, terrain, triangle soup}, depth
uniform in 8..11, fragment count log-normal (median 500k, sigma 1.5, capped at
16M). A fixed seeded pool of jobs is generated first; the timed stream replays
it at the given rate. Prints one JSON line per rate: p50/p99 latency (submit to
finished words on the host), voxels/s, and how many jobs overlapped.

  python -m dag_compression_fast_gb300.servebench --rates 100 300 1000 --jobs 60
"""
from __future__ import annotations

import argparse
import json
import sys
import threading
import time

import numpy as np


def make_jobs(count: int, seed: int):
    import dag_compression_fast_gb300 as D
    rng = np.random.default_rng(seed)
    jobs = []
    for i in range(count):
        kind = int(rng.integers(0, 3))
        depth = int(rng.integers(8, 12))
        target = min(16e6, float(np.exp(np.log(5e5) + 1.5 * rng.standard_normal())))
        g = 1 << depth
        if kind == 0:
            codes = D.gen_sphere_shell(depth, seed + i, target)
        elif kind == 1:
            codes = D.gen_terrain(depth, seed + i, min(1.0, target / (3.0 * g * g * 2.5)))
        else:
            codes = D.gen_triangle_soup(depth, seed + i, max(1, int(target / 32)))
        jobs.append((codes, depth, ["sphere", "terrain", "soup"][kind]))
    return jobs


def run_rate(srv, jobs, rate: float, seed: int):
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, len(jobs)))
    tickets = [None] * len(jobs)

    def submitter():
        t0 = time.perf_counter()
        for i, (codes, depth, _) in enumerate(jobs):
            delay = arrivals[i] - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            tickets[i] = srv.submit(codes, depth)

    start = time.perf_counter()
    th = threading.Thread(target=submitter)
    th.start()
    lat = []
    for i in range(len(jobs)):
        while tickets[i] is None:
            time.sleep(0.0002)
        _, ms = srv.wait(tickets[i])
        lat.append(ms)
    th.join()
    wall = time.perf_counter() - start
    frags = sum(int(c.size) for c, _, _ in jobs)
    return {"rate_per_s": rate, "jobs": len(jobs), "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "voxels_per_s": frags / wall, "wall_s": wall,
            "device_overlap": device_overlap([srv.timeline(t) for t in tickets])}


def device_overlap(intervals):
    """From the jobs' device intervals (CUDA events on each slot's stream):
    pairs of jobs whose work was on the GPU at the same time, and the sum of
    the intervals over their union (1.0: never more than one job at a time)."""
    iv = sorted((a, b) for a, b in intervals if b > a >= 0)
    pairs = sum(1 for i in range(len(iv)) for j in range(i + 1, len(iv)) if iv[j][0] < iv[i][1])
    union, cur_a, cur_b = 0.0, None, None
    for a, b in iv:
        if cur_b is None or a > cur_b:
            if cur_b is not None:
                union += cur_b - cur_a
            cur_a, cur_b = a, b
        else:
            cur_b = max(cur_b, b)
    if cur_b is not None:
        union += cur_b - cur_a
    total = sum(b - a for a, b in iv)
    return {"overlapping_pairs": pairs, "busy_ms": round(union, 3),
            "concurrency": round(total / union, 3) if union > 0 else None}


def main(argv=None) -> int:
    p = argparse.ArgumentParser()
    p.add_argument("--rates", type=float, nargs="+", default=[100.0, 300.0, 1000.0])
    p.add_argument("--jobs", type=int, default=60)
    p.add_argument("--slots", type=int, default=4)
    p.add_argument("--budget-gb", type=float, default=96.0)
    p.add_argument("--seed", type=int, default=0xDA6C0DE + 4)
    a = p.parse_args(argv)
    import dag_compression_fast_gb300 as D
    t0 = time.perf_counter()
    jobs = make_jobs(a.jobs, a.seed)
    gen_s = time.perf_counter() - t0
    srv = D.Server(0, slots=a.slots, hbm_budget_bytes=int(a.budget_gb * (1 << 30)))
    # Warm the slots with every job once, all at once: each slot grows its
    # arena and sees the call shapes, as a running server has. The rates
    # below then measure steady state; this pass's latencies are the cold
    # cost and are printed first.
    cold = run_rate(srv, jobs, 1e6, a.seed)
    print(json.dumps({"warmup_pass": True, "jobs": cold["jobs"], "p50_ms": cold["p50_ms"],
                      "p99_ms": cold["p99_ms"], "wall_s": cold["wall_s"]}), flush=True)
    for r in a.rates:
        res = run_rate(srv, jobs, r, a.seed + int(r))
        st = srv.stats()
        res.update({"slots": a.slots, "max_concurrent": st["max_concurrent"],
                    "fragments_total": sum(int(c.size) for c, _, _ in jobs),
                    "mix": {k: sum(1 for _, _, kk in jobs if kk == k) for k in ("sphere", "terrain", "soup")},
                    "generation_s": round(gen_s, 1)})
        print(json.dumps(res), flush=True)
    srv.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
