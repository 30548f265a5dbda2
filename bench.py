#!/usr/bin/env python
"""Benchmark: input voxels/s from Morton fragments to the final DAG on GB300.

Headline workload (the largest single-GPU configuration): a random triangle
soup in an 8192^3 grid (depth 13). 2M triangles with seeded uniform vertex
positions and edge lengths log-uniform in 1-16 voxels, conservatively
surface-voxelized (triangle/box separating-axis test) to ~65M uint64 Morton
fragments, shuffled (520 MB, larger than the 129 MB L2, so every step streams
from HBM). Low redundancy (about 5.8 fragments per 4^3 brick): the device
takes the radix-sort path. Seeded synthetic data stands in for the
reference's voxelized glTF scene.

Second workload, reported under "terrain_2048": the fBm terrain heightfield
of a 2048^3 grid (depth 11), ~31.5M fragments, on which the device takes the
fragment-grouping path.

One step = DAGCompression::CreateDAG + CreateFinalDAG through the dagc C ABI
(dagc_compress, both in one call), from device-resident fragments to the
device-resident uint32 DAG.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

--impl reference times the reference's algorithm on the host cores instead
(the CPU restatement of src/DAGCompression.cu, every host thread), on the
same workload, metric and config.
Multi-GPU runs (torchrun) are independent replicas: the path has no exchange
step on one volume, so each rank compresses its own copy ("weak" scaling).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import platform
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

METRIC = "input voxels/sec to final DAG; % HBM roofline; batched p50/p99 ms per chunk"
UNIT = "voxels/s"

SOUP = {"name": "triangle_soup_8192^3_depth13_2M_triangles", "depth": 13, "seed": 0xDA6C0DE + 3,
        "triangles": 2_000_000}
TERRAIN = {"name": "terrain_fbm_2048^3_depth11", "depth": 11, "seed": 0xDA6C0DE + 1}


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=60)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="dagc", choices=["dagc", "reference"])
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline sample budget")
    p.add_argument("--soak-seconds", type=float, default=1.0,
                   help="untimed steps run right before the timed region while the clocks are sampled")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-terrain", action="store_true", help="skip the second (terrain) workload")
    return p.parse_args()


def soup_codes() -> np.ndarray:
    import dag_compression_fast_gb300 as D
    return D.gen_triangle_soup(SOUP["depth"], SOUP["seed"], SOUP["triangles"])


def terrain_codes() -> np.ndarray:
    import dag_compression_fast_gb300 as D
    return D.gen_terrain(TERRAIN["depth"], TERRAIN["seed"])


def bench_config(n: int, world: int) -> dict:
    """The config both arms print (identical keys and values)."""
    return {"workload": SOUP["name"], "fragments": int(n), "depth": SOUP["depth"], "triangles": SOUP["triangles"],
            "seed": SOUP["seed"], "voxelization": "conservative (triangle/box separating-axis test)",
            "l2": f"inputs ({8 * n / 1e6:.0f} MB of fragments per step) larger than the 129 MB L2",
            "parallelism": f"replicas x{world}"}


def cpu_model() -> str:
    try:
        for line in open("/proc/cpuinfo"):
            k = line.split(":")[0].strip().lower()
            if k in ("model name", "cpu model", "hardware"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.TimeoutExpired):
        pass
    return platform.processor() or platform.machine()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("DAGC_BENCH_GLOO") is None else "gloo")
    return world, rank, local


def measured_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_figure(name: str, key: str, scale: float):
    """A per-item DRAM byte count from a committed ncu summary (measured on a
    smaller case), scaled by the item count of this workload."""
    path = os.path.join(REPO, "profiles", name)
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith(key + ":"):
            return float(line.split(":")[1]) * scale
    return None


def stage_roofline(prof, stage, kernel, peak, peak_kind, traffic):
    ms, launches, nbytes = prof[stage]
    achieved = (nbytes / 1e9) / (ms / 1e3) if ms > 0 else 0.0
    return {"kernel": kernel, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_source": peak_kind, "traffic": traffic,
            "algorithmic_bytes_per_launch": nbytes // max(launches, 1),
            "avg_launch_ms": ms / max(launches, 1), "launches": launches,
            "timing": "CUDA events around each launch on the call's stream, over profiled steps run right "
                      "after the timed region (same workload)"}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 100 ms in the background."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", str(self.device), "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": max(power) if power else None}


def time_oracle(codes: np.ndarray, depth: int, threads: int, budget_s: float, max_reps: int = 50):
    """CreateDAG + CreateFinalDAG of the CPU restatement, repeated until the budget is spent."""
    from oracle import oracle as O
    O.create_dag(codes[:1000], depth, threads)  # load + warm
    reps, t0 = 0, time.perf_counter()
    while True:
        O.final_dag(O.create_dag(codes, depth, threads))
        reps += 1
        el = time.perf_counter() - t0
        if el >= budget_s or reps >= max_reps:
            return codes.size * reps / el, reps, el


def cpu_baseline(codes: np.ndarray, budget_s: float):
    """The oracle (the reference's algorithm restated on the CPU) on the same
    fragments with every host thread, plus one thread on a bounded prefix."""
    threads = os.cpu_count() or 1
    depth = SOUP["depth"]
    value, reps, el = time_oracle(codes, depth, threads, budget_s)
    sample = codes[: min(codes.size, 4_000_000)]
    v1, reps1, el1 = time_oracle(sample, depth, 1, budget_s / 2, max_reps=3)
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "cpu_model": cpu_model(),
            "sample": f"full workload ({codes.size} fragments) x {reps} runs of CreateDAG+CreateFinalDAG, "
                      f"{el:.1f} s, oracle threads={threads}",
            "single_thread": {"value": v1, "unit": UNIT, "cores": 1,
                              "sample": f"first {sample.size} fragments of the shuffled workload x {reps1} runs, "
                                        f"{el1:.1f} s"}}


def run_reference(args, world, rank):
    if rank != 0:
        return
    codes = soup_codes()
    threads = os.cpu_count() or 1
    from oracle import oracle as O
    depth = SOUP["depth"]
    t0 = time.perf_counter()
    for _ in range(max(args.warmup, 1)):
        O.final_dag(O.create_dag(codes, depth, threads))
    per_step = (time.perf_counter() - t0) / max(args.warmup, 1)
    # Each step is a bounded sample of the workload: the whole workload while
    # the timed steps fit in ~2 minutes, else a prefix of the shuffled
    # fragments (a uniform random subset) sized to fit.
    budget_s = 120.0
    sample = codes
    if per_step * args.steps > budget_s:
        sample = codes[: max(1, int(codes.size * budget_s / (per_step * args.steps)))]
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.final_dag(O.create_dag(sample, depth, threads))
    el = time.perf_counter() - t0
    value = sample.size * args.steps / el
    what = ("full workload" if sample.size == codes.size else
            f"first {sample.size} of the {codes.size} shuffled fragments (a uniform random subset)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded triangle soup, stands in for the voxelized scene)",
        "config": bench_config(codes.size, world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "cpu_model": cpu_model(),
                         "sample": f"{what} per step, {args.steps} steps, oracle threads={threads}"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def group_roofline(prof, peak, peak_kind, n):
    group_kernels = {
        "group_sketch": ("group_probe + group_plan (sampled sketch, path choice)", "group_probe_terrain_d11.md"),
        "group_scatter": ("group_scatter (fragments by partition: one read, one write)",
                          "group_scatter_terrain_d11.md"),
        "group_aggregate": ("group_aggregate (per-partition tables in shared memory: one read)",
                            "group_aggregate_terrain_d11.md"),
    }
    top = max(group_kernels, key=lambda k: prof[k][0])
    label, prof_file = group_kernels[top]
    return stage_roofline(prof, top, label, peak, peak_kind, profile_figure(prof_file, "dram_bytes_per_fragment", n))


def stage_table(prof, steps):
    return {k: {"ms_per_step": v[0] / steps, "launches_per_step": v[1] / steps,
                "gbs": round((v[2] / 1e9) / (v[0] / 1e3), 1) if v[0] > 0 and v[2] else None}
            for k, v in prof.items() if v[1]}


def main():
    args = parse_args()
    if args.impl == "reference":
        # Host-only arm: rank 0 times it, the other ranks exit without work.
        run_reference(args, int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")))
        return
    world, rank, local = dist_setup()
    import torch
    import dag_compression_fast_gb300 as D
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"
    depth = SOUP["depth"]
    codes = soup_codes()
    n = int(codes.size)
    ctx = D.Context(local)
    d_codes = torch.from_numpy(codes.view(np.int64)).to(dev)
    stream = torch.cuda.current_stream()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def max_over_ranks(x: float) -> float:
        if world > 1:
            import torch.distributed as dist
            t = torch.tensor([x], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            return float(t.item())
        return x

    def step_on(frags, dp):
        # CreateDAG + CreateFinalDAG in one call (dagc_compress): the words
        # come straight from the call's level pools, no DAG copied out.
        words = ctx.compress(frags, dp)
        nw = words.n
        words.free()
        return nw

    for _ in range(max(args.warmup, 3)):
        n_words = step_on(d_codes, depth)
    counts = ctx.last_counts()

    # ---- timed region: device-resident fragments -> device-resident DAG ----
    # (the production path: each call's kernel sequence replays as a CUDA
    # graph). The clock sampler runs through an untimed soak of steps right
    # before the timed K steps and through them, so that it sees the clocks
    # under this load even when K steps take only a fraction of a second.
    sampler = ClockSampler(local)
    sampler.start()
    t_soak = time.perf_counter()
    soak_steps = 0
    while time.perf_counter() - t_soak < args.soak_seconds:
        step_on(d_codes, depth)
        soak_steps += 1
    launches0 = ctx.kernel_launches()
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step_on(d_codes, depth)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms = max_over_ranks(e0.elapsed_time(e1))
    launches = ctx.kernel_launches() - launches0
    clocks = sampler.stop()
    value = n * args.steps * world / (ms / 1e3)

    # ---- the same steps with CUDA events around every stage and digit pass ----
    ctx.profile(True)
    ctx.profile_reset()
    for _ in range(args.steps):
        step_on(d_codes, depth)
    torch.cuda.synchronize()
    ctx.profile(False)
    prof = ctx.profile_read()

    # ---- end to end: pinned host fragments -> host words, copies included ----
    h_codes = torch.from_numpy(codes.view(np.int64)).pin_memory()
    h_view = h_codes.numpy().view(np.uint64)
    h_words = torch.empty(n_words, dtype=torch.int32).pin_memory()
    lib = D.lib()
    sh = stream.cuda_stream
    nw = ctypes.c_uint64(0)
    for _ in range(2):
        ctx._check(lib.dagc_compress_host(ctx.handle, h_view.ctypes.data, n, depth, sh, h_words.data_ptr(),
                                          n_words, ctypes.byref(nw)))
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx._check(lib.dagc_compress_host(ctx.handle, h_view.ctypes.data, n, depth, sh, h_words.data_ptr(),
                                          n_words, ctypes.byref(nw)))
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e_sync = {"value": n * args.steps * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 8 * n,
                "d2h_bytes_per_step": 4 * int(nw.value),
                "mode": "dagc_compress_host, one call per step, each waiting for the previous"}

    # ---- end to end through the serving API: the same steps as jobs of a
    # three-slot server (dagc_server_submit_into / dagc_server_wait), at most
    # four in flight. Every step still copies its pinned host fragments in
    # and its words out (into pinned host buffers) inside the timed region; a
    # step's copies overlap other steps' kernels (two slots leave part of the
    # copies exposed: 6.1 against 5.1 ms per step on the soup). ----
    slots, window = 3, 4
    sv = D.Server(local, slots=slots, hbm_budget_bytes=256 << 30)
    outs = [torch.empty(n_words, dtype=torch.int32).pin_memory().numpy().view(np.uint32) for _ in range(window)]
    for i in range(max(args.warmup, 2)):
        sv.wait(sv.submit_into(h_view, depth, outs[i % window]))
    barrier()
    t0 = time.perf_counter()
    pending = []
    pipe_words = 0
    for i in range(args.steps):
        if len(pending) == window:
            w_out, _ = sv.wait(pending.pop(0))
            pipe_words = len(w_out)
        pending.append(sv.submit_into(h_view, depth, outs[i % window]))
    for tk in pending:
        w_out, _ = sv.wait(tk)
        pipe_words = len(w_out)
    pipe_s = max_over_ranks(time.perf_counter() - t0)
    sv.close()
    del h_codes, h_view, h_words
    if pipe_words != int(nw.value):
        raise RuntimeError("serving path returned a different word count")
    e2e_serving = {"value": n * args.steps * world / pipe_s, "unit": UNIT, "h2d_bytes_per_step": 8 * n,
                   "d2h_bytes_per_step": 4 * pipe_words,
                   "mode": f"serving API, {slots} slots, {window} jobs in flight: per step pinned host fragments -> "
                           "device -> pinned host words, steps overlapped (wall clock over K steps)"}
    # The headline e2e is the faster of the two ways through the public API.
    e2e = dict(e2e_serving if e2e_serving["value"] >= e2e_sync["value"] else e2e_sync)

    # ---- roofline of the dominant kernel of the path the device chose ----
    # Fragments with few per brick are radix-sorted (the digit pass
    # dominates); with many per brick they are grouped by hash.
    peak, peak_kind = measured_peaks()
    pass_traffic = profile_figure("onesweep_pass_keys_soup_d13.md", "dram_bytes_per_key_per_pass", n)
    if prof["fragment_pass"][2] > 0:
        roofline = stage_roofline(prof, "fragment_pass", "onesweep_pass (fragment sort digit pass, keys only)",
                                  peak, peak_kind, pass_traffic)
    else:
        roofline = group_roofline(prof, peak, peak_kind, n)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded triangle soup, stands in for the voxelized scene)",
        "config": bench_config(n, world),
        "counts": {"bricks": counts[1], "leaves": counts[2], "words": int(n_words),
                   "nodes_per_level": counts[3:]},
        "e2e": e2e,
        "e2e_sync": e2e_sync,
        "e2e_serving": e2e_serving,
        "roofline": roofline,
        "gpu_launches": int(launches),
        "stages": stage_table(prof, args.steps),
        "timed_region_s": ms / 1e3,
        "soak": {"steps": soak_steps, "seconds": args.soak_seconds},
    }
    if clocks:
        clocks["window"] = "untimed soak right before the timed region, then the timed region"
        clocks["ms_per_step_x_sm_mhz"] = round(ms / args.steps * clocks["sm_mhz"], 1)
        line["clocks"] = clocks
    del d_codes
    torch.cuda.empty_cache()

    # ---- second workload: the fBm terrain (grouping path) ----
    if not args.no_terrain:
        t_codes = terrain_codes()
        tn = int(t_codes.size)
        td = torch.from_numpy(t_codes.view(np.int64)).to(dev)
        tdepth = TERRAIN["depth"]
        for _ in range(max(args.warmup, 3)):
            step_on(td, tdepth)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            step_on(td, tdepth)
        e1.record(stream)
        torch.cuda.synchronize()
        tms = max_over_ranks(e0.elapsed_time(e1))
        ctx.profile(True)
        ctx.profile_reset()
        for _ in range(args.steps):
            step_on(td, tdepth)
        torch.cuda.synchronize()
        ctx.profile(False)
        tprof = ctx.profile_read()
        line["terrain_2048"] = {
            "workload": TERRAIN["name"], "fragments": tn, "depth": tdepth, "seed": TERRAIN["seed"],
            "value": tn * args.steps * world / (tms / 1e3), "unit": UNIT, "ms_per_step": tms / args.steps,
            "roofline": group_roofline(tprof, peak, peak_kind, tn) if tprof["group_scatter"][2] > 0 else
            stage_roofline(tprof, "fragment_pass", "onesweep_pass", peak, peak_kind, None),
            "stages": stage_table(tprof, args.steps),
        }
        del td

    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(codes, args.cpu_seconds)
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
