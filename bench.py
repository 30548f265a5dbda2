#!/usr/bin/env python
"""Benchmark: input voxels/s from Morton fragments to the final DAG on GB300.

Workload: the procedural terrain of a 2048^3 grid (depth 11): 4-octave fBm
heightfield, 3-voxel-thick surface, every voxel emitted U{1..4} times and
shuffled -> ~31.5M uint64 fragments (252 MB, larger than the 129 MB L2, so
every step streams from HBM). Seeded synthetic data stands in for the
reference's voxelized glTF scene.

One step = DAGCompression::CreateDAG + CreateFinalDAG through the dagc C ABI,
from device-resident fragments to the device-resident uint32 DAG.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

--impl reference times the reference's algorithm on the host cores instead
(the CPU oracle, all threads), same workload and metric.
Multi-GPU runs (torchrun) are independent replicas: the path has no exchange
step on one volume, so each rank compresses its own copy ("weak" scaling).
"""
from __future__ import annotations

import argparse
import json
import os
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
DEPTH = 11
SEED = 0xDA6C0DE + 1
WORKLOAD = "terrain_fbm_2048^3_depth11"
L2_NOTE = "inputs (252 MB of fragments per step) larger than the 129 MB L2"


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="dagc", choices=["dagc", "reference"])
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline sample budget")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


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
    """nvidia-smi clocks / throttle reasons sampled every 200 ms in the background."""

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
                 "-i", str(self.device), "-lms", "200"],
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
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(codes: np.ndarray, budget_s: float):
    """The oracle (the reference's algorithm restated on the CPU) on the same
    fragments with every host thread; repeated until the budget is spent."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    O.create_dag(codes[:1000], DEPTH, threads)  # load + warm
    reps, t0 = 0, time.perf_counter()
    while True:
        d = O.create_dag(codes, DEPTH, threads)
        O.final_dag(d)
        reps += 1
        el = time.perf_counter() - t0
        if el >= budget_s or reps >= 50:
            break
    return {"value": codes.size * reps / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"full workload ({codes.size} fragments) x {reps} runs of CreateDAG+CreateFinalDAG, "
                      f"{el:.1f} s, oracle threads={threads}"}


def run_reference(args, world, rank):
    if rank != 0:
        return
    import dag_compression_fast_gb300 as D
    codes = D.gen_terrain(DEPTH, SEED)
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        O.final_dag(O.create_dag(codes, DEPTH, threads))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.final_dag(O.create_dag(codes, DEPTH, threads))
    el = time.perf_counter() - t0
    value = codes.size * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded fBm terrain)",
        "config": {"workload": WORKLOAD, "fragments": int(codes.size), "depth": DEPTH},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"full workload per step, {args.steps} steps, oracle threads={threads}"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


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
    codes = D.gen_terrain(DEPTH, SEED)
    n = int(codes.size)
    ctx = D.Context(local)
    d_codes = torch.from_numpy(codes.view(np.int64)).to(dev)
    stream = torch.cuda.current_stream()

    def step():
        dag = ctx.create_dag(d_codes, DEPTH)
        words = ctx.create_final_dag(dag)
        nw = words.n
        words.free()
        return nw

    for _ in range(max(args.warmup, 3)):
        n_words = step()
    counts = ctx.last_counts()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- timed region: device-resident fragments -> device-resident DAG ----
    # (the production path: each call's kernel sequence replays as a CUDA graph)
    sampler = ClockSampler(local)
    sampler.start()
    launches0 = ctx.kernel_launches()
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    launches = ctx.kernel_launches() - launches0
    clocks = sampler.stop()
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = n * args.steps * world / (ms / 1e3)

    # ---- the same steps with CUDA events around every stage and digit pass ----
    ctx.profile(True)
    ctx.profile_reset()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    ctx.profile(False)
    prof = ctx.profile_read()

    # ---- end to end: pinned host fragments -> host words, copies included ----
    h_codes = torch.from_numpy(codes.view(np.int64)).pin_memory()
    h_view = h_codes.numpy().view(np.uint64)
    h_words = torch.empty(n_words, dtype=torch.int32).pin_memory()
    import ctypes
    lib = D.lib()
    sh = stream.cuda_stream
    nw = ctypes.c_uint64(0)
    for _ in range(2):
        ctx._check(lib.dagc_compress_host(ctx.handle, h_view.ctypes.data, n, DEPTH, sh, h_words.data_ptr(),
                                          n_words, ctypes.byref(nw)))
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ctx._check(lib.dagc_compress_host(ctx.handle, h_view.ctypes.data, n, DEPTH, sh, h_words.data_ptr(),
                                          n_words, ctypes.byref(nw)))
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_sync = {"value": n * args.steps * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 8 * n,
                "d2h_bytes_per_step": 4 * int(nw.value),
                "mode": "dagc_compress_host, one call per step, each waiting for the previous"}

    # ---- end to end through the serving API: the same steps as jobs of a
    # two-slot server (dagc_server_submit / dagc_server_wait). Every step still
    # copies its pinned host fragments in and its words out inside the timed
    # region; a step's host->device copy overlaps the previous step's kernels,
    # so the pace is the host link's (252 MB at ~211 GB/s). ----
    sv = D.Server(local, slots=2, hbm_budget_bytes=256 << 30)
    for _ in range(max(args.warmup, 2)):
        sv.wait(sv.submit(h_view, DEPTH))
    barrier()
    t0 = time.perf_counter()
    tickets = [sv.submit(h_view, DEPTH) for _ in range(args.steps)]
    pipe_words = 0
    for tk in tickets:
        w_out, _ = sv.wait(tk)
        pipe_words = len(w_out)
    pipe_s = time.perf_counter() - t0
    sv.close()
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([pipe_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        pipe_s = float(t.item())
    if pipe_words != int(nw.value):
        raise RuntimeError("serving path returned a different word count")
    e2e = {"value": n * args.steps * world / pipe_s, "unit": UNIT, "h2d_bytes_per_step": 8 * n,
           "d2h_bytes_per_step": 4 * pipe_words,
           "mode": "serving API, 2 slots: per step pinned host fragments -> device -> host words, "
                   "steps overlapped (wall clock over K steps)"}

    # ---- roofline of the dominant kernel of the path the device chose ----
    # Fragments with many per brick are grouped by hash (partition scatter +
    # per-partition tables); otherwise they are radix-sorted (the digit pass
    # dominates).
    peak, peak_kind = measured_peaks()
    pass_traffic = profile_figure("onesweep_pass_keys_20M_27bit.md", "dram_bytes_per_key_per_pass", n)
    group_kernels = {
        "group_sketch": ("group_probe + group_plan (sampled sketch, path choice)",
                         "group_probe_terrain_d11.md"),
        "group_scatter": ("group_scatter (fragments by partition: one read, one write)",
                          "group_scatter_terrain_d11.md"),
        "group_aggregate": ("group_aggregate (per-partition tables in shared memory: one read)",
                            "group_aggregate_terrain_d11.md"),
    }
    top = max(group_kernels, key=lambda k: prof[k][0])
    if prof[top][0] > prof["fragment_pass"][0]:
        label, prof_file = group_kernels[top]
        roofline = stage_roofline(prof, top, label, peak, peak_kind,
                                  profile_figure(prof_file, "dram_bytes_per_fragment", n))
        # The radix-sort path's digit pass on the same fragments, for reference
        # (it serves inputs with few fragments per brick).
        ctx.set_option(D.OPT_GROUP, 0)
        ctx.profile(True)
        ctx.profile_reset()
        for _ in range(2):
            step()
        torch.cuda.synchronize()
        ctx.profile(False)
        ctx.set_option(D.OPT_GROUP, 1)
        sort_prof = ctx.profile_read()
        roofline_sort = stage_roofline(sort_prof, "fragment_pass", "onesweep_pass (fragment sort, 8-bit digit, "
                                       "keys only; sort path forced)", peak, peak_kind, pass_traffic)
    else:
        roofline = stage_roofline(prof, "fragment_pass", "onesweep_pass (fragment sort, 8-bit digit, keys only)",
                                  peak, peak_kind, pass_traffic)
        roofline_sort = None
    stages = {k: {"ms_per_step": v[0] / args.steps, "launches_per_step": v[1] / args.steps,
                  "gbs": round((v[2] / 1e9) / (v[0] / 1e3), 1) if v[0] > 0 and v[2] else None}
              for k, v in prof.items() if v[1]}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded fBm terrain, stands in for the voxelized scene)",
        "config": {"workload": WORKLOAD, "fragments": n, "depth": DEPTH, "bricks": counts[1], "leaves": counts[2], "words": int(n_words),
                   "l2": L2_NOTE, "parallelism": f"replicas x{world}"},
        "e2e": e2e,
        "e2e_sync": e2e_sync,
        "roofline": roofline,
        "gpu_launches": int(launches),
        "stages": stages,
    }
    if roofline_sort:
        line["roofline_sort_pass"] = roofline_sort
    if clocks:
        line["clocks"] = clocks
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(codes, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
