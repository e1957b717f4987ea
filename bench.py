#!/usr/bin/env python3
"""Benchmark of the AoS hot path on one GB300 (replicas when N > 1).

Default workload, the width sweep: for s = 1..16 uint32 words (4..64-byte
structs), a 2 GiB array of N_s = 2^31 / (4 s) structs of seeded random words
is copied through this library's device API twice — once with
load/store_warp_contiguous and once with the block interface
(load/store_array_warp_contiguous) — and in both kernels a lane exits between
its load and its store when its struct's first word w has w % 625 == 624, so
about 5 % of 32-struct warp groups run non-converged and take the per-thread
fallback.  One step = those 32 launches.  GB/s counts bytes read + bytes
written (the skipped structs are not written).

Timed work uses inputs far larger than L2 (2 GiB per array), so no L2 flush
is needed between iterations.  `e2e` measures the same sweep through the
host-buffer entry point trv_copy_host (pinned host memory in and out inside
the timed region).  `--impl reference` times the CPU form of the path (the
oracle's multithreaded port) on the same metric.
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
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "AoS copy/gather GB/s & % HBM peak, batched vs per-call (bit-exact); p99 ms"
UNIT = "GB/s"
ARRAY_BYTES = 1 << 31
MODULUS = 625
SENTINEL = 0xA5
WORDS = list(range(1, 17))
CONFIG = {
    "workload": "width sweep: contiguous AoS copy, s=1..16 x uint32 (4-64 B), 2 GiB arrays, "
                "load/store_warp_contiguous + block interface, 5% warps diverged by early exit",
    "structs_per_width": {str(s): ARRAY_BYTES // (4 * s) for s in WORDS},
    "exit_predicate": "first word % 625 == 624",
    "launches_per_step": 32,
    "l2": "inputs larger than L2 (2 GiB arrays), no flush",
    "parallelism": "replicas",
}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=30)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["trove", "reference"], default="trove")
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--no-check", action="store_true")
    return p.parse_args()


# ---- distributed plumbing (replicas: each rank runs the whole workload) -----

def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if args.impl == "trove" else "gloo")
    return world, rank, local


def reduce_max(value: float, world: int, device=None) -> float:
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ---- peaks, clocks -------------------------------------------------------------

def hbm_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampled every 100 ms while the timed region runs."""
    QUERY = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.file.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.file.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(names, parts[3:7]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.file.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ---- the trove arm -------------------------------------------------------------

def sweep_plan():
    return [(s, 4 * s, ARRAY_BYTES // (4 * s)) for s in WORDS]


def verify_sweep(torch, tg, src, dst, plan):
    """One untimed pass with dst pre-filled; checks every width and both APIs
    on the device against an independent torch computation of the expected
    bytes.  Returns structs written per width."""
    written = {}
    for s, w, n in plan:
        words0 = src[: n * w].view(torch.int32).view(n, s)[:, 0].to(torch.int64) & 0xFFFFFFFF
        skip = (words0 % MODULUS) == (MODULUS - 1)
        written[s] = int(n - int(skip.sum()))
        srcv = src[: n * w].view(n, w)
        for path in (tg.PATH_WARP, tg.PATH_BLOCK):
            dst.fill_(SENTINEL)
            tg.copy_exit(dst, src, n, w, MODULUS, path=path)
            dv = dst[: n * w].view(n, w)
            ok = torch.equal(dv[~skip], srcv[~skip]) and bool((dv[skip] == SENTINEL).all())
            ok = ok and bool((dst[n * w:] == SENTINEL).all())
            if not ok:
                raise SystemExit(f"bench verification failed: width {w} B, path {path}")
    return written


def run_cpu_baseline(args, threads: int):
    """The oracle's multithreaded port on a bounded sample of the sweep."""
    import numpy as np

    import oracle
    sample_bytes = 128 << 20
    src = oracle.random_words(sample_bytes // 4, 0, threads=threads).view(np.uint8)
    dst = np.zeros_like(src)
    plan = [(s, 4 * s, sample_bytes // (4 * s)) for s in WORDS]
    total_bytes, elapsed, passes = 0, 0.0, 0
    while elapsed < args.cpu_seconds or passes == 0:
        for s, w, n in plan:
            for _api in range(2):
                t0 = time.perf_counter()
                oracle.run_mt(oracle.OP_COPY_EXIT, dst, src, None, n, w, threads, modulus=MODULUS)
                elapsed += time.perf_counter() - t0
                total_bytes += 2 * n * w
        passes += 1
    return {"value": total_bytes / elapsed / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{passes} passes of the sweep on a 128 MiB array per width (both APIs), "
                      f"early-exit copy with the same predicate, {threads} threads"}


def run_trove(args, world, rank, local):
    import torch

    import trove_gb300 as tg
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    tg.load(build_if_missing=True)
    plan = sweep_plan()
    src = torch.empty(ARRAY_BYTES + 256, dtype=torch.uint8, device=dev)
    dst = torch.empty_like(src)
    tg.fill_random_u32(src, (ARRAY_BYTES + 256) // 4, seed=0)
    written = {s: n for s, _, n in plan}
    if not args.no_check:
        written = verify_sweep(torch, tg, src, dst, plan)
    bytes_per_step = sum(n * w + written[s] * w for s, w, n in plan) * 2
    stream = torch.cuda.current_stream(dev)

    def step(events=None):
        for s, w, n in plan:
            for path in (tg.PATH_WARP, tg.PATH_BLOCK):
                if events is not None:
                    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                    tg.copy_exit(dst, src, n, w, MODULUS, path=path, stream=stream)
                    b.record(stream)
                    events.append(((s, path), a, b))
                else:
                    tg.copy_exit(dst, src, n, w, MODULUS, path=path, stream=stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    barrier(world)
    torch.cuda.synchronize(dev)
    clocks = Clocks(local)
    events = []
    t_start, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for _ in range(args.steps):
        step(events)
    t_end.record(stream)
    torch.cuda.synchronize(dev)
    clock_info = clocks.stop()
    barrier(world)
    local_ms = t_start.elapsed_time(t_end)
    ms = reduce_max(local_ms, world, dev)

    # per-kernel launch durations (CUDA events on the launching stream)
    per = {}
    for key, a, b in events:
        per.setdefault(key, []).append(a.elapsed_time(b))
    peak, peak_kind = hbm_peak()
    kernels = []
    for (s, path), times in per.items():
        w, n = 4 * s, ARRAY_BYTES // (4 * s)
        alg = n * w + written[s] * w
        avg = sum(times) / len(times)
        kernels.append({"kernel": f"copy_exit_{'warp' if path == tg.PATH_WARP else 'block'}_{w}B",
                        "launches": len(times), "total_ms": round(sum(times), 3), "avg_ms": round(avg, 4),
                        "bytes_per_launch": alg, "gbs": round(alg / avg / 1e6, 1),
                        "frac": round(alg / avg / 1e6 / peak, 4)})
    kernels.sort(key=lambda k: -k["total_ms"])
    top = kernels[0]
    traffic = None
    tfile = ROOT / "profiles" / "traffic.json"
    if tfile.exists():
        traffic = json.loads(tfile.read_text()).get(top["kernel"])

    # end to end through the host-buffer entry point (pinned in/out)
    e2e = None
    if args.e2e_steps > 0:
        h_src = torch.empty(ARRAY_BYTES, dtype=torch.uint8).pin_memory()
        h_dst = torch.empty(ARRAY_BYTES, dtype=torch.uint8).pin_memory()
        h_src.copy_(src[:ARRAY_BYTES].cpu())
        tg.copy_host(h_dst, h_src, ARRAY_BYTES // 64, 64)  # warm the staging buffers
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            for s, w, n in plan:
                tg.copy_host(h_dst, h_src, n, w)
        e2e_s = reduce_max(time.perf_counter() - t0, world, dev)
        e2e_bytes = args.e2e_steps * sum(2 * n * w for s, w, n in plan) * world
        if not torch.equal(h_dst[: plan[-1][2] * 64], h_src[: plan[-1][2] * 64]):
            raise SystemExit("e2e verification failed")
        per_step_io = sum(n * w for s, w, n in plan)
        e2e = {"value": round(e2e_bytes / e2e_s / 1e9, 2), "unit": UNIT, "h2d_bytes_per_step": per_step_io,
               "d2h_bytes_per_step": per_step_io, "steps": args.e2e_steps,
               "path": "trv_copy_host per width (pinned host buffers, chunked H2D/kernel/D2H overlap)"}
        del h_src, h_dst

    cpu = run_cpu_baseline(args, os.cpu_count() or 1) if rank == 0 and world == 1 else None
    value = bytes_per_step * args.steps * world / (ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded splitmix64 words)",
        "config": CONFIG,
        "fraction_of_hbm_peak": round(value / world / peak, 4), "peak_gbs": peak, "peak_kind": peak_kind,
        "roofline": {"bound": "hbm", "kernel": top["kernel"], "achieved": top["gbs"], "peak": peak,
                     "unit": "GB/s", "frac": top["frac"], "traffic": traffic,
                     "bytes_per_launch": top["bytes_per_launch"], "peak_kind": f"of {peak_kind}"},
        "kernels": kernels,
        "e2e": e2e,
        "gpu_launches": args.steps * len(plan) * 2,
        "clocks": clock_info,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---- the reference arm: the CPU form of the path ------------------------------

def run_reference(args, world, rank):
    if rank != 0:
        return
    import numpy as np

    import oracle
    threads = os.cpu_count() or 1
    sample_bytes = 64 << 20
    src = oracle.random_words(sample_bytes // 4, 0, threads=threads).view(np.uint8)
    dst = np.zeros_like(src)
    plan = [(s, 4 * s, sample_bytes // (4 * s)) for s in WORDS]

    def step():
        done = 0
        for s, w, n in plan:
            for _api in range(2):
                oracle.run_mt(oracle.OP_COPY_EXIT, dst, src, None, n, w, threads, modulus=MODULUS)
                done += 2 * n * w
        return done

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    total = sum(step() for _ in range(args.steps))
    el = time.perf_counter() - t0
    value = total / el / 1e9
    sample = (f"each step: the sweep on a 64 MiB array per width (both APIs), early-exit copy, "
              f"{threads} threads (oracle port: the reference has no CPU implementation)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(el * 1e3 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded splitmix64 words)", "config": CONFIG,
        "cpu_baseline": {"value": round(value, 2), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 2), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_trove(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
