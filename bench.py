#!/usr/bin/env python3
"""Benchmark of the AoS hot path on one GB300 (replicas when N > 1).

With no flags the run covers all five configs of the benchmark: the width
sweep is the headline (`value`, `roofline`, `e2e`, `cpu_baseline`), and
copy12, the 21 gathers, the 4096-array batch, the serving stream and the
AoS <-> SoA conversions follow as sub-records under `details.configs`
(`--configs` picks them, `none` for
the sweep alone), each with its own clocks, roofline, bit-exact check and
CPU baseline; copy12 and the gathers also time the reference Trove's own
kernels on the same buffers, and the gathers their random-block ceiling.

--workload sweep (default; the width sweep): for s = 1..16 uint32 words
  (4..64-byte structs), a 2 GiB array of N_s = 2^31 / (4 s) structs of seeded
  random words is copied through this library's device API twice — once with
  load/store_warp_contiguous, once with the block interface
  (load/store_array_warp_contiguous) — and in both kernels a lane exits between
  its load and its store when its struct's first word w has w % 625 == 624, so
  about 5 % of 32-struct warp groups run non-converged and take the per-thread
  fallback.  One step = those 32 launches.
--workload copy12: one contiguous copy of 2^20 structs of 12 B through
  load/store_warp_contiguous, L2 flushed before every timed launch (the
  array fits in L2); also reports the L2-resident rate of 100 launches
  replayed from a CUDA graph.
--workload layout: AoS -> SoA and SoA -> AoS of a 2 GiB array for s = 1..16
  words (trv_aos_to_soa / trv_soa_to_aos); one step = those 32 launches.
--workload gather: dst[i] = src[idx[i]] over 2^24 structs for widths
  {8,12,16,24,32,48,64} B and index patterns permutation / runs of 32 /
  identity; one step = those 21 gathers, L2 flushed before each (their
  sources are near L2's size), value from the summed gather times.
--workload batch: 4096 arrays, lengths log-uniform in [2^10, 2^22] structs,
  widths uniform from {4,12,20,36,64} B, 50 % copy / 40 % gather (uniform
  indices) / 10 % scatter (permutation); one step = the whole batch as one
  persistent launch replayed from a CUDA graph; the same work as one plain
  launch per array is timed beside it, each of its steps on its own, and
  `batched_vs_per_call` is its median step over the median batch launch.

GB/s counts bytes read + bytes written + index bytes.  Every array is far
larger than L2 or the step streams far more than L2 (129 MB), so no flush is
needed between iterations (copy12 and gather flush).  Launch shapes come from the library's autotuner,
run before the timed region (its cache is saved and reloaded).  `e2e` times the
same work with pinned host buffers in and out inside the timed region (the
sweep: its own 32 early-exit copies on pinned host arrays).
`--impl reference` times the CPU form of the path (the oracle's
multithreaded port; the reference has no CPU implementation of its own) on
the machine's cores: for the sweep one pass over the full 2 GiB arrays per step,
value = the median step.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "AoS copy/gather GB/s & % HBM peak, batched vs per-call (bit-exact); p99 ms"
UNIT = "GB/s"
ARRAY_BYTES = 1 << 31
MODULUS = 625
NOMINAL_HBM_GBS = 8000.0  # HBM3e nominal; the roofline's peak is the measured copy rate
SENTINEL = 0xA5
WORDS = list(range(1, 17))
GATHER_N = 1 << 24
GATHER_WIDTHS = [8, 12, 16, 24, 32, 48, 64]
GATHER_PATTERNS = ["perm", "runs", "identity"]
BATCH_COUNT = 4096
BATCH_WIDTHS = [4, 12, 20, 36, 64]
COPY12_N = 1 << 20
FLUSH_BYTES = 256 << 20  # written between timed launches whose working set would sit in L2


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=30)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["trove", "reference"], default="trove")
    p.add_argument("--workload", choices=["sweep", "copy12", "gather", "batch", "serve", "layout"], default="sweep")
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--configs", default="copy12,gather,batch,serve,layout",
                   help="with the sweep (the default workload): the other configs (and the AoS<->SoA layout "
                        "conversions) measured after it as sub-records under details.configs, comma-separated, "
                        "or 'none'")
    p.add_argument("--sub-cpu-seconds", type=float, default=3.0,
                   help="CPU-baseline seconds of each sub-record")
    p.add_argument("--no-check", action="store_true")
    p.add_argument("--no-tune", action="store_true")
    p.add_argument("--array-mib", type=int, default=ARRAY_BYTES >> 20,
                   help="sweep: bytes per array in MiB (default 2048; smaller only for profiling)")
    p.add_argument("--tune-cache", default=os.environ.get(
        "TROVE_GB300_TUNE_CACHE", str(Path.home() / ".cache" / "trove_gb300" / "autotune.json")))
    return p.parse_args()


# ---- distributed plumbing (replicas: each rank runs the whole workload) -----

def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        if args.impl == "trove":
            import torch
            torch.cuda.set_device(local)  # before NCCL binds the rank to a device
            dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        else:
            dist.init_process_group("gloo")
    return world, rank, local


def reduce_max(value: float, world: int, device=None) -> float:
    """Maximum of `value` over all ranks (the slowest replica's time)."""
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


class NvmlClocks:
    """SM / memory clocks and clock-event reasons read through NVML (the
    driver's libnvidia-ml, read-only queries) every 2 ms from a background
    thread while the timed region runs, so regions far shorter than
    nvidia-smi's sampling period are sampled too.  Raises OSError when NVML
    or the device cannot be opened."""
    CLOCK_SM, CLOCK_MEM = 1, 2  # nvmlClockType_t
    # clock-event reason bits of the NVML API
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, pci_bus_id: str | None, index: int):
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.lib = lib
        self.dev = ctypes.c_void_p()
        rc = -1
        if pci_bus_id:
            rc = lib.nvmlDeviceGetHandleByPciBusId_v2(pci_bus_id.encode(), ctypes.byref(self.dev))
        if rc != 0:
            rc = lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(index), ctypes.byref(self.dev))
        if rc != 0:
            lib.nvmlShutdown()
            raise OSError("no NVML handle for the device")
        self.reason_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
        mx = ctypes.c_uint(0)
        self.sm_max = float(mx.value) if lib.nvmlDeviceGetMaxClockInfo(self.dev, self.CLOCK_SM, ctypes.byref(mx)) == 0 \
            else None
        self.sm, self.mem, self.reasons = [], [], set()
        self.stop_flag = threading.Event()
        self.thread = threading.Thread(target=self._run, daemon=True)
        self.thread.start()

    def _run(self):
        sm, mem, why = ctypes.c_uint(0), ctypes.c_uint(0), ctypes.c_ulonglong(0)
        while True:
            if self.lib.nvmlDeviceGetClockInfo(self.dev, self.CLOCK_SM, ctypes.byref(sm)) == 0:
                self.sm.append(float(sm.value))
            if self.lib.nvmlDeviceGetClockInfo(self.dev, self.CLOCK_MEM, ctypes.byref(mem)) == 0:
                self.mem.append(float(mem.value))
            if self.reason_fn(self.dev, ctypes.byref(why)) == 0:
                for bit, name in self.REASONS.items():
                    if why.value & bit:
                        self.reasons.add(name)
            if self.stop_flag.wait(0.002):
                break

    def stop(self):
        self.stop_flag.set()
        self.thread.join()
        self.lib.nvmlShutdown()
        return {"sm_mhz": statistics.median(self.sm) if self.sm else None, "sm_max_mhz": self.sm_max,
                "mem_mhz": statistics.median(self.mem) if self.mem else None, "samples": len(self.sm),
                "reasons": sorted(self.reasons), "source": "nvml"}


def clock_sampler(torch, dev):
    """NVML poller when NVIDIA's management library opens, else nvidia-smi."""
    index = dev.index or 0
    try:
        p = torch.cuda.get_device_properties(dev)
        bus = "%08x:%02x:%02x.0" % (p.pci_domain_id, p.pci_bus_id, p.pci_device_id)
    except Exception:
        bus = None
    try:
        return NvmlClocks(bus, index)
    except (OSError, AttributeError):
        return Clocks(index)


class Clocks:
    """nvidia-smi sampled every 100 ms while the timed region runs (a region
    much shorter than that gets no sample: run it for more steps)."""
    QUERY = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap,clocks.mem")

    def __init__(self, index: int):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.skip = 0
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        # The sampler takes a moment to start: wait (at most 3 s) for its first
        # line, so a short timed region is sampled too, and drop what it
        # recorded before the region began.
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
            with open(self.file.name) as f:
                lines = f.read().splitlines()
            if lines:
                self.skip = len(lines)
                break
            time.sleep(0.02)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.file.seek(0)
        sm, smax, mem, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.file.read().splitlines()[self.skip:]:
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
            if len(parts) > 7:
                try:
                    mem.append(float(parts[7]))
                except ValueError:
                    pass
        os.unlink(self.file.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "mem_mhz": statistics.median(mem) if mem else None, "samples": len(sm), "reasons": sorted(reasons),
                "source": "nvidia-smi"}


def timed(torch, dev, stream, world, steps, step_fn, label_events=True):
    """Run `steps` steps between barriers and device syncs; returns (max ms
    over ranks, per-launch events, clock record)."""
    torch.cuda.synchronize(dev)
    barrier(world)
    torch.cuda.synchronize(dev)
    clocks = clock_sampler(torch, dev)
    events = [] if label_events else None
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(steps):
        step_fn(events)
    b.record(stream)
    torch.cuda.synchronize(dev)
    clock_info = clocks.stop()
    barrier(world)
    return reduce_max(a.elapsed_time(b), world, dev), events, clock_info


def launch_with_events(torch, stream, events, key, fn):
    if events is None:
        fn()
        return
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    fn()
    b.record(stream)
    events.append((key, a, b))


def kernel_table(events, bytes_of, peak):
    per = {}
    for key, a, b in events:
        per.setdefault(key, []).append(a.elapsed_time(b))
    rows = []
    for key, times in per.items():
        avg = sum(times) / len(times)
        alg = bytes_of(key)
        rows.append({"kernel": key, "launches": len(times), "total_ms": round(sum(times), 3),
                     "avg_ms": round(avg, 4), "bytes_per_launch": alg, "gbs": round(alg / avg / 1e6, 1),
                     "frac": round(alg / avg / 1e6 / peak, 4)})
    rows.sort(key=lambda r: -r["total_ms"])
    return rows


def host_mem_available() -> int:
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


def load_tune_cache(tg, path):
    try:
        if Path(path).exists():
            tg.autotune_load(path)
    except Exception:
        pass


def save_tune_cache(tg, path):
    try:
        Path(path).parent.mkdir(parents=True, exist_ok=True)
        tg.autotune_save(path)
    except Exception:
        pass


# ---- the reference Trove on the same GPU (a baseline leg) ----------------------

def reference_kernels():
    """The reference Trove's own kernels for this path, compiled for sm_103a
    from the reference's headers (the harness cubin the GPU tests also run,
    built where the reference checkout exists and shipped with the
    repository).  Returns (module, None) or (None, why)."""
    try:
        import oracle
        ref = oracle.reference_cubin()
    except Exception as e:  # noqa: BLE001 - reported in the record
        return None, f"reference cubin not loadable: {e}"
    if ref is None:
        return None, "reference cubin not present (built only where the reference checkout exists)"
    return ref, None


def flushed_launch_ms(torch, stream, flush, fn, reps):
    """Mean CUDA-event time of `reps` launches of fn, each after an L2 flush
    (outside its events)."""
    times = []
    for _ in range(reps):
        with torch.cuda.stream(stream):
            flush.fill_(1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        times.append((a, b))
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in times) / reps


# ---- workloads -------------------------------------------------------------------

class Sweep:
    name = "width sweep"
    config = {
        "workload": "width sweep: contiguous AoS copy, s=1..16 x uint32 (4-64 B), 2 GiB arrays, "
                    "load/store_warp_contiguous + block interface, 5% warps diverged by early exit",
        "structs_per_width": {str(s): ARRAY_BYTES // (4 * s) for s in WORDS},
        "exit_predicate": "first word % 625 == 624",
        "launches_per_step": 32,
        "l2": "inputs larger than L2 (2 GiB arrays), no flush",
        "parallelism": "replicas",
    }

    def __init__(self, torch, tg, dev, args):
        self.torch, self.tg, self.dev = torch, tg, dev
        self.array_bytes = args.array_mib << 20
        self.plan = [(s, 4 * s, self.array_bytes // (4 * s)) for s in WORDS]
        self.src = torch.empty(self.array_bytes + 256, dtype=torch.uint8, device=dev)
        self.dst = torch.empty_like(self.src)
        tg.fill_random_u32(self.src, (self.array_bytes + 256) // 4, seed=0)
        if self.array_bytes != ARRAY_BYTES:
            self.config = dict(self.config, structs_per_width={str(s): n for s, _, n in self.plan},
                               workload=self.config["workload"].replace("2 GiB", f"{args.array_mib} MiB"),
                               l2=self.config["l2"].replace("2 GiB", f"{args.array_mib} MiB"))
        self.written = {s: n for s, _, n in self.plan}
        self.tuned = {}
        self.steps = args.steps

    def tune(self):
        tg = self.tg
        for s, w, n in self.plan:
            for op, path in ((tg.OP_COPY_EXIT_WARP, tg.PATH_WARP), (tg.OP_COPY_EXIT_BLOCK, tg.PATH_BLOCK)):
                if tg.autotune_lookup(tg.SCOPE_CALL, op, w, n) is None:
                    tg.autotune_call(op, w, n)
                self.tuned[f"{'warp' if path == tg.PATH_WARP else 'block'}_{w}B"] = \
                    tg.autotune_lookup(tg.SCOPE_CALL, op, w, n)[0].unroll

    def verify(self):
        torch, tg = self.torch, self.tg
        for s, w, n in self.plan:
            words0 = self.src[: n * w].view(torch.int32).view(n, s)[:, 0].to(torch.int64) & 0xFFFFFFFF
            skip = (words0 % MODULUS) == (MODULUS - 1)
            self.written[s] = int(n - int(skip.sum()))
            srcv = self.src[: n * w].view(n, w)
            for path in (tg.PATH_WARP, tg.PATH_BLOCK):
                self.dst.fill_(SENTINEL)
                tg.copy_exit(self.dst, self.src, n, w, MODULUS, path=path)
                dv = self.dst[: n * w].view(n, w)
                ok = torch.equal(dv[~skip], srcv[~skip]) and bool((dv[skip] == SENTINEL).all())
                ok = ok and bool((self.dst[n * w:] == SENTINEL).all())
                if not ok:
                    raise SystemExit(f"bench verification failed: width {w} B, path {path}")

    def bytes_per_step(self):
        return sum(n * w + self.written[s] * w for s, w, n in self.plan) * 2

    def launches_per_step(self):
        return 2 * len(self.plan)

    def step(self, stream, events):
        torch, tg = self.torch, self.tg
        for s, w, n in self.plan:
            for path in (tg.PATH_WARP, tg.PATH_BLOCK):
                key = f"copy_exit_{'warp' if path == tg.PATH_WARP else 'block'}_{w}B"
                launch_with_events(torch, stream, events, key, lambda: tg.copy_exit(
                    self.dst, self.src, n, w, MODULUS, path=path, stream=stream))

    def kernel_bytes(self, key):
        w = int(key.rsplit("_", 1)[1][:-1])
        s, n = w // 4, self.array_bytes // w
        return n * w + self.written[s] * w

    def e2e(self, world, steps):
        """The timed workload itself with host buffers: the same 32 early-exit
        copies (both APIs, every width, same unrolls) through trv_copy_exit
        on pinned host arrays, which the copy kernel reads and writes in
        place over the CPU-GPU link (every byte of input crosses host ->
        device and every copied byte device -> host inside the timed
        region)."""
        torch, tg = self.torch, self.tg
        ab = self.array_bytes
        h_src = torch.empty(ab + 256, dtype=torch.uint8).pin_memory()
        h_dst = torch.empty(ab + 256, dtype=torch.uint8).pin_memory()
        h_src.copy_(self.src.cpu())
        h_dst.fill_(SENTINEL)
        tg.copy_exit(h_dst, h_src, ab // 64, 64, MODULUS, path=tg.PATH_WARP)  # pages the buffers in
        torch.cuda.synchronize(self.dev)
        h_dst.fill_(SENTINEL)
        stream = torch.cuda.current_stream(self.dev)
        barrier(world)
        torch.cuda.synchronize(self.dev)
        t0 = time.perf_counter()
        for _ in range(steps):
            for s, w, n in self.plan:
                for path in (tg.PATH_WARP, tg.PATH_BLOCK):
                    tg.copy_exit(h_dst, h_src, n, w, MODULUS, path=path, stream=stream)
        torch.cuda.synchronize(self.dev)
        el = reduce_max(time.perf_counter() - t0, world, self.dev)
        # earlier widths wrote bytes that later widths skip, so check one width
        # on its own: the widest, both APIs, into a fresh sentinel buffer
        s, w, n = self.plan[-1]
        for path in (tg.PATH_WARP, tg.PATH_BLOCK):
            h_dst.fill_(SENTINEL)
            tg.copy_exit(h_dst, h_src, n, w, MODULUS, path=path, stream=stream)
            torch.cuda.synchronize(self.dev)
            self._check_host_exit(h_dst, h_src, s, w, n)
        h2d = 2 * sum(n * w for s, w, n in self.plan)
        d2h = 2 * sum(self.written[s] * w for s, w, n in self.plan)
        return {"value": round(steps * (h2d + d2h) * world / el / 1e9, 2), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": steps,
                "path": "the step's 32 early-exit copies through trv_copy_exit (warp and block APIs) on pinned "
                        "host buffers, read and written in place by the copy kernels over the CPU-GPU link"}

    def _check_host_exit(self, h_dst, h_src, s, w, n):
        torch = self.torch
        words0 = h_src[: n * w].view(torch.int32).view(n, s)[:, 0].to(torch.int64) & 0xFFFFFFFF
        skip = (words0 % MODULUS) == (MODULUS - 1)
        dv, sv = h_dst[: n * w].view(n, w), h_src[: n * w].view(n, w)
        if not (torch.equal(dv[~skip], sv[~skip]) and bool((dv[skip] == SENTINEL).all())):
            raise SystemExit("e2e verification failed")

    def reference_gpu(self, kernels):
        """The reference's own early-exit copy (`exit_copy_<s>`:
        load_warp_contiguous / store_warp_contiguous with the warp_converged()
        fallback, one struct per thread, 256-thread blocks) and the
        compiler-generated AoS copy (`direct_copy_<s>`: r[i] = s[i]) on the
        same 2 GiB arrays, after checking that the reference writes the same
        bytes as this library's warp-API kernel; each timed the way the step
        times this library's kernels (CUDA events around back-to-back
        launches, inputs far larger than L2, as many launches as the timed
        region had), against copy_exit_warp_<w>B."""
        import ctypes
        torch, tg = self.torch, self.tg
        ref, why = reference_kernels()
        if ref is None:
            return {"unavailable": why}
        stream = torch.cuda.current_stream(self.dev)
        out = torch.empty_like(self.dst)
        own = {k["kernel"]: k for k in kernels}

        def launch_ms(fn, reps):
            fn()
            evs = []
            for _ in range(reps):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                fn()
                b.record(stream)
                evs.append((a, b))
            torch.cuda.synchronize(self.dev)
            return sum(a.elapsed_time(b) for a, b in evs) / reps

        rows, t_ref_sum, t_own_sum, alg_sum, t_dir_sum, dir_sum = [], 0.0, 0.0, 0, 0.0, 0
        for s, w, n in self.plan:
            grid = (n + 255) // 256
            args = [ctypes.c_void_p(self.src.data_ptr()), ctypes.c_void_p(out.data_ptr()), ctypes.c_longlong(n),
                    ctypes.c_uint32(MODULUS)]
            dargs = [ctypes.c_void_p(self.src.data_ptr()), ctypes.c_void_p(out.data_ptr())]

            def ref_exit():
                ref.launch(f"exit_copy_{s}", grid, 256, args, stream.cuda_stream)

            def ref_direct():  # whole blocks only: that kernel has no bounds check
                ref.launch(f"direct_copy_{s}", n // 256, 256, dargs, stream.cuda_stream)

            out.fill_(SENTINEL)
            self.dst.fill_(SENTINEL)
            ref_exit()
            tg.copy_exit(self.dst, self.src, n, w, MODULUS, path=tg.PATH_WARP, stream=stream)
            torch.cuda.synchronize(self.dev)
            if not torch.equal(out, self.dst):
                raise SystemExit(f"bench verification failed: reference and library exit copies differ ({w} B)")
            t_ref = launch_ms(ref_exit, self.steps)
            t_dir = launch_ms(ref_direct, 3)
            key = f"copy_exit_warp_{w}B"
            t_own = own[key]["avg_ms"]
            alg = self.kernel_bytes(key)
            dalg = 2 * (n // 256 * 256) * w
            rows.append({"width": w, "reference_gbs": round(alg / t_ref / 1e6, 1),
                         "this_gbs": round(alg / t_own / 1e6, 1), "ratio": round(t_ref / t_own, 3),
                         "compiler_gbs": round(dalg / t_dir / 1e6, 1)})
            t_ref_sum += t_ref
            t_own_sum += t_own
            alg_sum += alg
            t_dir_sum += t_dir
            dir_sum += dalg
        return {"kernel": "exit_copy_<s> (reference load/store_warp_contiguous + warp_converged fallback) and "
                          "direct_copy_<s> (compiler) vs copy_exit_warp_<w>B",
                "bit_exact_vs_library": True, "launches_per_width": self.steps,
                "l2": "inputs larger than L2, back-to-back launches, as this library's",
                "reference_gbs": round(alg_sum / t_ref_sum / 1e6, 1), "this_gbs": round(alg_sum / t_own_sum / 1e6, 1),
                "compiler_gbs": round(dir_sum / t_dir_sum / 1e6, 1), "ratio": round(t_ref_sum / t_own_sum, 3),
                "widths": rows}

    def extra(self):
        return {"tuned_unroll": self.tuned}


class Gather:
    """21 gathers per step.  Their sources (128 MiB-1 GiB) are near L2's size
    and overlap from one gather to the next, and a gather may leave source
    lines persisting in L2, so L2 is flushed before every gather (outside
    its events) and the value is bytes over the summed gather times."""
    name = "gather"
    kernel_timed = True
    config = {
        "workload": "random gather dst[i]=src[idx[i]], 2^24 structs, widths 8-64 B, "
                    "idx = permutation / runs of 32 (p=0.5) / identity",
        "structs": GATHER_N, "widths": GATHER_WIDTHS, "patterns": GATHER_PATTERNS,
        "l2": "L2 flushed (256 MiB write) before every gather; value = bytes / summed gather times",
        "parallelism": "replicas",
    }

    def __init__(self, torch, tg, dev, args):
        self.torch, self.tg, self.dev = torch, tg, dev
        n = GATHER_N
        self.src = torch.empty(n * 64 + 256, dtype=torch.uint8, device=dev)
        tg.fill_random_u32(self.src, (n * 64 + 256) // 4, seed=0)
        self.dst = torch.empty(n * 64, dtype=torch.uint8, device=dev)
        self.idx = {p: torch.empty(n, dtype=torch.int32, device=dev) for p in GATHER_PATTERNS}
        tg.fill_permutation(self.idx["perm"], n, 1)
        tg.fill_run_indices(self.idx["runs"], n, 2)
        self.idx["identity"].copy_(torch.arange(n, dtype=torch.int32, device=dev))
        self.flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)
        torch.cuda.synchronize(dev)
        self.tuned = {}
        self.steps = args.steps

    def tune(self):
        tg = self.tg
        for w in GATHER_WIDTHS:
            if tg.autotune_lookup(tg.SCOPE_CALL, tg.OP_GATHER, w, GATHER_N) is None:
                tg.autotune_call(tg.OP_GATHER, w, GATHER_N)
            c = tg.autotune_lookup(tg.SCOPE_CALL, tg.OP_GATHER, w, GATHER_N)[0]
            self.tuned[f"{w}B"] = {"path": c.path, "unroll": c.unroll, "cache_policy": c.cache_policy}

    def verify(self):
        torch, tg, n = self.torch, self.tg, GATHER_N
        for w in GATHER_WIDTHS:
            srcv = self.src[: n * w].view(n, w)
            for p in GATHER_PATTERNS:
                tg.gather(self.dst, self.src, n, self.idx[p], n, w)
                if not torch.equal(self.dst[: n * w].view(n, w), srcv[self.idx[p].long()]):
                    raise SystemExit(f"bench verification failed: gather {w} B {p}")

    def bytes_per_step(self):
        return sum((2 * w + 4) * GATHER_N for w in GATHER_WIDTHS) * len(GATHER_PATTERNS)

    def launches_per_step(self):
        return len(GATHER_WIDTHS) * len(GATHER_PATTERNS)

    def step(self, stream, events):
        for w in GATHER_WIDTHS:
            for p in GATHER_PATTERNS:
                with self.torch.cuda.stream(stream):
                    self.flush.fill_(1)
                launch_with_events(self.torch, stream, events, f"gather_{p}_{w}B", lambda: self.tg.gather(
                    self.dst, self.src, GATHER_N, self.idx[p], GATHER_N, w, stream=stream))

    def kernel_bytes(self, key):
        return (2 * int(key.rsplit("_", 1)[1][:-1]) + 4) * GATHER_N

    def e2e(self, world, steps):
        """Per gather: H2D of that step's indices and source, gather, D2H of
        the result, all through pinned host memory."""
        torch, tg, n = self.torch, self.tg, GATHER_N
        h_src = torch.empty(n * 64, dtype=torch.uint8).pin_memory()
        h_src.copy_(self.src[: n * 64].cpu())
        h_idx = {p: self.idx[p].cpu().pin_memory() for p in GATHER_PATTERNS}
        h_dst = torch.empty(n * 64, dtype=torch.uint8).pin_memory()
        d_idx = torch.empty(n, dtype=torch.int32, device=self.dev)
        stream = torch.cuda.current_stream(self.dev)
        barrier(world)
        t0 = time.perf_counter()
        h2d = d2h = 0
        for _ in range(steps):
            for w in GATHER_WIDTHS:
                for p in GATHER_PATTERNS:
                    self.src[: n * w].copy_(h_src[: n * w], non_blocking=True)
                    d_idx.copy_(h_idx[p], non_blocking=True)
                    tg.gather(self.dst, self.src, n, d_idx, n, w, stream=stream)
                    h_dst[: n * w].copy_(self.dst[: n * w], non_blocking=True)
                    h2d += n * w + 4 * n
                    d2h += n * w
        torch.cuda.synchronize(self.dev)
        el = reduce_max(time.perf_counter() - t0, world, self.dev)
        return {"value": round(steps * self.bytes_per_step() * world / el / 1e9, 2), "unit": UNIT,
                "h2d_bytes_per_step": h2d // steps, "d2h_bytes_per_step": d2h // steps, "steps": steps,
                "path": "per gather: pinned H2D of src + idx, trv_gather, pinned D2H of dst"}

    def reference_gpu(self, kernels):
        """The reference's coalesced_ptr gather kernel (tests/benchmark.cu:90-99
        pattern, one struct per thread, 256-thread blocks) and the
        compiler-generated gather on the same buffers, bit-compared with this
        library's output and timed the same way (L2 flushed before each
        launch, mean over as many launches as the timed region had)."""
        import ctypes
        torch, tg, n = self.torch, self.tg, GATHER_N
        ref, why = reference_kernels()
        if ref is None:
            return {"unavailable": why}
        stream = torch.cuda.current_stream(self.dev)
        out = torch.empty_like(self.dst)
        own = {k["kernel"]: k for k in kernels}
        cases, t_ref_sum, t_own_sum, t_dir_sum, alg_sum = [], 0.0, 0.0, 0.0, 0
        per_pattern = {p: [0.0, 0.0, 0] for p in GATHER_PATTERNS}
        for w in GATHER_WIDTHS:
            s = w // 4
            for p in GATHER_PATTERNS:
                args = [ctypes.c_void_p(self.idx[p].data_ptr()), ctypes.c_void_p(self.src.data_ptr()),
                        ctypes.c_void_p(out.data_ptr())]

                def ref_gather():
                    ref.launch(f"shfl_gather_{s}", n // 256, 256, args, stream.cuda_stream)

                def direct_gather():
                    ref.launch(f"direct_gather_{s}", n // 256, 256, args, stream.cuda_stream)

                out.zero_()
                ref_gather()
                self.dst.zero_()
                tg.gather(self.dst, self.src, n, self.idx[p], n, w, stream=stream)
                torch.cuda.synchronize(self.dev)
                if not torch.equal(out[: n * w], self.dst[: n * w]):
                    raise SystemExit(f"bench verification failed: reference and library gathers differ ({w} B {p})")
                t_ref = flushed_launch_ms(torch, stream, self.flush, ref_gather, self.steps)
                t_dir = flushed_launch_ms(torch, stream, self.flush, direct_gather, 3)
                key = f"gather_{p}_{w}B"
                t_own = own[key]["avg_ms"]
                alg = (2 * w + 4) * n
                cases.append({"case": key, "reference_gbs": round(alg / t_ref / 1e6, 1),
                              "this_gbs": round(alg / t_own / 1e6, 1), "ratio": round(t_ref / t_own, 3),
                              "compiler_gbs": round(alg / t_dir / 1e6, 1)})
                t_ref_sum += t_ref
                t_own_sum += t_own
                t_dir_sum += t_dir
                alg_sum += alg
                pp = per_pattern[p]
                pp[0] += t_ref
                pp[1] += t_own
                pp[2] += alg
        return {"kernel": "shfl_gather_<s> (reference coalesced_ptr gather) and direct_gather_<s> (compiler)",
                "bit_exact_vs_library": True, "launches_per_case": self.steps,
                "l2": "flushed before every launch, as this library's",
                "reference_gbs": round(alg_sum / t_ref_sum / 1e6, 1), "this_gbs": round(alg_sum / t_own_sum / 1e6, 1),
                "compiler_gbs": round(alg_sum / t_dir_sum / 1e6, 1), "ratio": round(t_ref_sum / t_own_sum, 3),
                "ratio_by_pattern": {p: round(v[0] / v[1], 3) for p, v in per_pattern.items()},
                "cases": cases}

    def ceiling(self, kernels, refrec):
        """Per gather, the memory system's ceiling for its rows
        (trv_probe_block_gather: every aligned block each row overlaps read
        whole, best of block sizes 32 / 64 / 128 with each L2 prefetch-size
        hint, indices read and n * width bytes written), as gather bytes per
        second, and each implementation's fraction of it.  Plus the plain
        rate of random reads of aligned 32 / 64 / 128-byte blocks."""
        torch, tg, n = self.torch, self.tg, GATHER_N
        stream = torch.cuda.current_stream(self.dev)
        own = {k["kernel"]: k for k in kernels}
        refc = {c["case"]: c for c in (refrec or {}).get("cases", [])}
        variants = [(b, h) for b in (32, 64, 128) for h in (0, 64, 128)]
        reps = 3
        cases = []
        for w in GATHER_WIDTHS:
            for p in GATHER_PATTERNS:
                alg = (2 * w + 4) * n
                best = None
                for b, h in variants:
                    def probe():
                        tg.probe_block_gather(self.dst, self.src, n, self.idx[p], n, w, b, h, stream=stream)
                    probe()
                    t = flushed_launch_ms(torch, stream, self.flush, probe, reps)
                    if best is None or t < best[0]:
                        best = (t, b, h)
                key = f"gather_{p}_{w}B"
                ceil = alg / best[0] / 1e6
                row = {"case": key, "ceiling_gbs": round(ceil, 1), "block_bytes": best[1], "l2_hint": best[2],
                       "this_frac": round(own[key]["gbs"] / ceil, 3)}
                if key in refc:
                    row["reference_frac"] = round(refc[key]["reference_gbs"] / ceil, 3)
                cases.append(row)
        # plain random reads of aligned blocks: rows of exactly one block, a
        # permutation of the rows, over 1 GiB at most
        blocks = {}
        perm_half = torch.empty(n // 2, dtype=torch.int32, device=self.dev)
        tg.fill_permutation(perm_half, n // 2, 5)
        for b in (32, 64, 128):
            rows = n if b * n <= (1 << 30) else n // 2
            ix = self.idx["perm"] if rows == n else perm_half
            best = None
            for h in (0, 64, 128):
                def probe():
                    tg.probe_block_gather(self.dst, self.src, rows, ix, rows, b, b, h, stream=stream)
                probe()
                t = flushed_launch_ms(torch, stream, self.flush, probe, reps)
                if best is None or t < best[0]:
                    best = (t, h)
            blocks[str(b)] = {"blocks": rows, "source_bytes": rows * b, "l2_hint": best[1],
                              "blocks_per_us": round(rows / best[0] / 1e3, 1),
                              "read_gbs": round(rows * b / best[0] / 1e6, 1)}
        del perm_half
        fr = [c["this_frac"] for c in cases if c["case"].startswith("gather_perm")]
        return {"probe": "trv_probe_block_gather", "reps": reps, "l2": "flushed before every launch",
                "this_frac_perm_min": min(fr), "this_frac_perm_mean": round(sum(fr) / len(fr), 3),
                "cases": cases, "random_block_reads": blocks}

    def extra(self):
        return {"tuned": self.tuned}


class Batch:
    name = "batch"
    config = {
        "workload": "4096 AoS arrays in one persistent launch (CUDA graph): len log-uniform [2^10, 2^22] "
                    "structs, width uniform {4,12,20,36,64} B, 50% copy / 40% gather (uniform idx) / "
                    "10% scatter (permutation); compared with one plain launch per array",
        "arrays": BATCH_COUNT, "widths": BATCH_WIDTHS, "seed": 4,
        "l2": "each step moves ~110 GB, no flush",
        "parallelism": "replicas",
    }

    def __init__(self, torch, tg, dev, args):
        import numpy as np
        self.torch, self.tg, self.dev = torch, tg, dev
        rng = np.random.default_rng(4)
        ops = rng.choice([0, 1, 2], size=BATCH_COUNT, p=[0.5, 0.4, 0.1])
        widths = rng.choice(BATCH_WIDTHS, size=BATCH_COUNT)
        lens = np.exp(rng.uniform(math.log(1 << 10), math.log(1 << 22), size=BATCH_COUNT)).astype(np.int64)
        gen = torch.Generator(device=dev)
        gen.manual_seed(4)
        self.tasks, self.keep = [], []
        for k in range(BATCH_COUNT):
            op, w, n = int(ops[k]), int(widths[k]), int(lens[k])
            src = torch.empty(n * w, dtype=torch.uint8, device=dev)
            tg.fill_random_u32(src, n * w // 4, seed=100 + k)
            dst = torch.empty_like(src)
            idx = None
            if op == 1:
                idx = torch.empty(n, dtype=torch.int32, device=dev)
                tg.fill_uniform_indices(idx, n, n, seed=200 + k)
            elif op == 2:
                idx = torch.randperm(n, generator=gen, device=dev, dtype=torch.int32)
            self.tasks.append(dict(op=op, width=w, n=n, src=src, dst=dst, idx=idx, bound=n))
        torch.cuda.synchronize(dev)  # inputs ready before any side stream reads them
        self.stream = torch.cuda.Stream(dev)
        self.batch = None
        self.per_call_ms = None
        self.tuned = False

    def tune(self):
        self.tg.autotune_batch(self.tasks)
        self.tuned = True

    def build(self):
        self.batch = self.tg.Batch(self.tasks)
        with self.torch.cuda.stream(self.stream):
            self.batch.capture(self.stream)

    def verify(self):
        torch = self.torch
        if self.batch is None:
            self.build()
        for t in self.tasks:
            t["dst"].fill_(SENTINEL)
        # the fills ran on the current stream; the batch stream does not wait
        # for it by itself (torch's side streams are non-blocking)
        self.stream.wait_stream(torch.cuda.current_stream(self.dev))
        self.batch.launch(self.stream)
        self.stream.synchronize()
        for k, t in enumerate(self.tasks):
            n, w = t["n"], t["width"]
            s, d = t["src"].view(n, w), t["dst"].view(n, w)
            if t["op"] == 0:
                ok = torch.equal(d, s)
            elif t["op"] == 1:
                ok = torch.equal(d, s[t["idx"].long()])
            else:
                ok = torch.equal(d[t["idx"].long()], s)
            if not ok:
                raise SystemExit(f"bench verification failed: batch task {k}")

    def bytes_per_step(self):
        return self.batch.info()[1]

    def launches_per_step(self):
        return 1

    def step(self, stream, events):
        launch_with_events(self.torch, self.stream, events, "batch_kernel", lambda: self.batch.launch(self.stream))

    def kernel_bytes(self, key):
        return self.bytes_per_step()

    def time_per_call(self, steps):
        """The same work as one plain launch per array, each step timed on its
        own with CUDA events (two warm-up steps first): its host-bound launch
        loop varies from run to run, so the median step is what is compared."""
        torch = self.torch
        for _ in range(2):
            self.tg.run_per_call(self.tasks, stream=self.stream)
        self.stream.synchronize()
        evs = []
        for _ in range(steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(self.stream)
            self.tg.run_per_call(self.tasks, stream=self.stream)
            b.record(self.stream)
            evs.append((a, b))
        self.stream.synchronize()
        self.per_call_steps = sorted(a.elapsed_time(b) for a, b in evs)
        self.per_call_ms = statistics.median(self.per_call_steps)

    def e2e(self, world, steps):
        """Per step: pinned H2D of every source and index array, the batch,
        pinned D2H of every destination.  Host memory bounds the sample: every
        k-th array (k chosen so the pinned copies fit in a quarter of the
        available host memory, at most 24 GB) forms its own batch."""
        torch, tg = self.torch, self.tg
        avail = host_mem_available()
        budget = min(24 << 30, avail // 4) if avail else (8 << 30)
        total = sum(2 * t["n"] * t["width"] + (4 * t["n"] if t["idx"] is not None else 0) for t in self.tasks)
        stride = max(1, math.ceil(total / budget))
        sub = self.tasks[::stride]
        hs = [(t["src"].cpu().pin_memory(), t["idx"].cpu().pin_memory() if t["idx"] is not None else None,
               torch.empty(t["dst"].numel(), dtype=torch.uint8).pin_memory()) for t in sub]
        b = tg.Batch(sub)
        sub_bytes = b.info()[1]
        barrier(world)
        t0 = time.perf_counter()
        h2d = d2h = 0
        with torch.cuda.stream(self.stream):
            for _ in range(steps):
                for t, (hsrc, hidx, hdst) in zip(sub, hs):
                    t["src"].copy_(hsrc, non_blocking=True)
                    h2d += hsrc.numel()
                    if hidx is not None:
                        t["idx"].copy_(hidx, non_blocking=True)
                        h2d += hidx.numel() * 4
                b.launch(self.stream)
                for t, (_, _, hdst) in zip(sub, hs):
                    hdst.copy_(t["dst"], non_blocking=True)
                    d2h += hdst.numel()
        self.stream.synchronize()
        el = reduce_max(time.perf_counter() - t0, world, self.dev)
        b.close()
        return {"value": round(steps * sub_bytes * world / el / 1e9, 2), "unit": UNIT,
                "h2d_bytes_per_step": h2d // steps, "d2h_bytes_per_step": d2h // steps, "steps": steps,
                "sample": f"every {stride}th array ({len(sub)} arrays) as its own batch",
                "path": "pinned H2D of all inputs, trv_batch_launch, pinned D2H of all outputs"}

    def extra(self):
        bps = self.bytes_per_step()
        return {"tiles": self.batch.info()[0], "autotuned": self.tuned,
                "per_call": {"ms_per_step": round(self.per_call_ms, 3), "statistic": "median step",
                             "min_ms": round(self.per_call_steps[0], 3), "max_ms": round(self.per_call_steps[-1], 3),
                             "steps": len(self.per_call_steps),
                             "value": round(bps / self.per_call_ms / 1e6, 2), "unit": UNIT,
                             "launches_per_step": BATCH_COUNT},
                "batch_median_ms": round(self._batch_ms, 4),
                "batched_vs_per_call": round(self.per_call_ms / self._batch_ms, 3)}


class Copy12:
    """The single contiguous copy: 2^20 structs of 3 x uint32, one launch.
    Its 24 MiB fit in L2, so a 256 MiB buffer is written between timed
    launches (outside each launch's events) and the value is bytes over the
    summed launch times: the cold-L2 rate of one launch."""
    name = "copy12"
    kernel_timed = True
    config = {
        "workload": "contiguous copy: 2^20 structs of 3 x uint32 (12 B), seed 0, one trv_copy launch through "
                    "load/store_warp_contiguous, 256 threads/block",
        "structs": COPY12_N, "width": 12,
        "l2": "L2 flushed (256 MiB write) before every timed launch; value = bytes / summed launch times",
        "parallelism": "replicas",
    }

    def __init__(self, torch, tg, dev, args):
        self.torch, self.tg, self.dev = torch, tg, dev
        self.src = torch.empty(COPY12_N * 12, dtype=torch.uint8, device=dev)
        tg.fill_random_u32(self.src, COPY12_N * 3, seed=0)
        self.dst = torch.empty_like(self.src)
        self.flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)
        self.unroll = 0  # the library's default until tuned
        self.tuned = {}
        self.steps = args.steps
        torch.cuda.synchronize(dev)

    def _launch_ms(self, unroll, reps=7):
        """Median time of one flushed launch at the given unroll."""
        torch = self.torch
        times = []
        for _ in range(reps):
            self.flush.fill_(1)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            self.tg.copy(self.dst, self.src, COPY12_N, 12, path="warp", unroll=unroll)
            b.record()
            torch.cuda.synchronize(self.dev)
            times.append(a.elapsed_time(b))
        return statistics.median(times)

    def tune(self):
        """The warp-contiguous path is fixed by the workload; only its unroll
        (structs per lane) is chosen, by timing each one."""
        for u in (1, 2, 4, 8):
            self.tuned[u] = round(self._launch_ms(u) * 1e3, 2)
        self.unroll = min(self.tuned, key=self.tuned.get)

    def verify(self):
        self.dst.fill_(SENTINEL)
        self.tg.copy(self.dst, self.src, COPY12_N, 12, path="warp")
        if not self.torch.equal(self.dst, self.src):
            raise SystemExit("bench verification failed: 12 B contiguous copy")

    def bytes_per_step(self):
        return 2 * COPY12_N * 12

    def launches_per_step(self):
        return 1

    def step(self, stream, events):
        with self.torch.cuda.stream(stream):
            self.flush.fill_(1)
        launch_with_events(self.torch, stream, events, "copy_warp_12B", lambda: self.tg.copy(
            self.dst, self.src, COPY12_N, 12, path="warp", unroll=self.unroll, stream=stream))

    def kernel_bytes(self, key):
        return self.bytes_per_step()

    def e2e(self, world, steps):
        """trv_copy_host on pinned host buffers, one call per step."""
        torch, tg = self.torch, self.tg
        h_src = self.src.cpu().pin_memory()
        h_dst = torch.empty_like(h_src).pin_memory()
        tg.copy_host(h_dst, h_src, COPY12_N, 12)
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(steps):
            tg.copy_host(h_dst, h_src, COPY12_N, 12)
        el = reduce_max(time.perf_counter() - t0, world, self.dev)
        if not torch.equal(h_dst, h_src):
            raise SystemExit("e2e verification failed")
        return {"value": round(steps * self.bytes_per_step() * world / el / 1e9, 2), "unit": UNIT,
                "h2d_bytes_per_step": COPY12_N * 12, "d2h_bytes_per_step": COPY12_N * 12, "steps": steps,
                "path": "trv_copy_host: pinned host buffers read and written in place by the copy kernel"}

    def reference_gpu(self, kernels):
        """The reference's load/store_warp_contiguous copy (one struct per
        thread, 4096 blocks of 256; tests/benchmark.cu:52-88 pattern) on the
        same buffers, bit-compared and timed the same way (L2 flushed before
        each launch, mean over as many launches as the timed region had)."""
        import ctypes
        torch = self.torch
        ref, why = reference_kernels()
        if ref is None:
            return {"unavailable": why}
        stream = torch.cuda.current_stream(self.dev)
        out = torch.full_like(self.dst, SENTINEL)
        args = [ctypes.c_void_p(self.src.data_ptr()), ctypes.c_void_p(out.data_ptr())]

        def ref_copy():
            ref.launch("shfl_copy_3", COPY12_N // 256, 256, args, stream.cuda_stream)

        def direct_copy():  # the compiler-generated AoS copy, r[i] = s[i]
            ref.launch("direct_copy_3", COPY12_N // 256, 256, args, stream.cuda_stream)

        ref_copy()
        torch.cuda.synchronize(self.dev)
        if not torch.equal(out, self.src):
            raise SystemExit("bench verification failed: reference 12 B copy")
        t_ref = flushed_launch_ms(torch, stream, self.flush, ref_copy, self.steps)
        t_dir = flushed_launch_ms(torch, stream, self.flush, direct_copy, self.steps)
        t_own = kernels[0]["avg_ms"]
        return {"kernel": "shfl_copy_3 (reference load/store_warp_contiguous), direct_copy_3 (compiler)",
                "bit_exact": True, "launches": self.steps, "l2": "flushed before every launch, as this library's",
                "reference_us": round(t_ref * 1e3, 2), "this_us": round(t_own * 1e3, 2),
                "compiler_us": round(t_dir * 1e3, 2),
                "reference_gbs": round(self.bytes_per_step() / t_ref / 1e6, 1),
                "this_gbs": round(self.bytes_per_step() / t_own / 1e6, 1),
                "compiler_gbs": round(self.bytes_per_step() / t_dir / 1e6, 1), "ratio": round(t_ref / t_own, 3)}

    def extra(self):
        """L2-resident rate: 100 back-to-back launches replayed from one CUDA
        graph (no flush), the way a caller chaining small copies sees it."""
        torch, tg = self.torch, self.tg
        k = 100
        side = torch.cuda.Stream(self.dev)
        side.wait_stream(torch.cuda.current_stream(self.dev))
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side, capture_error_mode="thread_local"):
            for _ in range(k):
                tg.copy(self.dst, self.src, COPY12_N, 12, path="warp", unroll=self.unroll, stream=side)
        for _ in range(3):
            g.replay()
        torch.cuda.synchronize(self.dev)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(side)
        with torch.cuda.stream(side):
            g.replay()
        b.record(side)
        torch.cuda.synchronize(self.dev)
        per = a.elapsed_time(b) / k
        return {"unroll": self.unroll, "us_per_launch_by_unroll": self.tuned,
                "graph_back_to_back": {"launches": k, "us_per_launch": round(per * 1e3, 2),
                                       "gbs": round(self.bytes_per_step() / per / 1e6, 1), "l2": "resident"}}


class Layout:
    """AoS -> SoA -> AoS on 2 GiB arrays of s = 1..16 words: one step is both
    conversions for every width (32 launches).  The AoS side moves through the
    device API (warp-contiguous rounds + transpose), the SoA side as s
    coalesced 32-bit planes."""
    name = "layout"
    config = {
        "workload": "AoS->SoA and SoA->AoS conversion (trv_aos_to_soa / trv_soa_to_aos), s=1..16 x uint32 "
                    "(4-64 B), 2 GiB arrays",
        "structs_per_width": {str(s): ARRAY_BYTES // (4 * s) for s in WORDS},
        "l2": "inputs larger than L2 (2 GiB arrays), no flush",
        "parallelism": "replicas",
    }

    def __init__(self, torch, tg, dev, args):
        self.torch, self.tg, self.dev = torch, tg, dev
        self.plan = [(s, 4 * s, ARRAY_BYTES // (4 * s)) for s in WORDS]
        self.aos = torch.empty(ARRAY_BYTES, dtype=torch.uint8, device=dev)
        tg.fill_random_u32(self.aos, ARRAY_BYTES // 4, seed=7)
        self.soa = torch.empty_like(self.aos)
        self.back = torch.empty_like(self.aos)
        self.tuned = {}
        torch.cuda.synchronize(dev)

    def tune(self):
        tg = self.tg
        for s, w, n in self.plan:
            for op, name in ((tg.OP_AOS_TO_SOA, "aos_to_soa"), (tg.OP_SOA_TO_AOS, "soa_to_aos")):
                if tg.autotune_lookup(tg.SCOPE_CALL, op, w, n) is None:
                    tg.autotune_call(op, w, n)
                self.tuned[f"{name}_{w}B"] = tg.autotune_lookup(tg.SCOPE_CALL, op, w, n)[0].unroll

    def verify(self):
        torch, tg = self.torch, self.tg
        for s, w, n in self.plan:
            tg.aos_to_soa(self.soa, self.aos, n, w)
            tg.soa_to_aos(self.back, self.soa, n, w)
            words = self.aos[: n * w].view(torch.int32).view(n, s)
            planes = self.soa[: n * w].view(torch.int32).view(s, n)
            ok = torch.equal(self.back[: n * w], self.aos[: n * w])
            ok = ok and all(torch.equal(planes[j], words[:, j]) for j in sorted({0, s - 1}))
            if not ok:
                raise SystemExit(f"bench verification failed: layout {w} B")

    def bytes_per_step(self):
        return sum(4 * n * w for s, w, n in self.plan)

    def launches_per_step(self):
        return 2 * len(self.plan)

    def step(self, stream, events):
        torch, tg = self.torch, self.tg
        for s, w, n in self.plan:
            launch_with_events(torch, stream, events, f"aos_to_soa_{w}B",
                               lambda: tg.aos_to_soa(self.soa, self.aos, n, w, stream=stream))
            launch_with_events(torch, stream, events, f"soa_to_aos_{w}B",
                               lambda: tg.soa_to_aos(self.back, self.soa, n, w, stream=stream))

    def kernel_bytes(self, key):
        w = int(key.rsplit("_", 1)[1][:-1])
        return 2 * (ARRAY_BYTES // w) * w

    def e2e(self, world, steps):
        return None

    def extra(self):
        return {"tuned_unroll": self.tuned}


SERVE_RATES = [2000, 5000, 10000, 20000, 50000]
SERVE_WIDTHS = [8, 12, 16, 28, 64]
SERVE_POOL = 1 << 23


def serve_requests(rate, seconds, seed, src_ptr, idx_ptr):
    """Seeded request stream: Poisson arrivals at `rate` per second for
    `seconds`; 50 % copy / 50 % gather, width uniform from SERVE_WIDTHS,
    length log-uniform in [256, 2^23] structs, sources and index windows at
    random offsets of the device-resident pools."""
    import numpy as np
    rng = np.random.default_rng(seed)
    count = max(1, int(rate * seconds))
    arrivals = np.cumsum(rng.exponential(1000.0 / rate, size=count))
    ops = rng.integers(0, 2, size=count)
    widths = rng.choice(SERVE_WIDTHS, size=count)
    lens = np.exp(rng.uniform(math.log(256), math.log(SERVE_POOL), size=count)).astype(np.int64)
    offs = (rng.random(size=count) * (SERVE_POOL - lens + 1)).astype(np.int64)
    reqs = []
    for k in range(count):
        w, n, off = int(widths[k]), int(lens[k]), int(offs[k])
        if ops[k] == 0:
            reqs.append({"op": 0, "width": w, "n": n, "src": src_ptr[w] + off * w, "src_n": n})
        else:
            reqs.append({"op": 1, "width": w, "n": n, "src": src_ptr[w], "src_n": SERVE_POOL, "idx": idx_ptr + 4 * off})
    return reqs, arrivals


class Serve:
    name = "serve"
    config = {
        "workload": "serving stream: Poisson arrivals at offered loads 2k-50k req/s, 50% copy / 50% gather, "
                    "len log-uniform [256, 2^23] structs, width from {8,12,16,28,64} B, uniform int32 indices, "
                    "device-resident sources, 64 GB HBM budget, continuous batching into the persistent kernel",
        "offered_loads_per_s": SERVE_RATES, "seconds_per_load": 1.0, "budget_bytes": 64 << 30,
        "max_inflight_batches": 4, "max_batch_requests": 1024,
        "l2": "each load moves tens of GB, no flush",
        "parallelism": "replicas",
    }

    def __init__(self, torch, tg, dev, args):
        self.torch, self.tg, self.dev = torch, tg, dev
        self.src = {}
        for w in SERVE_WIDTHS:
            t = torch.empty(SERVE_POOL * w, dtype=torch.uint8, device=dev)
            tg.fill_random_u32(t, SERVE_POOL * w // 4, seed=w)
            self.src[w] = t
        self.idx = torch.empty(SERVE_POOL, dtype=torch.int32, device=dev)
        tg.fill_uniform_indices(self.idx, SERVE_POOL, SERVE_POOL, seed=3)
        torch.cuda.synchronize(dev)  # the server's streams do not order after this one
        self.ptrs = {w: t.data_ptr() for w, t in self.src.items()}
        self.rows = []

    def tune(self):
        pass

    def verify(self):
        """300 requests served as a mixed stream must equal the same requests
        run alone, byte for byte."""
        torch, tg = self.torch, self.tg
        reqs, arr = serve_requests(20000, 0.015, 99, self.ptrs, self.idx.data_ptr())
        server = tg.Server(64 << 30, max_inflight=4, max_batch_requests=1024)
        ids, _ = server.replay(reqs, arr)
        for rid, r in zip(ids, reqs):
            res = server.wait(rid)
            n, w = r["n"], r["width"]
            got = torch.empty(n * w, dtype=torch.uint8, device=self.dev)
            tg.copy(got, res.dst, n, w)
            ref = torch.empty_like(got)
            if r["op"] == 0:
                tg.copy(ref, r["src"], n, w)
            else:
                tg.gather(ref, r["src"], r["src_n"], r["idx"], n, w)
            if not torch.equal(got, ref):
                raise SystemExit("bench verification failed: served request differs from the same request alone")
            server.release(rid)
        server.close()

    def run(self, seconds):
        tg = self.tg
        server = tg.Server(64 << 30, max_inflight=4, max_batch_requests=1024, release_when_done=True)
        # warm-up stream (not reported)
        reqs, arr = serve_requests(5000, 0.1, 1, self.ptrs, self.idx.data_ptr())
        server.replay(reqs, arr)
        total_bytes, total_ms = 0, 0.0
        for k, rate in enumerate(SERVE_RATES):
            reqs, arr = serve_requests(rate, seconds, 10 + k, self.ptrs, self.idx.data_ptr())
            _, st = server.replay(reqs, arr)
            span = st["last_done_ms"] - st["first_submit_ms"]
            self.rows.append({"offered_per_s": rate, "requests": st["completed"],
                              "achieved_per_s": round(st["completed"] / span * 1e3, 1),
                              "gbs": round(st["bytes"] / span / 1e6, 1), "p50_ms": round(st["p50_ms"], 3),
                              "p99_ms": round(st["p99_ms"], 3), "max_ms": round(st["max_ms"], 3),
                              "max_queued": st["max_queued"]})
            total_bytes += st["bytes"]
            total_ms += span
        stats = server.stats()
        server.close()
        return total_bytes, total_ms, stats


WORKLOADS = {"sweep": Sweep, "copy12": Copy12, "gather": Gather, "batch": Batch, "serve": Serve, "layout": Layout}


# ---- CPU baseline (the oracle's multithreaded port) ----------------------------

def cpu_sample(workload: str, threads: int, seconds: float, steps: int | None = None, full: bool = False,
               warmup: int = 1):
    """The CPU form of the workload (the oracle's multithreaded port) on a
    bounded sample: runs `steps` passes if given, else passes until `seconds`
    of work.  Returns (GB/s of the median pass, GB/s over all passes, passes,
    description).  `full`: the sweep on its real 2 GiB arrays instead of
    128 MiB ones."""
    import numpy as np

    import oracle
    if workload == "sweep":
        sample = ARRAY_BYTES if full else 128 << 20
        src = oracle.random_words(sample // 4, 0, threads=threads).view(np.uint8)
        dst = np.zeros_like(src)

        def one():
            done = 0
            for s in WORDS:
                w, n = 4 * s, sample // (4 * s)
                for _api in range(2):
                    oracle.run_mt(oracle.OP_COPY_EXIT, dst, src, None, n, w, threads, modulus=MODULUS)
                    done += 2 * n * w
            return done
        desc = (f"the sweep on a {sample >> 20} MiB array per width (both APIs), early-exit copy"
                + (" (the full workload)" if full else ""))
    elif workload == "layout":
        sample = 128 << 20
        src = oracle.random_words(sample // 4, 7, threads=threads).view(np.uint8)
        mid, back = np.zeros_like(src), np.zeros_like(src)

        def one():
            done = 0
            for s in WORDS:
                w, n = 4 * s, sample // (4 * s)
                oracle.run_mt(oracle.OP_AOS_TO_SOA, mid, src, None, n, w, threads)
                oracle.run_mt(oracle.OP_SOA_TO_AOS, back, mid, None, n, w, threads)
                done += 4 * n * w
            return done
        desc = "both conversions on a 128 MiB array per width"
    elif workload == "copy12":
        n = COPY12_N
        src = oracle.random_words(n * 3, 0, threads=threads).view(np.uint8)
        dst = np.zeros_like(src)

        def one():
            oracle.run_mt(oracle.OP_COPY, dst, src, None, n, 12, threads)
            return 2 * n * 12
        desc = "the 12 B copy of 2^20 structs (the whole workload)"
    elif workload == "gather":
        n = 1 << 21
        src = oracle.random_words(n * 16, 0, threads=threads).view(np.uint8)
        dst = np.zeros_like(src)
        idxs = {"perm": oracle.permutation(n, 1), "runs": oracle.run_indices(n, 2),
                "identity": np.arange(n, dtype=np.int32)}

        def one():
            done = 0
            for w in GATHER_WIDTHS:
                for p in GATHER_PATTERNS:
                    oracle.run_mt(oracle.OP_GATHER, dst, src, idxs[p], n, w, threads)
                    done += (2 * w + 4) * n
            return done
        desc = "the 21 gathers on 2^21 structs (1/8 of the workload's length)"
    elif workload == "serve":
        pool = 1 << 20
        srcs = {w: oracle.random_words(pool * w // 4, w, threads=threads).view(np.uint8) for w in SERVE_WIDTHS}
        pidx = oracle.uniform_indices(pool, pool, 3)
        rng = np.random.default_rng(10)
        sample = []
        for _ in range(200):
            w = int(rng.choice(SERVE_WIDTHS))
            n = int(np.exp(rng.uniform(math.log(256), math.log(pool))))
            off = int(rng.integers(0, pool - n + 1))
            sample.append((int(rng.integers(0, 2)), w, n, off))
        dst = np.zeros(pool * 64, np.uint8)

        def one():
            done = 0
            for op, w, n, off in sample:
                if op == 0:
                    oracle.run_mt(0, dst, srcs[w][off * w:], None, n, w, threads)
                    done += 2 * n * w
                else:
                    oracle.run_mt(1, dst, srcs[w], pidx[off:], n, w, threads)
                    done += 2 * n * w + 4 * n
            return done
        desc = "200 requests of the serving mix on 2^20-struct pools (lengths log-uniform up to 2^20)"
    else:
        rng = np.random.default_rng(4)
        ops = rng.choice([0, 1, 2], size=BATCH_COUNT, p=[0.5, 0.4, 0.1])
        widths = rng.choice(BATCH_WIDTHS, size=BATCH_COUNT)
        lens = np.exp(rng.uniform(math.log(1 << 10), math.log(1 << 22), size=BATCH_COUNT)).astype(np.int64)
        pick = list(range(0, BATCH_COUNT, 32))  # every 32nd array
        arrays = []
        for k in pick:
            n, w = int(lens[k]), int(widths[k])
            src = oracle.random_words(n * w // 4, 100 + k, threads=threads).view(np.uint8)
            idx = oracle.uniform_indices(n, n, 200 + k) if ops[k] == 1 else (
                oracle.permutation(n, 300 + k) if ops[k] == 2 else None)
            arrays.append((int(ops[k]), n, w, src, np.zeros_like(src), idx))

        def one():
            done = 0
            for op, n, w, src, dst, idx in arrays:
                oracle.run_mt(op, dst, src, idx, n, w, threads)
                done += 2 * n * w + (4 * n if op else 0)
            return done
        desc = "every 32nd array of the batch (128 arrays), same ops, widths and lengths"
    for _ in range(max(1, warmup)):  # warm caches and page in
        one()
    total, el, passes, rates, times = 0, 0.0, 0, [], []
    while (steps is not None and passes < steps) or (steps is None and (el < seconds or passes == 0)):
        t0 = time.perf_counter()
        moved = one()
        dt = time.perf_counter() - t0
        total += moved
        el += dt
        rates.append(moved / dt / 1e9)
        times.append(dt)
        passes += 1
    return (statistics.median(rates), total / el / 1e9, statistics.median(times),
            f"{passes} passes of {desc}, {threads} threads (oracle port); value = the median pass")


def run_reference(args, world, rank):
    """The reference arm: the CPU form of the path (the oracle's
    multithreaded port; the reference itself has no CPU implementation) on
    the machine's host cores.  For the sweep every step is one pass over the
    full 2 GiB arrays; value = the median step."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    med, mean, med_s, desc = cpu_sample(args.workload, threads, 0, steps=args.steps, warmup=args.warmup,
                                        full=args.workload == "sweep")
    cfg = WORKLOADS[args.workload].config
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": round(med, 2), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(med_s * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded splitmix64 words)", "config": cfg,
        "cpu_baseline": {"value": round(med, 2), "unit": UNIT, "cores": threads, "kind": "port",
                         "mean_over_passes": round(mean, 2),
                         "sample": desc + "; the reference has no CPU implementation of the path"},
        "e2e": {"value": round(med, 2), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def serve_record(torch, tg, dev, args, world, rank):
    """The serving workload: one open-loop replay per offered load; value =
    the bytes of all completed requests over the time from each stream's
    first submission to its last completion."""
    t_start = time.perf_counter()
    wl = Serve(torch, tg, dev, args)
    if not args.no_check:
        wl.verify()
    barrier(world)
    clocks = clock_sampler(torch, dev)
    total_bytes, total_ms, stats = wl.run(1.0)
    clock_info = clocks.stop()
    ms = reduce_max(total_ms, world, dev)
    peak, peak_kind = hbm_peak()
    value = total_bytes * world / (ms / 1e3) / 1e9
    top = max(wl.rows, key=lambda r: r["gbs"])
    rec = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": len(SERVE_RATES),
        "warmup": 1, "ms_per_step": round(ms / len(SERVE_RATES), 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded splitmix64 words)",
        "config": Serve.config, "bit_exact": not args.no_check,
        "fraction_of_hbm_peak": round(value / world / peak, 4), "peak_gbs": peak, "peak_kind": peak_kind,
        "roofline": {"bound": "hbm", "kernel": "batch_kernel (served)", "achieved": top["gbs"], "peak": peak,
                     "unit": "GB/s", "frac": round(top["gbs"] / peak, 4), "traffic": None,
                     "peak_kind": f"of {peak_kind}"},
        "latency_by_load": wl.rows, "p50_ms": {str(r["offered_per_s"]): r["p50_ms"] for r in wl.rows},
        "p99_ms": {str(r["offered_per_s"]): r["p99_ms"] for r in wl.rows},
        "e2e": None, "gpu_launches": int(stats["batches"]), "clocks": clock_info,
        "details": {"server": stats},
    }
    del wl
    rec["cpu_baseline"] = cpu_record("serve", args, world, rank)
    rec["wall_s"] = round(time.perf_counter() - t_start, 1)
    return rec


def cpu_record(workload, args, world, rank, seconds=None, single=False, full=False):
    """cpu_baseline of a record (rank 0, one GPU only)."""
    if rank != 0 or world != 1 or args.cpu_seconds <= 0:
        return None
    threads = os.cpu_count() or 1
    med, mean, _, desc = cpu_sample(workload, threads, args.cpu_seconds if seconds is None else seconds,
                                    full=full)
    rec = {"value": round(med, 2), "unit": UNIT, "cores": threads, "kind": "port", "mean_over_passes": round(mean, 2),
           "sample": desc}
    if single:
        med1, _, _, desc1 = cpu_sample(workload, 1, 0, steps=1, warmup=0)
        rec["single_thread"] = {"value": round(med1, 2), "unit": UNIT, "cores": 1, "sample": desc1}
    return rec


def measure(wl, torch, tg, dev, args, world, rank, e2e=True):
    """Tune, verify and time one workload; returns its JSON record."""
    t_start = time.perf_counter()
    if not args.no_tune:
        wl.tune()
        save_tune_cache(tg, args.tune_cache)
    if hasattr(wl, "build"):
        wl.build()
    if not args.no_check:
        wl.verify()
    stream = wl.stream if hasattr(wl, "stream") else torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        wl.step(stream, None)
    ms, events, clock_info = timed(torch, dev, stream, world, args.steps, lambda ev: wl.step(stream, ev))
    if getattr(wl, "kernel_timed", False):  # flushes ran between the launches: time the launches alone
        ms = reduce_max(sum(a.elapsed_time(b) for _, a, b in events), world, dev)
    peak, peak_kind = hbm_peak()
    bps = wl.bytes_per_step()
    value = bps * args.steps * world / (ms / 1e3) / 1e9
    kernels = kernel_table(events, wl.kernel_bytes, peak)
    top = kernels[0]
    traffic = None
    tfile = ROOT / "profiles" / "traffic.json"
    if tfile.exists():
        traffic = json.loads(tfile.read_text()).get(top["kernel"])
    if isinstance(wl, Batch):
        # both sides as the median step: the batch's launches from the timed
        # region, the per-call form's steps timed one by one
        wl._batch_ms = statistics.median(a.elapsed_time(b) for _, a, b in events)
        wl.time_per_call(max(5, args.steps // 2))
    rec = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded splitmix64 words)",
        "config": wl.config, "bit_exact": not args.no_check,
        "fraction_of_hbm_peak": round(value / world / peak, 4), "peak_gbs": peak, "peak_kind": peak_kind,
        "roofline": {"bound": "hbm", "kernel": top["kernel"], "achieved": top["gbs"], "peak": peak,
                     "unit": "GB/s", "frac": top["frac"], "traffic": traffic,
                     "bytes_per_launch": top["bytes_per_launch"], "peak_kind": f"of {peak_kind}",
                     "frac_of_nominal": round(top["gbs"] / NOMINAL_HBM_GBS, 4),
                     # DRAM bytes the kernel actually moves per launch (ncu) over its
                     # event-timed duration: how busy DRAM is, where random reads
                     # move whole DRAM blocks for narrower rows
                     "dram_frac": (round(traffic / (top["avg_ms"] * 1e6) / peak, 4) if traffic else None)},
        "kernels": kernels,
        "e2e": wl.e2e(world, args.e2e_steps) if e2e and args.e2e_steps > 0 else None,
        "gpu_launches": args.steps * wl.launches_per_step(),
        "clocks": clock_info,
        "details": wl.extra(),
    }
    if rank == 0 and hasattr(wl, "reference_gpu"):
        rec["reference_gpu"] = wl.reference_gpu(kernels)
    if hasattr(wl, "ceiling"):
        rec["ceiling"] = wl.ceiling(kernels, rec.get("reference_gpu"))
        # the dominant gather against the memory system's ceiling for its rows
        top_case = {c["case"]: c for c in rec["ceiling"]["cases"]}.get(top["kernel"])
        if top_case:
            rec["roofline"]["random_block_ceiling_gbs"] = top_case["ceiling_gbs"]
            rec["roofline"]["frac_of_random_block_ceiling"] = top_case["this_frac"]
    rec["wall_s"] = round(time.perf_counter() - t_start, 1)
    return rec


def targets(line, subs):
    """The benchmark's three targets, each with the figure this run measured."""
    out = {}
    ks = [k for k in line["kernels"] if k["kernel"].startswith("copy_exit_")]
    if ks:
        worst = min(k["gbs"] for k in ks)
        out["copy_at_85pct_of_hbm_peak_4_64B"] = {
            "slowest_kernel_gbs": worst, "frac_of_nominal_8000": round(worst / NOMINAL_HBM_GBS, 4),
            "frac_of_measured": round(worst / line["peak_gbs"], 4), "met": worst >= 0.85 * NOMINAL_HBM_GBS}
    g = subs.get("gather", {})
    rg = g.get("reference_gpu", {})
    if "ratio" in rg:
        out["random_gather_1p2x_reference"] = {
            "ratio": rg["ratio"], "ratio_by_pattern": rg.get("ratio_by_pattern"),
            "frac_of_random_block_ceiling_perm": {k: g["ceiling"][k] for k in ("this_frac_perm_min", "this_frac_perm_mean")}
            if "ceiling" in g else None,
            "met": rg.get("ratio_by_pattern", {}).get("perm", 0) >= 1.2}
    b = subs.get("batch", {}).get("details", {})
    if "batched_vs_per_call" in b:
        out["batched_2x_per_call"] = {"ratio": b["batched_vs_per_call"], "met": b["batched_vs_per_call"] >= 2.0}
    return out


def free_device(torch, dev):
    import gc
    gc.collect()
    torch.cuda.synchronize(dev)
    torch.cuda.empty_cache()


def run_trove(args, world, rank, local):
    import torch

    import trove_gb300 as tg
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    tg.load(build_if_missing=True)
    load_tune_cache(tg, args.tune_cache)
    if args.workload == "serve":
        line = serve_record(torch, tg, dev, args, world, rank)
    else:
        wl = WORKLOADS[args.workload](torch, tg, dev, args)
        line = measure(wl, torch, tg, dev, args, world, rank)
        del wl
        free_device(torch, dev)
        full = args.workload == "sweep" and args.array_mib == ARRAY_BYTES >> 20
        line["cpu_baseline"] = cpu_record(args.workload, args, world, rank, single=True, full=full)
    if args.workload == "sweep" and args.configs != "none":
        # the other configs of the benchmark, each measured the same way in
        # the same process, as sub-records (the headline stays the sweep)
        subs = {}
        sub_args = argparse.Namespace(**vars(args))
        sub_args.cpu_seconds = min(args.cpu_seconds, args.sub_cpu_seconds)
        for name in [c for c in args.configs.split(",") if c]:
            if name == "serve":
                subs[name] = serve_record(torch, tg, dev, sub_args, world, rank)
            else:
                wl = WORKLOADS[name](torch, tg, dev, sub_args)
                rec = measure(wl, torch, tg, dev, sub_args, world, rank, e2e=False)
                del wl
                free_device(torch, dev)
                rec["cpu_baseline"] = cpu_record(name, sub_args, world, rank)
                subs[name] = rec
            free_device(torch, dev)
        line["details"]["configs"] = subs
        line["gpu_launches"] += sum(r.get("gpu_launches") or 0 for r in subs.values())
        line["details"]["targets"] = targets(line, subs)
    if rank == 0:
        print(json.dumps(line), flush=True)


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
