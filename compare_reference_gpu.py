"""Side-by-side timing of the reference Trove and this library on one GPU.

Run it directly on a GB300, after
the library and the harness cubins are built:

    python compare_reference_gpu.py [--out FILE] [--reps N] [--tune]

The reference's kernels come from oracle/_ref/trove_ref_kernels.cubin, which
compiles oracle/trove_bench_kernels.cu (the reference's own test-kernel
patterns) against the reference's headers; it is built where the reference
checkout exists and travels with the repository.  This library is called
through its C ABI, as a user would: default launch shapes, or with --tune
the shapes its autotuner picks for each width.  Both sides run the same workloads on the
same buffers:

* the single 12-byte copy: 2^20 structs, one launch (reference kernel
  `shfl_copy_3`: load_warp_contiguous + store_warp_contiguous, one struct per
  thread; this library: trv_copy on the warp-contiguous path);
* the width sweep: s = 1..16 words, 2 GiB arrays of seeded random words, a
  lane leaving between load and store when its first word w has
  w % 625 == 624 (reference kernel `exit_copy_<s>`: load_warp_contiguous /
  store_warp_contiguous with the warp_converged() fallback; this library:
  trv_copy_exit on the warp-contiguous path), plus the compiler-generated
  AoS copy (`direct_copy_<s>`: r[i] = s[i]);
* the device-API gather (--part api_gather): the coalesced_ptr gather kernel
  source `shfl_gather_<s>` built against the reference's headers and against
  this repository's, widths 4..64 B, the three index patterns;
* warps with inactive lanes (--part partial): the coalesced_ptr gather and
  copy kernels `partial_gather_<s>` / `partial_copy_<s>`, in which a seeded
  10 / 30 / 50 % of the threads leave before the access, built against both
  header trees: the reference's 16/8/4/2-lane tile cascade against this
  library's per-lane handling of partial warps, 2^24 structs;
* one launch of each data-movement path (--part paths), for profiling the
  choice between them under ncu: this library's warp-contiguous transposing
  copy at 12, 24 and 64 B, its flat vector copy, its TMA bulk copy, its
  row-form and coalesced_ptr gathers at 12 and 64 B (random permutation),
  and the reference's shfl_copy and shfl_gather kernels at the same widths,
  each on arrays of 512 MiB (no timing, no comparison: just the launches);
* one launch each of the random-block probe and of the gathers it bounds
  (--part probe), for profiling them under ncu: 2^24 structs of 8 and 64 B
  gathered through a random permutation by trv_probe_block_gather (32-byte
  blocks for 8 B, 64-byte blocks with the 64-byte hint for 64 B), by
  trv_gather (the row-form shapes the autotuner picks for them) and by the
  reference's shfl_gather;
* the CPU-GPU link (--part host): copy-engine rates host -> device, device ->
  host and both at once on 2 GiB pinned buffers, and this library's copy and
  early-exit copy kernels reading and writing pinned host arrays in place
  (several paths, unrolls and grids), beside a staged pipeline (H2D, device
  copy, D2H on three streams); the ceiling of any host-buffer (e2e) figure;
* the gather: 2^24 structs, widths 8..64 B, a permutation, runs of 32 and
  the identity (reference kernel `shfl_gather_<s>`: coalesced_ptr; this
  library: trv_gather), plus the compiler-generated gather
  (`direct_gather_<s>`: r[i] = s[indices[i]]).

Every pair of outputs is compared bit for bit before anything is timed.
Timing: CUDA events around each launch on the launching stream, an L2 flush
(a 512 MiB write) between launches, median of `reps`.  GB/s counts bytes
read + written (+ 4 per index), the formula of the reference's
tests/benchmark.cu:283.
"""
import argparse
import ctypes
import json
import statistics
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

MODULUS = 625
SWEEP_BYTES = 1 << 31
GATHER_N = 1 << 24
GATHER_WIDTHS = [8, 12, 16, 24, 32, 48, 64]
SENTINEL = 0xA5


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=None)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--part", choices=["all", "copy12", "sweep", "gather", "api_gather", "partial", "paths", "host", "probe"], default="all")
    ap.add_argument("--tune", action="store_true",
                    help="run the library's autotuner for each width first (launch shapes as tuned)")
    args = ap.parse_args()

    import torch

    import oracle
    import trove_gb300 as tg

    tg.load()
    dev = torch.device("cuda", 0)
    torch.cuda.init()
    ref = oracle.reference_cubin()
    if ref is None:
        raise SystemExit("reference cubin not present (build it where the reference checkout exists)")
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    def timed(fn):
        for _ in range(3):
            fn()
        times = []
        for _ in range(args.reps):
            flush.fill_(1)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize(dev)
            times.append(a.elapsed_time(b))
        return statistics.median(times)

    def cubin(name, grid, *ptrs_and_scalars):
        ref.launch(name, grid, 256, list(ptrs_and_scalars), stream.cuda_stream)

    if args.part == "paths":
        return launch_paths(torch, tg, ref, dev, stream)
    if args.part == "host":
        return host_link(torch, tg, dev, args)
    if args.part == "probe":
        return launch_probe(torch, tg, ref, dev, stream)

    rows = []
    src = torch.empty(SWEEP_BYTES + 256, dtype=torch.uint8, device=dev)
    tg.fill_random_u32(src, (SWEEP_BYTES + 256) // 4, seed=0)
    d_ref = torch.empty(SWEEP_BYTES, dtype=torch.uint8, device=dev)
    d_own = torch.empty_like(d_ref)
    torch.cuda.synchronize(dev)

    if args.part in ("all", "copy12"):
        n, w = 1 << 20, 12
        ps, pr = ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(d_ref.data_ptr())

        def ref_copy():
            cubin("shfl_copy_3", n // 256, ps, pr)  # one struct per thread, 4096 blocks of 256

        def own_copy(unroll):
            return lambda: tg.copy(d_own, src, n, w, path="warp", unroll=unroll, stream=stream)

        ref_copy()
        own_copy(0)()
        torch.cuda.synchronize(dev)
        if not torch.equal(d_ref[: n * w], d_own[: n * w]):
            raise SystemExit("outputs differ: 12 B copy")
        t_ref = timed(ref_copy)
        by_unroll = {u: timed(own_copy(u)) for u in (1, 2, 4, 8)}  # structs per lane
        best = min(by_unroll, key=by_unroll.get)
        t_own = by_unroll[best]
        row = {"workload": "copy12", "width": w, "structs": n, "reference_us": round(t_ref * 1e3, 2),
               "this_us": round(t_own * 1e3, 2), "this_unroll": best,
               "this_us_by_unroll": {u: round(t * 1e3, 2) for u, t in by_unroll.items()},
               "reference_gbs": round(2 * n * w / t_ref / 1e6, 1),
               "this_gbs": round(2 * n * w / t_own / 1e6, 1), "ratio": round(t_ref / t_own, 3)}
        rows.append(row)
        print(json.dumps(row), flush=True)

    if args.part in ("all", "sweep"):
        for s in range(1, 17):
            w = 4 * s
            n = SWEEP_BYTES // w
            grid = (n + 255) // 256
            assert grid * 256 >= n and n * w <= SWEEP_BYTES
            ps, pr, po = (ctypes.c_void_p(t.data_ptr()) for t in (src, d_ref, d_own))

            def ref_exit():
                cubin(f"exit_copy_{s}", grid, ps, pr, ctypes.c_longlong(n), ctypes.c_uint(MODULUS))

            if args.tune:
                tg.autotune_call(tg.OP_COPY_EXIT_WARP, w, n)

            def own_exit():
                tg.copy_exit(d_own, src, n, w, MODULUS, path="warp", stream=stream)

            def ref_direct():
                cubin(f"direct_copy_{s}", n // 256, ps, pr)  # one struct per thread, whole blocks only

            d_ref.fill_(SENTINEL)
            d_own.fill_(SENTINEL)
            ref_exit()
            own_exit()
            torch.cuda.synchronize(dev)
            if not torch.equal(d_ref, d_own):
                raise SystemExit(f"outputs differ: width sweep {w} B")
            words0 = src[: n * w].view(torch.int32).view(n, s)[:, 0].to(torch.int64) & 0xFFFFFFFF
            skipped = int(((words0 % MODULUS) == (MODULUS - 1)).sum())
            alg = n * w + (n - skipped) * w
            t_ref, t_own = timed(ref_exit), timed(own_exit)
            t_dir = timed(ref_direct)
            row = {"workload": "sweep", "width": w, "structs": n,
                   "reference_gbs": round(alg / t_ref / 1e6, 1), "this_gbs": round(alg / t_own / 1e6, 1),
                   "ratio": round(t_ref / t_own, 3),
                   "compiler_aos_copy_gbs": round(2 * (n // 256 * 256) * w / t_dir / 1e6, 1)}
            rows.append(row)
            print(json.dumps(row), flush=True)

    if args.part in ("all", "gather"):
        n = GATHER_N
        idx = {p: torch.empty(n, dtype=torch.int32, device=dev) for p in ("perm", "runs", "identity")}
        tg.fill_permutation(idx["perm"], n, 1)
        tg.fill_run_indices(idx["runs"], n, 2)
        idx["identity"].copy_(torch.arange(n, dtype=torch.int32, device=dev))
        torch.cuda.synchronize(dev)
        for w in GATHER_WIDTHS:
            s = w // 4
            assert n * w <= SWEEP_BYTES
            if args.tune:
                tg.autotune_call(tg.OP_GATHER, w, n)
            for p, ix in idx.items():
                pi, ps, pr = (ctypes.c_void_p(t.data_ptr()) for t in (ix, src, d_ref))

                def ref_gather():
                    cubin(f"shfl_gather_{s}", n // 256, pi, ps, pr)

                def direct_gather():
                    cubin(f"direct_gather_{s}", n // 256, pi, ps, pr)

                def own_gather():
                    tg.gather(d_own, src, n, ix, n, w, stream=stream)

                ref_gather()
                own_gather()
                torch.cuda.synchronize(dev)
                if not torch.equal(d_ref[: n * w], d_own[: n * w]):
                    raise SystemExit(f"outputs differ: gather {w} B {p}")
                alg = (2 * w + 4) * n
                t_ref, t_own, t_dir = timed(ref_gather), timed(own_gather), timed(direct_gather)
                row = {"workload": "gather", "width": w, "pattern": p,
                       "reference_gbs": round(alg / t_ref / 1e6, 1), "this_gbs": round(alg / t_own / 1e6, 1),
                       "ratio": round(t_ref / t_own, 3), "compiler_aos_gather_gbs": round(alg / t_dir / 1e6, 1)}
                choice = tg.autotune_lookup(tg.SCOPE_CALL, tg.OP_GATHER, w, n)
                if choice is not None:
                    c = choice[0]
                    row["tuned"] = {"path": c.path, "unroll": c.unroll, "cache_policy": c.cache_policy}
                rows.append(row)
                print(json.dumps(row), flush=True)

    if args.part in ("all", "api_gather"):
        # The device API as users meet it: the same coalesced_ptr gather kernel
        # source built against both header trees.
        own = oracle.own_cubin()
        n = GATHER_N
        idx = {p: torch.empty(n, dtype=torch.int32, device=dev) for p in ("perm", "runs", "identity")}
        tg.fill_permutation(idx["perm"], n, 1)
        tg.fill_run_indices(idx["runs"], n, 2)
        idx["identity"].copy_(torch.arange(n, dtype=torch.int32, device=dev))
        torch.cuda.synchronize(dev)
        for s in range(1, 17):
            w = 4 * s
            for p, ix in idx.items():
                a_ref = [ctypes.c_void_p(ix.data_ptr()), ctypes.c_void_p(src.data_ptr()),
                         ctypes.c_void_p(d_ref.data_ptr())]
                a_own = [ctypes.c_void_p(ix.data_ptr()), ctypes.c_void_p(src.data_ptr()),
                         ctypes.c_void_p(d_own.data_ptr())]

                def ref_api():
                    cubin(f"shfl_gather_{s}", n // 256, *a_ref)

                def own_api():
                    own.launch(f"shfl_gather_{s}", n // 256, 256, a_own, stream.cuda_stream)

                ref_api()
                own_api()
                torch.cuda.synchronize(dev)
                if not torch.equal(d_ref[: n * w], d_own[: n * w]):
                    raise SystemExit(f"outputs differ: device-API gather {w} B {p}")
                alg = (2 * w + 4) * n
                t_ref, t_own = timed(ref_api), timed(own_api)
                row = {"workload": "api_gather", "width": w, "pattern": p,
                       "reference_gbs": round(alg / t_ref / 1e6, 1), "this_gbs": round(alg / t_own / 1e6, 1),
                       "ratio": round(t_ref / t_own, 3)}
                rows.append(row)
                print(json.dumps(row), flush=True)

    if args.part in ("all", "partial"):
        own = oracle.own_cubin()
        n = GATHER_N
        perm = torch.empty(n, dtype=torch.int32, device=dev)
        tg.fill_permutation(perm, n, 1)
        torch.cuda.synchronize(dev)
        for s in (2, 3, 4, 8, 12, 16):
            w = 4 * s
            for pct in (10, 30, 50):
                for kind in ("gather", "copy"):
                    ex = [ctypes.c_uint32(pct), ctypes.c_uint32(77)]
                    if kind == "gather":
                        a_ref = [ctypes.c_void_p(perm.data_ptr()), ctypes.c_void_p(src.data_ptr()),
                                 ctypes.c_void_p(d_ref.data_ptr()), *ex]
                        a_own = [ctypes.c_void_p(perm.data_ptr()), ctypes.c_void_p(src.data_ptr()),
                                 ctypes.c_void_p(d_own.data_ptr()), *ex]
                    else:
                        a_ref = [ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(d_ref.data_ptr()), *ex]
                        a_own = [ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(d_own.data_ptr()), *ex]
                    name = f"partial_{kind}_{s}"

                    def ref_k():
                        cubin(name, n // 256, *a_ref)

                    def own_k():
                        own.launch(name, n // 256, 256, a_own, stream.cuda_stream)

                    d_ref[: n * w].zero_()
                    d_own[: n * w].zero_()
                    ref_k()
                    own_k()
                    torch.cuda.synchronize(dev)
                    if not torch.equal(d_ref[: n * w], d_own[: n * w]):
                        raise SystemExit(f"outputs differ: {name} at {pct} %")
                    # bytes of the active rows (+ their indices for the gather)
                    active = n * (100 - pct) // 100
                    alg = active * (2 * w + (4 if kind == "gather" else 0))
                    t_ref, t_own = timed(ref_k), timed(own_k)
                    row = {"workload": "partial", "kind": kind, "width": w, "inactive_pct": pct,
                           "reference_gbs": round(alg / t_ref / 1e6, 1), "this_gbs": round(alg / t_own / 1e6, 1),
                           "ratio": round(t_ref / t_own, 3)}
                    rows.append(row)
                    print(json.dumps(row), flush=True)

    tg.check_device()
    if args.out:
        with open(args.out, "w") as f:
            json.dump({"gpu": torch.cuda.get_device_name(dev), "reps": args.reps, "tuned": args.tune, "rows": rows}, f,
                      indent=1)


def launch_probe(torch, tg, ref, dev, stream):
    """One launch each of the probe, trv_gather and the reference's gather on
    the same 2^24-struct permutation gathers (the profiling workload)."""
    n = GATHER_N
    src = torch.empty(n * 64 + 256, dtype=torch.uint8, device=dev)
    tg.fill_random_u32(src, (n * 64 + 256) // 4, seed=0)
    dst = torch.empty(n * 64, dtype=torch.uint8, device=dev)
    perm = torch.empty(n, dtype=torch.int32, device=dev)
    tg.fill_permutation(perm, n, 1)
    # the row-form shapes the autotuner picked for these gathers on this
    # round's boxes (given explicitly: tuning would add launches to profile)
    for w, block, hint, policy in ((8, 32, 0, 1), (64, 64, 64, 4)):
        tg.probe_block_gather(dst, src, n, perm, n, w, block, hint, stream=stream)
        tg.gather(dst, src, n, perm, n, w, path="warp", unroll=2, policy=policy, stream=stream)
        ref.launch(f"shfl_gather_{w // 4}", n // 256, 256,
                   [ctypes.c_void_p(perm.data_ptr()), ctypes.c_void_p(src.data_ptr()),
                    ctypes.c_void_p(dst.data_ptr())], stream.cuda_stream)
        torch.cuda.synchronize(dev)
    tg.check_device()
    print("probe and gathers launched", flush=True)


def host_link(torch, tg, dev, args):
    """Rates of the CPU-GPU link on 2 GiB pinned host buffers (median of
    `reps` CUDA-event-timed runs; GB/s = bytes read + written)."""
    nb = 2 << 30
    h_src = torch.empty(nb + 256, dtype=torch.uint8).pin_memory()
    h_dst = torch.empty(nb + 256, dtype=torch.uint8).pin_memory()
    h_src.random_(0, 255)
    d_a = torch.empty(nb + 256, dtype=torch.uint8, device=dev)
    d_b = torch.empty_like(d_a)
    rows = []

    def ev(fn):
        fn()
        torch.cuda.synchronize(dev)
        ts = []
        for _ in range(args.reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize(dev)
            ts.append(a.elapsed_time(b))
        return statistics.median(ts)

    def row(name, nbytes, fn):
        r = {"workload": "host", "case": name, "gbs": round(nbytes / ev(fn) / 1e6, 1)}
        rows.append(r)
        print(json.dumps(r), flush=True)

    s1, s2 = torch.cuda.Stream(dev), torch.cuda.Stream(dev)

    def both():
        with torch.cuda.stream(s1):
            d_a[:nb].copy_(h_src[:nb], non_blocking=True)
        with torch.cuda.stream(s2):
            h_dst[:nb].copy_(d_b[:nb], non_blocking=True)
        torch.cuda.current_stream(dev).wait_stream(s1)
        torch.cuda.current_stream(dev).wait_stream(s2)

    row("copy engine host->device", nb, lambda: d_a[:nb].copy_(h_src[:nb], non_blocking=True))
    row("copy engine device->host", nb, lambda: h_dst[:nb].copy_(d_a[:nb], non_blocking=True))
    row("copy engines both directions at once", 2 * nb, both)
    row("copy kernel reading host, writing device", nb, lambda: tg.copy(d_a, h_src, nb // 16, 16, path="vector"))
    row("copy kernel reading device, writing host", nb, lambda: tg.copy(h_dst, d_a, nb // 16, 16, path="vector"))
    for path, unrolls in (("vector", (2, 4, 8)), ("bulk", (0,)), ("warp", (1, 2, 4, 8))):
        for u in unrolls:
            row(f"in-place host copy, 16 B, {path} path, unroll {u}", 2 * nb,
                lambda: tg.copy(h_dst, h_src, nb // 16, 16, path=path, unroll=u))
    for grid in (152, 608, 2432):
        row(f"in-place host copy, 16 B, vector path, {grid} blocks", 2 * nb,
            lambda: tg.copy(h_dst, h_src, nb // 16, 16, path="vector", grid=grid))
    for w in (12, 64):
        n = nb // w
        for api in ("warp", "block"):
            for u in (1, 2, 4, 8):
                row(f"in-place host early-exit copy, {w} B, {api} API, unroll {u}", 2 * n * w,
                    lambda: tg.copy_exit(h_dst, h_src, n, w, MODULUS, path=api, unroll=u))

    def staged(w, chunk):
        per = chunk // w
        n_total = nb // w
        streams = [torch.cuda.Stream(dev) for _ in range(3)]
        for k, start in enumerate(range(0, n_total, per)):
            n = min(per, n_total - start)
            st, off = streams[k % 3], start * w
            with torch.cuda.stream(st):
                d_a[off: off + n * w].copy_(h_src[off: off + n * w], non_blocking=True)
                tg.copy_exit(d_b[off:], d_a[off:], n, w, MODULUS, path="warp", stream=st)
                h_dst[off: off + n * w].copy_(d_b[off: off + n * w], non_blocking=True)
        for st in streams:
            torch.cuda.current_stream(dev).wait_stream(st)

    for w in (12, 64):
        for chunk in (16 << 20, 64 << 20, 256 << 20):
            row(f"staged H2D + device early-exit copy + D2H, {w} B, {chunk >> 20} MiB pieces, 3 streams",
                2 * nb, lambda: staged(w, chunk))
    tg.check_device()
    if args.out:
        with open(args.out, "w") as f:
            json.dump({"gpu": torch.cuda.get_device_name(dev), "reps": args.reps, "rows": rows}, f, indent=1)


def launch_paths(torch, tg, ref, dev, stream):
    """One launch of every path on 512 MiB arrays (the profiling workload)."""
    nbytes = 512 << 20
    src = torch.empty(nbytes + 256, dtype=torch.uint8, device=dev)
    tg.fill_random_u32(src, (nbytes + 256) // 4, seed=0)
    dst = torch.empty_like(src)
    torch.cuda.synchronize(dev)
    for w in (12, 24, 64):
        n = nbytes // w
        tg.copy(dst, src, n, w, path="warp", stream=stream)
        ref.launch(f"shfl_copy_{w // 4}", n // 256, 256, [ctypes.c_void_p(src.data_ptr()),
                                                           ctypes.c_void_p(dst.data_ptr())], stream.cuda_stream)
    n = nbytes // 12
    tg.copy(dst, src, n, 12, path="vector", stream=stream)
    tg.copy(dst, src, n, 12, path="bulk", stream=stream)
    for w in (12, 64):
        n = nbytes // w // 256 * 256
        perm = torch.empty(n, dtype=torch.int32, device=dev)
        tg.fill_permutation(perm, n, 1)
        tg.gather(dst, src, n, perm, n, w, path="warp", stream=stream)
        tg.gather(dst, src, n, perm, n, w, path="coalesced", stream=stream)
        ref.launch(f"shfl_gather_{w // 4}", n // 256, 256,
                   [ctypes.c_void_p(perm.data_ptr()), ctypes.c_void_p(src.data_ptr()),
                    ctypes.c_void_p(dst.data_ptr())], stream.cuda_stream)
        torch.cuda.synchronize(dev)
        del perm
    torch.cuda.synchronize(dev)
    tg.check_device()
    print("paths launched", flush=True)


if __name__ == "__main__":
    main()
