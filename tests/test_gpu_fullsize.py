"""Full-size workloads, checked through size-independent properties (the
oracle would take minutes at these sizes):

* width sweep, 2 GiB arrays: every struct whose first word does not hit the
  exit predicate is copied, every other destination struct is untouched;
* gather over 2^24 structs: gather by a permutation then scatter by the same
  permutation restores the source (round trip), the identity gather is a
  copy, and a gather by any index set equals torch's own indexing;
* AoS -> SoA -> AoS round trip on 2 GiB;
* the batched kernel on arrays drawn like the 4096-array workload (lengths
  log-uniform up to 2^22 structs), against per-array torch results.
Inputs come from the library's seeded generators; torch on the GPU computes
the expected results here.
"""
import math

import numpy as np
import pytest

import trove_gb300 as tg

pytestmark = pytest.mark.gpu

SWEEP_BYTES = 1 << 31
MODULUS = 625
SENTINEL = 0xA5
N = 1 << 24


@pytest.fixture(scope="module")
def big(cuda):
    torch = cuda
    src = torch.empty(SWEEP_BYTES + 256, dtype=torch.uint8, device="cuda")
    tg.fill_random_u32(src, (SWEEP_BYTES + 256) // 4, seed=11)
    dst = torch.empty(SWEEP_BYTES, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    yield src, dst
    del src, dst
    torch.cuda.empty_cache()


@pytest.mark.parametrize("width", [4, 12, 24, 44, 64])
@pytest.mark.parametrize("path", ["warp", "block"])
def test_sweep_full_size(cuda, big, width, path):
    torch = cuda
    src, dst = big
    n = SWEEP_BYTES // width
    s = width // 4
    dst.fill_(SENTINEL)
    tg.copy_exit(dst, src, n, width, MODULUS, path=path)
    torch.cuda.synchronize()
    first = src[: n * width].view(torch.int32).view(n, s)[:, 0].to(torch.int64) & 0xFFFFFFFF
    skip = (first % MODULUS) == (MODULUS - 1)
    d, v = dst[: n * width].view(n, width), src[: n * width].view(n, width)
    assert 0 < int(skip.sum()) < n // 100
    assert torch.equal(d[~skip], v[~skip])
    assert bool((d[skip] == SENTINEL).all())
    assert bool((dst[n * width:] == SENTINEL).all())
    tg.check_device()


@pytest.mark.parametrize("width", [8, 12, 16, 24, 32, 48, 64])
def test_gather_full_size(cuda, big, width):
    torch = cuda
    src, dst = big
    perm = torch.empty(N, dtype=torch.int32, device="cuda")
    runs = torch.empty(N, dtype=torch.int32, device="cuda")
    tg.fill_permutation(perm, N, 1)
    tg.fill_run_indices(runs, N, 2)
    view = src[: N * width]
    # permutation round trip: gather then scatter back
    g = torch.empty(N * width, dtype=torch.uint8, device="cuda")
    tg.gather(g, view, N, perm, N, width)
    back = torch.full((N * width,), SENTINEL, dtype=torch.uint8, device="cuda")
    tg.scatter(back, N, g, perm, N, width)
    torch.cuda.synchronize()
    assert torch.equal(back, view)
    # any index set equals torch indexing; identity is a copy
    for idx in (runs, torch.arange(N, dtype=torch.int32, device="cuda")):
        tg.gather(g, view, N, idx, N, width)
        torch.cuda.synchronize()
        assert torch.equal(g.view(N, width), view.view(N, width)[idx.long()])
    del g, back, perm, runs
    tg.check_device()


@pytest.mark.parametrize("width", [4, 12, 28, 64])
def test_aos_soa_round_trip_full_size(cuda, big, width):
    torch = cuda
    src, dst = big
    n = SWEEP_BYTES // width
    tg.aos_to_soa(dst, src, n, width)
    torch.cuda.synchronize()
    s = width // 4
    # plane j holds word j of every struct: spot-check a strided sample of planes
    words = src[: n * width].view(torch.int32).view(n, s)
    planes = dst[: n * width].view(torch.int32).view(s, n)
    for j in sorted({0, s // 2, s - 1}):
        assert torch.equal(planes[j], words[:, j])
    back = torch.empty(n * width, dtype=torch.uint8, device="cuda")
    tg.soa_to_aos(back, dst, n, width)
    torch.cuda.synchronize()
    assert torch.equal(back, src[: n * width])
    del back


def test_batch_full_length_distribution(cuda):
    """512 arrays drawn like the 4096-array workload (same length, width and
    op distributions), each checked against torch."""
    torch = cuda
    rng = np.random.default_rng(4)
    count = 512
    ops = rng.choice([0, 1, 2], size=count, p=[0.5, 0.4, 0.1])
    widths = rng.choice([4, 12, 20, 36, 64], size=count)
    lens = np.exp(rng.uniform(math.log(1 << 10), math.log(1 << 22), size=count)).astype(np.int64)
    tasks = []
    for k in range(count):
        op, w, n = int(ops[k]), int(widths[k]), int(lens[k])
        src = torch.empty(n * w, dtype=torch.uint8, device="cuda")
        tg.fill_random_u32(src, n * w // 4, seed=500 + k)
        idx = None
        if op == 1:
            idx = torch.empty(n, dtype=torch.int32, device="cuda")
            tg.fill_uniform_indices(idx, n, n, seed=600 + k)
        elif op == 2:
            idx = torch.empty(n, dtype=torch.int32, device="cuda")
            tg.fill_permutation(idx, n, 700 + k)
        dst = torch.full((n * w,), SENTINEL, dtype=torch.uint8, device="cuda")
        tasks.append(dict(op=op, width=w, n=n, src=src, dst=dst, idx=idx, bound=n))
    torch.cuda.synchronize()
    b = tg.Batch(tasks)
    stream = torch.cuda.Stream()  # graph capture needs a stream other than the legacy default
    b.capture(stream)
    b.launch(stream)
    stream.synchronize()
    for k, t in enumerate(tasks):
        n, w = t["n"], t["width"]
        s, d = t["src"].view(n, w), t["dst"].view(n, w)
        if t["op"] == 0:
            ok = torch.equal(d, s)
        elif t["op"] == 1:
            ok = torch.equal(d, s[t["idx"].long()])
        else:
            ok = torch.equal(d[t["idx"].long()], s)
        assert ok, (k, t["op"], w, n)
    b.close()


def test_copy_beyond_2_31_structs(cuda):
    """More than 2^31 structs (4-byte, 8.6 GB a side) through trv_copy's default
    path, the flat vector and warp-contiguous paths and a batch copy task:
    every offset is 64-bit."""
    torch = cuda
    n = (1 << 31) + 4099
    src = torch.empty(n * 4, dtype=torch.uint8, device="cuda")
    tg.fill_random_u32(src, n, seed=12)
    dst = torch.empty_like(src)
    for kw in ({}, {"path": "vector"}, {"path": "warp"}):
        dst.zero_()
        tg.copy(dst, src, n, 4, **kw)
        torch.cuda.synchronize()
        assert torch.equal(dst, src), kw
    dst.zero_()
    b = tg.Batch([dict(op=tg.OP_COPY, width=4, n=n, src=src, dst=dst)])
    b.launch()
    torch.cuda.synchronize()
    assert torch.equal(dst, src)
    b.close()
    del src, dst
    torch.cuda.empty_cache()


@pytest.mark.parametrize("width,rows", [(8, 5 << 27), (36, (1 << 27) + 37), (64, (1 << 27) + 37),
                                        (128, (1 << 26) + 37)])
def test_index_ops_beyond_4_gib(cuda, width, rows):
    """Gathers from and scatters into an array of more than 4 GiB, so that most
    rows' byte offsets need more than 32 bits: every C ABI path, the batch's
    staged and register movers and the allocation-free batch, against torch's
    own indexing.  The scatters write distinct rows, each check restores the
    rows it overwrote, and at the end the whole array must equal a fresh copy
    of its seeded contents (no row outside the index set was touched)."""
    torch = cuda
    n = (1 << 20) + 13
    big = torch.empty(rows * width, dtype=torch.uint8, device="cuda")
    tg.fill_random_u32(big, rows * width // 4, seed=width)
    view = big.view(rows, width)
    idx = torch.empty(n, dtype=torch.int32, device="cuda")
    tg.fill_uniform_indices(idx, n, rows, seed=width + 1)
    assert int((idx.long() * width >= (1 << 32)).sum()) > n // 10
    expect = view[idx.long()]
    out = torch.empty(n * width, dtype=torch.uint8, device="cuda")
    # the struct-typed paths cover widths up to 64 bytes
    paths = ["auto", "warp", "coalesced", "direct", "vector"] if width <= 64 else ["auto", "warp", "vector"]
    for path in paths:
        out.fill_(SENTINEL)
        tg.gather(out, big, rows, idx, n, width, path=path)
        torch.cuda.synchronize()
        assert torch.equal(out.view(n, width), expect), ("gather", path)

    # distinct destination rows spread over the whole array, in random order
    gen = torch.Generator(device="cuda")
    gen.manual_seed(width)
    step = (rows - 1) // n
    didx = (torch.arange(n, device="cuda", dtype=torch.int64) * step + 5)
    didx = didx[torch.randperm(n, generator=gen, device="cuda")].to(torch.int32)
    saved = view[didx.long()].clone()
    payload = torch.empty(n * width, dtype=torch.uint8, device="cuda")
    tg.fill_random_u32(payload, n * width // 4, seed=width + 2)
    for path in paths:
        tg.scatter(big, rows, payload, didx, n, width, path=path)
        torch.cuda.synchronize()
        assert torch.equal(view[didx.long()], payload.view(n, width)), ("scatter", path)
        view[didx.long()] = saved

    if width <= 64:  # the batch's movers serve widths up to 64 bytes
        for opts in ({}, {"blocks_per_sm": 2, "gather_policy": 1, "scatter_policy": 1}):
            # one batch each: a gather from the array and a scatter into it
            # in one batch would race
            out.fill_(SENTINEL)
            b = tg.Batch([dict(op=tg.OP_GATHER, width=width, n=n, src=big, dst=out, idx=idx, bound=rows)], **opts)
            b.launch()
            torch.cuda.synchronize()
            b.close()
            assert torch.equal(out.view(n, width), expect), ("batch gather", opts)
            b = tg.Batch([dict(op=tg.OP_SCATTER, width=width, n=n, src=payload, dst=big, idx=didx, bound=rows)],
                         **opts)
            b.launch()
            torch.cuda.synchronize()
            b.close()
            assert torch.equal(view[didx.long()], payload.view(n, width)), ("batch scatter", opts)
            view[didx.long()] = saved
        out.fill_(SENTINEL)
        tg.run_static([dict(op=tg.OP_GATHER, width=width, n=n, src=big, dst=out, idx=idx, bound=rows)])
        torch.cuda.synchronize()
        assert torch.equal(out.view(n, width), expect), "static batch gather"

    fresh = torch.empty_like(big)
    tg.fill_random_u32(fresh, rows * width // 4, seed=width)
    assert torch.equal(big, fresh)
    del big, fresh, view, out, payload, saved, expect
    torch.cuda.empty_cache()
    tg.check_device()
