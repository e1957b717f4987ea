"""The reference's own test-kernel patterns (oracle/trove_bench_kernels.cu)
on the GPU, compiled against this repository's headers and against the
reference's headers (a prebuilt cubin per TILE_SIZE 32/16/8/4/2, shipped
with the repository).  Both must match the CPU oracle bit for bit, which also
shows that kernels written for the reference recompile unchanged against
include/trove.  Beyond the reference's own tests: struct sizes of 20, 24
(composite int4 schedule) and 33 words, warp_load / warp_store /
uncoalesced_store, warp_converged<N> and thread_tile<N>, coalesced_ptr on
warps with inactive lanes, and (this repository's headers only, as the
reference's ptr.h does not compile it) reference-to-reference assignment
through coalesced_ptr."""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

N = 256 * 40
TILES = (32, 16, 8, 4, 2)
SIZES = list(range(1, 17)) + [20, 24, 33]
_loaded = {}


def modules(tile=32):
    """[(tree, cubin)] at TILE_SIZE `tile`; the reference's cubin is required."""
    if tile not in _loaded:
        mods = [("own", oracle.own_cubin(tile))]
        ref = oracle.reference_cubin(tile)
        if ref is not None:
            mods.append(("reference", ref))
        _loaded[tile] = mods
    return _loaded[tile]


@pytest.fixture(scope="module")
def cubins(cuda):
    return modules()


def lane_hash(i, seed):
    """The partial-warp kernels' exit hash (trove_bench_kernels.cu lane_hash)."""
    x = (np.asarray(i, np.uint64) * np.uint64(0x9E3779B1) + np.uint64(seed)) & np.uint64(0xFFFFFFFF)
    x ^= x >> np.uint64(15)
    x = (x * np.uint64(0x85EBCA6B)) & np.uint64(0xFFFFFFFF)
    x ^= x >> np.uint64(13)
    return x


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1).copy()).cuda()


def ptr(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("tile", TILES)
def test_reference_cubin_shipped(cuda, tile):
    """The reference's kernels must be on the GPU machine: a missing cubin is
    a failure, not a skip, so the comparison cannot drop out unnoticed."""
    names = [n for n, _ in modules(tile)]
    assert "reference" in names, f"oracle/_ref reference cubin for TILE_SIZE {tile} is missing"


@pytest.mark.parametrize("tile", TILES)
@pytest.mark.parametrize("s", SIZES)
def test_benchmark_kernels(cuda, s, tile):
    torch = cuda
    w = 4 * s
    src_h = oracle.random_structs(N, w, seed=s)
    perm = oracle.permutation(N, s + 1)
    runs = oracle.run_indices(N, s + 2)
    for name, mod in modules(tile):
        src = dev(torch, src_h)
        out = torch.zeros(N * w, dtype=torch.uint8, device="cuda")
        mod.launch(f"shfl_store_{s}", N // 256, 256, [ptr(out)])
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy().view(np.int32), oracle.counting(N, s)), (name, s)

        sums = torch.zeros(N, dtype=torch.int32, device="cuda")
        mod.launch(f"shfl_load_{s}", N // 256, 256, [ptr(src), ptr(sums)])
        torch.cuda.synchronize()
        assert np.array_equal(sums.cpu().numpy(), oracle.load_sum(src_h, N, s)), (name, s)

        for kind in ["shfl_copy", "direct_copy"]:
            out.zero_()
            mod.launch(f"{kind}_{s}", N // 256, 256, [ptr(src), ptr(out)])
            torch.cuda.synchronize()
            assert np.array_equal(out.cpu().numpy(), src_h.reshape(-1)), (name, kind, s)

        if tile != 32:
            continue  # coalesced_ptr does not depend on TILE_SIZE: its kernels run once

        for idx_h in (perm, runs):
            idx = torch.from_numpy(idx_h).cuda()
            expect = oracle.gather(np.zeros(N * w, np.uint8), src_h, idx_h, N, w)
            for kind in ["shfl_gather", "direct_gather"]:
                out.zero_()
                mod.launch(f"{kind}_{s}", N // 256, 256, [ptr(idx), ptr(src), ptr(out)])
                torch.cuda.synchronize()
                assert np.array_equal(out.cpu().numpy(), expect), (name, kind, s)

        idx = torch.from_numpy(perm).cuda()
        expect = oracle.scatter(np.zeros(N * w, np.uint8), src_h, perm, N, w)
        for kind in ["shfl_scatter", "direct_scatter"]:
            out.zero_()
            mod.launch(f"{kind}_{s}", N // 256, 256, [ptr(idx), ptr(src), ptr(out)])
            torch.cuda.synchronize()
            assert np.array_equal(out.cpu().numpy(), expect), (name, kind, s)


@pytest.mark.parametrize("tile", TILES)
@pytest.mark.parametrize("s", [1, 3, 5, 8, 12, 16, 20, 24, 33])
def test_block_and_exit_kernels(cuda, s, tile):
    torch = cuda
    w = 4 * s
    l = 256 * 7 + 17  # partial tail warp -> non-converged fallback
    for name, mod in modules(tile):
        out = torch.zeros(l * w, dtype=torch.uint8, device="cuda")
        mod.launch(f"block_write_{s}", 5, 256, [ptr(out), ctypes.c_int(l)])
        torch.cuda.synchronize()
        counting = oracle.counting(l, s)
        assert np.array_equal(out.cpu().numpy().view(np.int32), counting), (name, s)
        cp = torch.zeros_like(out)
        mod.launch(f"block_copy_{s}", 5, 256, [ptr(out), ptr(cp), ctypes.c_int(l)])
        torch.cuda.synchronize()
        assert np.array_equal(cp.cpu().numpy().view(np.int32), counting), (name, s)

        n = 256 * 30 + 5
        src_h = oracle.random_structs(n, w, seed=100 + s)
        init = np.full(n * w, 0xA5, np.uint8)
        expect, _ = oracle.copy_exit(init, src_h, n, w, 7)
        dst = dev(torch, init)
        mod.launch(f"exit_copy_{s}", (n + 255) // 256, 256,
                   [ptr(dev(torch, src_h)), ptr(dst), ctypes.c_longlong(n), ctypes.c_uint32(7)])
        torch.cuda.synchronize()
        assert np.array_equal(dst.cpu().numpy(), expect), (name, s)


@pytest.mark.parametrize("s", [1, 2, 3, 5, 8, 16, 24])
def test_memory_kernels(cuda, cubins, s):
    """warp_load(p, lane, 32) / warp_store(a, q, lane, 32) round-trip each
    warp's 32*s words; uncoalesced_store(a, u + s*i) writes thread i's s
    words in a row (reference memory.h:136-168); odd warps use the volatile
    overloads."""
    torch = cuda
    nthreads = 256 * 8
    words = oracle.random_words(nthreads * s, seed=40 + s).view(np.int32)
    warps = words.reshape(nthreads // 32, s, 32)  # word k of lane l at [warp, k, l]
    expect_u = warps.transpose(0, 2, 1).reshape(-1)  # thread i = 32 warp + l holds a[k] = word k
    for name, mod in cubins:
        src = dev(torch, words)
        r = torch.zeros_like(src)
        u = torch.zeros_like(src)
        mod.launch(f"memory_rw_{s}", nthreads // 256, 256, [ptr(src), ptr(r), ptr(u)])
        torch.cuda.synchronize()
        assert np.array_equal(r.cpu().numpy().view(np.int32), words), (name, s)
        assert np.array_equal(u.cpu().numpy().view(np.int32), expect_u), (name, s)


def test_warp_converged_and_thread_tile(cuda, cubins):
    """warp_converged<32/16/8/4/2> in warps with chosen active lanes, and
    thread_tile<N>: id, size and shfl from rank (id + 3) % N."""
    torch = cuda
    rng = np.random.default_rng(3)
    masks = [0xFFFFFFFF, 0xFFFF0000, 0x0000FFFF, 0xFF00FF00, 0x0F0F0F0F, 0x33333333, 0x55555555,
             0xFFFFFFFE, 0x7FFFFFFF, 0x00000001, 0x80000000, 0x0000FF00, 0xF0F0F0F0, 0xCCCCCCCC]
    masks += [int(x) for x in rng.integers(1, 1 << 32, size=64 - len(masks), dtype=np.uint64)]
    masks_h = np.array(masks, np.uint32)
    expect = np.full(64 * 32, 0xFF, np.uint8)
    for wi, m in enumerate(masks):
        for lane in range(32):
            if not (m >> lane) & 1:
                continue
            bits = 0
            for k, n in enumerate((32, 16, 8, 4, 2)):
                g = ((1 << n) - 1) << (lane & ~(n - 1)) if n < 32 else 0xFFFFFFFF
                if (m & g) == g:
                    bits |= 1 << k
            expect[32 * wi + lane] = bits
    nthreads = 256 * 4
    tid = np.arange(nthreads)
    v = tid * 7 + 1
    expect_tile = np.empty((nthreads, 5), np.int64)
    for k, n in enumerate((32, 16, 8, 4, 2)):
        rank = tid & (n - 1)
        src = (tid & ~(n - 1)) + (rank + 3) % n
        expect_tile[:, k] = v[src] * 1024 + rank * 32 + n
    for name, mod in cubins:
        out = torch.full((64 * 32,), 0xFF, dtype=torch.uint8, device="cuda")
        mod.launch("converged_probe", (64 * 32) // 256, 256, [ptr(dev(torch, masks_h)), ptr(out)])
        tiles = torch.zeros(nthreads * 5, dtype=torch.int32, device="cuda")
        mod.launch("tile_shfl_probe", nthreads // 256, 256, [ptr(tiles)])
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), expect), name
        assert np.array_equal(tiles.cpu().numpy().reshape(nthreads, 5), expect_tile), name


@pytest.mark.parametrize("s", [1, 2, 3, 4, 5, 8, 12, 16, 24])
@pytest.mark.parametrize("pct", [10, 50])
def test_partial_warp_coalesced_ptr(cuda, cubins, s, pct):
    """coalesced_ptr gathers and copies in warps where a seeded pct % of the
    lanes left first: the reference's 16/8/4/2-lane cascade and this
    library's per-lane fallback must both move exactly the active rows."""
    torch = cuda
    w = 4 * s
    src_h = oracle.random_structs(N, w, seed=60 + s)
    perm = oracle.permutation(N, 61 + s)
    seed = 1000 + s
    active = (lane_hash(np.arange(N), seed) % np.uint64(100)) >= np.uint64(pct)
    exp_g = np.zeros((N, w), np.uint8)
    exp_g[active] = src_h[perm[active]]
    exp_c = np.zeros((N, w), np.uint8)
    exp_c[active] = src_h[active]
    for name, mod in cubins:
        src = dev(torch, src_h)
        idx = torch.from_numpy(perm).cuda()
        out = torch.zeros(N * w, dtype=torch.uint8, device="cuda")
        mod.launch(f"partial_gather_{s}", N // 256, 256,
                   [ptr(idx), ptr(src), ptr(out), ctypes.c_uint32(pct), ctypes.c_uint32(seed)])
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), exp_g.reshape(-1)), (name, s, pct)
        out.zero_()
        mod.launch(f"partial_copy_{s}", N // 256, 256,
                   [ptr(src), ptr(out), ctypes.c_uint32(pct), ctypes.c_uint32(seed)])
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), exp_c.reshape(-1)), (name, s, pct)


@pytest.mark.parametrize("s", [1, 3, 4, 8, 12, 16, 24, 33])
def test_coalesced_ref_to_ref_assignment(cuda, s):
    """D[i] = S[idx[i]] and D[idx[i]] = S[i] with both sides coalesced_ptr
    (ptr.h coalesced_ref::operator=(const coalesced_ref&)); the reference's
    ptr.h:47-72 does not compile this, so only this repository's build runs."""
    torch = cuda
    w = 4 * s
    own = oracle.own_cubin()
    src_h = oracle.random_structs(N, w, seed=80 + s)
    for idx_h in (oracle.permutation(N, 81 + s), oracle.run_indices(N, 82 + s)):
        src = dev(torch, src_h)
        idx = torch.from_numpy(idx_h).cuda()
        out = torch.zeros(N * w, dtype=torch.uint8, device="cuda")
        own.launch(f"refref_gather_{s}", N // 256, 256, [ptr(idx), ptr(src), ptr(out)])
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), oracle.gather(np.zeros(N * w, np.uint8), src_h, idx_h, N, w)), s
    perm = oracle.permutation(N, 83 + s)
    src = dev(torch, src_h)
    out = torch.zeros(N * w, dtype=torch.uint8, device="cuda")
    own.launch(f"refref_scatter_{s}", N // 256, 256, [ptr(torch.from_numpy(perm).cuda()), ptr(src), ptr(out)])
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), oracle.scatter(np.zeros(N * w, np.uint8), src_h, perm, N, w)), s
