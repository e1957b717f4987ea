"""GPU parity: every C ABI path against the CPU oracle, bit-exact, through
the C ABI.  Sizes are small enough for the oracle to finish in seconds; the
full-size workloads are checked through size-independent properties in
test_gpu_fullsize.py."""
import numpy as np
import pytest

import oracle
import trove_gb300 as tg

pytestmark = pytest.mark.gpu

WIDTHS = list(range(4, 65, 4))
SENTINEL = 0xA5


def to_dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1).copy()).cuda()


def to_host(t):
    return t.cpu().numpy()


def guarded(torch, nbytes, offset=0, guard=256):
    """Device byte buffer with sentinel guard bands; returns (buffer, view
    start) so writes outside [start, start + nbytes) can be detected."""
    buf = torch.full((guard + offset + nbytes + guard,), SENTINEL, dtype=torch.uint8, device="cuda")
    return buf, guard + offset


def check_guards(buf, start, nbytes):
    h = to_host(buf)
    assert (h[:start] == SENTINEL).all(), "write before the destination"
    assert (h[start + nbytes:] == SENTINEL).all(), "write past the destination"
    return h[start:start + nbytes]


@pytest.mark.parametrize("width", WIDTHS)
def test_copy_struct_paths(cuda, width):
    torch = cuda
    for n in [1, 31, 33, 4097, 65539]:
        src_h = oracle.random_structs(n, width, seed=width * 1000 + n)
        src = to_dev(torch, src_h)
        expect = oracle.copy(src_h, n, width)
        for path in ["warp", "block", "direct", "vector", "auto", "bulk"]:
            for unroll in ([1, 2, 4, 8] if path in ("warp", "block", "direct", "vector") else [0]):
                for chunk in ([0, 4096, 48 << 10] if path == "bulk" else [0]):
                    buf, start = guarded(torch, n * width)
                    tg.copy(buf[start:], src, n, width, path=path, unroll=unroll, chunk=chunk)
                    got = check_guards(buf, start, n * width)
                    assert np.array_equal(got, expect), (width, n, path, unroll, chunk)
    tg.check_device()


@pytest.mark.parametrize("offset", [4, 8, 12])
@pytest.mark.parametrize("width", [8, 12, 16, 24, 32, 48, 64])
def test_copy_misaligned(cuda, width, offset):
    """Struct arrays not aligned to their widest word; the flat path with
    source and destination at different alignments."""
    torch = cuda
    n = 3001
    src_h = oracle.random_structs(n, width, seed=offset * 7 + width)
    sbuf, sstart = guarded(torch, n * width, offset=offset)
    sbuf[sstart:sstart + n * width] = to_dev(torch, src_h)
    for path in ["warp", "block", "vector", "auto", "bulk"]:
        for doff in [(offset * 3) % 16, offset]:
            dbuf, dstart = guarded(torch, n * width, offset=doff)
            if path == "bulk" and doff % 16 != offset % 16:
                with pytest.raises(tg.TroveError, match="alignment"):
                    tg.copy(dbuf[dstart:], sbuf[sstart:], n, width, path=path)
                continue
            tg.copy(dbuf[dstart:], sbuf[sstart:], n, width, path=path)
            got = check_guards(dbuf, dstart, n * width)
            assert np.array_equal(got, src_h.reshape(-1)), (path, width, offset, doff)
    tg.check_device()


@pytest.mark.parametrize("nbytes_width", [(1, 1), (3, 7), (5, 3), (100, 13), (7, 132), (1000, 100)])
def test_copy_odd_widths(cuda, nbytes_width):
    torch = cuda
    n, width = nbytes_width
    src_h = np.frombuffer(oracle.random_words((n * width + 3) // 4, 9).tobytes()[:n * width], np.uint8)
    src = to_dev(torch, src_h)
    buf, start = guarded(torch, n * width, offset=1)
    tg.copy(buf[start:], src, n, width)
    assert np.array_equal(check_guards(buf, start, n * width), src_h)
    with pytest.raises(tg.TroveError):
        tg.copy(buf[start:], src, n, width, path="warp")


@pytest.mark.parametrize("path", ["warp", "block"])
@pytest.mark.parametrize("width", WIDTHS)
def test_copy_exit(cuda, width, path):
    torch = cuda
    for n, modulus in [(20000, 7), (100003, 625), (4096, 0), (77, 3)]:
        src_h = oracle.random_structs(n, width, seed=width + n + modulus)
        init = np.full(n * width, SENTINEL, np.uint8)
        expect, written = oracle.copy_exit(init, src_h, n, width, modulus)
        src = to_dev(torch, src_h)
        dst = to_dev(torch, init)
        tg.copy_exit(dst, src, n, width, modulus, path=path)
        assert np.array_equal(to_host(dst), expect), (width, n, modulus, path)
        if modulus == 625:
            assert 0 < n - written < n // 100


def index_sets(n, seed):
    return {
        "perm": oracle.permutation(n, seed),
        "runs": oracle.run_indices(n, seed),
        "uniform": oracle.uniform_indices(n, n, seed),
        "identity": np.arange(n, dtype=np.int32),
    }


@pytest.mark.parametrize("width", WIDTHS)
def test_gather(cuda, width):
    torch = cuda
    for n in [33, 5000, 65536 + 17]:
        src_h = oracle.random_structs(n, width, seed=width * 31 + n)
        src = to_dev(torch, src_h)
        init = np.full(n * width, SENTINEL, np.uint8)
        for name, idx_h in index_sets(n, seed=n + width).items():
            idx = torch.from_numpy(idx_h).cuda()
            expect = oracle.gather(init, src_h, idx_h, n, width)
            for path in ["warp", "coalesced", "direct", "auto", "vector"]:
                for unroll in ([1, 2, 4, 8] if path in ("warp", "coalesced", "direct") else [0]):
                    dst = to_dev(torch, init)
                    tg.gather(dst, src, n, idx, n, width, path=path, unroll=unroll)
                    assert np.array_equal(to_host(dst), expect), (width, n, name, path, unroll)


@pytest.mark.parametrize("width", [4, 8, 12, 24, 64, 100])
def test_row_form_cache_policies(cuda, width):
    """Every cache policy of the row-form gather / scatter moves the same
    bytes as the oracle."""
    torch = cuda
    n = 65536 + 17
    src_h = oracle.random_structs(n, width, seed=width + 3)
    src = to_dev(torch, src_h)
    init = np.full(n * width, SENTINEL, np.uint8)
    sets = index_sets(n, seed=width)
    for policy in range(6):
        for name, idx_h in sets.items():
            idx = torch.from_numpy(idx_h).cuda()
            dst = to_dev(torch, init)
            tg.gather(dst, src, n, idx, n, width, path="warp", policy=policy)
            assert np.array_equal(to_host(dst), oracle.gather(init, src_h, idx_h, n, width)), (policy, name)
    perm_h = sets["perm"]
    for policy in range(7):
        dst = to_dev(torch, init)
        tg.scatter(dst, n, src, torch.from_numpy(perm_h).cuda(), n, width, path="warp", policy=policy)
        assert np.array_equal(to_host(dst), oracle.scatter(init, src_h, perm_h, n, width)), policy
    with pytest.raises(tg.TroveError):
        tg.gather(dst, src, n, idx, n, width, path="warp", policy=6)
    with pytest.raises(tg.TroveError):
        tg.scatter(dst, n, src, torch.from_numpy(perm_h).cuda(), n, width, path="warp", policy=7)


@pytest.mark.parametrize("width", [8, 12, 20, 24])
def test_scatter_destination_passes(cuda, width):
    """Scatters onto destinations above 64 MiB in destination passes (cache
    policy 6; the default for structs of at most 16 bytes): every row lands
    once, skipped indices leave the destination alone, a partial scatter
    keeps the rest."""
    torch = cuda
    n = (1 << 23) + 17  # 8-24 B: 64-192 MiB destinations, 2-3 passes
    src_h = oracle.random_structs(n, width, seed=width + 40)
    src = to_dev(torch, src_h)
    idx_h = oracle.permutation(n, width + 41)
    idx_h[5] = -1
    idx_h[77] = n + 3
    ok = (idx_h >= 0) & (idx_h < n)
    expect = np.full((n, width), SENTINEL, np.uint8)
    expect[idx_h[ok]] = src_h[ok]
    idx = torch.from_numpy(idx_h).cuda()
    for kw in ({}, {"path": "warp", "policy": 6}, {"path": "warp", "policy": 1}):
        dst = torch.full((n * width,), SENTINEL, dtype=torch.uint8, device="cuda")
        tg.scatter(dst, n, src, idx, n, width, **kw)
        assert np.array_equal(to_host(dst).reshape(n, width), expect), kw
    # a third of the rows, in passes on request
    m = n // 3
    expect = np.full((n, width), SENTINEL, np.uint8)
    sel = idx_h[:m]
    okm = (sel >= 0) & (sel < n)
    expect[sel[okm]] = src_h[:m][okm]
    dst = torch.full((n * width,), SENTINEL, dtype=torch.uint8, device="cuda")
    tg.scatter(dst, n, src, idx, m, width, path="warp", policy=6)
    assert np.array_equal(to_host(dst).reshape(n, width), expect)


@pytest.mark.parametrize("width", [4, 12, 16, 36, 64])
def test_gather_out_of_range_indices_are_skipped(cuda, width):
    torch = cuda
    n = 4099
    src_h = oracle.random_structs(n, width, seed=5)
    idx_h = oracle.uniform_indices(n, n, 6)
    bad = np.arange(n) % 97 == 3
    idx_h = idx_h.copy()
    idx_h[bad] = np.where(np.arange(bad.sum()) % 2 == 0, -5, n + 10)
    init = np.full(n * width, SENTINEL, np.uint8)
    expect = init.reshape(n, width).copy()
    expect[~bad] = src_h[idx_h[~bad]]
    for path in ["warp", "coalesced", "direct", "vector"]:
        dst = to_dev(torch, init)
        tg.gather(dst, to_dev(torch, src_h), n, torch.from_numpy(idx_h).cuda(), n, width, path=path)
        assert np.array_equal(to_host(dst), expect.reshape(-1)), path


@pytest.mark.parametrize("width", WIDTHS)
def test_scatter(cuda, width):
    torch = cuda
    for n in [33, 5000, 65536 + 17]:
        src_h = oracle.random_structs(n, width, seed=width * 17 + n)
        src = to_dev(torch, src_h)
        init = np.full(n * width, SENTINEL, np.uint8)
        for name in ["perm", "identity"]:
            idx_h = index_sets(n, seed=n)[name]
            idx = torch.from_numpy(idx_h).cuda()
            expect = oracle.scatter(init, src_h, idx_h, n, width)
            for path in ["warp", "coalesced", "direct", "auto", "vector"]:
                for unroll in ([1, 2, 4, 8] if path in ("warp", "coalesced") else [0]):
                    dst = to_dev(torch, init)
                    tg.scatter(dst, n, src, idx, n, width, path=path, unroll=unroll)
                    assert np.array_equal(to_host(dst), expect), (width, n, name, path, unroll)


def test_scatter_out_of_range_indices_are_skipped(cuda):
    torch = cuda
    n, width = 2000, 20
    src_h = oracle.random_structs(n, width, seed=8)
    idx_h = oracle.permutation(n, 9).copy()
    idx_h[::13] = -1
    keep = idx_h >= 0
    init = np.full(n * width, SENTINEL, np.uint8)
    expect = init.reshape(n, width).copy()
    expect[idx_h[keep]] = src_h[keep]
    for path in ["warp", "coalesced", "direct", "vector"]:
        dst = to_dev(torch, init)
        tg.scatter(dst, n, to_dev(torch, src_h), torch.from_numpy(idx_h).cuda(), n, width, path=path)
        assert np.array_equal(to_host(dst), expect.reshape(-1)), path


@pytest.mark.parametrize("width", [8, 12, 16, 24, 32, 48, 64])
def test_index_ops_misaligned(cuda, width):
    """Source and destination 4 bytes past a 16-byte boundary: the row-form
    kernels drop to 4-byte words, the coalesced_ptr kernels to the widest
    word every pointer allows."""
    torch = cuda
    n = 3001
    src_h = oracle.random_structs(n, width, seed=width)
    sbuf = torch.zeros(n * width + 64, dtype=torch.uint8, device="cuda")
    sbuf[4:4 + n * width] = to_dev(torch, src_h)
    idx_h = oracle.permutation(n, 3)
    idx = torch.from_numpy(idx_h).cuda()
    init = np.full(n * width, SENTINEL, np.uint8)
    g_expect = oracle.gather(init, src_h, idx_h, n, width)
    s_expect = oracle.scatter(init, src_h, idx_h, n, width)
    for path in ["warp", "coalesced", "direct", "auto"]:
        dbuf = torch.full((n * width + 64,), SENTINEL, dtype=torch.uint8, device="cuda")
        tg.gather(dbuf[4:], sbuf[4:], n, idx, n, width, path=path)
        assert np.array_equal(to_host(dbuf)[4:4 + n * width], g_expect), ("gather", path)
        dbuf.fill_(SENTINEL)
        tg.scatter(dbuf[4:], n, sbuf[4:], idx, n, width, path=path)
        assert np.array_equal(to_host(dbuf)[4:4 + n * width], s_expect), ("scatter", path)


def test_fill_matches_oracle_stream(cuda):
    torch = cuda
    for nwords, seed in [(1, 0), (1000, 0), (1 << 20, 12345)]:
        t = torch.empty(nwords, dtype=torch.int32, device="cuda")
        tg.fill_random_u32(t, nwords, seed)
        assert np.array_equal(to_host(t).view(np.uint32), oracle.random_words(nwords, seed))


def test_uniform_indices_match_oracle(cuda):
    torch = cuda
    for n, bound, seed in [(1, 1, 0), (5000, 77, 3), (1 << 20, 1 << 20, 9)]:
        t = torch.empty(n, dtype=torch.int32, device="cuda")
        tg.fill_uniform_indices(t, n, bound, seed)
        assert np.array_equal(to_host(t), oracle.uniform_indices(n, bound, seed))


def test_run_indices_and_permutation_match_oracle(cuda):
    """The gather workload's index patterns, generated by the library, equal
    the oracle's generators (ragged last chunk included)."""
    torch = cuda
    for n, seed in [(32, 0), (33, 4), (100003, 2), (1 << 20, 7)]:
        t = torch.empty(n, dtype=torch.int32, device="cuda")
        tg.fill_run_indices(t, n, seed)
        assert np.array_equal(to_host(t), oracle.run_indices(n, seed))
    for n, seed in [(1, 0), (2, 5), (100003, 1), (1 << 20, 3)]:
        t = torch.empty(n, dtype=torch.int32, device="cuda")
        tg.fill_permutation(t, n, seed)
        assert np.array_equal(to_host(t), oracle.permutation(n, seed))
    with pytest.raises(tg.TroveError):
        tg.fill_run_indices(t, 31, 0)


def test_copy_host(cuda):
    torch = cuda
    for n, width, pinned in [(1, 12, False), (100003, 12, True), ((96 << 20) // 28 + 5, 28, True)]:
        src_h = torch.from_numpy(oracle.random_structs(n, width, seed=n).reshape(-1).copy())
        if pinned:
            src_h = src_h.pin_memory()
        dst_h = torch.zeros_like(src_h)
        if pinned:
            dst_h = dst_h.pin_memory()
        tg.copy_host(dst_h, src_h, n, width)
        assert torch.equal(dst_h, src_h)


def test_config1_contiguous_copy_12B(cuda):
    """N = 2^20 structs of 3 x uint32 (12 B), words from seed 0, through
    load/store_warp_contiguous (one launch, 256 threads per block), bit-exact
    against the CPU host loop."""
    torch = cuda
    n, width = 1 << 20, 12
    src_h = oracle.random_structs(n, width, seed=0)
    src = to_dev(torch, src_h)
    dst = torch.zeros_like(src)
    tg.copy(dst, src, n, width, path="warp")
    torch.cuda.synchronize()
    assert np.array_equal(to_host(dst), oracle.copy(src_h, n, width))


@pytest.mark.parametrize("width", WIDTHS)
def test_aos_soa_round_trip(cuda, width):
    torch = cuda
    s = width // 4
    for n in [1, 33, 4097, 100003]:
        aos_h = oracle.random_structs(n, width, seed=width + 7 * n)
        soa_expect = oracle.aos_to_soa(aos_h, n, s)
        assert np.array_equal(soa_expect.reshape(s, n), aos_h.view(np.uint32).reshape(n, s).T)
        aos = to_dev(torch, aos_h)
        for unroll, grid in [(0, 0), (1, 0), (2, 0), (4, 0), (8, 0), (2, -1), (1, 7)]:
            soa = torch.empty(n * width, dtype=torch.uint8, device="cuda")
            tg.aos_to_soa(soa, aos, n, width, unroll=unroll, grid=grid)
            assert np.array_equal(to_host(soa).view(np.uint32), soa_expect), (width, n, unroll, grid)
            back = torch.zeros_like(aos)
            tg.soa_to_aos(back, soa, n, width, unroll=unroll, grid=grid)
            assert np.array_equal(to_host(back), aos_h.reshape(-1)), (width, n, unroll, grid)


@pytest.mark.parametrize("width", [68, 96, 128, 132, 200, 256])
def test_index_ops_wide_structs(cuda, width):
    """Widths above 64 bytes: row-form kernels with a run-time word count."""
    torch = cuda
    n = 3000
    src_h = oracle.random_structs(n, width, seed=width)
    src = to_dev(torch, src_h)
    init = np.full(n * width, SENTINEL, np.uint8)
    for name, idx_h in index_sets(n, seed=width).items():
        idx = torch.from_numpy(idx_h).cuda()
        for path in ["auto", "warp"]:
            dst = to_dev(torch, init)
            tg.gather(dst, src, n, idx, n, width, path=path)
            assert np.array_equal(to_host(dst), oracle.gather(init, src_h, idx_h, n, width)), (name, path)
        if name in ("perm", "identity"):
            dst = to_dev(torch, init)
            tg.scatter(dst, n, src, idx, n, width)
            assert np.array_equal(to_host(dst), oracle.scatter(init, src_h, idx_h, n, width)), name
    bad = oracle.uniform_indices(n, n, 1).copy()
    bad[::7] = -3
    dst = to_dev(torch, init)
    tg.gather(dst, src, n, torch.from_numpy(bad).cuda(), n, width)
    e = init.reshape(n, width).copy()
    ok = bad >= 0
    e[ok] = src_h[bad[ok]]
    assert np.array_equal(to_host(dst), e.reshape(-1))
