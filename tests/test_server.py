"""Serving: admission against an HBM budget, continuous batching into the
persistent kernel, per-request results.  Every request's output served in a
mixed, overlapping stream must be byte-identical to the same request run
alone (trv_copy / trv_gather), and to the oracle."""
import ctypes

import numpy as np
import pytest

import oracle
import trove_gb300 as tg

WIDTHS = [8, 12, 16, 28, 64]


def read_device(ptr, nbytes):
    """Device bytes at a raw address, through the CUDA driver (independent of
    the library under test)."""
    cu = ctypes.CDLL("libcuda.so.1")
    out = np.empty(nbytes, np.uint8)
    rc = cu.cuMemcpyDtoH_v2(out.ctypes.data_as(ctypes.c_void_p), ctypes.c_uint64(ptr), ctypes.c_size_t(nbytes))
    assert rc == 0, rc
    return out


def test_server_argument_errors(trove_lib):
    """Refused before any device work: a zero budget, negative or oversized
    slot counts and task tables."""
    for kw in ({}, {"max_inflight": -1}, {"max_inflight": 65}, {"max_batch_requests": (1 << 16) + 1},
               {"max_batch_requests": (1 << 31) - 1}, {"tile_bytes": -1}):
        with pytest.raises(tg.TroveError, match="invalid argument"):
            tg.Server(0 if not kw else 1 << 20, **kw)


@pytest.fixture(scope="module")
def pools(cuda):
    torch = cuda
    n = 1 << 18
    src = {w: torch.from_numpy(oracle.random_structs(n, w, seed=w).reshape(-1).copy()).cuda() for w in WIDTHS}
    idx_h = oracle.uniform_indices(n, n, 5)
    return n, src, torch.from_numpy(idx_h).cuda(), idx_h


def make_requests(pools, count, seed, max_len):
    n_pool, src, idx, _ = pools
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(count):
        w = int(rng.choice(WIDTHS))
        n = int(np.exp(rng.uniform(np.log(1), np.log(max_len))))
        off = int(rng.integers(0, n_pool - n + 1))
        if rng.random() < 0.5:
            reqs.append(dict(op=tg.OP_COPY, width=w, n=n, src=src[w].data_ptr() + off * w, src_n=n))
        else:
            reqs.append(dict(op=tg.OP_GATHER, width=w, n=n, src=src[w], src_n=n_pool, idx=idx.data_ptr() + 4 * off))
    return reqs


def alone(torch, r):
    out = torch.empty(r["n"] * r["width"], dtype=torch.uint8, device="cuda")
    if r["op"] == tg.OP_COPY:
        tg.copy(out, r["src"], r["n"], r["width"])
    else:
        tg.gather(out, r["src"], r["src_n"], r["idx"], r["n"], r["width"])
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.gpu
def test_results_same_alone_and_in_the_mix(cuda, pools):
    torch = cuda
    reqs = make_requests(pools, 400, seed=1, max_len=60000)
    expect = [alone(torch, r) for r in reqs]
    # oracle for a few of them
    n_pool, src, _, idx_h = pools
    for r, e in list(zip(reqs, expect))[:20]:
        w, n = r["width"], r["n"]
        src_h = src[w].cpu().numpy().reshape(n_pool, w)
        if r["op"] == tg.OP_COPY:
            off = (r["src"] - src[w].data_ptr()) // w
            assert np.array_equal(e, src_h[off:off + n].reshape(-1))
        else:
            off = (r["idx"] - pools[2].data_ptr()) // 4
            assert np.array_equal(e, src_h[idx_h[off:off + n]].reshape(-1))
    server = tg.Server(1 << 30, max_inflight=3, max_batch_requests=32)
    rng = np.random.default_rng(2)
    arrivals = np.cumsum(rng.exponential(1.0 / 20.0, size=len(reqs)))  # ~20 requests per ms
    ids, st = server.replay(reqs, arrivals)
    assert st["completed"] == len(reqs)
    assert st["batches"] > 1
    batches = set()
    for rid, r, e in zip(ids, reqs, expect):
        res = server.wait(rid)
        assert res.status == 0
        batches.add(res.batch)
        got = read_device(res.dst, r["n"] * r["width"])
        assert np.array_equal(got, e), (r["op"], r["width"], r["n"])
        assert res.submit_ms <= res.launch_ms <= res.done_ms
        server.release(rid)
    assert len(batches) > 1
    assert st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    stats = server.stats()
    assert stats["budget_in_use"] == 0
    server.close()


@pytest.mark.gpu
def test_budget_admission_and_reuse(cuda, pools):
    torch = cuda
    reqs = make_requests(pools, 60, seed=3, max_len=40000)
    big = max(r["n"] * r["width"] for r in reqs)
    budget = 2 * big + 4096  # at most a few outputs resident at once
    server = tg.Server(budget, max_inflight=2, max_batch_requests=8, release_when_done=True)
    ids, st = server.replay(reqs, np.zeros(len(reqs)))  # all arrive at once
    assert st["completed"] == len(reqs)
    stats = server.stats()
    assert stats["max_queued"] > 1
    assert stats["budget_in_use"] == 0
    server.close()
    server = tg.Server(1 << 20)
    too_big = dict(op=tg.OP_COPY, width=64, n=(1 << 20) // 64 + 1, src=pools[1][64], src_n=(1 << 20) // 64 + 1)
    with pytest.raises(tg.TroveError) as e:
        server.submit(too_big)
    assert e.value.status == 6  # TRV_ERR_BUDGET
    with pytest.raises(tg.TroveError):
        server.submit(dict(op=tg.OP_SCATTER, width=12, n=5, src=pools[1][12], src_n=5))
    server.close()


@pytest.mark.gpu
def test_poll_wait_release_cycle(cuda, pools):
    torch = cuda
    r = make_requests(pools, 1, seed=7, max_len=1000)[0]
    e = alone(torch, r)
    server = tg.Server(1 << 24)
    rid = server.submit(r)
    res = server.wait(rid, 10000)
    assert res.status == 0 and server.poll(rid).status == 0
    assert np.array_equal(read_device(res.dst, r["n"] * r["width"]), e)
    server.release(rid)
    with pytest.raises(tg.TroveError):
        server.release(rid)
    server.close()


@pytest.mark.gpu
def test_gather_with_out_of_range_indices(cuda, pools):
    """Server gathers skip indices outside [0, src_n): the in-range rows equal
    the oracle's, and a run of such requests neither faults nor disturbs the
    requests beside it."""
    torch = cuda
    n_pool, src, _, _ = pools
    rng = np.random.default_rng(11)
    server = tg.Server(1 << 28, max_inflight=2, max_batch_requests=16)
    reqs, idx_keep, expect_ok = [], [], []
    for k, w in enumerate(WIDTHS * 2):
        n = int(rng.integers(100, 5000))
        idx_h = rng.integers(0, n_pool, size=n).astype(np.int32)
        bad = rng.random(n) < 0.2
        idx_h[bad] = np.where(rng.random(int(bad.sum())) < 0.5, -1 - k, n_pool + k).astype(np.int32)
        idx = torch.from_numpy(idx_h).cuda()
        idx_keep.append(idx)
        reqs.append(dict(op=tg.OP_GATHER, width=w, n=n, src=src[w], src_n=n_pool, idx=idx))
        src_h = src[w].cpu().numpy().reshape(n_pool, w)
        expect_ok.append((~bad, src_h[np.where(bad, 0, idx_h)]))
    torch.cuda.synchronize()
    ids = [server.submit(r) for r in reqs]
    for rid, r, (ok, rows) in zip(ids, reqs, expect_ok):
        res = server.wait(rid)
        assert res.status == 0
        got = read_device(res.dst, r["n"] * r["width"]).reshape(r["n"], r["width"])
        assert np.array_equal(got[ok], rows[ok]), (r["width"], r["n"])
        server.release(rid)
    server.close()
    tg.check_device()
