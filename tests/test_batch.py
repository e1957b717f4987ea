"""Batched execution (one persistent launch for many arrays) and the
autotuner cache.  The cache tests run on CPU; batch tests need a GPU and check
every task bit-exact against the oracle, launched plainly, as a CUDA graph
replay, and against one launch per task."""
import json

import numpy as np
import pytest

import oracle
import trove_gb300 as tg

SENTINEL = 0xA5


def test_autotune_cache_roundtrip(trove_lib, tmp_path):
    tg.autotune_clear()
    assert tg.autotune_lookup(tg.SCOPE_CALL, tg.OP_COPY, 12, 1 << 20) is None
    entries = [
        {"scope": 0, "op": 0, "width": 12, "bucket": 10, "path": 3, "unroll": 4, "grid": 0, "chunk": 0,
         "tile_bytes": 0, "cache_policy": 0, "gbs": 7100.0},
        {"scope": 1, "op": 1, "width": 36, "bucket": 8, "path": 0, "unroll": 0, "grid": 0, "chunk": 0,
         "tile_bytes": 131072, "cache_policy": 1, "gbs": 3000.5},
        {"scope": 0, "op": 3, "width": 20, "bucket": 13, "path": 1, "unroll": 8, "grid": 0, "chunk": 0,
         "tile_bytes": 0, "gbs": 6800.0},
    ]
    src = tmp_path / "in.json"
    src.write_text(json.dumps(entries))
    tg.autotune_load(src)
    got, tile = tg.autotune_lookup(tg.SCOPE_CALL, tg.OP_COPY, 12, 1 << 20)  # bucket(2^20) == 10
    assert (got.path, got.unroll) == (3, 4) and tile == 0
    got, tile = tg.autotune_lookup(tg.SCOPE_BATCH, tg.OP_GATHER, 36, 1 << 16)
    assert tile == 131072 and got.cache_policy == 1
    assert tg.autotune_lookup(tg.SCOPE_CALL, 3, 20, 1 << 26)[0].unroll == 8
    assert tg.autotune_lookup(tg.SCOPE_CALL, tg.OP_COPY, 12, 1 << 12) is None  # other bucket
    out = tmp_path / "out.json"
    tg.autotune_save(out)
    back = {(e["scope"], e["op"], e["width"], e["bucket"]): e for e in json.loads(out.read_text())}
    assert len(back) == 3
    assert back[(1, 1, 36, 8)]["tile_bytes"] == 131072
    assert back[(0, 3, 20, 13)]["unroll"] == 8
    tg.autotune_clear()
    assert tg.autotune_lookup(tg.SCOPE_CALL, tg.OP_COPY, 12, 1 << 20) is None
    with pytest.raises(tg.TroveError):
        tg.autotune_load(tmp_path / "missing.json")


def test_autotune_load_rejects_malformed_files(trove_lib, tmp_path):
    """A cache file is input: an unclosed entry or a file with no entries is
    refused, an empty array is fine, and a loaded entry whose launch shape is
    out of range is refused when a call would use it (a TMA chunk of 1 GiB,
    whose ring size would overflow), before anything reaches a device."""
    tg.autotune_clear()
    for text, ok in [('[{"scope": 0, "op": 0', False), ("garbage", False), ("[]", True)]:
        f = tmp_path / "c.json"
        f.write_text(text)
        if ok:
            tg.autotune_load(f)
        else:
            with pytest.raises(tg.TroveError) as e:
                tg.autotune_load(f)
            assert e.value.status == 1
    f = tmp_path / "chunk.json"
    f.write_text(json.dumps([{"scope": 0, "op": 0, "width": 16, "bucket": 10, "path": 4, "unroll": 0,
                              "grid": 0, "chunk": 1 << 30, "tile_bytes": 0, "cache_policy": 0}]))
    tg.autotune_load(f)
    ok = 0x100000
    with pytest.raises(tg.TroveError) as e:
        tg.copy(ok, ok + (64 << 20), 1 << 20, 16)  # AUTO takes the cached TMA shape
    assert e.value.status == 1
    tg.autotune_clear()


def test_batch_argument_errors(trove_lib):
    ok = 0x100000
    bad_tasks = [
        [dict(op=7, width=12, n=5, src=ok, dst=ok)],
        [dict(op=0, width=13, n=5, src=ok, dst=ok)],
        [dict(op=0, width=68, n=5, src=ok, dst=ok)],
        [dict(op=0, width=12, n=5, src=0, dst=ok)],
        [dict(op=1, width=12, n=5, src=ok, dst=ok, idx=None, bound=5)],
        [dict(op=1, width=12, n=5, src=ok + 2, dst=ok, idx=ok, bound=5)],
    ]
    for tasks, status in zip(bad_tasks, [1, 2, 2, 1, 1, 3]):
        with pytest.raises(tg.TroveError) as e:
            tg.Batch(tasks)
        assert e.value.status == status
    for bad_path in ["bulk", "warp"]:
        with pytest.raises(tg.TroveError):
            tg.Batch([dict(op=0, width=12, n=5, src=ok, dst=ok)], copy_path=bad_path)
    for bad in (dict(gather_policy=2), dict(gather_policy=8), dict(scatter_policy=4), dict(scatter_policy=-1)):
        with pytest.raises(tg.TroveError) as e:
            tg.Batch([dict(op=0, width=12, n=5, src=ok, dst=ok)], **bad)
        assert e.value.status == 1


def test_static_batch_argument_errors(trove_lib):
    """trv_batch_run_static validates the tasks and options before touching a
    device: the same task errors as trv_batch_create, the task limit, and an
    empty batch is a no-op."""
    ok = 0x100000
    for tasks, status in [([dict(op=7, width=12, n=5, src=ok, dst=ok)], 1),
                          ([dict(op=0, width=13, n=5, src=ok, dst=ok)], 2),
                          ([dict(op=0, width=12, n=5, src=0, dst=ok)], 1),
                          ([dict(op=1, width=12, n=5, src=ok + 2, dst=ok, idx=ok, bound=5)], 3),
                          ([dict(op=0, width=4, n=1, src=ok, dst=ok)] * (tg.STATIC_BATCH_MAX_TASKS + 1), 2)]:
        with pytest.raises(tg.TroveError) as e:
            tg.run_static(tasks)
        assert e.value.status == status
    with pytest.raises(tg.TroveError) as e:
        tg.run_static([dict(op=0, width=12, n=5, src=ok, dst=ok)], gather_policy=3)
    assert e.value.status == 1
    tg.run_static([])
    tg.run_static([dict(op=0, width=12, n=0, src=ok, dst=ok)])  # no tiles: nothing to launch


def make_workload(torch, count, seed, widths=(4, 12, 20, 36, 64), max_len=20000):
    """Mixed tasks with their expected outputs (oracle)."""
    rng = np.random.default_rng(seed)
    tasks, expect, outs = [], [], []
    for k in range(count):
        op = int(rng.choice([0, 0, 0, 0, 0, 1, 1, 1, 1, 2]))
        w = int(rng.choice(widths))
        n = int(np.exp(rng.uniform(np.log(1), np.log(max_len))))
        if k % 17 == 0:
            n = 0
        src_h = oracle.random_structs(max(n, 1), w, seed=seed * 1000 + k)[:n]
        init = np.full(max(n, 1) * w, SENTINEL, np.uint8)
        src = torch.from_numpy(src_h.reshape(-1).copy()).cuda() if n else torch.zeros(w, dtype=torch.uint8,
                                                                                        device="cuda")
        dst = torch.from_numpy(init.copy()).cuda()
        idx_t, bound = None, 0
        if op == 0:
            e = init.copy()
            e[: n * w] = src_h.reshape(-1)
        elif op == 1:
            idx_h = oracle.uniform_indices(n, max(n, 1), seed + k) if n else np.zeros(1, np.int32)
            if n > 10:
                idx_h[3] = -1  # skipped
                idx_h[7] = n + 5  # skipped
            idx_t = torch.from_numpy(idx_h.copy()).cuda()
            bound = n
            e = init.copy().reshape(-1, w)
            ok = (idx_h[:n] >= 0) & (idx_h[:n] < n)
            e[:n][ok] = src_h[idx_h[:n][ok]]
            e = e.reshape(-1)
        else:
            idx_h = oracle.permutation(n, seed + k) if n else np.zeros(1, np.int32)
            bound = n
            if n > 10:  # skipped: the destination keeps its sentinel at those rows
                idx_h[5] = -1
                idx_h[9] = n + 3
                ok = (idx_h[:n] >= 0) & (idx_h[:n] < n)
                e = init.copy().reshape(-1, w)
                e[idx_h[:n][ok]] = src_h[ok]
                e = e.reshape(-1)
            else:
                e = oracle.scatter(init, src_h, idx_h, n, w) if n else init.copy()
            idx_t = torch.from_numpy(idx_h.copy()).cuda()
        tasks.append(dict(op=op, width=w, n=n, src=src, dst=dst, idx=idx_t, bound=bound))
        expect.append(e)
        outs.append(dst)
    return tasks, expect


def reset(tasks):
    for t in tasks:
        t["dst"].fill_(SENTINEL)


def check(tasks, expect):
    for k, (t, e) in enumerate(zip(tasks, expect)):
        got = t["dst"].cpu().numpy()
        assert np.array_equal(got, e), (k, t["op"], t["width"], t["n"])


@pytest.mark.gpu
@pytest.mark.parametrize("gather_policy,scatter_policy", [(0, 0), (1, 1), (4, 5), (5, 1), (1, 5), (6, 5), (7, 5)])
@pytest.mark.parametrize("copy_path", ["vector", "auto"])
@pytest.mark.parametrize("tile_bytes", [0, 4096, 1 << 20])
def test_batch_matches_oracle(cuda, copy_path, tile_bytes, gather_policy, scatter_policy):
    torch = cuda
    tasks, expect = make_workload(torch, 120, seed=3)
    b = tg.Batch(tasks, tile_bytes=tile_bytes, copy_path=copy_path, gather_policy=gather_policy,
                 scatter_policy=scatter_policy)
    tiles, nbytes = b.info()
    assert tiles > 0 and nbytes > 0
    b.launch()
    torch.cuda.synchronize()
    check(tasks, expect)
    b.close()


@pytest.mark.gpu
def test_batch_graph_replay_and_per_call(cuda):
    torch = cuda
    tasks, expect = make_workload(torch, 200, seed=9, widths=tuple(range(4, 65, 4)))
    stream = torch.cuda.Stream()
    b = tg.Batch(tasks, tile_bytes=8192)
    with torch.cuda.stream(stream):
        b.capture(stream)
        for _ in range(3):
            reset(tasks)
            b.launch(stream)
            stream.synchronize()
            check(tasks, expect)
    reset(tasks)
    tg.run_per_call(tasks)
    torch.cuda.synchronize()
    check(tasks, expect)
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("blocks_per_sm", [2, 4])
@pytest.mark.parametrize("policy", [1, 5])
def test_batch_register_budgets(cuda, blocks_per_sm, policy):
    """Both kernel builds (2 and 4 resident blocks per SM) with register-held
    and shared-memory-staged gather / scatter rows, at several tile sizes."""
    torch = cuda
    tasks, expect = make_workload(torch, 80, seed=21, widths=tuple(range(4, 65, 4)))
    for tile_bytes in (0, 2048, 1 << 18):
        reset(tasks)
        b = tg.Batch(tasks, tile_bytes=tile_bytes, blocks_per_sm=blocks_per_sm, gather_policy=policy,
                     scatter_policy=policy)
        b.launch()
        torch.cuda.synchronize()
        check(tasks, expect)
        b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("policy", [1, 5])
def test_batch_misaligned_arrays(cuda, policy):
    """Arrays 4 or 8 bytes past a 16-byte boundary (slices of larger buffers):
    the movers fall back from their 16- and 8-byte words and vectors."""
    torch = cuda
    tasks, expect = [], []
    rng = np.random.default_rng(31)
    for k, (op, w, n, so, do) in enumerate([(0, 12, 4097, 4, 8), (0, 64, 3000, 8, 4), (1, 16, 5000, 4, 4),
                                            (1, 64, 2500, 8, 0), (1, 20, 4099, 0, 4), (2, 16, 5000, 4, 8),
                                            (2, 12, 4096, 8, 4), (2, 64, 1500, 0, 8)]):
        src_h = oracle.random_structs(n, w, seed=500 + k)
        sbuf = torch.zeros(n * w + 16, dtype=torch.uint8, device="cuda")
        sbuf[so:so + n * w] = torch.from_numpy(src_h.reshape(-1).copy()).cuda()
        dbuf = torch.full((n * w + 16,), SENTINEL, dtype=torch.uint8, device="cuda")
        init = np.full(n * w, SENTINEL, np.uint8)
        idx_t = None
        if op == 0:
            e = src_h.reshape(-1).copy()
        elif op == 1:
            idx_h = rng.integers(0, n, size=n).astype(np.int32)
            idx_h[11] = -1
            e = init.reshape(-1, w).copy()
            ok = idx_h >= 0
            e[ok] = src_h[idx_h[ok]]
            e = e.reshape(-1)
            idx_t = torch.from_numpy(idx_h).cuda()
        else:
            idx_h = oracle.permutation(n, 600 + k)
            e = oracle.scatter(init, src_h, idx_h, n, w)
            idx_t = torch.from_numpy(idx_h.copy()).cuda()
        tasks.append(dict(op=op, width=w, n=n, src=sbuf[so:], dst=dbuf[do:], idx=idx_t, bound=n, keep=(sbuf, dbuf, do)))
        expect.append(e)
    b = tg.Batch(tasks, gather_policy=policy, scatter_policy=policy)
    b.launch()
    torch.cuda.synchronize()
    for k, (t, e) in enumerate(zip(tasks, expect)):
        sbuf, dbuf, do = t["keep"]
        got = dbuf.cpu().numpy()
        assert np.array_equal(got[do:do + e.size], e), k
        assert (got[:do] == SENTINEL).all() and (got[do + e.size:] == SENTINEL).all(), k
    b.close()


@pytest.mark.gpu
def test_batch_runs_of_empty_tasks(cuda):
    """Long runs of tasks without tiles between real ones (equal tile-prefix
    values): the kernel's task search must land every tile on its task."""
    torch = cuda
    made, made_expect = make_workload(torch, 12, seed=41)
    pairs = [(t, e) for t, e in zip(made, made_expect) if t["n"] > 0]
    tasks, want = [], []
    dummy = torch.zeros(64, dtype=torch.uint8, device="cuda")
    for k, (t, e) in enumerate(pairs):
        for _ in range((50, 300, 1, 77, 200)[k % 5]):
            tasks.append(dict(op=k % 3, width=12, n=0, src=dummy, dst=dummy, idx=None, bound=0))
        tasks.append(t)
        want.append((t, e))
    for _ in range(123):
        tasks.append(dict(op=0, width=4, n=0, src=dummy, dst=dummy))
    for tile_bytes in (0, 2048):
        for t, _ in want:
            t["dst"].fill_(SENTINEL)
        b = tg.Batch(tasks, tile_bytes=tile_bytes)
        b.launch()
        torch.cuda.synchronize()
        for t, e in want:
            assert np.array_equal(t["dst"].cpu().numpy(), e), (t["op"], t["width"], t["n"])
        b.close()


@pytest.mark.gpu
def test_batch_grid_override_and_empty(cuda):
    torch = cuda
    tasks, expect = make_workload(torch, 40, seed=5)
    for grid in [1, 3, 1000]:
        reset(tasks)
        tg.Batch(tasks, grid=grid, tile_bytes=2048).launch()
        torch.cuda.synchronize()
        check(tasks, expect)
    empty = tg.Batch([])
    assert empty.info() == (0, 0)
    empty.launch()


@pytest.mark.gpu
def test_autotune_on_gpu(cuda, tmp_path):
    torch = cuda
    tg.autotune_clear()
    n, w = 1 << 18, 12
    for op in (tg.OP_COPY, tg.OP_GATHER, 3, 4, tg.OP_AOS_TO_SOA, tg.OP_SOA_TO_AOS):
        tg.autotune_call(op, w, n)
        assert tg.autotune_lookup(tg.SCOPE_CALL, op, w, n) is not None, op
    src_h = oracle.random_structs(n, w, seed=1)
    src = torch.from_numpy(src_h.reshape(-1).copy()).cuda()
    dst = torch.zeros_like(src)
    tg.copy(dst, src, n, w)  # AUTO consults the cache
    idx_h = oracle.permutation(n, 2)
    gd = torch.zeros_like(src)
    tg.gather(gd, src, n, torch.from_numpy(idx_h).cuda(), n, w)
    init = np.full(n * w, SENTINEL, np.uint8)
    ed = torch.from_numpy(init).cuda()
    tg.copy_exit(ed, src, n, w, 625, path="warp")
    torch.cuda.synchronize()
    assert np.array_equal(dst.cpu().numpy(), src_h.reshape(-1))
    assert np.array_equal(gd.cpu().numpy(), oracle.gather(np.zeros(n * w, np.uint8), src_h, idx_h, n, w))
    assert np.array_equal(ed.cpu().numpy(), oracle.copy_exit(init, src_h, n, w, 625)[0])
    soa = torch.zeros_like(src)
    tg.aos_to_soa(soa, src, n, w)  # unroll from the cache
    back = torch.zeros_like(src)
    tg.soa_to_aos(back, soa, n, w)
    torch.cuda.synchronize()
    assert np.array_equal(soa.cpu().numpy().view(np.uint32), oracle.aos_to_soa(src_h, n, w // 4))
    assert np.array_equal(back.cpu().numpy(), src_h.reshape(-1))
    tasks, expect = make_workload(torch, 60, seed=11)
    tg.autotune_batch(tasks)
    reset(tasks)
    tg.Batch(tasks).launch()
    torch.cuda.synchronize()
    check(tasks, expect)
    tg.autotune_save(tmp_path / "cache.json")
    assert json.loads((tmp_path / "cache.json").read_text())
    tg.autotune_clear()
