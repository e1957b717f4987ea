"""trv_batch_run_static: the batch entry point that allocates no device
memory, for callers that cannot call cudaMalloc (it synchronizes the whole
device; a process whose device memory is reserved up front by another
allocator may have none to spare).  Its results must equal the allocating
entry point's (trv_batch_create + trv_batch_launch) byte for byte, on two
calls in a row, since every call reuses the same library-owned device array.
Collected last so that a run stopping at the first failure has run the rest."""
import numpy as np
import pytest

import oracle
import trove_gb300 as tg

pytestmark = pytest.mark.gpu

SENTINEL = 0x5A


def workload(torch, count, seed):
    rng = np.random.default_rng(seed)
    tasks = []
    for k in range(count):
        op = int(rng.choice([0, 0, 1, 1, 2]))
        w = int(rng.choice([4, 8, 12, 20, 36, 48, 64]))
        n = int(np.exp(rng.uniform(0, np.log(30000))))
        src = torch.from_numpy(oracle.random_structs(n, w, seed=seed * 977 + k).reshape(-1).copy()).cuda()
        dst = torch.full((n * w,), SENTINEL, dtype=torch.uint8, device="cuda")
        idx = None
        if op == 1:
            idx = torch.from_numpy(oracle.uniform_indices(n, n, seed + k)).cuda()
        elif op == 2:
            idx = torch.from_numpy(oracle.permutation(n, seed + k)).cuda()
        tasks.append(dict(op=op, width=w, n=n, src=src, dst=dst, idx=idx, bound=n))
    return tasks


def outputs(tasks):
    return [t["dst"].cpu().numpy().copy() for t in tasks]


def reset(tasks):
    for t in tasks:
        t["dst"].fill_(SENTINEL)


def test_static_batch_equals_allocating_batch(cuda):
    torch = cuda
    tasks = workload(torch, 300, seed=21)
    b = tg.Batch(tasks, tile_bytes=16384)
    b.launch()
    torch.cuda.synchronize()
    expect = outputs(tasks)
    b.close()
    for call in range(2):
        reset(tasks)
        tg.run_static(tasks, tile_bytes=16384)
        torch.cuda.synchronize()
        for k, (got, e) in enumerate(zip(outputs(tasks), expect)):
            assert np.array_equal(got, e), (call, k, tasks[k]["op"], tasks[k]["width"], tasks[k]["n"])
    # a different batch through the same array right after, with default tiles
    more = workload(torch, 40, seed=22)
    b = tg.Batch(more)
    b.launch()
    torch.cuda.synchronize()
    expect = outputs(more)
    b.close()
    reset(more)
    tg.run_static(more)
    torch.cuda.synchronize()
    for got, e in zip(outputs(more), expect):
        assert np.array_equal(got, e)
    # register-held rows at the 128-register budget, through the same array
    reset(more)
    tg.run_static(more, blocks_per_sm=2, gather_policy=1, scatter_policy=1)
    torch.cuda.synchronize()
    for got, e in zip(outputs(more), expect):
        assert np.array_equal(got, e)


def test_static_batch_allocates_nothing(cuda):
    """Once the kernels are loaded (first call), further calls change neither
    the device's free memory nor torch's allocator counters."""
    torch = cuda
    tasks = workload(torch, 60, seed=23)
    tg.run_static(tasks)
    tg.run_static(tasks, blocks_per_sm=2, gather_policy=1, scatter_policy=1)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0, reserved0 = torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
    for _ in range(3):
        tg.run_static(tasks)
        tg.run_static(tasks, blocks_per_sm=2, gather_policy=1, scatter_policy=1)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert (torch.cuda.memory_allocated(), torch.cuda.memory_reserved()) == (alloc0, reserved0)


def test_static_batch_refuses_capture(cuda):
    """The plan is copied from host memory that lives only for the call, so a
    capturing stream is refused before anything is enqueued."""
    torch = cuda
    src = torch.arange(64, dtype=torch.uint8, device="cuda")
    dst = torch.zeros_like(src)
    one = dict(op=0, width=4, n=16, src=src, dst=dst)
    tg.run_static([one])  # first call (address look-up) outside any capture
    torch.cuda.synchronize()
    assert torch.equal(dst, src)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    status = None
    with torch.cuda.graph(g, stream=side, capture_error_mode="thread_local"):
        try:
            tg.run_static([one], stream=side)
        except tg.TroveError as e:
            status = e.status
        dst.add_(1)  # keeps the captured graph non-empty
    assert status == 2  # TRV_ERR_UNSUPPORTED
    torch.cuda.synchronize()
    assert torch.equal(dst, src)  # the graph was captured, never replayed
    dst.zero_()
    tg.run_static([one], stream=side)  # the stream works normally afterwards
    side.synchronize()
    assert torch.equal(dst, src)


def test_static_batch_limit(cuda):
    torch = cuda
    src = torch.zeros(64, dtype=torch.uint8, device="cuda")
    dst = torch.zeros_like(src)
    one = dict(op=0, width=4, n=16, src=src, dst=dst)
    with pytest.raises(tg.TroveError) as e:
        tg.run_static([one] * (tg.STATIC_BATCH_MAX_TASKS + 1))
    assert e.value.status == 2  # TRV_ERR_UNSUPPORTED
    tg.run_static([one] * tg.STATIC_BATCH_MAX_TASKS)
    torch.cuda.synchronize()
    assert torch.equal(dst, src)
