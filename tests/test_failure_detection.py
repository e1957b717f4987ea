"""Failure detection without faulting the GPU.

* The TMA bulk path bounds every mbarrier wait.  A host-side hook shrinks the
  copy loop's poll budget to zero, so the first wait gives up at once while
  its load is still in flight: the kernel must set the device flag
  (trv_check_device -> TRV_ERR_DEVICE_FLAG), still drain its own transfers,
  and leave the context usable (the next copy is bit-exact).
* The server's wait is bounded on the host: a request held back by the HBM
  budget makes trv_server_wait return TRV_ERR_TIMEOUT, and the request
  completes once the budget is released.
"""
import numpy as np
import pytest

import oracle
import trove_gb300 as tg

DEVICE_FLAG = 11  # TRV_ERR_DEVICE_FLAG
TIMEOUT = 7  # TRV_ERR_TIMEOUT


def test_wait_hook_exported(trove_lib):
    assert hasattr(trove_lib, "trv_debug_set_bulk_wait_polls")
    tg.debug_set_bulk_wait_polls(0xFFFFFFFF)  # the default: no device work


@pytest.mark.gpu
def test_bulk_wait_timeout_sets_flag_and_context_survives(cuda):
    torch = cuda
    width, n = 16, (8 << 20) // 16
    src_h = oracle.random_structs(n, width, seed=41).reshape(-1)
    src = torch.from_numpy(src_h.copy()).cuda()
    dst = torch.zeros_like(src)
    tg.check_device()  # starts clear
    tg.debug_set_bulk_wait_polls(0)
    try:
        tg.copy(dst, src, n, width, path="bulk")
        with pytest.raises(tg.TroveError) as e:
            tg.check_device()
        assert e.value.status == DEVICE_FLAG
    finally:
        tg.debug_set_bulk_wait_polls(0xFFFFFFFF)
    tg.check_device()  # reading the flag cleared it
    dst.zero_()
    tg.copy(dst, src, n, width, path="bulk")
    tg.check_device()
    assert np.array_equal(dst.cpu().numpy(), src_h)


@pytest.mark.gpu
def test_server_wait_times_out_while_budget_is_held(cuda):
    torch = cuda
    width, n = 16, 1 << 14
    nbytes = n * width
    src_h = oracle.random_structs(n, width, seed=43).reshape(-1)
    src = torch.from_numpy(src_h.copy()).cuda()
    req = dict(op=tg.OP_COPY, width=width, n=n, src=src, src_n=n)
    server = tg.Server(nbytes)  # room for exactly one output
    try:
        first = server.submit(req)
        assert server.wait(first, 10000).status == 0
        second = server.submit(req)
        with pytest.raises(tg.TroveError) as e:
            server.wait(second, 200)
        assert e.value.status == TIMEOUT
        assert server.poll(second) is None  # TRV_ERR_BUSY: still queued
        server.release(first)
        res = server.wait(second, 10000)
        assert res.status == 0
        out = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        tg.copy(out, res.dst, n, width)
        assert np.array_equal(out.cpu().numpy(), src_h)
        server.release(second)
    finally:
        server.close()
