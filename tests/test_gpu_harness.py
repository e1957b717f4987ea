"""The reference's own test-kernel patterns (oracle/trove_bench_kernels.cu)
on the GPU, compiled against this repository's headers and — where the
prebuilt cubin is present — against the reference's headers.  Both must
match the CPU oracle bit for bit, which also shows that kernels written for
the reference recompile unchanged against include/trove."""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

N = 256 * 40


def modules():
    mods = [("own", oracle.own_cubin())]
    ref = oracle.reference_cubin()
    if ref is not None:
        mods.append(("reference", ref))
    return mods


@pytest.fixture(scope="module")
def cubins(cuda):
    return modules()


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1).copy()).cuda()


def ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def test_reference_cubin_shipped(cubins):
    names = [n for n, _ in cubins]
    if "reference" not in names:
        pytest.skip("reference cubin not present (built only where the reference checkout exists)")


@pytest.mark.parametrize("s", list(range(1, 17)))
def test_benchmark_kernels(cuda, cubins, s):
    torch = cuda
    w = 4 * s
    src_h = oracle.random_structs(N, w, seed=s)
    perm = oracle.permutation(N, s + 1)
    runs = oracle.run_indices(N, s + 2)
    for name, mod in cubins:
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


@pytest.mark.parametrize("s", [1, 3, 5, 8, 12, 16])
def test_block_and_exit_kernels(cuda, cubins, s):
    torch = cuda
    w = 4 * s
    l = 256 * 7 + 17  # partial tail warp -> non-converged fallback
    for name, mod in cubins:
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
