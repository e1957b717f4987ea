"""CPU oracle for the AoS hot path — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, and only to verify results (or, for the baseline, as the timed CPU
form).  The product library never imports it.

  * the C restatement (aos_oracle.c) through ctypes: seeded inputs, copy,
    gather, scatter, early-exit copy, the reference's known answers and the
    R2C index semantics;
  * the host lane emulator builds (emu/): the reference's own headers and this
    repository's headers run on 32 emulated lanes;
  * a CUDA driver-API loader for the harness cubins (trove_bench_kernels.cu
    compiled against either header tree).
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import build_oracle as _b

_c = None
_u8p = ctypes.c_void_p


def _p(a) -> int:
    return 0 if a is None else int(a.ctypes.data)


def lib():
    """The C oracle, built on first use."""
    global _c
    if _c is None:
        c = ctypes.CDLL(str(_b.build_oracle_lib()))
        c.orc_word.restype = ctypes.c_uint32
        c.orc_word.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        c.orc_fill_u32.argtypes = [_u8p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int]
        c.orc_permutation.argtypes = [_u8p, ctypes.c_uint64, ctypes.c_uint64]
        c.orc_uniform_indices.argtypes = [_u8p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64]
        c.orc_run_indices.argtypes = [_u8p, ctypes.c_uint64, ctypes.c_uint64]
        for name in ("orc_copy",):
            getattr(c, name).argtypes = [_u8p, _u8p, ctypes.c_uint64, ctypes.c_uint32]
        for name in ("orc_gather", "orc_scatter"):
            getattr(c, name).argtypes = [_u8p, _u8p, _u8p, ctypes.c_uint64, ctypes.c_uint32]
        c.orc_copy_exit.restype = ctypes.c_uint64
        c.orc_copy_exit.argtypes = [_u8p, _u8p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32]
        c.orc_counting.argtypes = [_u8p, ctypes.c_uint64, ctypes.c_int]
        c.orc_load_sum.argtypes = [_u8p, _u8p, ctypes.c_uint64, ctypes.c_int]
        c.orc_r2c_source.argtypes = [ctypes.c_int, ctypes.c_int, _u8p, _u8p]
        c.orc_aos_to_soa.argtypes = [_u8p, _u8p, ctypes.c_uint64, ctypes.c_int]
        c.orc_run_mt.argtypes = [ctypes.c_int, _u8p, _u8p, _u8p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int]
        _c = c
    return _c


# ---- seeded inputs ---------------------------------------------------------

def word(seed: int, k: int) -> int:
    return lib().orc_word(seed, k)


def random_words(nwords: int, seed: int, threads: int = 1) -> np.ndarray:
    out = np.empty(nwords, np.uint32)
    lib().orc_fill_u32(_p(out), nwords, seed, threads)
    return out


def random_structs(n: int, width: int, seed: int, threads: int = 1) -> np.ndarray:
    """n structs of `width` bytes (a multiple of 4) as an (n, width) uint8 array."""
    assert width % 4 == 0
    return random_words(n * width // 4, seed, threads).view(np.uint8).reshape(n, width)


def permutation(n: int, seed: int) -> np.ndarray:
    out = np.empty(n, np.int32)
    lib().orc_permutation(_p(out), n, seed)
    return out


def uniform_indices(n: int, bound: int, seed: int) -> np.ndarray:
    out = np.empty(n, np.int32)
    lib().orc_uniform_indices(_p(out), n, bound, seed)
    return out


def run_indices(n: int, seed: int) -> np.ndarray:
    out = np.empty(n, np.int32)
    lib().orc_run_indices(_p(out), n, seed)
    return out


# ---- the path's semantics ---------------------------------------------------

def _bytes(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a)
    return a.view(np.uint8).reshape(-1)


def copy(src: np.ndarray, n: int, width: int) -> np.ndarray:
    s = _bytes(src)
    out = np.zeros(n * width, np.uint8)
    lib().orc_copy(_p(out), _p(s), n, width)
    return out


def gather(dst_init: np.ndarray, src: np.ndarray, idx: np.ndarray, n: int, width: int) -> np.ndarray:
    """dst[i] = src[idx[i]]; dst_init must already hold the skipped structs.
    Indices must be valid (the C ABI's skip rule is applied by the caller)."""
    out = _bytes(dst_init).copy()
    lib().orc_gather(_p(out), _p(_bytes(src)), _p(np.ascontiguousarray(idx, np.int32)), n, width)
    return out


def scatter(dst_init: np.ndarray, src: np.ndarray, idx: np.ndarray, n: int, width: int) -> np.ndarray:
    out = _bytes(dst_init).copy()
    lib().orc_scatter(_p(out), _p(_bytes(src)), _p(np.ascontiguousarray(idx, np.int32)), n, width)
    return out


def copy_exit(dst_init: np.ndarray, src: np.ndarray, n: int, width: int, modulus: int):
    out = _bytes(dst_init).copy()
    written = lib().orc_copy_exit(_p(out), _p(_bytes(src)), n, width, modulus)
    return out, int(written)


def counting(n: int, s: int) -> np.ndarray:
    out = np.empty(n * s, np.int32)
    lib().orc_counting(_p(out), n, s)
    return out


def load_sum(src: np.ndarray, n: int, s: int) -> np.ndarray:
    out = np.empty(n, np.int32)
    lib().orc_load_sum(_p(np.ascontiguousarray(src).view(np.int32)), _p(out), n, s)
    return out


def memory_op(s: int, kind: int, offset: int, stride: int, data: np.ndarray, out_init) -> np.ndarray:
    """trove/memory.h restated (reference memory.h:136-168 and the
    warp_load_array / warp_store_array / uncoalesced_store_array recursions
    above it): warp_load(p, offset, stride)[k] = p[offset + k * stride]
    (kinds 0 and 1, the volatile overload); warp_store writes
    p[offset + k * stride] = a[k] (kind 2); uncoalesced_store writes
    p[k] = a[k], its stride unused (kind 3)."""
    out = np.array(out_init, np.int32)
    d = np.asarray(data, np.int32)
    k = np.arange(s)
    if kind in (0, 1):
        out[:s] = d[offset + k * stride]
    elif kind == 2:
        out[offset + k * stride] = d[:s]
    else:
        out[:s] = d[:s]
    return out


def aos_to_soa(aos: np.ndarray, n: int, s: int) -> np.ndarray:
    out = np.empty(n * s, np.uint32)
    lib().orc_aos_to_soa(_p(out), _p(np.ascontiguousarray(aos).view(np.uint32)), n, s)
    return out


def r2c_source(n: int, m: int):
    lane = np.empty(n * m, np.int32)
    elem = np.empty(n * m, np.int32)
    lib().orc_r2c_source(n, m, _p(lane), _p(elem))
    return lane.reshape(n, m), elem.reshape(n, m)


OP_COPY, OP_GATHER, OP_SCATTER, OP_COPY_EXIT, OP_AOS_TO_SOA, OP_SOA_TO_AOS = 0, 1, 2, 3, 4, 5


def run_mt(op: int, dst: np.ndarray, src: np.ndarray, idx, n: int, width: int, threads: int, modulus: int = 0):
    """The timed CPU form: static split of n structs over `threads` threads
    (OP_COPY_EXIT applies the early-exit predicate with `modulus`)."""
    third = modulus if op == OP_COPY_EXIT else _p(idx)
    lib().orc_run_mt(op, _p(dst), _p(src), third, n, width, threads)


# ---- host lane emulator builds ----------------------------------------------

class Emu:
    """ctypes view of emu/api_cases.cpp built against one header tree."""

    def __init__(self, path: Path):
        self.path = Path(path)
        c = ctypes.CDLL(str(path))
        v, i32 = ctypes.c_void_p, ctypes.c_int
        c.emu_transpose.argtypes = [i32, i32, i32, i32, v]
        c.emu_rotate.argtypes = [i32, i32, v, v]
        c.emu_copy.argtypes = [i32, i32, v, v, i32]
        c.emu_store_counting.argtypes = [i32, v, i32]
        c.emu_load_sum.argtypes = [i32, v, v, i32]
        c.emu_gather.argtypes = [i32, v, v, v, i32]
        c.emu_scatter.argtypes = [i32, v, v, v, i32]
        c.emu_block.argtypes = [i32, i32, v, v, i32]
        c.emu_copy_exit.argtypes = [i32, i32, v, v, ctypes.c_longlong, ctypes.c_uint32]
        c.emu_warp_converged.argtypes = [i32, ctypes.c_uint32, v]
        c.emu_memory.argtypes = [i32, i32, i32, i32, v, v]
        self.c = c

    def transpose(self, direction: str, n: int, m: int, data: np.ndarray) -> np.ndarray:
        """data: (n, m, words) int32, transposed in a copy."""
        d = np.ascontiguousarray(data, np.int32).copy()
        rc = self.c.emu_transpose(0 if direction == "r2c" else 1, n, m, d.shape[2], _p(d))
        assert rc == 0, rc
        return d

    def rotate(self, values: np.ndarray, a: int) -> np.ndarray:
        v = np.ascontiguousarray(values, np.int32)
        out = np.empty_like(v)
        assert self.c.emu_rotate(len(v), a, _p(v), _p(out)) == 0
        return out

    def copy(self, s: int, tile: int, src: np.ndarray, n: int) -> np.ndarray:
        out = np.zeros(n * s, np.int32)
        assert self.c.emu_copy(s, tile, _p(np.ascontiguousarray(src)), _p(out), n) == 0
        return out

    def store_counting(self, s: int, n: int) -> np.ndarray:
        out = np.zeros(n * s, np.int32)
        assert self.c.emu_store_counting(s, _p(out), n) == 0
        return out

    def load_sum(self, s: int, src: np.ndarray, n: int) -> np.ndarray:
        out = np.zeros(n, np.int32)
        assert self.c.emu_load_sum(s, _p(np.ascontiguousarray(src)), _p(out), n) == 0
        return out

    def gather(self, s: int, src: np.ndarray, idx: np.ndarray, n: int, dst_init=None) -> np.ndarray:
        out = np.zeros(n * s, np.int32) if dst_init is None else np.array(dst_init, np.int32)
        assert self.c.emu_gather(s, _p(np.ascontiguousarray(src)), _p(np.ascontiguousarray(idx, np.int32)),
                                 _p(out), n) == 0
        return out

    def scatter(self, s: int, src: np.ndarray, idx: np.ndarray, n: int, dst_init) -> np.ndarray:
        out = np.array(dst_init, np.int32)
        assert self.c.emu_scatter(s, _p(np.ascontiguousarray(src)), _p(np.ascontiguousarray(idx, np.int32)),
                                  _p(out), n) == 0
        return out

    def block(self, s: int, write: bool, src, l: int) -> np.ndarray:
        out = np.zeros(l * s, np.int32)
        assert self.c.emu_block(s, 1 if write else 0, _p(src), _p(out), l) == 0
        return out

    def copy_exit(self, s: int, api: int, src: np.ndarray, n: int, modulus: int, dst_init) -> np.ndarray:
        out = np.array(dst_init, np.int32)
        assert self.c.emu_copy_exit(s, api, _p(np.ascontiguousarray(src)), _p(out), n, modulus) == 0
        return out

    def memory(self, s: int, kind: int, offset: int, stride: int, data: np.ndarray, out_init) -> np.ndarray:
        """trove/memory.h: kind 0 warp_load (1: volatile), 2 warp_store,
        3 uncoalesced_store; data is the source buffer (kinds 0-1) or the
        s values stored (kinds 2-3)."""
        out = np.array(out_init, np.int32)
        assert self.c.emu_memory(s, kind, offset, stride, _p(np.ascontiguousarray(data, np.int32)), _p(out)) == 0
        return out

    def warp_converged(self, N: int, active: int) -> np.ndarray:
        out = np.full(32, 255, np.uint8)
        assert self.c.emu_warp_converged(N, active, _p(out)) == 0
        return out


def own_emulator() -> Emu:
    return Emu(_b.build_own_emu())


def reference_emulator() -> Emu | None:
    p = _b.build_ref_emu()
    return Emu(p) if p is not None else None


# ---- harness cubins on the GPU (CUDA driver API) -----------------------------

class Cubin:
    """Loads one of the harness cubins into the current CUDA context."""

    def __init__(self, path: Path, device: int = 0):
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.path = Path(path)
        self._check(self.cu.cuInit(0), "cuInit")
        ctx = ctypes.c_void_p()
        self._check(self.cu.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:  # bind the device's primary context (the one the runtime API uses)
            dev = ctypes.c_int()
            self._check(self.cu.cuDeviceGet(ctypes.byref(dev), device), "cuDeviceGet")
            self._check(self.cu.cuDevicePrimaryCtxRetain(ctypes.byref(ctx), dev), "cuDevicePrimaryCtxRetain")
            self._check(self.cu.cuCtxSetCurrent(ctx), "cuCtxSetCurrent")
        mod = ctypes.c_void_p()
        self._check(self.cu.cuModuleLoad(ctypes.byref(mod), str(self.path).encode()), "cuModuleLoad")
        self.mod = mod
        self._fns = {}

    def _check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUresult {rc} ({self.path.name})")

    def function(self, name: str):
        if name not in self._fns:
            f = ctypes.c_void_p()
            self._check(self.cu.cuModuleGetFunction(ctypes.byref(f), self.mod, name.encode()), name)
            self._fns[name] = f
        return self._fns[name]

    def launch(self, name: str, grid: int, block: int, args, stream: int = 0):
        f = self.function(name)
        holders = list(args)
        params = (ctypes.c_void_p * len(holders))(
            *[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in holders])
        self._check(self.cu.cuLaunchKernel(f, grid, 1, 1, block, 1, 1, 0, ctypes.c_void_p(stream), params, None),
                    f"cuLaunchKernel({name})")


def own_cubin(tile: int = 32) -> Cubin:
    """The harness kernels built against this repository's headers at
    TILE_SIZE `tile`."""
    return Cubin(_b.build_own_cubin(tile))


def reference_cubin(tile: int = 32) -> Cubin | None:
    """The same kernels built against the reference's headers, or None where
    that prebuilt cubin is absent."""
    p = _b.build_ref_cubin(tile)
    return Cubin(p) if p is not None and Path(p).exists() else None
