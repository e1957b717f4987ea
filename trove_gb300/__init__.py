"""trove_gb300 — Python binding of the GB300 AoS load/store library's C ABI.

The library itself is CUDA C++ (trove_gb300/csrc, device API in include/trove,
C ABI in include/trove_gb300.h).  This module only loads
trove_gb300/_lib/libtrove_gb300.so with ctypes and forwards calls; there is no
Python or CPU implementation of any operation, and a missing library is an
error, never a fallback.

Arguments that name memory accept a torch tensor, a numpy array (host memory
only, for copy_host) or a raw integer address.  `n` counts structs and
`width` is the struct size in bytes.  Calls are asynchronous on `stream`
(default: torch's current stream on the current device when torch is loaded,
else the legacy default stream) and raise TroveError on a non-zero status.
"""
from __future__ import annotations

import ctypes
import sys

from . import _build

PATH_AUTO = 0
PATH_WARP = 1
PATH_BLOCK = 2
PATH_VECTOR = 3
PATH_BULK = 4
PATH_DIRECT = 5
PATH_COALESCED = 6

PATHS = {"auto": PATH_AUTO, "warp": PATH_WARP, "block": PATH_BLOCK, "vector": PATH_VECTOR,
         "bulk": PATH_BULK, "direct": PATH_DIRECT, "coalesced": PATH_COALESCED}

TRV_OK = 0


class TroveError(RuntimeError):
    """A C ABI call returned a non-zero trv_status."""

    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        lib = _lib
        text = lib.trv_status_string(status).decode() if lib is not None else str(status)
        msg = f"{where}: {text} (status {status})"
        if detail:
            msg += f"; {detail}"
        super().__init__(msg)


class Launch(ctypes.Structure):
    """trv_launch: optional path / unroll / block / grid choice (0 = choose)."""
    _fields_ = [("path", ctypes.c_int32), ("unroll", ctypes.c_int32),
                ("block_threads", ctypes.c_int32), ("grid_blocks", ctypes.c_int32),
                ("chunk_bytes", ctypes.c_int32)]


_lib = None

_SIGNATURES = {
    "trv_status_string": (ctypes.c_char_p, [ctypes.c_int32]),
    "trv_version": (ctypes.c_int32, []),
    "trv_last_cuda_error": (ctypes.c_int32, []),
    "trv_check_device": (ctypes.c_int32, [ctypes.c_void_p]),
    "trv_copy": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                  ctypes.c_void_p]),
    "trv_copy_ex": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                     ctypes.POINTER(Launch), ctypes.c_void_p]),
    "trv_copy_exit": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                       ctypes.c_uint32, ctypes.c_int32, ctypes.c_void_p]),
    "trv_copy_exit_ex": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                          ctypes.c_uint32, ctypes.POINTER(Launch), ctypes.c_void_p]),
    "trv_gather": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                                    ctypes.c_uint64, ctypes.c_uint32, ctypes.c_void_p]),
    "trv_gather_ex": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                                       ctypes.c_uint64, ctypes.c_uint32, ctypes.POINTER(Launch),
                                       ctypes.c_void_p]),
    "trv_scatter": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_uint64, ctypes.c_uint32, ctypes.c_void_p]),
    "trv_scatter_ex": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_uint64, ctypes.c_uint32, ctypes.POINTER(Launch),
                                        ctypes.c_void_p]),
    "trv_fill_random_u32": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64,
                                             ctypes.c_void_p]),
    "trv_copy_host": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32]),
}


def library_path():
    return _build.LIB


def exported_symbols():
    """Names of the C ABI functions this binding declares."""
    return sorted(_SIGNATURES)


def load(build_if_missing: bool = False):
    """Load libtrove_gb300.so (building it first if asked).  Raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not path.exists():
        if not build_if_missing:
            raise RuntimeError(f"{path} is not built; run __graft_entry__.build() (no CPU fallback exists)")
        _build.build()
    lib = ctypes.CDLL(str(path))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _addr(x) -> int:
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return int(x.data_ptr())
    if hasattr(x, "ctypes"):
        return int(x.ctypes.data)
    raise TypeError(f"cannot take the address of {type(x).__name__}")


def _stream(stream) -> int:
    if stream is None:
        torch = sys.modules.get("torch")
        if torch is not None and torch.cuda.is_available() and torch.cuda.is_initialized():
            return int(torch.cuda.current_stream().cuda_stream)
        return 0
    if isinstance(stream, int):
        return stream
    return int(stream.cuda_stream)


def _check(rc: int, where: str):
    if rc != TRV_OK:
        detail = ""
        if rc == 4:
            detail = f"cudaError {load().trv_last_cuda_error()}"
        raise TroveError(rc, where, detail)


def _launch(path, unroll, block, grid, chunk=0):
    if isinstance(path, str):
        path = PATHS[path]
    if not (path or unroll or block or grid or chunk):
        return None
    return ctypes.byref(Launch(int(path), int(unroll), int(block), int(grid), int(chunk)))


def copy(dst, src, n: int, width: int, *, path=PATH_AUTO, unroll: int = 0, block: int = 0, grid: int = 0,
         chunk: int = 0, stream=None):
    """dst[i] = src[i] for n structs of `width` bytes (trv_copy_ex)."""
    lib = load()
    _check(lib.trv_copy_ex(_addr(dst), _addr(src), n, width, _launch(path, unroll, block, grid, chunk),
                           _stream(stream)), "trv_copy")


def check_device(stream=None):
    """Synchronize and raise if a kernel's bounded wait gave up."""
    _check(load().trv_check_device(_stream(stream)), "trv_check_device")


def copy_exit(dst, src, n: int, width: int, modulus: int, *, path=PATH_WARP, unroll: int = 0, grid: int = 0,
              stream=None):
    """Copy skipping structs whose first word w has w % modulus == modulus - 1."""
    if isinstance(path, str):
        path = PATHS[path]
    cfg = Launch(int(path), int(unroll), 0, int(grid), 0)
    _check(load().trv_copy_exit_ex(_addr(dst), _addr(src), n, width, modulus, ctypes.byref(cfg), _stream(stream)),
           "trv_copy_exit")


def gather(dst, src, src_n: int, idx, n: int, width: int, *, path=PATH_AUTO, unroll: int = 0, block: int = 0,
           grid: int = 0, stream=None):
    """dst[i] = src[idx[i]] (trv_gather_ex); out-of-range indices are skipped."""
    _check(load().trv_gather_ex(_addr(dst), _addr(src), src_n, _addr(idx), n, width,
                                _launch(path, unroll, block, grid), _stream(stream)), "trv_gather")


def scatter(dst, dst_n: int, src, idx, n: int, width: int, *, path=PATH_AUTO, unroll: int = 0, block: int = 0,
            grid: int = 0, stream=None):
    """dst[idx[i]] = src[i] (trv_scatter_ex); out-of-range indices are skipped."""
    _check(load().trv_scatter_ex(_addr(dst), dst_n, _addr(src), _addr(idx), n, width,
                                 _launch(path, unroll, block, grid), _stream(stream)), "trv_scatter")


def fill_random_u32(dst, nwords: int, seed: int, *, stream=None):
    """dst[k] = word k of the seeded splitmix64 stream."""
    _check(load().trv_fill_random_u32(_addr(dst), nwords, seed, _stream(stream)), "trv_fill_random_u32")


def copy_host(dst_host, src_host, n: int, width: int):
    """Host-buffer copy through the device; returns when dst_host is written."""
    _check(load().trv_copy_host(_addr(dst_host), _addr(src_host), n, width), "trv_copy_host")
