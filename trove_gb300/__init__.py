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
                ("chunk_bytes", ctypes.c_int32), ("cache_policy", ctypes.c_int32)]


OP_COPY = 0
OP_GATHER = 1
OP_SCATTER = 2
OP_COPY_EXIT_WARP = 3   # autotuner keys of the early-exit copy
OP_COPY_EXIT_BLOCK = 4
OP_AOS_TO_SOA = 5       # autotuner keys of the layout conversions
OP_SOA_TO_AOS = 6
SCOPE_CALL = 0
SCOPE_BATCH = 1


class Task(ctypes.Structure):
    """trv_task: one array of a batch."""
    _fields_ = [("op", ctypes.c_int32), ("width", ctypes.c_uint32), ("n", ctypes.c_uint64),
                ("src", ctypes.c_void_p), ("dst", ctypes.c_void_p), ("idx", ctypes.c_void_p),
                ("bound", ctypes.c_uint64)]


class BatchOptions(ctypes.Structure):
    _fields_ = [("tile_bytes", ctypes.c_int32), ("copy_path", ctypes.c_int32), ("grid_blocks", ctypes.c_int32),
                ("blocks_per_sm", ctypes.c_int32), ("gather_policy", ctypes.c_int32),
                ("scatter_policy", ctypes.c_int32)]


_lib = None

_SIGNATURES = {
    "trv_status_string": (ctypes.c_char_p, [ctypes.c_int32]),
    "trv_version": (ctypes.c_int32, []),
    "trv_last_cuda_error": (ctypes.c_int32, []),
    "trv_check_device": (ctypes.c_int32, [ctypes.c_void_p]),
    "trv_debug_set_bulk_wait_polls": (ctypes.c_int32, [ctypes.c_uint32]),
    "trv_set_l2_fetch_granularity": (ctypes.c_int32, [ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]),
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
    "trv_aos_to_soa": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                        ctypes.c_void_p]),
    "trv_soa_to_aos": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                        ctypes.c_void_p]),
    "trv_aos_to_soa_ex": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                           ctypes.POINTER(Launch), ctypes.c_void_p]),
    "trv_soa_to_aos_ex": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                           ctypes.POINTER(Launch), ctypes.c_void_p]),
    "trv_fill_uniform_indices": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64,
                                                  ctypes.c_void_p]),
    "trv_fill_run_indices": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p]),
    "trv_fill_permutation": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p]),
    "trv_copy_host": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32]),
    "trv_batch_create": (ctypes.c_int32, [ctypes.POINTER(Task), ctypes.c_uint64, ctypes.POINTER(BatchOptions),
                                          ctypes.POINTER(ctypes.c_void_p)]),
    "trv_batch_launch": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p]),
    "trv_batch_capture": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p]),
    "trv_batch_info": (ctypes.c_int32, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64),
                                        ctypes.POINTER(ctypes.c_uint64)]),
    "trv_batch_destroy": (ctypes.c_int32, [ctypes.c_void_p]),
    "trv_run_per_call": (ctypes.c_int32, [ctypes.POINTER(Task), ctypes.c_uint64, ctypes.c_void_p]),
    "trv_probe_block_gather": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                                                ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int32,
                                                ctypes.c_void_p]),
    "trv_batch_run_static": (ctypes.c_int32, [ctypes.POINTER(Task), ctypes.c_uint64, ctypes.POINTER(BatchOptions),
                                              ctypes.c_void_p]),
    "trv_autotune_call": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_void_p]),
    "trv_autotune_batch": (ctypes.c_int32, [ctypes.POINTER(Task), ctypes.c_uint64, ctypes.c_void_p]),
    "trv_autotune_lookup": (ctypes.c_int32, [ctypes.c_int32, ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint64,
                                             ctypes.POINTER(Launch), ctypes.POINTER(ctypes.c_int32)]),
    "trv_autotune_clear": (ctypes.c_int32, []),
    "trv_autotune_save": (ctypes.c_int32, [ctypes.c_char_p]),
    "trv_autotune_load": (ctypes.c_int32, [ctypes.c_char_p]),
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


def _launch(path, unroll, block, grid, chunk=0, policy=0):
    if isinstance(path, str):
        path = PATHS[path]
    if not (path or unroll or block or grid or chunk or policy):
        return None
    return ctypes.byref(Launch(int(path), int(unroll), int(block), int(grid), int(chunk), int(policy)))


def copy(dst, src, n: int, width: int, *, path=PATH_AUTO, unroll: int = 0, block: int = 0, grid: int = 0,
         chunk: int = 0, stream=None):
    """dst[i] = src[i] for n structs of `width` bytes (trv_copy_ex)."""
    lib = load()
    _check(lib.trv_copy_ex(_addr(dst), _addr(src), n, width, _launch(path, unroll, block, grid, chunk),
                           _stream(stream)), "trv_copy")


def set_l2_fetch_granularity(nbytes: int) -> int:
    """Set the context's L2 fetch granularity hint (32, 64 or 128 bytes);
    returns the previous value."""
    prev = ctypes.c_int32()
    _check(load().trv_set_l2_fetch_granularity(int(nbytes), ctypes.byref(prev)), "trv_set_l2_fetch_granularity")
    return prev.value


def debug_set_bulk_wait_polls(polls: int):
    """Testing hook: poll budget of the bulk copy's waits (0xFFFFFFFF: default)."""
    _check(load().trv_debug_set_bulk_wait_polls(polls & 0xFFFFFFFF), "trv_debug_set_bulk_wait_polls")


def check_device(stream=None):
    """Synchronize and raise if a kernel's bounded wait gave up."""
    _check(load().trv_check_device(_stream(stream)), "trv_check_device")


def copy_exit(dst, src, n: int, width: int, modulus: int, *, path=PATH_WARP, unroll: int = 0, grid: int = 0,
              stream=None):
    """Copy skipping structs whose first word w has w % modulus == modulus - 1."""
    if isinstance(path, str):
        path = PATHS[path]
    cfg = Launch(int(path), int(unroll), 0, int(grid), 0, 0)
    _check(load().trv_copy_exit_ex(_addr(dst), _addr(src), n, width, modulus, ctypes.byref(cfg), _stream(stream)),
           "trv_copy_exit")


def gather(dst, src, src_n: int, idx, n: int, width: int, *, path=PATH_AUTO, unroll: int = 0, block: int = 0,
           grid: int = 0, policy: int = 0, stream=None):
    """dst[i] = src[idx[i]] (trv_gather_ex); out-of-range indices are skipped."""
    _check(load().trv_gather_ex(_addr(dst), _addr(src), src_n, _addr(idx), n, width,
                                _launch(path, unroll, block, grid, 0, policy), _stream(stream)), "trv_gather")


def scatter(dst, dst_n: int, src, idx, n: int, width: int, *, path=PATH_AUTO, unroll: int = 0, block: int = 0,
            grid: int = 0, policy: int = 0, stream=None):
    """dst[idx[i]] = src[i] (trv_scatter_ex); out-of-range indices are skipped."""
    _check(load().trv_scatter_ex(_addr(dst), dst_n, _addr(src), _addr(idx), n, width,
                                 _launch(path, unroll, block, grid, 0, policy), _stream(stream)), "trv_scatter")


def probe_block_gather(dst, src, src_n: int, idx, n: int, width: int, block_bytes: int, l2_hint: int = 0, *,
                       stream=None):
    """Reads the block_bytes-aligned blocks every row src[idx[i]] overlaps, the
    indices, and writes n * width bytes (trv_probe_block_gather): the memory
    system's ceiling for a gather of those rows."""
    _check(load().trv_probe_block_gather(_addr(dst), _addr(src), src_n, _addr(idx), n, width, block_bytes,
                                         l2_hint, _stream(stream)), "trv_probe_block_gather")


def fill_random_u32(dst, nwords: int, seed: int, *, stream=None):
    """dst[k] = word k of the seeded splitmix64 stream."""
    _check(load().trv_fill_random_u32(_addr(dst), nwords, seed, _stream(stream)), "trv_fill_random_u32")


def aos_to_soa(dst_soa, src_aos, n: int, width: int, *, unroll: int = 0, grid: int = 0, stream=None):
    """soa[j * n + i] = field j of struct i (32-bit fields)."""
    cfg = Launch(0, int(unroll), 0, int(grid), 0, 0)
    _check(load().trv_aos_to_soa_ex(_addr(dst_soa), _addr(src_aos), n, width, ctypes.byref(cfg), _stream(stream)),
           "trv_aos_to_soa")


def soa_to_aos(dst_aos, src_soa, n: int, width: int, *, unroll: int = 0, grid: int = 0, stream=None):
    """Field j of struct i = soa[j * n + i] (32-bit fields)."""
    cfg = Launch(0, int(unroll), 0, int(grid), 0, 0)
    _check(load().trv_soa_to_aos_ex(_addr(dst_aos), _addr(src_soa), n, width, ctypes.byref(cfg), _stream(stream)),
           "trv_soa_to_aos")


def fill_uniform_indices(idx, n: int, bound: int, seed: int, *, stream=None):
    """idx[i] uniform in [0, bound) from the seeded stream (same as the oracle)."""
    _check(load().trv_fill_uniform_indices(_addr(idx), n, bound, seed, _stream(stream)), "trv_fill_uniform_indices")


def fill_run_indices(idx, n: int, seed: int, *, stream=None):
    """Run pattern: per aligned chunk of 32, a run (p = 1/2) or 32 uniform draws."""
    _check(load().trv_fill_run_indices(_addr(idx), n, seed, _stream(stream)), "trv_fill_run_indices")


def fill_permutation(idx, n: int, seed: int, *, stream=None):
    """Seeded Fisher-Yates permutation of 0..n-1 (host-generated, copied in)."""
    _check(load().trv_fill_permutation(_addr(idx), n, seed, _stream(stream)), "trv_fill_permutation")


def copy_host(dst_host, src_host, n: int, width: int):
    """Host-buffer copy; returns when dst_host is written."""
    _check(load().trv_copy_host(_addr(dst_host), _addr(src_host), n, width), "trv_copy_host")


# ---- batched execution -------------------------------------------------------

def make_tasks(tasks) -> "ctypes.Array":
    """Task array from Task objects or dicts with keys op, width, n, src, dst,
    idx, bound (addresses may be tensors)."""
    arr = (Task * len(tasks))()
    for k, t in enumerate(tasks):
        if isinstance(t, Task):
            arr[k] = t
            continue
        arr[k] = Task(int(t["op"]), int(t["width"]), int(t["n"]), _addr(t["src"]), _addr(t["dst"]),
                      _addr(t.get("idx")), int(t.get("bound", 0)))
    return arr


class Batch:
    """A planned batch (trv_batch): launch() runs every task in one
    persistent kernel; capture() records it as a CUDA graph first."""

    def __init__(self, tasks, *, tile_bytes: int = 0, copy_path=PATH_AUTO, grid: int = 0, blocks_per_sm: int = 0,
                 gather_policy: int = 0, scatter_policy: int = 0):
        if isinstance(copy_path, str):
            copy_path = PATHS[copy_path]
        self._tasks = make_tasks(tasks)
        opt = BatchOptions(int(tile_bytes), int(copy_path), int(grid), int(blocks_per_sm), int(gather_policy),
                           int(scatter_policy))
        h = ctypes.c_void_p()
        _check(load().trv_batch_create(self._tasks, len(self._tasks), ctypes.byref(opt), ctypes.byref(h)),
               "trv_batch_create")
        self._h = h

    def launch(self, stream=None):
        _check(load().trv_batch_launch(self._h, _stream(stream)), "trv_batch_launch")

    def capture(self, stream):
        _check(load().trv_batch_capture(self._h, _stream(stream)), "trv_batch_capture")

    def info(self):
        tiles, nbytes = ctypes.c_uint64(), ctypes.c_uint64()
        _check(load().trv_batch_info(self._h, ctypes.byref(tiles), ctypes.byref(nbytes)), "trv_batch_info")
        return tiles.value, nbytes.value

    def close(self):
        if self._h:
            _check(load().trv_batch_destroy(self._h), "trv_batch_destroy")
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


STATIC_BATCH_MAX_TASKS = 4096


def run_static(tasks, *, tile_bytes: int = 0, grid: int = 0, blocks_per_sm: int = 0, gather_policy: int = 0,
               scatter_policy: int = 0, stream=None):
    """Plan and run a batch in one call without allocating device memory
    (trv_batch_run_static), for callers that must not call cudaMalloc: it
    synchronizes the whole device, and a process whose device memory is
    reserved up front by another allocator may have none to spare.  Uses one
    library-owned device array of at most STATIC_BATCH_MAX_TASKS task entries,
    shared by every call on the device: calls whose work overlaps on the GPU
    race and must be ordered by the caller."""
    arr = make_tasks(tasks)
    opt = BatchOptions(int(tile_bytes), PATH_AUTO, int(grid), int(blocks_per_sm), int(gather_policy),
                       int(scatter_policy))
    _check(load().trv_batch_run_static(arr, len(arr), ctypes.byref(opt), _stream(stream)), "trv_batch_run_static")


def run_per_call(tasks, stream=None):
    """One plain launch per task (the batch's baseline)."""
    arr = make_tasks(tasks)
    _check(load().trv_run_per_call(arr, len(arr), _stream(stream)), "trv_run_per_call")


# ---- autotuner ----------------------------------------------------------------

def autotune_call(op: int, width: int, n: int, stream=None):
    _check(load().trv_autotune_call(op, width, n, _stream(stream)), "trv_autotune_call")


def autotune_batch(tasks, stream=None):
    arr = make_tasks(tasks)
    _check(load().trv_autotune_batch(arr, len(arr), _stream(stream)), "trv_autotune_batch")


def autotune_lookup(scope: int, op: int, width: int, n: int):
    """(Launch, tile_bytes) cached for the key, or None."""
    out, tile = Launch(), ctypes.c_int32()
    rc = load().trv_autotune_lookup(scope, op, width, n, ctypes.byref(out), ctypes.byref(tile))
    if rc == 8:
        return None
    _check(rc, "trv_autotune_lookup")
    return out, tile.value


def autotune_clear():
    _check(load().trv_autotune_clear(), "trv_autotune_clear")


def autotune_save(path):
    _check(load().trv_autotune_save(str(path).encode()), "trv_autotune_save")


def autotune_load(path):
    _check(load().trv_autotune_load(str(path).encode()), "trv_autotune_load")


# ---- serving ------------------------------------------------------------------------

class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_inflight", ctypes.c_int32),
                ("max_batch_requests", ctypes.c_int32), ("tile_bytes", ctypes.c_int32),
                ("release_when_done", ctypes.c_int32)]


class Request(ctypes.Structure):
    _fields_ = [("op", ctypes.c_int32), ("width", ctypes.c_uint32), ("n", ctypes.c_uint64),
                ("src", ctypes.c_void_p), ("src_n", ctypes.c_uint64), ("idx", ctypes.c_void_p)]


class Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("batch", ctypes.c_int32), ("dst", ctypes.c_void_p),
                ("submit_ms", ctypes.c_double), ("launch_ms", ctypes.c_double), ("done_ms", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_uint64) for k in ("submitted", "admitted", "completed", "rejected", "batches",
                                               "max_queued", "bytes", "budget_in_use")] + \
               [(k, ctypes.c_double) for k in ("p50_ms", "p99_ms", "mean_ms", "max_ms", "first_submit_ms",
                                               "last_done_ms")]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


_SIGNATURES.update({
    "trv_server_create": (ctypes.c_int32, [ctypes.POINTER(ServerConfig), ctypes.POINTER(ctypes.c_void_p)]),
    "trv_server_submit": (ctypes.c_int32, [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_uint64)]),
    "trv_server_poll": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint64, ctypes.POINTER(Result)]),
    "trv_server_wait": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double, ctypes.POINTER(Result)]),
    "trv_server_release": (ctypes.c_int32, [ctypes.c_void_p, ctypes.c_uint64]),
    "trv_server_stats_get": (ctypes.c_int32, [ctypes.c_void_p, ctypes.POINTER(ServerStats)]),
    "trv_server_replay": (ctypes.c_int32, [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_double),
                                           ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64),
                                           ctypes.POINTER(ServerStats)]),
    "trv_server_destroy": (ctypes.c_int32, [ctypes.c_void_p]),
})


def make_request(r) -> Request:
    if isinstance(r, Request):
        return r
    return Request(int(r["op"]), int(r["width"]), int(r["n"]), _addr(r["src"]), int(r.get("src_n", 0)),
                   _addr(r.get("idx")))


class Server:
    """trv_server: admission against an HBM budget, continuous batching into
    the persistent kernel, per-request latency."""

    def __init__(self, budget_bytes: int, *, max_inflight: int = 0, max_batch_requests: int = 0,
                 tile_bytes: int = 0, release_when_done: bool = False):
        cfg = ServerConfig(int(budget_bytes), int(max_inflight), int(max_batch_requests), int(tile_bytes),
                           1 if release_when_done else 0)
        h = ctypes.c_void_p()
        _check(load().trv_server_create(ctypes.byref(cfg), ctypes.byref(h)), "trv_server_create")
        self._h = h

    def submit(self, req) -> int:
        rid = ctypes.c_uint64()
        _check(load().trv_server_submit(self._h, ctypes.byref(make_request(req)), ctypes.byref(rid)),
               "trv_server_submit")
        return rid.value

    def poll(self, rid: int):
        res = Result()
        rc = load().trv_server_poll(self._h, rid, ctypes.byref(res))
        if rc == 9:
            return None
        _check(rc, "trv_server_poll")
        return res

    def wait(self, rid: int, timeout_ms: float = 60000.0) -> Result:
        res = Result()
        _check(load().trv_server_wait(self._h, rid, timeout_ms, ctypes.byref(res)), "trv_server_wait")
        return res

    def release(self, rid: int):
        _check(load().trv_server_release(self._h, rid), "trv_server_release")

    def stats(self) -> dict:
        st = ServerStats()
        _check(load().trv_server_stats_get(self._h, ctypes.byref(st)), "trv_server_stats")
        return st.as_dict()

    def replay(self, requests, arrival_ms):
        """Open-loop replay; returns (ids, stats dict) for these requests."""
        n = len(requests)
        arr = (Request * n)(*[make_request(r) for r in requests])
        times = (ctypes.c_double * n)(*[float(t) for t in arrival_ms])
        ids = (ctypes.c_uint64 * n)()
        st = ServerStats()
        _check(load().trv_server_replay(self._h, arr, times, n, ids, ctypes.byref(st)), "trv_server_replay")
        return list(ids), st.as_dict()

    def close(self):
        if self._h:
            h, self._h = self._h, None
            _check(load().trv_server_destroy(h), "trv_server_destroy")

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
