"""C ABI: the library loads, exports every function include/trove_gb300.h
declares, and rejects bad arguments before touching the GPU.  CPU only: no
call here reaches a kernel launch."""
import ctypes
import re
from pathlib import Path

import pytest

import trove_gb300 as tg

HEADER = Path(__file__).resolve().parent.parent / "include" / "trove_gb300.h"


def declared():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:const char\*|int32_t)\s+(trv_\w+)\(", text, re.M)))


def test_header_declares_the_binding(trove_lib):
    assert declared() == tg.exported_symbols()


def test_library_exports_every_declared_symbol(trove_lib):
    for name in declared():
        assert hasattr(trove_lib, name), name


def test_status_strings(trove_lib):
    assert trove_lib.trv_status_string(0) == b"ok"
    assert b"invalid" in trove_lib.trv_status_string(1)
    assert trove_lib.trv_status_string(999) == b"unknown status"
    assert trove_lib.trv_version() >= 100


def rc_of(fn):
    try:
        fn()
    except tg.TroveError as e:
        return e.status
    return 0


def test_argument_errors_need_no_gpu(trove_lib):
    bad = 0x1002  # non-null, not 4-byte aligned; never dereferenced
    ok = 0x100000
    # n == 0 is a no-op
    assert rc_of(lambda: tg.copy(0, 0, 0, 12)) == 0
    assert rc_of(lambda: tg.gather(0, 0, 0, 0, 0, 12)) == 0
    # null pointers / zero width / overflow
    assert rc_of(lambda: tg.copy(0, ok, 5, 12)) == 1
    assert rc_of(lambda: tg.copy(ok, ok, 5, 0)) == 1
    assert rc_of(lambda: tg.copy(ok, ok, 1 << 62, 16)) == 1
    assert rc_of(lambda: tg.gather(ok, ok, 10, 0, 5, 12)) == 1
    assert rc_of(lambda: tg.scatter(ok, 10, ok, 0, 5, 12)) == 1
    # struct paths need 4-byte multiples up to 64 bytes, and 4-byte alignment
    assert rc_of(lambda: tg.copy(ok, ok, 5, 12, path="warp", unroll=3)) == 1
    assert rc_of(lambda: tg.copy(ok, ok, 5, 13, path="warp")) == 2
    assert rc_of(lambda: tg.copy(ok, ok, 5, 68, path="block")) == 2
    assert rc_of(lambda: tg.copy(bad, ok, 5, 12, path="warp")) == 3
    assert rc_of(lambda: tg.copy_exit(ok, bad, 5, 12, 625, path="block")) == 3
    assert rc_of(lambda: tg.copy_exit(ok, ok, 5, 12, 625, path="vector")) == 2
    assert rc_of(lambda: tg.gather(ok, ok, 10, bad, 5, 12)) == 3
    assert rc_of(lambda: tg.gather(ok, ok, 10, ok, 5, 12, path="bulk")) == 2
    assert rc_of(lambda: tg.scatter(ok, 10, ok, ok, 5, 12, path="block")) == 2
    assert rc_of(lambda: tg.copy_exit(ok, ok, 5, 12, 625, path="warp", unroll=5)) == 1
    assert rc_of(lambda: tg.copy(ok, ok, 5, 12, block=128)) == 2
    # TMA bulk chunks: multiples of 16 whose 4-stage ring fits shared memory
    assert rc_of(lambda: tg.copy(ok, ok, 5, 12, path="bulk", chunk=24)) == 1
    assert rc_of(lambda: tg.copy(ok, ok, 5, 12, path="bulk", chunk=64 << 10)) == 1
    assert rc_of(lambda: tg.copy(ok, ok, 5, 12, path="bulk", chunk=1 << 30)) == 1
    assert rc_of(lambda: tg.fill_random_u32(0, 5, 1)) == 1
    assert rc_of(lambda: tg.copy_host(0, ok, 5, 4)) == 1
    assert rc_of(lambda: tg.aos_to_soa(ok, ok, 5, 68)) == 2
    assert rc_of(lambda: tg.soa_to_aos(ok, bad, 5, 12)) == 3
    assert rc_of(lambda: tg.aos_to_soa(0, ok, 5, 12)) == 1
    assert rc_of(lambda: tg.set_l2_fetch_granularity(48)) == 1
    # layout _ex forms, seeded index generators
    assert rc_of(lambda: tg.aos_to_soa(ok, ok, 0, 12, unroll=3)) == 0  # n == 0 first
    assert rc_of(lambda: tg.aos_to_soa(ok, ok, 5, 12, unroll=3)) == 1
    assert rc_of(lambda: tg.fill_run_indices(ok, 31, 0)) == 1  # runs need n >= 32
    assert rc_of(lambda: tg.fill_run_indices(bad, 64, 0)) == 3
    assert rc_of(lambda: tg.fill_run_indices(ok, 1 << 31, 0)) == 1
    assert rc_of(lambda: tg.fill_permutation(0, 5, 0)) == 1
    assert rc_of(lambda: tg.fill_permutation(bad, 5, 0)) == 3
    assert rc_of(lambda: tg.fill_permutation(ok, 0, 0)) == 0
    assert rc_of(lambda: tg.gather(ok, ok, 10, ok, 5, 12, path="warp", policy=6)) == 1
    # the random-block probe: n a multiple of 32, 4-byte widths up to 128,
    # block sizes 32 / 64 / 128, hints none / 64 / 128, block-aligned source
    assert rc_of(lambda: tg.probe_block_gather(ok, ok, 64, ok, 0, 12, 64)) == 0
    assert rc_of(lambda: tg.probe_block_gather(ok, ok, 64, ok, 48, 12, 64)) == 1
    assert rc_of(lambda: tg.probe_block_gather(ok, ok, 64, ok, 64, 14, 64)) == 1
    assert rc_of(lambda: tg.probe_block_gather(ok, ok, 64, ok, 64, 132, 64)) == 1
    assert rc_of(lambda: tg.probe_block_gather(ok, ok, 64, 0, 64, 12, 64)) == 1
    assert rc_of(lambda: tg.probe_block_gather(ok, ok, 64, ok, 64, 12, 16)) == 2
    assert rc_of(lambda: tg.probe_block_gather(ok, ok, 64, ok, 64, 12, 64, 32)) == 2
    assert rc_of(lambda: tg.probe_block_gather(ok, ok + 32, 64, ok, 64, 12, 64)) == 3
    assert rc_of(lambda: tg.probe_block_gather(ok + 8, ok, 64, ok, 64, 12, 64)) == 3


def test_error_carries_status_text(trove_lib):
    with pytest.raises(tg.TroveError, match="invalid argument"):
        tg.copy(0, 0x100000, 5, 12)


def test_missing_library_is_an_error(monkeypatch, tmp_path):
    import importlib
    mod = importlib.reload(tg)
    monkeypatch.setattr(mod._build, "LIB", tmp_path / "absent.so")
    with pytest.raises(RuntimeError, match="not built"):
        mod.load()
    importlib.reload(tg)


def test_header_is_plain_c(trove_lib, tmp_path):
    """The boundary header compiles as C11 with every warning an error, and a
    C program using it links against the library (no C++ in the ABI)."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not found")
    prog = tmp_path / "use.c"
    prog.write_text(
        "#include <trove_gb300.h>\n"
        "int main(void) {\n"
        "    trv_launch cfg = {TRV_PATH_AUTO, 0, 0, 0, 0, 0};\n"
        "    trv_task t = {TRV_OP_COPY, 12, 0, 0, 0, 0, 0};\n"
        "    trv_batch* b = 0;\n"
        "    (void)trv_batch_create(&t, 0, 0, &b);\n"
        "    return trv_copy_ex(0, 0, 0, 12, &cfg, 0) == TRV_OK ? 0 : 1;\n"
        "}\n")
    lib = tg.library_path()
    r = subprocess.run([gcc, "-std=c11", "-Wall", "-Wextra", "-Werror", f"-I{HEADER.parent}", str(prog),
                        f"-L{lib.parent}", "-ltrove_gb300", "-o", str(tmp_path / "use")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
