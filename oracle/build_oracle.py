"""Build recipe of the oracle — TEST INFRASTRUCTURE ONLY.

Outputs (all git-ignored):
  oracle/_build/libaos_oracle.so        gcc: the C restatement (aos_oracle.c)
  oracle/_build/libtrove_emu.so         g++: emu/api_cases.cpp on this repo's
                                        include/ under the host lane emulator
  oracle/_build/trove_own_kernels.cubin nvcc: trove_bench_kernels.cu on include/
                                        (TILE_SIZE 32; _t16/_t8/_t4/_t2 for
                                        the other tile sizes)
  oracle/_ref/libtrove_ref_emu.so       g++: emu/api_cases.cpp on the
                                        reference's headers, in place
  oracle/_ref/trove_ref_kernels.cubin   nvcc: trove_bench_kernels.cu on the
                                        reference's headers, in place (and
                                        _t16/_t8/_t4/_t2)
The two oracle/_ref outputs need the reference checkout, which exists only
where the repository is developed; on a GPU machine the prebuilt cubin is
used as shipped.  The reference's own build system is never run: its headers
are compiled directly from where they lie, with the shims in oracle/emu
standing in for cooperative_groups and thrust on the host.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
# The reference checkout sits beside this repository unless TROVE_REFERENCE names it.
REFERENCE = Path(os.environ.get("TROVE_REFERENCE", str(ROOT.parent / "reference")))
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

ORACLE_LIB = BUILD / "libaos_oracle.so"
OWN_EMU = BUILD / "libtrove_emu.so"
OWN_CUBIN = BUILD / "trove_own_kernels.cubin"
REF_EMU = REF_OUT / "libtrove_ref_emu.so"
REF_CUBIN = REF_OUT / "trove_ref_kernels.cubin"
# TILE_SIZE values of the harness cubins (the reference's tests/Makefile knob)
TILES = (32, 16, 8, 4, 2)


def _tiled(path: Path, tile: int) -> Path:
    return path if tile == 32 else path.with_name(f"{path.stem}_t{tile}{path.suffix}")


def _stale(out: Path, *deps: Path) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    for d in deps:
        files = [d] if d.is_file() else [p for p in d.rglob("*") if p.is_file()]
        if any(f.stat().st_mtime > t for f in files):
            return True
    return False


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    return None


def build_oracle_lib() -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    src = HERE / "aos_oracle.c"
    if _stale(ORACLE_LIB, src):
        tmp = ORACLE_LIB.with_suffix(".tmp")
        _run(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-pthread", str(src), "-o", str(tmp)])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def _emu_cmd(include_args, out):
    return ["g++", "-std=c++20", "-O1", "-fPIC", "-shared", "-pthread", "-include",
            str(HERE / "emu" / "lane_emu.h"), *include_args, str(HERE / "emu" / "api_cases.cpp"), "-o", str(out)]


def build_own_emu() -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    if _stale(OWN_EMU, HERE / "emu", ROOT / "include" / "trove"):
        tmp = OWN_EMU.with_suffix(".tmp")
        _run(_emu_cmd([f"-I{ROOT / 'include'}"], tmp))
        os.replace(tmp, OWN_EMU)
    return OWN_EMU


def reference_present() -> bool:
    return (REFERENCE / "trove" / "aos.h").is_file()


def build_ref_emu() -> Path | None:
    if not reference_present():
        return REF_EMU if REF_EMU.exists() else None
    REF_OUT.mkdir(parents=True, exist_ok=True)
    if _stale(REF_EMU, HERE / "emu", REFERENCE / "trove"):
        tmp = REF_EMU.with_suffix(".tmp")
        _run(_emu_cmd([f"-I{HERE / 'emu'}", f"-I{REFERENCE}"], tmp))
        os.replace(tmp, REF_EMU)
    return REF_EMU


def _cubin(include_dir: Path, out: Path, deps, tile: int, defines=()):
    nvcc = _nvcc()
    if nvcc is None:
        return None
    out.parent.mkdir(parents=True, exist_ok=True)
    if _stale(out, HERE / "trove_bench_kernels.cu", HERE / "build_oracle.py", *deps):
        tmp = out.with_suffix(".tmp")
        _run([nvcc, "-std=c++17", "-cubin", *ARCH, "-O3", "-lineinfo", f"-DTILE_SIZE={tile}", *defines,
              f"-I{include_dir}", str(HERE / "trove_bench_kernels.cu"), "-o", str(tmp)])
        os.replace(tmp, out)
    return out


def build_own_cubin(tile: int = 32):
    return _cubin(ROOT / "include", _tiled(OWN_CUBIN, tile), [ROOT / "include" / "trove"], tile,
                  defines=("-DTRV_OWN_TREE",))


def build_ref_cubin(tile: int = 32):
    out = _tiled(REF_CUBIN, tile)
    if not reference_present():
        return out if out.exists() else None
    return _cubin(REFERENCE, out, [REFERENCE / "trove"], tile)


def build(emulators: bool = False):
    """Build the C oracle and the GPU harness cubins (every tile size, both
    header trees; the reference's only where its checkout exists); the
    host-emulator libraries only when `emulators` (the CPU test suite builds
    those on demand)."""
    jobs = [build_oracle_lib]
    for t in TILES:
        jobs += [lambda t=t: build_own_cubin(t), lambda t=t: build_ref_cubin(t)]
    if emulators:
        jobs += [build_own_emu, build_ref_emu]
    with ThreadPoolExecutor(len(jobs)) as ex:
        return [f.result() for f in [ex.submit(j) for j in jobs]]


if __name__ == "__main__":
    for p in build(emulators=True):
        print(p)
