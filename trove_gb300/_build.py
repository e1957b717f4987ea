"""Build recipe of the CUDA library (sm_103a only).

Compiles trove_gb300/csrc into trove_gb300/_lib/libtrove_gb300.so with nvcc:
one object per struct width for the template-heavy kernels (so the build runs
in parallel), then one shared-library link.  Rebuilds only when a source,
header or flag changed.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "trove_gb300" / "csrc"
INCLUDE = ROOT / "include"
OUT_DIR = ROOT / "trove_gb300" / "_lib"
OBJ_DIR = ROOT / "trove_gb300" / "_lib" / "obj"
LIB = OUT_DIR / "libtrove_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-O2", *ARCH,
              f"-I{INCLUDE}", f"-I{CSRC}"]
WIDTHS = range(1, 17)


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the trove_gb300 CUDA library cannot be built")


def _units():
    """(object name, source, extra flags) for every translation unit."""
    units = [(f"width_ops_{s:02d}.o", CSRC / "width_ops.cu", [f"-DTRV_WIDTH={s}"]) for s in WIDTHS]
    for src in sorted(CSRC.glob("*.cu")):
        if src.name != "width_ops.cu":
            units.append((src.stem + ".o", src, []))
    for src in sorted(CSRC.glob("*.cpp")):
        units.append((src.stem + ".o", src, ["-x", "cu"]))
    return units


def _fingerprint() -> str:
    h = hashlib.sha256()
    for p in sorted([*CSRC.rglob("*"), *INCLUDE.rglob("*")]):
        if p.is_file():
            h.update(str(p.relative_to(ROOT)).encode())
            h.update(p.read_bytes())
    h.update(" ".join(NVCC_FLAGS).encode())
    return h.hexdigest()


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Build (if stale) and return the path of libtrove_gb300.so."""
    stamp = OUT_DIR / ".fingerprint"
    fp = _fingerprint()
    if LIB.exists() and stamp.exists() and stamp.read_text() == fp:
        return LIB
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    cc = nvcc()
    units = _units()
    jobs = jobs or max(1, min(len(units), os.cpu_count() or 4))

    def compile_one(unit):
        obj, src, extra = unit
        cmd = [cc, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(OBJ_DIR / obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(compile_one, units))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *[str(OBJ_DIR / o) for o in objs]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    stamp.write_text(fp)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
