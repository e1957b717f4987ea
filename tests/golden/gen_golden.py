"""Generate the golden fixtures from the reference's own code.

Runs the reference's trove headers (compiled in place by
oracle/build_oracle.py against the host lane emulator, oracle/emu) on seeded
inputs and records what they produce:
  transposes.npz  r2c/c2r outputs for every tile size and element count,
                  rotate() outputs (structured data, stored in full);
  golden.json     for every other case (including trove/memory.h's
                  warp_load / warp_store / uncoalesced_store): the inputs'
                  recipe (seeds, sizes, index pattern) and the SHA-256 of
                  the reference's output bytes, plus small outputs in full.
Needs the reference checkout, so it runs where the repository is developed;
the fixtures are committed and the tests only read them.

    python tests/golden/gen_golden.py
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

import oracle  # noqa: E402

WIDTHS = [1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 20, 24, 33]
TILES = [32, 16, 8, 4, 2]


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def transpose_inputs(n: int, m: int, words: int):
    rows = np.zeros((n, m, words), np.int32)
    cols = np.zeros((n, m, words), np.int32)
    for L in range(n):
        for k in range(m):
            rows[L, k, :] = (k * n + L) * 16 + np.arange(words)
    for l in range(n):
        for j in range(m):
            cols[l, j, :] = (l * m + j) * 16 + np.arange(words)
    return rows, cols


def transpose_cases():
    for n in TILES:
        for m in range(2, n + 1):
            for words in ([1, 2, 4] if n == 32 and m <= 8 else [1]):
                yield n, m, words


def index_pattern(kind: str, n: int, seed: int) -> np.ndarray:
    if kind == "perm":
        return oracle.permutation(n, seed)
    if kind == "runs":
        return oracle.run_indices(n, seed)
    if kind == "uniform":
        return oracle.uniform_indices(n, n, seed)
    if kind == "identity":
        return np.arange(n, dtype=np.int32)
    raise ValueError(kind)


def case_inputs(case: dict):
    """Regenerate a case's inputs from its recipe (also used by the tests)."""
    s, n = case["s"], case["n"]
    src = oracle.random_words(n * s, case["seed"]).view(np.int32)
    idx = index_pattern(case["pattern"], n, case["seed"] + 1) if "pattern" in case else None
    init = oracle.random_words(n * s, case["seed"] + 2).view(np.int32) if case.get("init") else None
    return src, idx, init


def memory_inputs(case: dict):
    """Inputs of a memory.h case: the source buffer (loads) or the stored
    values (stores), and the output buffer's initial contents."""
    words = oracle.random_words(case["len"], case["seed"]).view(np.int32)
    init = oracle.random_words(case["len"], case["seed"] + 1).view(np.int32)
    if case["op"] >= 2:
        return words[: case["s"]].copy(), init
    return words, np.zeros(case["s"], np.int32)


def main():
    ref = oracle.reference_emulator()
    if ref is None:
        raise SystemExit("reference checkout not found; golden fixtures cannot be regenerated here")
    arrays = {}
    for n, m, words in transpose_cases():
        rows, cols = transpose_inputs(n, m, words)
        arrays[f"r2c_{n}_{m}_{words}"] = ref.transpose("r2c", n, m, rows)
        arrays[f"c2r_{n}_{m}_{words}"] = ref.transpose("c2r", n, m, cols)
    for m in range(1, 33):
        base = np.arange(m, dtype=np.int32) * 3 + 1
        arrays[f"rotate_{m}"] = np.stack([ref.rotate(base, a) for a in range(m)])
    old = HERE / "transposes.npz"
    unchanged = False
    if old.exists():
        prev = dict(np.load(old))
        unchanged = prev.keys() == arrays.keys() and all(np.array_equal(prev[k], arrays[k]) for k in arrays)
    if not unchanged:  # rewrite only on a change (the archive itself is not byte-stable)
        np.savez_compressed(old, **arrays)

    cases = []
    seed = 1000
    for s in WIDTHS:
        for tile in TILES:
            seed += 10
            c = dict(kind="copy", s=s, tile=tile, n=96, seed=seed)
            src, _, _ = case_inputs(c)
            c["sha256"] = digest(ref.copy(s, tile, src, c["n"]))
            cases.append(c)
        seed += 10
        c = dict(kind="store_counting", s=s, n=64, seed=seed)
        c["sha256"] = digest(ref.store_counting(s, c["n"]))
        cases.append(c)
        seed += 10
        c = dict(kind="load_sum", s=s, n=64, seed=seed)
        src, _, _ = case_inputs(c)
        out = ref.load_sum(s, src, c["n"])
        c["sha256"] = digest(out)
        c["out"] = out.tolist()
        cases.append(c)
        for pattern in ["perm", "runs", "uniform", "identity"]:
            for n in [96, 77]:
                seed += 10
                c = dict(kind="gather", s=s, n=n, seed=seed, pattern=pattern, init=True)
                src, idx, init = case_inputs(c)
                c["sha256"] = digest(ref.gather(s, src, idx, n, init))
                cases.append(c)
        for pattern in ["perm", "identity"]:
            for n in [96, 77]:
                seed += 10
                c = dict(kind="scatter", s=s, n=n, seed=seed, pattern=pattern, init=True)
                src, idx, init = case_inputs(c)
                c["sha256"] = digest(ref.scatter(s, src, idx, n, init))
                cases.append(c)
        for write in [1, 0]:
            seed += 10
            l = 32 * 5 + 17
            c = dict(kind="block", s=s, n=l, write=write, seed=seed)
            src = oracle.counting(l, s)
            c["sha256"] = digest(ref.block(s, bool(write), src, l))
            cases.append(c)
        for api in [0, 1]:
            seed += 10
            c = dict(kind="copy_exit", s=s, n=32 * 6 + 9, api=api, modulus=7, seed=seed, init=True)
            src, _, init = case_inputs(c)
            c["sha256"] = digest(ref.copy_exit(s, api, src, c["n"], 7, init))
            cases.append(c)
    for s in WIDTHS:  # trove/memory.h: warp_load, warp_store, uncoalesced_store
        for kind in range(4):
            for offset, stride in [(0, 1), (3, 5), (7, 32)]:
                seed += 10
                c = dict(kind="memory", s=s, op=kind, offset=offset, stride=stride, seed=seed,
                         len=offset + s * stride + 8)
                data, init = memory_inputs(c)
                out = ref.memory(s, kind, offset, stride, data, init)
                c["sha256"] = digest(out)
                cases.append(c)
    masks = [0xFFFFFFFF, 0x0000FFFF, 0xFFFF0000, 0x00FF00FF, 0x0F0F0F0F, 0x33333333, 0x55555555,
             0xFFFFFFFE, 0x7FFFFFFF, 0x000000FF, 0xF0F0F0F0, 0x0000000F]
    for N in [32, 16, 8, 4, 2]:
        for mask in masks:
            out = ref.warp_converged(N, mask)
            cases.append(dict(kind="warp_converged", N=N, mask=mask, out=out.tolist()))
    with open(HERE / "golden.json", "w") as f:
        json.dump({"generator": "tests/golden/gen_golden.py", "cases": cases}, f, indent=0)
    print(f"{len(arrays)} arrays, {len(cases)} cases")


if __name__ == "__main__":
    main()
