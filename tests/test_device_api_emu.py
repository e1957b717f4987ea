"""This repository's device API (include/trove) run on the host lane
emulator against the golden fixtures recorded from the reference: every
transposition, copy, known-answer kernel, coalesced_ptr gather/scatter, block
interface case, warp_converged result and memory.h load/store must be
identical.  CPU only."""
import hashlib

import numpy as np
import pytest

import oracle
from tests.golden.gen_golden import case_inputs, memory_inputs, transpose_cases, transpose_inputs


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def emu():
    return oracle.own_emulator()


def run_case(emu, c):
    s, n = c["s"], c["n"]
    src, idx, init = case_inputs(c)
    k = c["kind"]
    if k == "copy":
        return emu.copy(s, c["tile"], src, n)
    if k == "store_counting":
        return emu.store_counting(s, n)
    if k == "load_sum":
        return emu.load_sum(s, src, n)
    if k == "gather":
        return emu.gather(s, src, idx, n, init)
    if k == "scatter":
        return emu.scatter(s, src, idx, n, init)
    if k == "block":
        return emu.block(s, bool(c["write"]), oracle.counting(n, s), n)
    if k == "copy_exit":
        return emu.copy_exit(s, c["api"], src, n, c["modulus"], init)
    raise ValueError(k)


def test_transposes_match_reference(emu, golden_arrays):
    for n, m, words in transpose_cases():
        rows, cols = transpose_inputs(n, m, words)
        assert np.array_equal(emu.transpose("r2c", n, m, rows), golden_arrays[f"r2c_{n}_{m}_{words}"]), (n, m)
        assert np.array_equal(emu.transpose("c2r", n, m, cols), golden_arrays[f"c2r_{n}_{m}_{words}"]), (n, m)


def test_rotate_matches_reference(emu, golden_arrays):
    for m in range(1, 33):
        base = np.arange(m, dtype=np.int32) * 3 + 1
        for a in range(m):
            assert np.array_equal(emu.rotate(base, a), golden_arrays[f"rotate_{m}"][a])


@pytest.mark.parametrize("kind", ["copy", "store_counting", "load_sum", "gather", "scatter", "block",
                                  "copy_exit"])
def test_kernels_match_reference(emu, golden_cases, kind):
    for c in (c for c in golden_cases if c["kind"] == kind):
        assert digest(run_case(emu, c)) == c["sha256"], c


def test_warp_converged_matches_reference(emu, golden_cases):
    for c in (c for c in golden_cases if c["kind"] == "warp_converged"):
        assert emu.warp_converged(c["N"], c["mask"]).tolist() == c["out"], c


@pytest.mark.parametrize("s", [2, 3, 4, 6, 8, 12, 16])
def test_misaligned_views(emu, s):
    """Struct arrays that start 4 bytes past a 16-byte boundary: the widest
    word is chosen from the actual alignment, so results stay exact (the
    reference assumes sizeof-derived alignment and is not run here)."""
    n = 96
    raw = oracle.random_words(n * s + 4, 77)
    src = raw[1:1 + n * s].view(np.int32)  # 4-byte offset view
    assert src.ctypes.data % 16 != 0
    out = emu.copy(s, 32, src, n)
    assert np.array_equal(out, src)
    idx = oracle.permutation(n, 5)
    g = emu.gather(s, src, idx, n)
    assert np.array_equal(g.reshape(n, s), src.reshape(n, s)[idx])


def test_memory_functions_match_reference(emu, golden_cases):
    """warp_load (and its volatile overload), warp_store, uncoalesced_store."""
    cases = [c for c in golden_cases if c["kind"] == "memory"]
    assert len(cases) == 19 * 4 * 3
    for c in cases:
        data, init = memory_inputs(c)
        out = emu.memory(c["s"], c["op"], c["offset"], c["stride"], data, init)
        assert digest(out) == c["sha256"], c
