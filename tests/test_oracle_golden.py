"""Pin the CPU oracle against the golden fixtures recorded from the
reference's own code (tests/golden/gen_golden.py).  CPU only."""
import hashlib

import numpy as np
import pytest

import oracle
from tests.golden.gen_golden import case_inputs, transpose_cases, transpose_inputs


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def oracle_output(case):
    """What the oracle says the reference computes for a golden case."""
    s, n = case["s"], case["n"]
    width = 4 * s
    src, idx, init = case_inputs(case)
    kind = case["kind"]
    if kind == "copy":
        return oracle.copy(src, n, width)
    if kind == "store_counting":
        return oracle.counting(n, s)
    if kind == "load_sum":
        return oracle.load_sum(src, n, s)
    if kind == "gather":
        return oracle.gather(init, src, idx, n, width)
    if kind == "scatter":
        return oracle.scatter(init, src, idx, n, width)
    if kind == "block":
        return oracle.counting(n, s)  # write: counting; copy of counting: counting
    if kind == "copy_exit":
        out, _ = oracle.copy_exit(init, src, n, width, case["modulus"])
        return out
    raise ValueError(kind)


def test_golden_fixture_is_complete(golden_cases, golden_arrays):
    kinds = {c["kind"] for c in golden_cases}
    assert kinds == {"copy", "store_counting", "load_sum", "gather", "scatter", "block", "copy_exit",
                     "warp_converged", "memory"}
    assert len(golden_arrays) == 2 * len(list(transpose_cases())) + 32


@pytest.mark.parametrize("kind", ["copy", "store_counting", "load_sum", "gather", "scatter", "block",
                                  "copy_exit"])
def test_oracle_matches_reference(golden_cases, kind):
    cases = [c for c in golden_cases if c["kind"] == kind]
    assert cases
    for c in cases:
        out = oracle_output(c)
        assert digest(out) == c["sha256"], c
        if "out" in c:
            assert out.tolist() == c["out"]


def test_oracle_transpose_semantics(golden_arrays):
    """r2c: column (l, j) holds row-form word l*m+j; c2r is the inverse."""
    for n, m, words in transpose_cases():
        rows, cols = transpose_inputs(n, m, words)
        lane, elem = oracle.r2c_source(n, m)
        expect_cols = rows[lane, elem]
        assert np.array_equal(golden_arrays[f"r2c_{n}_{m}_{words}"], expect_cols), (n, m, words)
        assert np.array_equal(golden_arrays[f"c2r_{n}_{m}_{words}"], rows), (n, m, words)
        assert np.array_equal(expect_cols, cols)


def test_rotate_semantics(golden_arrays):
    for m in range(1, 33):
        base = np.arange(m, dtype=np.int32) * 3 + 1
        got = golden_arrays[f"rotate_{m}"]
        for a in range(m):
            assert np.array_equal(got[a], np.roll(base, -a)), (m, a)


def test_warp_converged_semantics(golden_cases):
    for c in (c for c in golden_cases if c["kind"] == "warp_converged"):
        N, mask = c["N"], c["mask"]
        for lane in range(32):
            if not (mask >> lane) & 1:
                assert c["out"][lane] == 255  # lane did not run
                continue
            group = ((1 << N) - 1) << (lane & ~(N - 1))
            assert c["out"][lane] == int((mask & group) == group), (N, hex(mask), lane)


def test_seeded_generators_are_stable():
    # Values fixed at the time the fixtures were recorded.
    w = oracle.random_words(4, 0)
    assert w.dtype == np.uint32 and len(set(w.tolist())) == 4
    assert oracle.word(0, 3) == int(w[3])
    p = oracle.permutation(1000, 5)
    assert sorted(p.tolist()) == list(range(1000))
    r = oracle.run_indices(1024, 9)
    assert r.min() >= 0 and r.max() < 1024
    runs = sum(all(r[c * 32 + k] == r[c * 32] + k for k in range(32)) for c in range(32))
    assert 4 <= runs <= 28  # about half of the 32 chunks are runs
    mt = oracle.random_words(1 << 16, 3, threads=4)
    assert np.array_equal(mt, oracle.random_words(1 << 16, 3))


def test_copy_exit_counts():
    src = oracle.random_structs(5000, 12, 11)
    init = np.zeros_like(src)
    out, written = oracle.copy_exit(init, src, 5000, 12, 625)
    words0 = src.view(np.uint32)[:, 0]
    skip = (words0 % 625) == 624
    assert written == 5000 - skip.sum()
    o = out.reshape(5000, 12)
    assert np.array_equal(o[~skip], src[~skip]) and not o[skip].any()


def test_multithreaded_forms_agree():
    n, w = 10007, 20
    src = oracle.random_structs(n, w, 3)
    idx = oracle.permutation(n, 4)
    for op, expect in [(oracle.OP_COPY, src.reshape(-1)),
                       (oracle.OP_GATHER, oracle.gather(np.zeros(n * w, np.uint8), src, idx, n, w)),
                       (oracle.OP_SCATTER, oracle.scatter(np.zeros(n * w, np.uint8), src, idx, n, w))]:
        dst = np.zeros(n * w, np.uint8)
        oracle.run_mt(op, dst, src, idx if op else None, n, w, 7)
        assert np.array_equal(dst, expect)


def test_multithreaded_layouts_agree():
    n, w = 10007, 28
    s = w // 4
    src = oracle.random_structs(n, w, 5)
    soa = np.zeros(n * w, np.uint8)
    oracle.run_mt(oracle.OP_AOS_TO_SOA, soa, src, None, n, w, 7)
    assert np.array_equal(soa.view(np.uint32), oracle.aos_to_soa(src, n, s))
    back = np.zeros(n * w, np.uint8)
    oracle.run_mt(oracle.OP_SOA_TO_AOS, back, soa, None, n, w, 5)
    assert np.array_equal(back, src.reshape(-1))


def test_memory_restatement_matches_reference(golden_cases):
    from tests.golden.gen_golden import memory_inputs
    for c in (c for c in golden_cases if c["kind"] == "memory"):
        data, init = memory_inputs(c)
        out = oracle.memory_op(c["s"], c["op"], c["offset"], c["stride"], data, init)
        assert hashlib.sha256(np.ascontiguousarray(out).tobytes()).hexdigest() == c["sha256"], c
