"""trv_probe_block_gather, the random-read ceiling that gathers are compared
against: on a small case its output must equal a host restatement of what
each lane reads and folds (so it reads exactly the aligned blocks every row
overlaps, and writes n * width bytes and nothing past them)."""
import numpy as np
import pytest

import oracle
import trove_gb300 as tg

pytestmark = pytest.mark.gpu


def expected(src_bytes, idx, src_n, n, width, block):
    """Lane l of the warp owning rows 32 w .. 32 w + 31 folds (XOR) the
    16-byte vectors of its slots q = l + 32 r, r < K: row q // K, block
    (q % K) // (block / 16) past that row's first, vector (q % K) % (block / 16)
    of it, idle past the row's last block or for an invalid index; vector k
    of the warp's 2 * width output vectors is lane k % 32's fold."""
    vpb = block // 16
    k_slots = ((width - 1) // block + 2) * vpb
    words = src_bytes.view(np.uint32)
    out = np.zeros((n * width) // 4, np.uint32).reshape(-1, 4)
    for w in range(n // 32):
        rows = idx[32 * w: 32 * w + 32]
        fold = np.zeros((32, 4), np.uint32)
        fold[:, 0] = np.arange(32, dtype=np.uint32)
        for lane in range(32):
            for r in range(k_slots):
                q = lane + 32 * r
                j, slot = divmod(q, k_slots)
                row = int(rows[j])
                if row < 0 or row >= src_n:
                    continue
                start = row * width
                b0, b1 = start // block, (start + width - 1) // block
                blk = b0 + slot // vpb
                if blk > b1:
                    continue
                v0 = (blk * block + (slot % vpb) * 16) // 4
                assert v0 + 4 <= len(words)  # inside the allocation
                fold[lane] ^= words[v0: v0 + 4]
        base = (32 * w * width) // 16
        for kk in range(2 * width):
            out[base + kk] = fold[kk % 32]
    return out.reshape(-1).view(np.uint8)


@pytest.mark.parametrize("width", [8, 12, 20, 64, 128])
@pytest.mark.parametrize("block,hint", [(32, 0), (64, 64), (128, 128), (64, 0)])
def test_probe_reads_the_blocks_rows_overlap(cuda, width, block, hint):
    torch = cuda
    n, src_n = 128, 1000
    # src_n rows, rounded up to whole blocks (the probe reads whole blocks)
    nbytes = -(-src_n * width // block) * block
    src_h = oracle.random_words(nbytes // 4, seed=width).view(np.uint8)
    idx_h = oracle.uniform_indices(n, src_n, seed=block + width)
    idx_h[5] = -1
    idx_h[77] = src_n + 3  # out of range: reads nothing
    src = torch.from_numpy(src_h.copy()).cuda()
    idx = torch.from_numpy(idx_h).cuda()
    dst = torch.full((n * width + 256,), 0x5A, dtype=torch.uint8, device="cuda")
    tg.probe_block_gather(dst, src, src_n, idx, n, width, block, hint)
    torch.cuda.synchronize()
    got = dst.cpu().numpy()
    assert np.array_equal(got[: n * width], expected(src_h, idx_h, src_n, n, width, block))
    assert (got[n * width:] == 0x5A).all()
