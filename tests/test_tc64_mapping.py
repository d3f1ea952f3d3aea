"""The FP64-width tensor pass's thread mapping (tensor64.cu: 1024 threads, two
groups of 16 warps, a quarter of a column per thread), replayed on the CPU for
K = 3 and 4: in the digit steps every (operand row, K index) of a group's
digit operand is written exactly once, by 16- or 8-byte stores inside the
operand; the column maximum's shuffle partners (lanes ^ 8, ^ 16) hold the same
column; in the accumulator steps every thread reads TMEM lanes of its own
warp's quadrant and columns inside its group's 8-order set, and the group
reads every (lane, column) of that set exactly once."""
import pytest


def kmajor(row, k, sbo):
    # byte offset of element (row, k) of a K-major BF16 operand (pass.h: tc_kmajor_offset)
    return (row >> 3) * sbo + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2


@pytest.mark.parametrize("K", [3, 4])
def test_tc64_thread_mapping(K):
    D = 1 << K
    R, G, NV = 2 * D, 128 // D, D // 2
    SBO, A_BYTES, SET = 16 * R, 128 * R * 2, 8 * R
    for g in range(2):
        written, cells, colmax_writer = set(), {}, set()
        for gtid in range(512):
            tid = 512 * g + gtid
            w, l = tid >> 5, tid & 31
            assert w >> 4 == g
            wg = w & 15
            # digit steps
            mc, qc = 8 * wg + (l & 7), l >> 3
            hc, cc = qc >> 1, qc & 1
            assert 0 <= mc < 128 and mc // G < D
            k0 = hc * D + cc * NV
            off, nbytes = kmajor(mc, k0, SBO), 2 * NV
            assert off % nbytes == 0 and off + nbytes <= A_BYTES
            for i in range(NV):
                assert kmajor(mc, k0 + i, SBO) == off + 2 * i
                assert (mc, k0 + i) not in written
                written.add((mc, k0 + i))
            if qc == 0:
                colmax_writer.add(mc)
            for x in (8, 16):
                assert 8 * wg + ((l ^ x) & 7) == mc
            # accumulator steps
            m, q = 32 * (w & 3) + l, (wg >> 2) & 3
            half, chunk = q >> 1, q & 1
            assert 32 * (w & 3) <= m < 32 * (w & 3) + 32  # the warp's TMEM lane quadrant
            for c in range(NV):
                for o in range(8):
                    col = half * D + chunk * NV + c + o * R
                    assert col < SET
                    assert (m, col) not in cells
                    cells[(m, col)] = tid
        assert len(written) == 128 * R
        assert len(colmax_writer) == 128
        assert len(cells) == 128 * SET
