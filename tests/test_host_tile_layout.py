"""Shared-memory layout of the tile FFT (fft_fast.cu) checked on the CPU.

A restatement of the kernel's staged-line layout (ppos, tile_lp, the step-A
scratch stride) and of its shared-memory access patterns, with a bank model:
a warp's 8-byte accesses are served per half-warp, each half taking as many
wavefronts as the largest number of distinct 4-byte words that fall in one of
the 32 banks.  Every access of the line FFT and of the transposed tile side
must take the minimum (2 wavefronts per warp access), except the R = 2 row
loads (N = 64, 2-way) and a few of the real-pair reads of element N - j.
"""
import pytest


def ilog2(x):
    return x.bit_length() - 1


def brev(x, bits):
    return int(format(x, "0%db" % bits)[::-1], 2) if bits else 0


def scratch_stride(R):
    return 32 + 32 // R


def pad_a(R):
    return 1 if R >= 16 else 0


def pad_b(R):
    if R >= 32:
        return 0
    if R >= 16:
        return ((R // 2 - R * R - R) % 16 + 16) % 16
    return R // 2 if R >= 4 else 1


def ppos(R, j):
    return j + pad_a(R) * (j >> ilog2(R)) + pad_b(R) * (j >> (2 * ilog2(R)))


def tile_lp(R, real):
    N = 32 * R
    lp = max(ppos(R, N - 1) + 1, R * scratch_stride(R))
    return ((lp + 13) // 16) * 16 + 2 if real else (lp | 1)


def line_out_index(R, lane, r):
    P = 32 // R
    return lane // P + R * brev(r, ilog2(R)) + R * R * brev(lane % P, ilog2(P))


def wavefronts(elems):
    """8-byte elements addressed by the 32 lanes -> wavefronts of the warp access."""
    tot = 0
    for g0 in (0, 16):
        banks = {}
        for a in elems[g0:g0 + 16]:
            for w in (2 * a, 2 * a + 1):
                banks.setdefault(w % 32, set()).add(w)
        tot += max(len(v) for v in banks.values())
    return tot


@pytest.mark.parametrize("R", [2, 4, 8, 16, 32])
def test_positions_fit_and_are_distinct(R):
    N = 32 * R
    pos = [ppos(R, j) for j in range(N)]
    assert len(set(pos)) == N
    for real in (False, True):
        assert max(pos) < tile_lp(R, real)
        assert R * scratch_stride(R) <= tile_lp(R, real)


@pytest.mark.parametrize("R", [2, 4, 8, 16, 32])
def test_line_fft_accesses_conflict_free(R):
    LR, P, S = ilog2(R), 32 // R, scratch_stride(R)
    for r in range(R):  # step A scratch stores, step-A twiddles, step B loads
        assert wavefronts([brev(r, LR) * S + lane for lane in range(32)]) == 2
        assert wavefronts([brev(r, LR) * 32 + lane for lane in range(32)]) == 2
        assert wavefronts([(lane // P) * S + P * r + lane % P for lane in range(32)]) == 2
        # staged-tile stores of the FFT outputs
        assert wavefronts([ppos(R, line_out_index(R, lane, r)) for lane in range(32)]) == 2
        # row loads of the transposed-to-contiguous tiles
        w = wavefronts([ppos(R, lane + 32 * r) for lane in range(32)])
        assert w == (4 if R == 2 else 2)


@pytest.mark.parametrize("R", [2, 4, 8, 16, 32])
def test_transposed_side_conflict_free(R):
    N, TL = 32 * R, 16
    NV = TL * N // 2 // 256
    LPc, LPr = tile_lp(R, False), tile_lp(R, True)
    extra_zm = 0
    for warp in range(8):
        for u in range(NV):
            e2 = [warp * 32 + lane + u * 256 for lane in range(32)]
            lj = [((e % (TL // 2)) * 2, e // (TL // 2)) for e in e2]
            for dl in (0, 1):  # complex: lines l and l + 1 of element j
                assert wavefronts([(l + dl) * LPc + ppos(R, j) for l, j in lj]) == 2
            # real pairs: row l / 2, elements j and N - j
            assert wavefronts([(l // 2) * LPr + ppos(R, j) for l, j in lj]) == 2
            extra_zm += wavefronts([(l // 2) * LPr + ppos(R, (N - j) & (N - 1)) for l, j in lj]) - 2
    # the mirrored reads (element N - j) cross the padding boundaries backwards: a few 2-way accesses
    assert extra_zm <= (8 * NV * 2) // (2 if R == 2 else 8)
