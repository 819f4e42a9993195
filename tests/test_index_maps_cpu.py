"""CPU checks of the index arithmetic of the TMA-fed separable kernel
(`k_sep2d_tma` in csrc/ifx_fir.cu), restated here: every item map covers its
cells exactly once, every shared-memory read stays inside the buffer that
holds it, and the row pass's 16-byte loads are free of bank conflicts.  These
are the checks a kernel's launch geometry gets on the CPU before it runs on a
GPU; they fail when the restatement and its invariants drift apart."""
import pytest

TX, NB, NBY = 64, 16, 8          # kStTX, kStNB, kStNBY
KMAX = 36                        # kCorrKmax


def st_pitch(n):
    """Smallest pitch >= n floats that is 4 mod 8 (st_pitch)."""
    p = (n + 3) & ~3
    return p if (p & 7) else p + 4


def row_items(rows):
    return 64 * (rows >> 4) + 32 * (((rows & 15) + 7) >> 3)


def row_item(it, rows):
    lane, grp, full = it & 31, it >> 5, 2 * (rows >> 4)
    if grp < full:
        return 16 * (grp >> 1) + 4 * (lane >> 3) + ((lane >> 1) & 3), NB * (2 * (grp & 1) + (lane & 1))
    return 8 * grp + (lane & 7), NB * (lane >> 3)


@pytest.mark.parametrize("rows", list(range(1, 120)))
def test_row_pass_items_cover_rows_once_without_bank_conflicts(rows):
    n = row_items(rows)
    assert n % 32 == 0
    seen = {}
    for it in range(n):
        r, c0 = row_item(it, rows)
        if r >= rows:
            continue
        for i in range(NB):
            seen[(r, c0 + i)] = seen.get((r, c0 + i), 0) + 1
    assert len(seen) == rows * TX and max(seen.values()) == 1
    # each 8-lane phase of a warp's 16-byte loads touches 8 distinct 16-byte bank groups
    for pitch in (68, 76, 84, 92, 100):
        for it0 in range(0, n, 8):
            groups = {((r * pitch + c0) // 4) % 8 for r, c0 in (row_item(it, rows) for it in range(it0, it0 + 8))}
            assert len(groups) == 8


@pytest.mark.parametrize("ty", [32, 40, 48, 56, 64])
def test_pass_reads_stay_inside_their_buffers(ty):
    """Both pass orders, every factor length: the row pass reads at most
    4*ceil((NB+k-1)/4) values from a 16-byte aligned window start, the column
    pass NB+k-1 rows; the y-first column pass fills columns up to CV (odd CV
    writes column CV, inside the pitch)."""
    for kx in range(1, KMAX + 1):
        for ky in range(1, KMAX + 1):
            RV, CV = ty + ky - 1, TX + kx - 1
            SP = st_pitch(CV + 3)                              # input tile pitch (Float32 box width)
            reach = 4 * ((NB + kx - 1 + 3) // 4)               # values the row pass loads per item
            # x first: row pass over RV rows of the input, column pass over I (RV rows, pitch 68)
            for it in range(row_items(RV)):
                r, c0 = row_item(it, RV)
                if r < RV:
                    assert c0 + reach <= SP
            for it in range((TX // 2) * (ty // NBY)):
                rs, c = divmod(it, TX // 2)
                assert rs * NBY + NBY + ky - 1 <= RV and 2 * c + 1 < st_pitch(TX)
            # y first: column pass over CV columns into I (ty rows, pitch st_pitch(CV+3))
            si = st_pitch(CV + 3)
            cp = (CV + 1) >> 1
            for it in range(cp * (ty // NBY)):
                rs, c = divmod(it, cp)
                assert rs * NBY + NBY + ky - 1 <= RV and 2 * c + 1 < min(SP, si)
            for it in range(row_items(ty)):
                r, c0 = row_item(it, ty)
                if r < ty:
                    assert c0 + reach <= si


def test_column_pass_items_cover_tile_once():
    for ty in (32, 40, 48, 56, 64):
        seen = set()
        for it in range((TX // 2) * (ty // NBY)):
            rs, c = divmod(it, TX // 2)
            for i in range(NBY):
                for j in (0, 1):
                    cell = (rs * NBY + i, 2 * c + j)
                    assert cell not in seen
                    seen.add(cell)
        assert len(seen) == ty * TX
