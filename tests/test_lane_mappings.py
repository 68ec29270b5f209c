"""Index logic of two GPU mappings, simulated lane by lane on the CPU.

* bsr4_row (csrc/bsr4.cuh): 4 lanes per block row; lane q takes the row's blocks
  s+q, s+q+4, ... whole, U at a time with the blocks past the row's end masked off,
  then two exchange steps (lanes q^2, then q^1) leave entry q of the row's product in
  lane q.
* multidot32w_kernel (csrc/k_krylov.cu): the float4 entries of the vectors cut into
  tiles of T x 256, CTA b taking tiles b, b + G, ...; every entry must be read by
  exactly one thread of one CTA."""
import numpy as np
import pytest


def bsr4_lane_partials(rowPtr, colPtr, val, x, row, U):
    """The four lanes' partial 4-vectors of one block row, as the kernel forms them."""
    s, e = rowPtr[row], rowPtr[row + 1]
    parts = np.zeros((4, 4))
    for q in range(4):
        k = s + q
        while k < e:
            for u in range(U):
                kk = k + 4 * u
                if kk < e:  # masked batch
                    parts[q] += val[kk] @ x[colPtr[kk]]
            k += 4 * U
    return parts


def exchange(parts):
    """The two shuffle steps of bsr4_row on the lanes' (a0, a1, a2, a3)."""
    out = np.zeros(4)
    k = np.zeros((4, 2))
    for q in range(4):  # lanes q and q^2: q & 2 keeps rows 2, 3, the others rows 0, 1
        hi = (q & 2) != 0
        own = parts[q][[2, 3]] if hi else parts[q][[0, 1]]
        other = parts[q ^ 2][[2, 3]] if hi else parts[q ^ 2][[0, 1]]
        k[q] = own + other
    for q in range(4):  # lanes q and q^1: the odd lane keeps the second of its two rows
        odd = (q & 1) != 0
        out[q] = (k[q][1] if odd else k[q][0]) + (k[q ^ 1][1] if odd else k[q ^ 1][0])
    return out


@pytest.mark.parametrize("U", [1, 2, 4])
def test_bsr4_row_gives_every_entry_of_the_product(U):
    rng = np.random.default_rng(5)
    n = 60
    lens = rng.integers(0, 40, n)  # empty rows and rows longer than 4U blocks included
    rowPtr = np.concatenate([[0], np.cumsum(lens)])
    colPtr = rng.integers(0, n, rowPtr[-1])
    val = rng.standard_normal((rowPtr[-1], 4, 4))
    x = rng.standard_normal((n, 4))
    ref = np.zeros((n, 4))
    for r in range(n):
        for k in range(rowPtr[r], rowPtr[r + 1]):
            ref[r] += val[k] @ x[colPtr[k]]
    got = np.array([exchange(bsr4_lane_partials(rowPtr, colPtr, val, x, r, U)) for r in range(n)])
    assert np.allclose(got, ref, rtol=1e-13, atol=1e-12)


@pytest.mark.parametrize("n4,G,T", [(1369121, 608, 3), (660469, 608, 3), (1000, 608, 3), (769, 1, 3),
                                    (5, 4, 3), (123457, 37, 4)])
def test_dot_tiles_cover_every_entry_once(n4, G, T):
    tile = T * 256
    count = np.zeros(n4, np.int32)
    for b in range(G):
        base = b * tile
        while base < n4:
            for t in range(T):
                k0 = base + t * 256
                k = np.arange(k0, min(k0 + 256, n4))
                count[k] += 1
            base += G * tile
    assert (count == 1).all()
