"""CPU checks of the bandwidth-reducing order the cylinder Newton solve uses
(broadcast_gb300.linsolve.folded_ring_order): a permutation, and the periodic
O-mesh Jacobian pattern (cells within 3 in i, periodic, and in j) banded with
kl = ku <= 15 im + 35 in it, against ~5 im jm in the natural (i, j, e) order."""
import numpy as np
import pytest


def _pattern(im, jm):
    """(row, col) of the Jacobian's structural non-zeros, rows (i, j, e), i slowest."""
    i, j, di, dj, e, f = np.meshgrid(np.arange(im), np.arange(jm), np.arange(-3, 4), np.arange(-3, 4), np.arange(5),
                                     np.arange(5), indexing="ij")
    jj = j + dj
    ok = (jj >= 0) & (jj < jm)
    ii = (i + di) % im
    row = e + 5 * j + 5 * jm * i
    col = f + 5 * jj + 5 * jm * ii
    return row[ok], col[ok]


@pytest.mark.parametrize("im,jm", [(28, 21), (7, 9), (64, 10), (13, 13)])
def test_folded_order_is_a_permutation_and_bands_the_periodic_stencil(im, jm):
    from broadcast_gb300.linsolve import folded_ring_order
    p = folded_ring_order(im, jm)
    n = 5 * im * jm
    assert p.dtype == np.int32 and np.array_equal(np.sort(p), np.arange(n))
    r, c = _pattern(im, jm)
    natural = int(np.abs(r - c).max())
    folded = int(np.abs(p[r].astype(np.int64) - p[c]).max())
    assert folded <= 15 * im + 35
    if im > 7:
        assert folded < natural
