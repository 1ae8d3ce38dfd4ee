"""The halo argument of the tiled red-black smoother (snac_gb300/csrc/k_mg_fused.cu), checked on the CPU.

A tile sweeps its cells in shared memory with zero values beyond its edge.  After t half-sweeps, only cells
within t of the edge can differ from a global sweep, so the output cells, 4 cells in from the edge, are exact
after the 2 nu = 4 half-sweeps of one launch.  The pre-smoother starts from x = 0: its first half-sweep sees
zero neighbours everywhere (the cells beyond the tile are still zero too), so after t half-sweeps only cells
within t - 1 of the edge can differ.  That leaves the neighbours of every output cell exact as well, which is
what lets the pre-smoother form the residual of its output cells and restrict it without a wider tile.

The sweeps here run in numpy (float64, one fixed operation order shared by the tile and the global sweep), on
random diagonally dominant 5-point operators; no GPU is needed.
"""
import numpy as np
import pytest


def half_sweep(x, b, ce, cw, cn, cs, inv, color, parity=0):
    """One red-black half-sweep over the cells with (i + j + parity) % 2 == color (parity: that of the array's
    origin in the global grid, so a tile keeps the global colouring); x[j, i] with zero values outside."""
    n1, n0 = x.shape
    xp = np.zeros((n1 + 2, n0 + 2))
    xp[1:-1, 1:-1] = x
    acc = ce * xp[1:-1, 2:]
    acc = acc + cw * xp[1:-1, :-2]
    acc = acc + cn * xp[2:, 1:-1]
    acc = acc + cs * xp[:-2, 1:-1]
    jj, ii = np.indices(x.shape)
    upd = (ii + jj + parity) % 2 == color
    out = x.copy()
    out[upd] = ((b - acc) * inv)[upd]
    return out


def residual(x, b, ce, cw, cn, cs, d):
    n1, n0 = x.shape
    xp = np.zeros((n1 + 2, n0 + 2))
    xp[1:-1, 1:-1] = x
    acc = ce * xp[1:-1, 2:]
    acc = acc + cw * xp[1:-1, :-2]
    acc = acc + cn * xp[2:, 1:-1]
    acc = acc + cs * xp[:-2, 1:-1]
    return b - (d * x + acc)


def operator(rng, n1, n0):
    ce = -rng.uniform(0.5, 1.5, (n1, n0))
    cn = -rng.uniform(0.5, 1.5, (n1, n0))
    ce[:, -1] = 0.0
    cn[-1, :] = 0.0
    cw = np.zeros_like(ce)
    cw[:, 1:] = ce[:, :-1]
    cs = np.zeros_like(cn)
    cs[1:, :] = cn[:-1, :]
    d = -(ce + cw + cn + cs) + rng.uniform(0.0, 0.5, (n1, n0))
    return ce, cw, cn, cs, d


def sweeps(x, b, ops, nhalf, parity=0):
    ce, cw, cn, cs, d = ops
    for t in range(nhalf):
        x = half_sweep(x, b, ce, cw, cn, cs, 1.0 / d, t % 2, parity)
    return x


def distance_to_edge(h, w):
    jj, ii = np.indices((h, w))
    return np.minimum(np.minimum(ii, w - 1 - ii), np.minimum(jj, h - 1 - jj))


@pytest.mark.parametrize("seed,j0,i0", [(0, 7, 11), (1, 20, 3), (2, 13, 30)])
def test_zero_start_tile_is_exact_one_ring_further(seed, j0, i0):
    rng = np.random.default_rng(seed)
    n1, n0, h, w, nhalf = 60, 90, 24, 40, 4
    ops = operator(rng, n1, n0)
    b = rng.standard_normal((n1, n0))
    glob = sweeps(np.zeros((n1, n0)), b, ops, nhalf)
    win = (slice(j0, j0 + h), slice(i0, i0 + w))
    tile_ops = tuple(o[win] for o in ops)
    tile = sweeps(np.zeros((h, w)), b[win], tile_ops, nhalf, (i0 + j0) % 2)
    dist = distance_to_edge(h, w)
    # from zero, only cells within nhalf - 1 = 3 of the edge can differ ...
    np.testing.assert_array_equal(tile[dist >= nhalf - 1], glob[win][dist >= nhalf - 1])
    # ... so the residual of every output cell (4 in from the edge) is the global one, bit for bit
    rt = residual(tile, b[win], *tile_ops)
    rg = residual(glob, b, *ops)[win]
    np.testing.assert_array_equal(rt[dist >= nhalf], rg[dist >= nhalf])
    # the ring at distance nhalf - 2 does differ: the bound is tight
    assert np.any(tile[dist == nhalf - 2] != glob[win][dist == nhalf - 2])


def test_nonzero_start_needs_the_full_halo():
    """With a nonzero start (the post-smoother adds the coarse correction first) the cells within nhalf of the
    edge may all differ; the output cells, nhalf in from the edge, are still exact."""
    rng = np.random.default_rng(3)
    n1, n0, h, w, nhalf = 60, 90, 24, 40, 4
    ops = operator(rng, n1, n0)
    b = rng.standard_normal((n1, n0))
    x0 = rng.standard_normal((n1, n0))
    glob = sweeps(x0, b, ops, nhalf)
    win = (slice(10, 10 + h), slice(20, 20 + w))
    tile = sweeps(x0[win].copy(), b[win], tuple(o[win] for o in ops), nhalf, (10 + 20) % 2)
    dist = distance_to_edge(h, w)
    np.testing.assert_array_equal(tile[dist >= nhalf], glob[win][dist >= nhalf])
    assert np.any(tile[dist == nhalf - 1] != glob[win][dist == nhalf - 1])
