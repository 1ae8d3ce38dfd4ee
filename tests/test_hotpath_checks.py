"""The numpy wrappers check every array against the extents lo/hi imply before any C call (an array of the
wrong shape, order or type would otherwise be read or written past its end by the library).  CPU only: every
case raises before the library is called."""
import numpy as np
import pytest

from snac_gb300 import hotpath

LO, HI = (1, 1, 1), (8, 6, 4)
N = (8, 6, 4)


def halo(order="F", n=N):
    return np.zeros(tuple(x + 2 for x in n), order=order)


def metric(a):
    return np.ones(N[a] + 2)


def test_fillps_rejects_wrong_arrays():
    u, v, w, p = halo(), halo(), halo(), halo()
    m = [metric(0), metric(1), metric(2)]
    with pytest.raises(ValueError, match="u: shape"):
        hotpath.fillps(LO, HI, *m, 0.1, halo(n=(8, 6, 5)), v, w, p)
    with pytest.raises(ValueError, match="v: Fortran-ordered"):
        hotpath.fillps(LO, HI, *m, 0.1, u, halo(order="C"), w, p)
    with pytest.raises(ValueError, match="w: float64"):
        hotpath.fillps(LO, HI, *m, 0.1, u, v, w.astype(np.float32), p)
    with pytest.raises(ValueError, match="dyf: shape"):
        hotpath.fillps(LO, HI, m[0], np.ones(N[1] + 1), m[2], 0.1, u, v, w, p)
    with pytest.raises(ValueError, match="three axes"):
        hotpath.fillps(LO, (8, 0, 4), *m, 0.1, u, v, w, p)


def test_rk_mom_checks_interior_and_halo_arrays():
    f = [halo() for _ in range(4)]
    m = [metric(a // 2) for a in range(6)]
    r = [np.zeros(N, order="F") for _ in range(3)]
    with pytest.raises(ValueError, match="dvdtrko: shape"):
        hotpath.rk_mom((0.5, 0.0), LO, HI, *m, 0.01, (0, 0, 0), (0, 0, 0), 0.0, None, 1e-3, *f, r[0],
                       np.zeros((8, 6, 3), order="F"), r[2])


def test_boundary_wrappers_check_tables_and_planes():
    u, v, w, p = halo(), halo(), halo(), halo()
    with pytest.raises(ValueError, match="tr: shape"):
        hotpath.set_open_bc_uvw(0, LO, HI, 2, 1e-3, 0.1, u, v, w, p, np.zeros((10, 8, 2), order="F"))
    with pytest.raises(ValueError, match="is_bound: shape"):
        hotpath.boundp([["D", "D"]] * 3, LO, HI, np.zeros((3, 2)), np.zeros((2, 3)), np.zeros((3, 2)), 0,
                       metric(0), metric(1), metric(2), p)
    with pytest.raises(ValueError, match="rhsy: shape"):
        hotpath.updt_rhs(LO, HI, [[1, 1]] * 3, np.zeros((6, 4, 2), order="F"), np.zeros((6, 4, 2), order="F"),
                         np.zeros((8, 6, 2), order="F"), p)
