"""The reference's hot-path subroutines, one block at a time, on numpy arrays.

Each function keeps the argument list of the Fortran subroutine it replaces
(rk.f90, fillps.f90, correc.f90, updt_pressure.f90, bound.f90, chkdt.f90,
chkdiv.f90, fft.f90) and works in place on Fortran-ordered float64 arrays
with the reference's halo conventions, exactly as SNaC's driver passes them.
The work runs in the CUDA kernels of libsnac_gb300.so (see include/snac_gpu.h).

The C entry points take bare pointers and size every copy from lo/hi, so an array of the wrong shape, order
or type would make them read or write past the caller's buffer.  Every wrapper here therefore checks each
array against the extents the Fortran declaration implies before calling: halo'd fields (lo-1:hi+1)^3,
interior arrays (lo:hi)^3, 1-D metrics (lo-1:hi+1), BC planes and traction planes; a mismatch raises
ValueError naming the argument, and nothing reaches the library.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import check, dptr, iarr, darr


def _extents(lo, hi):
    n = tuple(int(h) - int(l) + 1 for l, h in zip(lo, hi))
    if len(n) != 3 or min(n) < 1:
        raise ValueError(f"lo={tuple(lo)} hi={tuple(hi)}: three axes with hi >= lo expected")
    return n


def _arr(a, shape, name):
    """Pointer to a float64 array of exactly `shape`, Fortran-ordered (any order for 1-D)."""
    if not isinstance(a, np.ndarray) or a.dtype != np.float64:
        raise ValueError(f"{name}: float64 numpy array expected")
    if a.shape != tuple(shape):
        raise ValueError(f"{name}: shape {tuple(shape)} expected, got {a.shape}")
    if a.ndim > 1 and not a.flags["F_CONTIGUOUS"]:
        raise ValueError(f"{name}: Fortran-ordered (column-major) array expected")
    if a.ndim == 1 and not a.flags["C_CONTIGUOUS"]:
        raise ValueError(f"{name}: contiguous array expected")
    return dptr(a)


def _halo(a, n, name):
    return _arr(a, tuple(x + 2 for x in n), name)


def _interior(a, n, name):
    return _arr(a, n, name)


def _metrics(n, **m):
    """1-D metric arrays d?c / d?f over (lo-1:hi+1) of their axis (x, y or z from the name's second letter)."""
    axis = {"x": 0, "y": 1, "z": 2}
    return [_arr(a, (n[axis[k[1]]] + 2,), k) for k, a in m.items()]


def _plane(a, n, ax, name, sides=2):
    """A plane over the two axes other than ax, (n_t1 + 2) x (n_t2 + 2) x sides."""
    t1, t2 = [q for q in range(3) if q != ax]
    return _arr(a, (n[t1] + 2, n[t2] + 2, sides), name)


def rk_mom(rkpar, lo, hi, dxc, dxf, dyc, dyf, dzc, dzf, dt, bforce, gacc, beta, s1, visc, u, v, w, p,
           dudtrko, dvdtrko, dwdtrko, impdiff=False, boussinesq=False):
    """rk.f90:7-128 (rk_mom)."""
    n = _extents(lo, hi)
    mt = _metrics(n, dxc=dxc, dxf=dxf, dyc=dyc, dyf=dyf, dzc=dzc, dzf=dzf)
    check(capi.lib().snac_rk_mom(darr(rkpar), iarr(lo), iarr(hi), *mt, float(dt), darr(bforce), darr(gacc),
                                 float(beta), _halo(s1, n, "s1") if s1 is not None else capi.DP(), float(visc),
                                 _halo(u, n, "u"), _halo(v, n, "v"), _halo(w, n, "w"), _halo(p, n, "p"),
                                 _interior(dudtrko, n, "dudtrko"), _interior(dvdtrko, n, "dvdtrko"),
                                 _interior(dwdtrko, n, "dwdtrko"), int(impdiff), int(boussinesq)))


def rk_scal(rkpar, lo, hi, dxc, dxf, dyc, dyf, dzc, dzf, dt, alpha, vol_all, u, v, w, is_forced, scalf, ssource,
            dsdtrko, s, impdiff=False):
    """rk.f90:130-204 (rk_scal); returns f (scalf - bulk mean, or 0)."""
    n = _extents(lo, hi)
    mt = _metrics(n, dxc=dxc, dxf=dxf, dyc=dyc, dyf=dyf, dzc=dzc, dzf=dzf)
    f = C.c_double(0.0)
    check(capi.lib().snac_rk_scal(darr(rkpar), iarr(lo), iarr(hi), *mt, float(dt), float(alpha), float(vol_all),
                                  _halo(u, n, "u"), _halo(v, n, "v"), _halo(w, n, "w"), int(is_forced), float(scalf),
                                  float(ssource), _interior(dsdtrko, n, "dsdtrko"), _halo(s, n, "s"), C.byref(f),
                                  int(impdiff)))
    return f.value


def fillps(lo, hi, dxf, dyf, dzf, dt, u, v, w, p, fft_axis=0):
    """fillps.f90:7-54."""
    n = _extents(lo, hi)
    mt = _metrics(n, dxf=dxf, dyf=dyf, dzf=dzf)
    check(capi.lib().snac_fillps(iarr(lo), iarr(hi), *mt, float(dt), _halo(u, n, "u"), _halo(v, n, "v"),
                                 _halo(w, n, "w"), _halo(p, n, "p"), int(fft_axis)))


def correc(lo, hi, dxc, dyc, dzc, dt, p, u, v, w):
    """correc.f90:7-48."""
    n = _extents(lo, hi)
    mt = _metrics(n, dxc=dxc, dyc=dyc, dzc=dzc)
    check(capi.lib().snac_correc(iarr(lo), iarr(hi), *mt, float(dt), _halo(p, n, "p"), _halo(u, n, "u"),
                                 _halo(v, n, "v"), _halo(w, n, "w")))


def updt_pressure(lo, hi, dxc, dxf, dyc, dyf, dzc, dzf, alpha, pp, p, impdiff=False):
    """updt_pressure.f90:7-47."""
    n = _extents(lo, hi)
    mt = _metrics(n, dxc=dxc, dxf=dxf, dyc=dyc, dyf=dyf, dzc=dzc, dzf=dzf)
    check(capi.lib().snac_updt_pressure(iarr(lo), iarr(hi), *mt, float(alpha), _halo(pp, n, "pp"), _halo(p, n, "p"),
                                        int(impdiff)))


def updt_rhs(lo, hi, is_bound, rhsx, rhsy, rhsz, p):
    """bound.f90:543-585; is_bound[dir][side]; rhs? are (n_t1, n_t2, 0:1) interior planes."""
    n = _extents(lo, hi)
    isb = (C.c_int * 6)(*[int(is_bound[a][s]) for a in range(3) for s in range(2)])
    check(capi.lib().snac_updt_rhs(iarr(lo), iarr(hi), isb, _arr(rhsx, (n[1], n[2], 2), "rhsx"),
                                   _arr(rhsy, (n[0], n[2], 2), "rhsy"), _arr(rhsz, (n[0], n[1], 2), "rhsz"),
                                   _halo(p, n, "p")))


def chkdt(lo, hi, dxc, dxf, dyc, dyf, dzc, dzf, visc, u, v, w, impdiff=False):
    """chkdt.f90:8-56 for one block; returns dtmax."""
    n = _extents(lo, hi)
    mt = _metrics(n, dxc=dxc, dxf=dxf, dyc=dyc, dyf=dyf, dzc=dzc, dzf=dzf)
    out = C.c_double()
    check(capi.lib().snac_chkdt(iarr(lo), iarr(hi), *mt, float(visc), _halo(u, n, "u"), _halo(v, n, "v"),
                                _halo(w, n, "w"), int(impdiff), C.byref(out)))
    return out.value


def chkdiv(lo, hi, dxf, dyf, dzf, u, v, w, vol):
    """chkdiv.f90:8-44 for one block; returns (divtot, divmax)."""
    n = _extents(lo, hi)
    mt = _metrics(n, dxf=dxf, dyf=dyf, dzf=dzf)
    a = C.c_double(); b = C.c_double()
    check(capi.lib().snac_chkdiv(iarr(lo), iarr(hi), *mt, _halo(u, n, "u"), _halo(v, n, "v"), _halo(w, n, "w"),
                                 float(vol), C.byref(a), C.byref(b)))
    return a.value, b.value


def set_bc(ctype, ibound, lo, hi, idir, centered, rvalue, dr, p):
    """bound.f90:108-248 (set_bc) on one face."""
    n = _extents(lo, hi)
    if int(idir) not in (1, 2, 3) or int(ibound) not in (0, 1):
        raise ValueError("idir must be 1..3 and ibound 0 or 1")
    check(capi.lib().snac_set_bc(ctype.encode(), int(ibound), iarr(lo), iarr(hi), int(idir), int(centered),
                                 float(rvalue), float(dr), _halo(p, n, "p")))


def _cbc(a):
    """C order of a Fortran cbc(0:1,3[,3]) character array given as nested lists indexed [c][d][s] or [d][s]."""
    return "".join(np.asarray(a, dtype="U1").ravel()).encode()


def _ints(a, shape, name):
    r = np.ascontiguousarray(a, dtype=np.int32)
    if r.shape != shape:
        raise ValueError(f"{name}: shape {shape} expected, got {r.shape}")
    return r


def bounduvw(cbc, lo, hi, bc, is_correc, is_bound, nb, myrank, dxc, dxf, dyc, dyf, dzc, dzf, u, v, w):
    """bound.f90:8-66 (bounduvw) for one block: cbc[c][d][s], bc[c][d][s], is_bound[d][s], nb[d][s]."""
    n = _extents(lo, hi)
    mt = _metrics(n, dxc=dxc, dxf=dxf, dyc=dyc, dyf=dyf, dzc=dzc, dzf=dzf)
    b = np.ascontiguousarray(bc, dtype=np.float64)
    if b.shape != (3, 3, 2):
        raise ValueError(f"bc: shape (3, 3, 2) expected, got {b.shape}")
    ib, nbr = _ints(is_bound, (3, 2), "is_bound"), _ints(nb, (3, 2), "nb")
    check(capi.lib().snac_bounduvw(_cbc(cbc), iarr(lo), iarr(hi), dptr(b), int(is_correc),
                                   ib.ctypes.data_as(capi.IP), nbr.ctypes.data_as(capi.IP), int(myrank), *mt,
                                   _halo(u, n, "u"), _halo(v, n, "v"), _halo(w, n, "w")))


def boundp(cbc, lo, hi, bc, is_bound, nb, myrank, dxc, dyc, dzc, p):
    """bound.f90:68-106 (boundp) for one block: cbc[d][s], bc[d][s], is_bound[d][s], nb[d][s]."""
    n = _extents(lo, hi)
    mt = _metrics(n, dxc=dxc, dyc=dyc, dzc=dzc)
    b = np.ascontiguousarray(bc, dtype=np.float64)
    if b.shape != (3, 2):
        raise ValueError(f"bc: shape (3, 2) expected, got {b.shape}")
    ib, nbr = _ints(is_bound, (3, 2), "is_bound"), _ints(nb, (3, 2), "nb")
    check(capi.lib().snac_boundp(_cbc(cbc), iarr(lo), iarr(hi), dptr(b), ib.ctypes.data_as(capi.IP),
                                 nbr.ctypes.data_as(capi.IP), int(myrank), *mt, _halo(p, n, "p")))


def set_open_bc_uvw(ibound, lo, hi, idir, visc, dr, u, v, w, p, tr):
    """bound.f90:250-328; tr is the traction plane of axis idir, (n_t1 + 2, n_t2 + 2, 2)."""
    n = _extents(lo, hi)
    check(capi.lib().snac_set_open_bc_uvw(int(ibound), iarr(lo), iarr(hi), int(idir), float(visc), float(dr),
                                          _halo(u, n, "u"), _halo(v, n, "v"), _halo(w, n, "w"), _halo(p, n, "p"),
                                          _plane(tr, n, int(idir) - 1, "tr")))


def set_open_bc_p(ibound, lo, hi, idir, drc, drf, alpha, p):
    """bound.f90:330-375; drc = (drc(0), drc(1))."""
    n = _extents(lo, hi)
    check(capi.lib().snac_set_open_bc_p(int(ibound), iarr(lo), iarr(hi), int(idir), _arr(np.asarray(drc, float), (2,), "drc"),
                                        float(drf), float(alpha), _halo(p, n, "p")))


def cmpt_estimated_traction(ibound, lo, hi, idir, visc, dr, u, v, w, p, tr):
    """bound.f90:377-436; tr as in set_open_bc_uvw."""
    n = _extents(lo, hi)
    check(capi.lib().snac_cmpt_estimated_traction(int(ibound), iarr(lo), iarr(hi), int(idir), float(visc), float(dr),
                                                  _halo(u, n, "u"), _halo(v, n, "v"), _halo(w, n, "w"),
                                                  _halo(p, n, "p"), _plane(tr, n, int(idir) - 1, "tr")))


def outflow(is_outflow_bound, is_estimated_traction, lo, hi, dl, dl_h, visc, u, v, w, p, tr_x, tr_y, tr_z):
    """bound.f90:479-515: masks and dl, dl_h indexed [idir-1][ibound]."""
    n = _extents(lo, hi)
    ob, et = _ints(is_outflow_bound, (3, 2), "is_outflow_bound"), _ints(is_estimated_traction, (3, 2), "is_estimated_traction")
    check(capi.lib().snac_outflow(ob.ctypes.data_as(capi.IP), et.ctypes.data_as(capi.IP), iarr(lo), iarr(hi),
                                  _arr(np.ascontiguousarray(dl, float), (3, 2), "dl"),
                                  _arr(np.ascontiguousarray(dl_h, float), (3, 2), "dl_h"), float(visc),
                                  _halo(u, n, "u"), _halo(v, n, "v"), _halo(w, n, "w"), _halo(p, n, "p"),
                                  _plane(tr_x, n, 0, "tr_x"), _plane(tr_y, n, 1, "tr_y"), _plane(tr_z, n, 2, "tr_z")))


def outflow_p(is_outflow_bound, lo, hi, dlc, dlf, alpha, p):
    """bound.f90:517-541: dlc indexed [idir-1][ibound][0:1], dlf [idir-1][ibound]."""
    n = _extents(lo, hi)
    ob = _ints(is_outflow_bound, (3, 2), "is_outflow_bound")
    check(capi.lib().snac_outflow_p(ob.ctypes.data_as(capi.IP), iarr(lo), iarr(hi),
                                    _arr(np.ascontiguousarray(dlc, float), (3, 2, 2), "dlc"),
                                    _arr(np.ascontiguousarray(dlf, float), (3, 2), "dlf"), float(alpha),
                                    _halo(p, n, "p")))


def fft(kind, idir, arr, q=0):
    """fft.f90:85-94 on an interior array arr(n1,n2,n3) along idir (1..3), in place."""
    if arr.ndim != 3:
        raise ValueError("arr: a 3-D interior array expected")
    n = arr.shape
    check(capi.lib().snac_fft(int(kind), int(idir), iarr(n), int(q), _arr(arr, n, "arr")))


def find_fft(bc, centered):
    kf = C.c_int(); kb = C.c_int(); norm = np.zeros(2)
    check(capi.lib().snac_find_fft(bc.encode(), int(centered), C.byref(kf), C.byref(kb), dptr(norm)))
    return kf.value, kb.value, norm


def eigenvalues(n, bc, centered):
    lam = np.zeros(n)
    check(capi.lib().snac_eigenvalues(int(n), bc.encode(), int(centered), dptr(lam)))
    return lam


def initgrid(lo, hi, gt, gr, lmin, lmax):
    n = hi - lo + 3
    drc, drf, rc, rf = (np.zeros(n) for _ in range(4))
    check(capi.lib().snac_initgrid(int(lo), int(hi), int(gt), float(gr), float(lmin), float(lmax), dptr(drc), dptr(drf),
                                   dptr(rc), dptr(rf)))
    return drc, drf, rc, rf
