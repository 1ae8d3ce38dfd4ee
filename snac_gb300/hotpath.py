"""The reference's hot-path subroutines, one block at a time, on numpy arrays.

Each function keeps the argument list of the Fortran subroutine it replaces
(rk.f90, fillps.f90, correc.f90, updt_pressure.f90, bound.f90, chkdt.f90,
chkdiv.f90, fft.f90) and works in place on Fortran-ordered float64 arrays
with the reference's halo conventions, exactly as SNaC's driver passes them.
The work runs in the CUDA kernels of libsnac_gb300.so (see include/snac_gpu.h).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import check, dptr, iarr, darr


def _f(a):
    assert a.dtype == np.float64 and (a.flags["F_CONTIGUOUS"] or a.ndim == 1), "Fortran-ordered float64 expected"
    return dptr(a)


def rk_mom(rkpar, lo, hi, dxc, dxf, dyc, dyf, dzc, dzf, dt, bforce, gacc, beta, s1, visc, u, v, w, p,
           dudtrko, dvdtrko, dwdtrko, impdiff=False, boussinesq=False):
    """rk.f90:7-128 (rk_mom)."""
    check(capi.lib().snac_rk_mom(darr(rkpar), iarr(lo), iarr(hi), _f(dxc), _f(dxf), _f(dyc), _f(dyf), _f(dzc), _f(dzf),
                                 float(dt), darr(bforce), darr(gacc), float(beta), _f(s1) if s1 is not None else capi.DP(),
                                 float(visc), _f(u), _f(v), _f(w), _f(p), _f(dudtrko), _f(dvdtrko), _f(dwdtrko),
                                 int(impdiff), int(boussinesq)))


def rk_scal(rkpar, lo, hi, dxc, dxf, dyc, dyf, dzc, dzf, dt, alpha, vol_all, u, v, w, is_forced, scalf, ssource,
            dsdtrko, s, impdiff=False):
    """rk.f90:130-204 (rk_scal); returns f (scalf - bulk mean, or 0)."""
    f = C.c_double(0.0)
    check(capi.lib().snac_rk_scal(darr(rkpar), iarr(lo), iarr(hi), _f(dxc), _f(dxf), _f(dyc), _f(dyf), _f(dzc), _f(dzf),
                                  float(dt), float(alpha), float(vol_all), _f(u), _f(v), _f(w), int(is_forced),
                                  float(scalf), float(ssource), _f(dsdtrko), _f(s), C.byref(f), int(impdiff)))
    return f.value


def fillps(lo, hi, dxf, dyf, dzf, dt, u, v, w, p, fft_axis=0):
    """fillps.f90:7-54."""
    check(capi.lib().snac_fillps(iarr(lo), iarr(hi), _f(dxf), _f(dyf), _f(dzf), float(dt), _f(u), _f(v), _f(w), _f(p),
                                 int(fft_axis)))


def correc(lo, hi, dxc, dyc, dzc, dt, p, u, v, w):
    """correc.f90:7-48."""
    check(capi.lib().snac_correc(iarr(lo), iarr(hi), _f(dxc), _f(dyc), _f(dzc), float(dt), _f(p), _f(u), _f(v), _f(w)))


def updt_pressure(lo, hi, dxc, dxf, dyc, dyf, dzc, dzf, alpha, pp, p, impdiff=False):
    """updt_pressure.f90:7-47."""
    check(capi.lib().snac_updt_pressure(iarr(lo), iarr(hi), _f(dxc), _f(dxf), _f(dyc), _f(dyf), _f(dzc), _f(dzf),
                                        float(alpha), _f(pp), _f(p), int(impdiff)))


def updt_rhs(lo, hi, is_bound, rhsx, rhsy, rhsz, p):
    """bound.f90:543-585; is_bound[dir][side]."""
    isb = (C.c_int * 6)(*[int(is_bound[a][s]) for a in range(3) for s in range(2)])
    check(capi.lib().snac_updt_rhs(iarr(lo), iarr(hi), isb, _f(rhsx), _f(rhsy), _f(rhsz), _f(p)))


def chkdt(lo, hi, dxc, dxf, dyc, dyf, dzc, dzf, visc, u, v, w, impdiff=False):
    """chkdt.f90:8-56 for one block; returns dtmax."""
    out = C.c_double()
    check(capi.lib().snac_chkdt(iarr(lo), iarr(hi), _f(dxc), _f(dxf), _f(dyc), _f(dyf), _f(dzc), _f(dzf), float(visc),
                                _f(u), _f(v), _f(w), int(impdiff), C.byref(out)))
    return out.value


def chkdiv(lo, hi, dxf, dyf, dzf, u, v, w, vol):
    """chkdiv.f90:8-44 for one block; returns (divtot, divmax)."""
    a = C.c_double(); b = C.c_double()
    check(capi.lib().snac_chkdiv(iarr(lo), iarr(hi), _f(dxf), _f(dyf), _f(dzf), _f(u), _f(v), _f(w), float(vol),
                                 C.byref(a), C.byref(b)))
    return a.value, b.value


def set_bc(ctype, ibound, lo, hi, idir, centered, rvalue, dr, p):
    """bound.f90:108-248 (set_bc) on one face."""
    check(capi.lib().snac_set_bc(ctype.encode(), int(ibound), iarr(lo), iarr(hi), int(idir), int(centered),
                                 float(rvalue), float(dr), _f(p)))


def _cbc(a):
    """C order of a Fortran cbc(0:1,3[,3]) character array given as nested lists indexed [c][d][s] or [d][s]."""
    return "".join(np.asarray(a, dtype="U1").ravel()).encode()


def bounduvw(cbc, lo, hi, bc, is_correc, is_bound, nb, myrank, dxc, dxf, dyc, dyf, dzc, dzf, u, v, w):
    """bound.f90:8-66 (bounduvw) for one block: cbc[c][d][s], bc[c][d][s], is_bound[d][s], nb[d][s]."""
    b = np.ascontiguousarray(bc, dtype=np.float64)
    ib = np.ascontiguousarray(is_bound, dtype=np.int32)
    nbr = np.ascontiguousarray(nb, dtype=np.int32)
    check(capi.lib().snac_bounduvw(_cbc(cbc), iarr(lo), iarr(hi), dptr(b), int(is_correc),
                                   ib.ctypes.data_as(capi.IP), nbr.ctypes.data_as(capi.IP), int(myrank),
                                   dptr(dxc), dptr(dxf), dptr(dyc), dptr(dyf), dptr(dzc), dptr(dzf), _f(u), _f(v),
                                   _f(w)))


def boundp(cbc, lo, hi, bc, is_bound, nb, myrank, dxc, dyc, dzc, p):
    """bound.f90:68-106 (boundp) for one block: cbc[d][s], bc[d][s], is_bound[d][s], nb[d][s]."""
    b = np.ascontiguousarray(bc, dtype=np.float64)
    ib = np.ascontiguousarray(is_bound, dtype=np.int32)
    nbr = np.ascontiguousarray(nb, dtype=np.int32)
    check(capi.lib().snac_boundp(_cbc(cbc), iarr(lo), iarr(hi), dptr(b), ib.ctypes.data_as(capi.IP),
                                 nbr.ctypes.data_as(capi.IP), int(myrank), dptr(dxc), dptr(dyc), dptr(dzc), _f(p)))


def fft(kind, idir, arr, q=0):
    """fft.f90:85-94 on an interior array arr(n1,n2,n3) along idir (1..3), in place."""
    n = arr.shape
    check(capi.lib().snac_fft(int(kind), int(idir), iarr(n), int(q), _f(arr)))


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
