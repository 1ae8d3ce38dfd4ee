"""All blocks of a case resident on the GPU: the domain layer of the C ABI.

``Domain(case)`` runs the set-up of main.f90:188-886 (placement, grids, BC
planes, solver set-up) in the library; the per-stage routines and whole RK3
steps (main.f90:893-1069) then run on the device without host round trips.
Only one domain exists at a time (the library keeps module-level state, like
the reference's Fortran modules).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import check, dptr


class Domain:
    def __init__(self, case, precision: int = 0, nu: int = 0, device: int = 0, use_graph: int = 0, nu_coarse: int = 0,
                 **solver):
        """solver: further snac_options fields (inner_iters, inner_tol, inner_adapt, refine_steps, mg_fuse,
        mg_cta_level, mg_tile, mg_waves, mg_red_batch, mg_lnu, tma, pdl, mg_inv, mg_restrict); 0 or absent selects
        the library default."""
        L = capi.lib()
        self.case = case
        c, arr, keep = capi.fill_descs(case)
        opt = capi.Options(precision=int(precision), use_graph=int(use_graph), nu=int(nu), device=int(device),
                           nu_coarse=int(nu_coarse))
        names = {f[0] for f in capi.Options._fields_}
        for k, v in solver.items():
            if k not in names:
                raise TypeError(f"unknown solver option {k}")
            setattr(opt, k, v)
        check(L.snac_init(C.byref(c), arr, C.byref(opt)))
        self._keep = keep
        self.nblocks = len(case.blocks)
        self.geom = [self.geometry(ib) for ib in range(self.nblocks)]

    def close(self):
        capi.lib().snac_finalize()

    def geometry(self, ib):
        lo = (C.c_int * 3)(); hi = (C.c_int * 3)(); nb = (C.c_int * 6)(); isb = (C.c_int * 6)()
        check(capi.lib().snac_block_geometry(ib, lo, hi, nb, isb))
        return dict(lo=tuple(lo), hi=tuple(hi), nb=[[nb[2 * a], nb[2 * a + 1]] for a in range(3)],
                    is_bound=[[isb[2 * a], isb[2 * a + 1]] for a in range(3)])

    def shape(self, ib, kind):
        lo, hi = self.geom[ib]["lo"], self.geom[ib]["hi"]
        n = [hi[a] - lo[a] + 1 for a in range(3)]
        if capi.DUDTRKO <= kind <= capi.DWDTRKO or kind >= capi.DSDTRKO0:
            return tuple(n)
        return tuple(x + 2 for x in n)

    def get(self, ib, kind) -> np.ndarray:
        a = np.zeros(self.shape(ib, kind), order="F")
        check(capi.lib().snac_get_field(ib, kind, dptr(a)))
        return a

    def set_many(self, items):
        """items: (block, kind, Fortran-ordered float64 array) triples, copied to the device in one call."""
        items = list(items)
        n = len(items)
        ib = (C.c_int * n)(*[i[0] for i in items])
        kd = (C.c_int * n)(*[i[1] for i in items])
        for _, _, a in items:
            if not (a.flags.f_contiguous and a.dtype == np.float64):
                raise ValueError("set_many needs Fortran-ordered float64 arrays")
        hp = (C.c_void_p * n)(*[a.ctypes.data for _, _, a in items])
        check(capi.lib().snac_set_fields(n, ib, kd, hp))

    def get_many(self, items):
        """items: (block, kind, Fortran-ordered float64 array) triples, filled from the device in one call."""
        items = list(items)
        n = len(items)
        ib = (C.c_int * n)(*[i[0] for i in items])
        kd = (C.c_int * n)(*[i[1] for i in items])
        for _, _, a in items:
            if not (a.flags.f_contiguous and a.dtype == np.float64 and a.flags.writeable):
                raise ValueError("get_many needs writeable Fortran-ordered float64 arrays")
        hp = (C.c_void_p * n)(*[a.ctypes.data for _, _, a in items])
        check(capi.lib().snac_get_fields(n, ib, kd, hp))

    def set(self, ib, kind, a: np.ndarray):
        a = np.asfortranarray(a, dtype=np.float64)
        assert a.shape == self.shape(ib, kind)
        check(capi.lib().snac_set_field(ib, kind, dptr(a)))

    def grid(self, ib, axis, which):
        lo, hi = self.geom[ib]["lo"], self.geom[ib]["hi"]
        out = np.zeros(hi[axis] - lo[axis] + 3)
        check(capi.lib().snac_get_grid(ib, axis, which, dptr(out)))
        return out

    @property
    def vol_all(self):
        return capi.lib().snac_vol_all()

    # per-stage routines (every block)
    def rk_mom(self, irk):
        check(capi.lib().snac_rk_mom_all(int(irk)))

    def bounduvw(self, is_correc=False):
        check(capi.lib().snac_bounduvw_all(int(is_correc)))

    def inflow(self, is_correc=False):
        check(capi.lib().snac_inflow_all(int(is_correc)))

    def boundp(self, kind=capi.P):
        check(capi.lib().snac_boundp_all(int(kind)))

    def fillps(self, dtrk):
        check(capi.lib().snac_fillps_all(float(dtrk)))

    def updt_rhs(self):
        check(capi.lib().snac_updt_rhs_all())

    def solve_pressure(self):
        return capi.lib().snac_solve_pressure()

    def correc(self, dtrk):
        check(capi.lib().snac_correc_all(float(dtrk)))

    def updt_pressure(self, alpha):
        check(capi.lib().snac_updt_pressure_all(float(alpha)))

    def chkdt(self):
        out = C.c_double()
        check(capi.lib().snac_chkdt_all(C.byref(out)))
        return out.value

    def chkdiv(self):
        a = C.c_double(); b = C.c_double()
        check(capi.lib().snac_chkdiv_all(C.byref(a), C.byref(b)))
        return a.value, b.value

    def kinetic_energy(self):
        out = C.c_double()
        check(capi.lib().snac_kinetic_energy(C.byref(out)))
        return out.value

    def step(self, n=1, allow_not_converged=False):
        rc = capi.lib().snac_step(int(n))
        if rc == capi.ERR_NOT_CONVERGED and allow_not_converged:
            return rc
        check(rc)
        return rc

    def checkpoint_save(self, prefix):
        """load_one('w') of every field of every block: <prefix>_b_###_{u,v,w,p,s_###}.bin"""
        check(capi.lib().snac_checkpoint_save(str(prefix).encode()))

    def checkpoint_load(self, prefix):
        check(capi.lib().snac_checkpoint_load(str(prefix).encode()))

    def out1d(self, ib, kind, idir):
        """(coordinates, profile) of out1d along idir (1..3)"""
        n = self.case.blocks[ib].ng[idir - 1]
        x = np.zeros(n); p = np.zeros(n)
        check(capi.lib().snac_out1d(int(ib), int(kind), int(idir), x.ctypes.data_as(capi.DP), p.ctypes.data_as(capi.DP)))
        return x, p

    def autotune(self, steps: int = 3):
        """Time the solver-setting candidates from a snapshot of the state and keep the fastest (the state is
        restored); returns the chosen settings and the times per step before and after."""
        r = capi.TuneResult()
        check(capi.lib().snac_autotune(int(steps), C.byref(r)))
        return dict(precision=r.precision, inner_iters=r.inner_iters, nu_coarse=r.nu_coarse, ms_per_step=r.ms_per_step,
                    ms_before=r.ms_before, candidates=r.ncand, mg_tile=r.mg_tile, mg_waves=r.mg_waves,
                    mg_cta_level=r.mg_cta_level, refine_steps=r.refine_steps)

    def stats(self):
        s = capi.StepStats()
        check(capi.lib().snac_get_stats(C.byref(s)))
        return dict(istep=s.istep, time=s.time, dt=s.dt, iters=s.solve_iters_max, residual=s.solve_residual_max,
                    solves=s.solves, device_ms=s.device_ms, helm_iters=s.helm_iters_max,
                    helm_residual=s.helm_residual_max)

    @property
    def dt(self):
        out = C.c_double()
        check(capi.lib().snac_get_dt(C.byref(out)))
        return out.value

    @dt.setter
    def dt(self, v):
        check(capi.lib().snac_set_dt(float(v)))
