"""ctypes wrapper of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline / reference legs of bench.py; never by the snac_gb300 package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
MAX_SCAL = 4

U, V, W, P, PP, PO, DUDTRKO, DVDTRKO, DWDTRKO = range(9)
S0 = 9
DSDTRKO0 = 20
G_DXC, G_DXF, G_XC, G_XF = range(4)

(R2HC, HC2R, REDFT00, REDFT01, REDFT10, REDFT11, RODFT00, RODFT01, RODFT10, RODFT11) = (0, 1, 3, 4, 5, 6, 7, 8, 9, 10)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc only; make rebuilds only what changed)."""
    subprocess.run(["make", "-s", "-C", _HERE] + (["-B"] if force else []), check=True)
    return _LIB_PATH


class BlockDesc(C.Structure):
    _fields_ = [("ng", C.c_int * 3), ("lmin", C.c_double * 3), ("lmax", C.c_double * 3), ("gt", C.c_int * 3),
                ("gr", C.c_double * 3), ("cbcvel", ((C.c_char * 2) * 3) * 3), ("bcvel", ((C.c_double * 2) * 3) * 3),
                ("cbcpre", (C.c_char * 2) * 3), ("bcpre", (C.c_double * 2) * 3),
                ("cbcscal", ((C.c_char * 2) * 3) * MAX_SCAL), ("bcscal", ((C.c_double * 2) * 3) * MAX_SCAL),
                ("grid_file", C.POINTER(C.c_double) * 3), ("inflow_type", (C.c_int * 2) * 3)]


class CaseDesc(C.Structure):
    _fields_ = [("nblocks", C.c_int), ("visci", C.c_double), ("cfl", C.c_double), ("dtmax", C.c_double),
                ("dt_f", C.c_double), ("bforce", C.c_double * 3), ("gacc", C.c_double * 3), ("beta", C.c_double),
                ("nscal", C.c_int), ("alphai", C.c_double * MAX_SCAL), ("ssource", C.c_double * MAX_SCAL),
                ("scalf", C.c_double * MAX_SCAL), ("is_sforced", C.c_int * MAX_SCAL), ("icheck", C.c_int),
                ("fft_axis", C.c_int), ("impdiff", C.c_int), ("boussinesq", C.c_int), ("tol", C.c_double),
                ("maxiter", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        L.or_create.restype = C.c_void_p
        L.or_create.argtypes = [C.POINTER(CaseDesc), C.POINTER(BlockDesc), C.c_char_p, C.c_int]
        L.or_destroy.argtypes = [C.c_void_p]
        L.or_field.restype = dp
        L.or_field.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.or_grid.restype = dp
        L.or_grid.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
        L.or_block_geometry.argtypes = [C.c_void_p, C.c_int, ip, ip, ip, ip]
        L.or_vol_all.restype = C.c_double
        L.or_vol_all.argtypes = [C.c_void_p]
        for n in ("or_checkpoint_save", "or_checkpoint_load"):
            getattr(L, n).argtypes = [C.c_void_p, C.c_char_p]
            getattr(L, n).restype = C.c_int
        L.or_time_istep.argtypes = [C.c_void_p, dp, C.POINTER(C.c_int)]
        L.or_out1d.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, dp, dp, C.c_char_p]
        L.or_out1d.restype = C.c_int
        L.or_fortran_e15_7.argtypes = [C.c_double, C.c_char_p]
        for n in ("or_bounduvw", "or_boundp", "or_inflow"):
            getattr(L, n).argtypes = [C.c_void_p, C.c_int]
        L.or_fillps_all.argtypes = [C.c_void_p, C.c_double]
        L.or_impdiff_solve.argtypes = [C.c_void_p, C.c_int, C.c_double]
        L.or_updt_rhs_all.argtypes = [C.c_void_p]
        L.or_solve_pressure.argtypes = [C.c_void_p]
        L.or_correc_all.argtypes = [C.c_void_p, C.c_double]
        L.or_updt_pressure_all.argtypes = [C.c_void_p, C.c_double]
        L.or_chkdt.restype = C.c_double
        L.or_chkdt.argtypes = [C.c_void_p]
        L.or_chkdiv.argtypes = [C.c_void_p, dp, dp]
        L.or_kinetic_energy.restype = C.c_double
        L.or_kinetic_energy.argtypes = [C.c_void_p]
        L.or_step.argtypes = [C.c_void_p, C.c_int]
        L.or_dt.restype = C.c_double
        L.or_dt.argtypes = [C.c_void_p]
        L.or_set_dt.argtypes = [C.c_void_p, C.c_double]
        L.or_istep.argtypes = [C.c_void_p]
        L.or_time.restype = C.c_double
        L.or_time.argtypes = [C.c_void_p]
        L.or_last_iterations.argtypes = [C.c_void_p]
        L.or_last_residual.restype = C.c_double
        L.or_last_residual.argtypes = [C.c_void_p]
        L.or_set_threads.argtypes = [C.c_int]
        L.or_r2r.argtypes = [C.c_int, C.c_int, dp, dp]
        L.or_find_fft.argtypes = [C.c_char_p, C.c_int, ip, ip, dp]
        L.or_eigenvalues.argtypes = [C.c_int, C.c_char_p, C.c_int, dp]
        L.or_initgrid.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, dp, dp, dp, dp]
        d = C.c_double
        i = C.c_int
        L.or_rk_mom.argtypes = [dp, ip, ip, dp, dp, dp, dp, dp, dp, d, dp, dp, d, dp, d, dp, dp, dp, dp, dp, dp, dp, i, i]
        L.or_rk_scal.argtypes = [dp, ip, ip, dp, dp, dp, dp, dp, dp, d, d, d, dp, dp, dp, i, d, d, dp, dp, dp, i]
        L.or_fillps.argtypes = [ip, ip, dp, dp, dp, d, dp, dp, dp, dp, i]
        L.or_correc.argtypes = [ip, ip, dp, dp, dp, d, dp, dp, dp, dp]
        L.or_updt_pressure.argtypes = [ip, ip, dp, dp, dp, dp, dp, dp, d, dp, dp, i]
        L.or_chkdt_local.argtypes = [ip, ip, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp]
        L.or_chkdiv_local.argtypes = [ip, ip, dp, dp, dp, dp, dp, dp, d, dp, dp]
        L.or_updt_rhs.argtypes = [ip, ip, ip, dp, dp, dp, dp]
        L.or_set_bc.argtypes = [C.c_char, i, ip, ip, i, i, d, d, dp]
        L.or_cmpt_vorticity.argtypes = [ip, dp, dp, dp, dp, dp, dp, dp, dp, dp]
        L.or_cmpt_strain_rate.argtypes = [ip, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp]
        L.or_cmpt_rotation_rate.argtypes = [ip, dp, dp, dp, dp, dp, dp, dp]
        L.or_cmpt_q_criterion.argtypes = [ip, dp, dp, dp]
        d_ = C.c_double
        L.or_set_open_bc_uvw.argtypes = [i, ip, ip, i, d_, d_, dp, dp, dp, dp, dp]
        L.or_set_open_bc_p.argtypes = [i, ip, ip, i, dp, d_, d_, dp]
        L.or_cmpt_estimated_traction.argtypes = [i, ip, ip, i, d_, d_, dp, dp, dp, dp, dp]
        L.or_outflow.argtypes = [ip, ip, ip, ip, dp, dp, d_, dp, dp, dp, dp, dp, dp, dp]
        L.or_outflow_p.argtypes = [ip, ip, ip, dp, dp, d_, dp]
        L.or_bounduvw_block.argtypes = [C.c_char_p, ip, ip, dp, i, ip, ip, i, dp, dp, dp, dp, dp, dp, dp, dp, dp]
        L.or_boundp_block.argtypes = [C.c_char_p, ip, ip, dp, ip, ip, i, dp, dp, dp, dp]
        L.or_r2r_lines.argtypes = [i, i, i, C.c_long, C.c_long, dp]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


def fill_descs(case, block_cls=BlockDesc, case_cls=CaseDesc):
    """Translate a snac_gb300.cases.Case into the C input structs (keeps grid arrays alive)."""
    nb = len(case.blocks)
    arr = (block_cls * nb)()
    keep = []
    for ib, b in enumerate(case.blocks):
        d = arr[ib]
        for a in range(3):
            d.ng[a] = int(b.ng[a]); d.lmin[a] = float(b.lmin[a]); d.lmax[a] = float(b.lmax[a])
            d.gt[a] = int(b.gt[a]); d.gr[a] = float(b.gr[a])
            for s in range(2):
                d.cbcpre[a][s] = b.cbcpre[a][s].encode()
                d.bcpre[a][s] = float(b.bcpre[a][s])
                for c in range(3):
                    d.cbcvel[c][a][s] = b.cbcvel[c][a][s].encode()
                    d.bcvel[c][a][s] = float(b.bcvel[c][a][s])
                for sc in range(MAX_SCAL):
                    if b.cbcscal is not None and sc < len(b.cbcscal):
                        d.cbcscal[sc][a][s] = b.cbcscal[sc][a][s].encode()
                        d.bcscal[sc][a][s] = float(b.bcscal[sc][a][s])
                    else:
                        d.cbcscal[sc][a][s] = b"N"
                        d.bcscal[sc][a][s] = 0.0
            for s in range(2):
                d.inflow_type[a][s] = int(b.inflow_type[a][s])
            gf = b.grid_file[a]
            if gf is not None:
                g = np.ascontiguousarray(gf, dtype=np.float64)
                keep.append(g)
                d.grid_file[a] = g.ctypes.data_as(C.POINTER(C.c_double))
            else:
                d.grid_file[a] = C.POINTER(C.c_double)()
    c = case_cls()
    c.nblocks = nb
    c.visci, c.cfl, c.dtmax, c.dt_f = case.visci, case.cfl, case.dtmax, case.dt_f
    for a in range(3):
        c.bforce[a] = case.bforce[a]; c.gacc[a] = case.gacc[a]
    c.beta = case.beta
    c.nscal = case.nscal
    for s in range(MAX_SCAL):
        c.alphai[s] = case.alphai[s] if s < len(case.alphai) else 1.0
        c.ssource[s] = case.ssource[s] if s < len(case.ssource) else 0.0
        c.scalf[s] = case.scalf[s] if s < len(case.scalf) else 0.0
        c.is_sforced[s] = int(case.is_sforced[s]) if s < len(case.is_sforced) else 0
    c.icheck = case.icheck
    c.fft_axis = case.fft_axis
    c.impdiff = case.impdiff
    c.boussinesq = case.boussinesq
    c.tol = case.tol
    c.maxiter = case.maxiter
    return c, arr, keep


class OracleDomain:
    """All blocks of a case on the CPU, with the reference's per-step routines."""

    def __init__(self, case, threads: int = 0):
        L = lib()
        if threads:
            L.or_set_threads(threads)
        self.case = case
        c, arr, keep = fill_descs(case)
        err = C.create_string_buffer(512)
        h = L.or_create(C.byref(c), arr, err, 512)
        if not h:
            raise RuntimeError("oracle: " + err.value.decode())
        self.h = h
        self.nblocks = len(case.blocks)
        self.geom = [self.geometry(ib) for ib in range(self.nblocks)]

    def close(self):
        if self.h:
            lib().or_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def geometry(self, ib):
        lo = (C.c_int * 3)(); hi = (C.c_int * 3)(); nb = (C.c_int * 6)(); isb = (C.c_int * 6)()
        lib().or_block_geometry(self.h, ib, lo, hi, nb, isb)
        return dict(lo=tuple(lo), hi=tuple(hi), nb=[[nb[2 * a], nb[2 * a + 1]] for a in range(3)],
                    is_bound=[[isb[2 * a], isb[2 * a + 1]] for a in range(3)])

    def field(self, ib: int, kind: int) -> np.ndarray:
        """Live view (Fortran order) of a block field; halo'd unless it is an RK storage array."""
        p = lib().or_field(self.h, ib, kind)
        if not p:
            raise KeyError(kind)
        lo, hi = self.geom[ib]["lo"], self.geom[ib]["hi"]
        n = [hi[a] - lo[a] + 1 for a in range(3)]
        halo = not (DUDTRKO <= kind <= DWDTRKO or kind >= DSDTRKO0)
        shape = tuple(x + 2 for x in n) if halo else tuple(n)
        cnt = int(np.prod(shape))
        buf = np.ctypeslib.as_array(p, shape=(cnt,))
        return buf.reshape(shape, order="F")

    def grid(self, ib: int, axis: int, which: int) -> np.ndarray:
        lo, hi = self.geom[ib]["lo"], self.geom[ib]["hi"]
        n = hi[axis] - lo[axis] + 3
        return np.ctypeslib.as_array(lib().or_grid(self.h, ib, axis, which), shape=(n,))

    def bounduvw(self, is_correc=False):
        lib().or_bounduvw(self.h, int(is_correc))

    def inflow(self, is_correc=False):
        lib().or_inflow(self.h, int(is_correc))

    def checkpoint_save(self, prefix):
        rc = lib().or_checkpoint_save(self.h, str(prefix).encode())
        if rc:
            raise IOError(f"oracle checkpoint save failed ({rc})")

    def checkpoint_load(self, prefix):
        rc = lib().or_checkpoint_load(self.h, str(prefix).encode())
        if rc:
            raise IOError(f"oracle checkpoint load failed ({rc})")

    def out1d(self, ib, kind, idir, fname=None):
        n = self.case.blocks[ib].ng[idir - 1]
        x = np.zeros(n); p = np.zeros(n)
        dpp = C.POINTER(C.c_double)
        rc = lib().or_out1d(self.h, int(ib), int(kind), int(idir), x.ctypes.data_as(dpp), p.ctypes.data_as(dpp),
                            None if fname is None else str(fname).encode())
        if rc:
            raise IOError("oracle out1d failed")
        return x, p

    @property
    def time_istep(self):
        t = C.c_double(); i = C.c_int()
        lib().or_time_istep(self.h, C.byref(t), C.byref(i))
        return t.value, i.value

    def boundp(self, kind=P):
        lib().or_boundp(self.h, kind)

    def step(self, n=1):
        rc = lib().or_step(self.h, n)
        if rc < 0:
            raise RuntimeError(f"oracle step failed ({rc})")
        return rc

    def chkdt(self):
        return lib().or_chkdt(self.h)

    def chkdiv(self):
        a = C.c_double(); b = C.c_double()
        lib().or_chkdiv(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def kinetic_energy(self):
        return lib().or_kinetic_energy(self.h)

    @property
    def dt(self):
        return lib().or_dt(self.h)

    @dt.setter
    def dt(self, v):
        lib().or_set_dt(self.h, v)

    @property
    def istep(self):
        return lib().or_istep(self.h)

    @property
    def time(self):
        return lib().or_time(self.h)

    @property
    def vol_all(self):
        return lib().or_vol_all(self.h)

    def last_solve(self):
        return lib().or_last_iterations(self.h), lib().or_last_residual(self.h)


def r2r(kind: int, x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    lib().or_r2r(kind, x.size, _ptr(x), _ptr(y))
    return y


def eigenvalues(n: int, bc: str, centered: bool) -> np.ndarray:
    lam = np.zeros(n)
    rc = lib().or_eigenvalues(n, bc.encode(), int(centered), _ptr(lam))
    if rc:
        raise ValueError(bc)
    return lam


def find_fft(bc: str, centered: bool):
    kf = C.c_int(); kb = C.c_int(); norm = np.zeros(2)
    lib().or_find_fft(bc.encode(), int(centered), C.byref(kf), C.byref(kb), _ptr(norm))
    return kf.value, kb.value, norm


def fortran_e15_7(v: float) -> str:
    """The oracle's Fortran E15.7 formatter (output.f90's '(2E15.7)' fields)."""
    out = C.create_string_buffer(128)
    lib().or_fortran_e15_7(float(v), out)
    return out.value.decode()
