"""ctypes binding of include/snac_gpu.h (libsnac_gb300.so).

This is the reference-side view of the library: the same entry points a
Fortran driver binds with iso_c_binding, callable from Python with numpy
arrays laid out like the reference's Fortran arrays (order='F', halo 1).
The library has no CPU path: without the compiled extension or a CUDA
device every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _build

MAX_SCAL = 4
OK, ERR_ARG, ERR_CUDA, ERR_NOT_CONVERGED, ERR_NAN, ERR_TIMEOUT, ERR_BOUNDS, ERR_STATE, ERR_UNSUPPORTED, ERR_NOMEM, ERR_IO = range(11)
U, V, W, P, PP, PO, DUDTRKO, DVDTRKO, DWDTRKO = range(9)
S0, DSDTRKO0 = 9, 20
G_DXC, G_DXF, G_XC, G_XF = range(4)
R2HC, HC2R, REDFT00, REDFT01, REDFT10, REDFT11, RODFT00, RODFT01, RODFT10, RODFT11 = (0, 1, 3, 4, 5, 6, 7, 8, 9, 10)


class SnacError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"snac error {code}: {msg}")
        self.code = code


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


class Options(C.Structure):
    _fields_ = [("precision", C.c_int), ("use_graph", C.c_int), ("nu", C.c_int), ("device", C.c_int),
                ("nu_coarse", C.c_int), ("inner_iters", C.c_int), ("inner_tol", C.c_double),
                ("inner_adapt", C.c_int), ("refine_steps", C.c_int), ("mg_fuse", C.c_int),
                ("mg_cta_level", C.c_int), ("mg_tile", C.c_int), ("mg_waves", C.c_int), ("mg_red_batch", C.c_int),
                ("mg_lnu", C.c_int), ("tma", C.c_int), ("pdl", C.c_int), ("mg_inv", C.c_int),
                ("mg_restrict", C.c_int)]


class TuneResult(C.Structure):
    _fields_ = [("precision", C.c_int), ("inner_iters", C.c_int), ("nu_coarse", C.c_int), ("ms_per_step", C.c_double),
                ("ms_before", C.c_double), ("ncand", C.c_int), ("mg_tile", C.c_int), ("mg_waves", C.c_int),
                ("mg_cta_level", C.c_int), ("refine_steps", C.c_int)]


class StepStats(C.Structure):
    _fields_ = [("istep", C.c_int), ("time", C.c_double), ("dt", C.c_double), ("solve_iters_max", C.c_int),
                ("solve_residual_max", C.c_double), ("solves", C.c_int), ("device_ms", C.c_double),
                ("helm_iters_max", C.c_int), ("helm_residual_max", C.c_double)]


_lib = None
DP = C.POINTER(C.c_double)
FP = C.POINTER(C.c_float)
IP = C.POINTER(C.c_int)

# every entry point declared in include/snac_gpu.h with its ctypes signature
PROTOTYPES = {
    "snac_last_error": (C.c_char_p, []),
    "snac_device_count": (C.c_int, [IP]),
    "snac_probe_peaks": (C.c_int, [DP, DP]),
    "snac_profile_kernel": (C.c_int, [C.c_int]),
    "snac_profile_read": (C.c_int, [IP, DP]),
    "snac_launch_count": (C.c_int, [C.POINTER(C.c_longlong)]),
    "snac_bench_smoother": (C.c_int, [C.c_int, C.c_int, DP, DP]),
    "snac_register": (C.c_int, [C.c_void_p, C.c_size_t]),
    "snac_unregister": (C.c_int, [C.c_void_p]),
    "snac_update_device": (C.c_int, [C.c_void_p]),
    "snac_update_host": (C.c_int, [C.c_void_p]),
    "snac_rk_mom": (C.c_int, [DP, IP, IP, DP, DP, DP, DP, DP, DP, C.c_double, DP, DP, C.c_double, DP, C.c_double,
                              DP, DP, DP, DP, DP, DP, DP, C.c_int, C.c_int]),
    "snac_rk_scal": (C.c_int, [DP, IP, IP, DP, DP, DP, DP, DP, DP, C.c_double, C.c_double, C.c_double, DP, DP, DP,
                               C.c_int, C.c_double, C.c_double, DP, DP, DP, C.c_int]),
    "snac_fillps": (C.c_int, [IP, IP, DP, DP, DP, C.c_double, DP, DP, DP, DP, C.c_int]),
    "snac_correc": (C.c_int, [IP, IP, DP, DP, DP, C.c_double, DP, DP, DP, DP]),
    "snac_updt_pressure": (C.c_int, [IP, IP, DP, DP, DP, DP, DP, DP, C.c_double, DP, DP, C.c_int]),
    "snac_updt_rhs": (C.c_int, [IP, IP, IP, DP, DP, DP, DP]),
    "snac_chkdt": (C.c_int, [IP, IP, DP, DP, DP, DP, DP, DP, C.c_double, DP, DP, DP, C.c_int, DP]),
    "snac_chkdiv": (C.c_int, [IP, IP, DP, DP, DP, DP, DP, DP, C.c_double, DP, DP]),
    "snac_chkdiv_noalloc": (C.c_int, [IP, IP, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_double, C.c_void_p, DP, DP]),
    "snac_set_bc": (C.c_int, [C.c_char, C.c_int, IP, IP, C.c_int, C.c_int, C.c_double, C.c_double, DP]),
    "snac_cmpt_vorticity": (C.c_int, [IP, DP, DP, DP, DP, DP, DP, DP, DP, DP]),
    "snac_cmpt_strain_rate": (C.c_int, [IP, DP, DP, DP, DP, DP, DP, DP, DP, DP, DP]),
    "snac_cmpt_rotation_rate": (C.c_int, [IP, DP, DP, DP, DP, DP, DP, DP]),
    "snac_cmpt_q_criterion": (C.c_int, [IP, DP, DP, DP]),
    "snac_q_criterion": (C.c_int, [IP, DP, DP, DP, DP, DP, DP, DP, DP, DP, DP]),
    "snac_bounduvw": (C.c_int, [C.c_char_p, IP, IP, DP, C.c_int, IP, IP, C.c_int, DP, DP, DP, DP, DP, DP, DP, DP,
                                DP]),
    "snac_boundp": (C.c_int, [C.c_char_p, IP, IP, DP, IP, IP, C.c_int, DP, DP, DP, DP]),
    "snac_fft": (C.c_int, [C.c_int, C.c_int, IP, C.c_int, DP]),
    "snac_find_fft": (C.c_int, [C.c_char_p, C.c_int, IP, IP, DP]),
    "snac_eigenvalues": (C.c_int, [C.c_int, C.c_char_p, C.c_int, DP]),
    "snac_initgrid": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, DP, DP, DP, DP]),
    "snac_init": (C.c_int, [C.POINTER(CaseDesc), C.POINTER(BlockDesc), C.POINTER(Options)]),
    "snac_finalize": (C.c_int, []),
    "snac_check_case": (C.c_int, [C.POINTER(CaseDesc), C.POINTER(BlockDesc), IP, C.POINTER(C.c_long)]),
    "snac_block_geometry": (C.c_int, [C.c_int, IP, IP, IP, IP]),
    "snac_get_grid": (C.c_int, [C.c_int, C.c_int, C.c_int, DP]),
    "snac_set_field": (C.c_int, [C.c_int, C.c_int, DP]),
    "snac_get_field": (C.c_int, [C.c_int, C.c_int, DP]),
    "snac_vol_all": (C.c_double, []),
    "snac_rk_mom_all": (C.c_int, [C.c_int]),
    "snac_bounduvw_all": (C.c_int, [C.c_int]),
    "snac_boundp_all": (C.c_int, [C.c_int]),
    "snac_inflow_all": (C.c_int, [C.c_int]),
    "snac_fillps_all": (C.c_int, [C.c_double]),
    "snac_impdiff_solve": (C.c_int, [C.c_int, C.c_double, C.c_double]),
    "snac_updt_rhs_all": (C.c_int, []),
    "snac_solve_pressure": (C.c_int, []),
    "snac_correc_all": (C.c_int, [C.c_double]),
    "snac_updt_pressure_all": (C.c_int, [C.c_double]),
    "snac_chkdt_all": (C.c_int, [DP]),
    "snac_chkdiv_all": (C.c_int, [DP, DP]),
    "snac_kinetic_energy": (C.c_int, [DP]),
    "snac_step": (C.c_int, [C.c_int]),
    "snac_read_namelists": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int, C.POINTER(CaseDesc),
                                      C.POINTER(BlockDesc), C.c_int]),
    "snac_checkpoint_save": (C.c_int, [C.c_char_p]),
    "snac_checkpoint_load": (C.c_int, [C.c_char_p]),
    "snac_out1d": (C.c_int, [C.c_int, C.c_int, C.c_int, DP, DP]),
    "snac_cnn_conv3x3": (C.c_int, [FP, C.c_int, C.c_int, C.c_int, FP, FP, C.c_int, FP]),
    "snac_cnn_set_poll_limit": (C.c_int, [C.c_long]),
    "snac_guess_grad": (C.c_int, [FP, FP, C.c_int, C.c_int, C.c_int, FP, FP, DP]),
    "snac_set_open_bc_uvw": (C.c_int, [C.c_int, IP, IP, C.c_int, C.c_double, C.c_double, DP, DP, DP, DP, DP]),
    "snac_set_open_bc_p": (C.c_int, [C.c_int, IP, IP, C.c_int, DP, C.c_double, C.c_double, DP]),
    "snac_cmpt_estimated_traction": (C.c_int, [C.c_int, IP, IP, C.c_int, C.c_double, C.c_double, DP, DP, DP, DP, DP]),
    "snac_outflow": (C.c_int, [IP, IP, IP, IP, DP, DP, C.c_double, DP, DP, DP, DP, DP, DP, DP]),
    "snac_outflow_p": (C.c_int, [IP, IP, IP, DP, DP, C.c_double, DP]),
    "snac_bounds_checked": (C.c_int, []),
    "snac_bounds_selftest": (C.c_int, []),
    "snac_unet_nparams": (C.c_int, []),
    "snac_unet_forward": (C.c_int, [FP, C.c_int, C.c_int, C.c_int, C.c_int, FP, FP]),
    "snac_unet_grad": (C.c_int, [FP, FP, C.c_int, C.c_int, C.c_int, C.c_int, FP, FP, DP]),
    "snac_unet_set_poll_limit": (C.c_int, [C.c_long]),
    "snac_guess_mode": (C.c_int, [C.c_int]),
    "snac_guess_train": (C.c_int, [C.c_int, C.c_double, DP, DP, IP]),
    "snac_guess_measure": (C.c_int, [C.c_int, DP, DP]),
    "snac_autotune": (C.c_int, [C.c_int, C.POINTER(TuneResult)]),
    "snac_tune_inject_failure": (C.c_int, [C.c_int]),
    "snac_set_fields": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_void_p)]),
    "snac_get_fields": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_void_p)]),
    "snac_out1d_write": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int]),
    "snac_out3d_write": (C.c_int, [C.c_char_p, C.c_int, C.c_int]),
    "snac_get_stats": (C.c_int, [C.POINTER(StepStats)]),
    "snac_set_dt": (C.c_int, [C.c_double]),
    "snac_get_dt": (C.c_int, [DP]),
}


def lib_path() -> str:
    return _build.LIB


def lib(build_if_missing: bool = True):
    """Load libsnac_gb300.so (compiling it in-tree first when absent); with SNAC_BOUNDS_CHECK=1 in the
    environment, the bounds-check build libsnac_gb300_checked.so instead."""
    global _lib
    if _lib is None:
        checked = os.environ.get("SNAC_BOUNDS_CHECK", "0") not in ("", "0")
        path = _build.LIB_CHECKED if checked else _build.LIB
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError(f"snac_gb300 extension not built: {path}")
            _build.build_checked() if checked else _build.build()
        L = C.CDLL(path)
        for name, (res, args) in PROTOTYPES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int):
    if rc != OK:
        raise SnacError(rc, lib().snac_last_error().decode())
    return rc


def dptr(a: np.ndarray):
    if a is None:
        return DP()
    assert a.dtype == np.float64, a.dtype
    assert a.flags["F_CONTIGUOUS"] or a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(DP)


def iarr(v, n=3):
    return (C.c_int * n)(*[int(x) for x in v])


def darr(v):
    v = list(v)
    return (C.c_double * len(v))(*[float(x) for x in v])


def device_count() -> int:
    n = C.c_int(0)
    rc = lib().snac_device_count(C.byref(n))
    return n.value if rc == OK else 0


def fill_descs(case):
    """snac_gb300.cases.Case -> (CaseDesc, BlockDesc array, kept arrays)."""
    nb = len(case.blocks)
    arr = (BlockDesc * nb)()
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
                d.grid_file[a] = g.ctypes.data_as(DP)
            else:
                d.grid_file[a] = DP()
    c = CaseDesc()
    c.nblocks = nb
    c.visci, c.cfl, c.dtmax, c.dt_f = case.visci, case.cfl, case.dtmax, case.dt_f
    for a in range(3):
        c.bforce[a] = case.bforce[a]
        c.gacc[a] = case.gacc[a]
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
