"""param.f90:88-240 on the host: snac_read_namelists fills snac_case / snac_block_desc from dns.nml and
blocks.nml as the reference reads them (defaults, array sections in Fortran order, repeat counts,
logicals, comments).  No device is needed."""
import ctypes as C

import numpy as np
import pytest

from snac_gb300 import capi, cases


def _fmt(v):
    if isinstance(v, str):
        return f"'{v}'"
    return repr(float(v)) if isinstance(v, float) else str(v)


def write_namelists(case, dirpath, style=0):
    """dns.nml / blocks.nml for a case; style varies the namelist syntax the reader must accept."""
    nb = len(case.blocks)
    d = ["&dns ! global parameters",
         f"cfl = {case.cfl}, dtmax = {case.dtmax}, dt_f = {case.dt_f}",
         f"visci = {case.visci}",
         "nstep = 100, time_max = 10., tw_max = 0.1",
         "stop_type(1:3) = T, F, F",
         "restart = .false., is_overwrite_save = T, nsaves_max = 0",
         f"icheck = {case.icheck}, iout0d = 10, iout1d = 20, iout2d = 0, iout3d = 100, isave = 1000",
         "bforce(1:3) = " + ", ".join(repr(float(x)) for x in case.bforce),
         "gacc = " + ", ".join(repr(float(x)) for x in case.gacc),
         f"nscal = {case.nscal}", "/", ""]
    if case.nscal:
        d += ["&scalar",
              "alphai(1:%d) = " % case.nscal + ", ".join(repr(float(x)) for x in case.alphai[:case.nscal]),
              f"beta = {case.beta}",
              "iniscal = " + ", ".join("'zer'" for _ in range(case.nscal)),
              "ssource = " + ", ".join(repr(float(x)) for x in case.ssource[:case.nscal]),
              "is_sforced = " + ", ".join(".true." if x else ".false." for x in case.is_sforced[:case.nscal]),
              "scalf = " + ", ".join(repr(float(x)) for x in case.scalf[:case.nscal]), "/", ""]
    d += ["&hypre", f"hypre_solver_i = 2, hypre_tol = {case.tol}, hypre_maxiter = {case.maxiter}", "/"]
    b = ["&blocks", f"nblocks = {nb}"]
    for ib, blk in enumerate(case.blocks, start=1):
        b.append(f"block_dims(1:3,{ib}) = 1, 1, 1")
        if style == 0:
            b.append(f"block_ng(1:3,{ib}) = " + ", ".join(str(x) for x in blk.ng))
        else:
            b.append(f"block_ng (1:3, {ib}) = " + ", ".join(str(x) for x in blk.ng))
        b.append(f"block_lmin(1:3,{ib}) = " + ", ".join(repr(float(x)) for x in blk.lmin))
        b.append(f"block_lmax(1:3,{ib}) = " + ", ".join(repr(float(x)) for x in blk.lmax))
        b.append(f"block_gt(1:3,{ib}) = " + ", ".join(str(x) for x in blk.gt))
        b.append(f"block_gr(1:3,{ib}) = " + ", ".join(repr(float(x)) for x in blk.gr))
        for c in range(3):
            b.append(f"block_cbcvel(0:1,1:3,{c + 1},{ib}) = " +
                     ", ".join(f"'{blk.cbcvel[c][a][s]}'" for a in range(3) for s in range(2)))
            vals = [float(blk.bcvel[c][a][s]) for a in range(3) for s in range(2)]
            if style == 1 and all(v == 0.0 for v in vals):
                b.append(f"block_bcvel(0:1,1:3,{c + 1},{ib}) = 6*0.d0")
            else:
                b.append(f"block_bcvel(0:1,1:3,{c + 1},{ib}) = " + ", ".join(repr(v) for v in vals))
        b.append(f"block_cbcpre(0:1,1:3,{ib}) = " + ", ".join(f"'{blk.cbcpre[a][s]}'" for a in range(3) for s in range(2)))
        b.append(f"block_bcpre(0:1,1:3,{ib}) = " + ", ".join(repr(float(blk.bcpre[a][s])) for a in range(3) for s in range(2)))
        for q in range(case.nscal):
            b.append(f"block_cbcscal(0:1,1:3,{q + 1},{ib}) = " +
                     ", ".join(f"'{blk.cbcscal[q][a][s]}'" for a in range(3) for s in range(2)))
            b.append(f"block_bcscal(0:1,1:3,{q + 1},{ib}) = " +
                     ", ".join(repr(float(blk.bcscal[q][a][s])) for a in range(3) for s in range(2)))
        b.append(f"block_inflow_type(0:1,1:3,{ib}) = " + ", ".join(str(blk.inflow_type[a][s]) for a in range(3) for s in range(2)))
        b.append(f"block_inivel({ib}) = 'zer' ! initial velocity")
    b.append("/")
    (dirpath / "dns.nml").write_text("\n".join(d) + "\n")
    (dirpath / "blocks.nml").write_text("\n".join(b) + "\n")


@pytest.mark.parametrize("which,style", [("channel", 0), ("channel_scalar", 1), ("lbox", 1), ("kovasznay", 0),
                                         ("dhc", 0)])
def test_read_namelists_matches_case(tmp_path, which, style):
    case = {"channel": lambda: cases.channel_4block(), "channel_scalar": lambda: cases.channel_4block_scalar(),
            "lbox": lambda: cases.l_shaped_box(n=16, nz=8), "kovasznay": lambda: cases.kovasznay(),
            "dhc": lambda: cases.dhc_reference_test()}[which]()
    write_namelists(case, tmp_path, style)
    want_c, want_b, _ = capi.fill_descs(case)
    got_c = capi.CaseDesc()
    got_b = (capi.BlockDesc * 8)()
    rc = capi.lib().snac_read_namelists(str(tmp_path / "dns.nml").encode(), str(tmp_path / "blocks.nml").encode(),
                                        case.fft_axis, case.impdiff, case.boussinesq, C.byref(got_c), got_b, 8)
    assert rc == 0, capi.lib().snac_last_error()
    for name, _ in capi.CaseDesc._fields_:
        a, b = getattr(got_c, name), getattr(want_c, name)
        if hasattr(a, "__len__"):
            n = case.nscal if name in ("alphai", "ssource", "scalf", "is_sforced") else len(a)
            assert list(a)[:n] == list(b)[:n], name
        else:
            assert a == b, name
    for ib in range(len(case.blocks)):
        for name, _ in capi.BlockDesc._fields_:
            if name == "grid_file":
                continue
            a = np.array(getattr(got_b[ib], name)).ravel()
            b = np.array(getattr(want_b[ib], name)).ravel()
            if name in ("cbcscal", "bcscal"):
                a, b = a[:6 * case.nscal], b[:6 * case.nscal]
            assert a.tolist() == b.tolist(), (ib, name)


def test_read_namelists_defaults_and_errors(tmp_path):
    (tmp_path / "dns.nml").write_text("&dns\ncfl = 0.5, dtmax = 1.e5\nicheck = 10\n/\n")
    (tmp_path / "blocks.nml").write_text("&blocks\nnblocks = 1\nblock_ng(1:3,1) = 8, 8, 8\n/\n")
    c = capi.CaseDesc()
    b = (capi.BlockDesc * 2)()
    L = capi.lib()
    assert L.snac_read_namelists(str(tmp_path / "dns.nml").encode(), str(tmp_path / "blocks.nml").encode(),
                                 0, 0, 0, C.byref(c), b, 2) == 0
    assert c.visci == 1.0 and c.dt_f == -1.0 and c.nscal == 0            # param.f90:108-114
    assert c.tol == float(np.float32(1e-4)) and c.maxiter == 50        # hypre defaults, param.f90:15-17
    assert bytes(b[0].cbcvel[0][0]) == b"DD" and bytes(b[0].cbcpre[2]) == b"NN"  # param.f90:125-126
    assert list(b[0].lmax) == [1.0, 1.0, 1.0] and list(b[0].ng) == [8, 8, 8]
    # _BOUSSINESQ_BUOYANCY without scalars is an input error (param.f90:155-162)
    assert L.snac_read_namelists(str(tmp_path / "dns.nml").encode(), str(tmp_path / "blocks.nml").encode(),
                                 0, 0, 1, C.byref(c), b, 2) == capi.ERR_ARG
    assert L.snac_read_namelists(str(tmp_path / "nope.nml").encode(), str(tmp_path / "blocks.nml").encode(),
                                 0, 0, 0, C.byref(c), b, 2) == capi.ERR_IO
