"""Oracle building blocks against independent definitions (numpy / scipy)."""
import numpy as np
import pytest
import scipy.fft as sfft

from snac_gb300 import cases


def test_r2hc_matches_numpy(oracle_mod):
    O = oracle_mod
    rng = np.random.default_rng(1)
    for n in (1, 2, 5, 8, 16, 33):
        x = rng.standard_normal(n)
        y = O.r2r(O.R2HC, x)
        X = np.fft.rfft(x)
        hc = np.zeros(n)
        hc[: n // 2 + 1] = X.real
        for k in range(1, (n + 1) // 2):
            hc[n - k] = X[k].imag
        np.testing.assert_allclose(y, hc, atol=1e-12 * max(1, n))
        np.testing.assert_allclose(O.r2r(O.HC2R, y), n * x, atol=1e-11 * n)


@pytest.mark.parametrize("kind,stype,sk", [("REDFT10", "dct", 2), ("REDFT01", "dct", 3), ("REDFT11", "dct", 4),
                                           ("RODFT10", "dst", 2), ("RODFT01", "dst", 3), ("RODFT11", "dst", 4),
                                           ("REDFT00", "dct", 1), ("RODFT00", "dst", 1)])
def test_dct_dst_match_scipy(oracle_mod, kind, stype, sk):
    """FFTW's unnormalised kinds equal scipy's type-1..4 DCT/DST with norm=None."""
    O = oracle_mod
    rng = np.random.default_rng(2)
    for n in (2, 3, 8, 12):
        x = rng.standard_normal(n)
        y = O.r2r(getattr(O, kind), x)
        ref = (sfft.dct if stype == "dct" else sfft.dst)(x, type=sk)
        np.testing.assert_allclose(y, ref, atol=1e-11 * n)


@pytest.mark.parametrize("bc", ["FF", "NN", "DD", "ND"])
def test_eigenvalues_diagonalise_1d_operator(oracle_mod, bc):
    """fft.f90:151-189: the modified wavenumbers of the centred 1-D operator with the BC folding of solver.f90."""
    O = oracle_mod
    n = 12
    lam = O.eigenvalues(n, bc, True)
    # 1-D operator with unit spacing, folded boundaries (N: +1, centred D: -1) or periodic
    A = np.zeros((n, n))
    for i in range(n):
        A[i, i] = -2.0
        if i > 0: A[i, i - 1] = 1.0
        if i < n - 1: A[i, i + 1] = 1.0
    if bc == "FF":
        A[0, -1] = A[-1, 0] = 1.0
    else:
        s = {"N": 1.0, "D": -1.0}
        A[0, 0] += s[bc[0]]
        A[-1, -1] += s[bc[1]]
    ev = np.sort(np.linalg.eigvalsh(A))
    np.testing.assert_allclose(np.sort(lam), ev, atol=1e-12)


def test_dn_pair_has_no_eigenvalues(oracle_mod):
    """The reference's eigenvalues() has no 'DN' case (fft.f90:159-188)."""
    with pytest.raises(ValueError):
        oracle_mod.eigenvalues(8, "DN", True)


def test_initgrid_matches_python(oracle_mod):
    import ctypes as C
    O = oracle_mod
    n = 40
    drc, drf, rc, rf = (np.zeros(n + 2) for _ in range(4))
    P = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    O.lib().or_initgrid(1, n, 0, 1.8, 0.0, 2.0, P(drc), P(drf), P(rc), P(rf))
    g = cases.global_axis_grid(n, 0.0, 2.0, 1.8)
    np.testing.assert_allclose(rf, g[0], rtol=0, atol=1e-15)
    np.testing.assert_allclose(drf, g[2], rtol=0, atol=1e-15)
    np.testing.assert_allclose(drc, g[3], rtol=0, atol=1e-15)


def test_block_placement_channel(oracle_mod):
    d = oracle_mod.OracleDomain(cases.channel_4block(nx=(8, 16), ny=(4, 8), nz=8))
    assert [g["lo"] for g in d.geom] == [(1, 1, 1), (9, 1, 1), (1, 5, 1), (9, 5, 1)]
    assert d.geom[0]["nb"] == [[1, 1], [-1, 2], [0, 0]]
    assert d.geom[3]["is_bound"] == [[0, 0], [0, 1], [0, 0]]


def test_bad_connectivity_rejected(oracle_mod):
    c = cases.ldc_reference_test()
    c.blocks[0].bcpre[1][1] = 3.0  # y+ friend of block 1 points at block 3, which does not point back
    with pytest.raises(RuntimeError):
        oracle_mod.OracleDomain(c)


def test_oracle_solver_exact_on_manufactured(oracle_mod):
    """A divergence-free projection: after one pressure solve + correction the divergence vanishes."""
    O = oracle_mod
    d = O.OracleDomain(cases.lid_driven_cavity(16))
    rng = np.random.default_rng(3)
    for k in (O.U, O.V, O.W):
        f = d.field(0, k)
        f[...] = rng.standard_normal(f.shape)
    d.bounduvw(False)
    O.lib().or_fillps_all(d.h, 0.1)
    O.lib().or_updt_rhs_all(d.h)
    O.lib().or_solve_pressure(d.h)
    d.boundp(O.PP)
    O.lib().or_correc_all(d.h, 0.1)
    d.bounduvw(True)
    assert d.chkdiv()[1] < 1e-9


def test_oracle_impdiff_matches_explicit_small_dt(oracle_mod):
    """IMPDIFF (Crank-Nicolson diffusion through the Helmholtz solves) and explicit RK3 diffusion are two
    discretisations of the same equations: at a small dt their solutions differ at second order in dt.
    Checks the BC planes, the staggered extents hif and the shift of the oracle's Helmholtz problems."""
    from snac_gb300 import capi
    out = {}
    for imp in (0, 1):
        case = cases.heated_cavity(n=(12, 12, 8), stretch=1.2, ra=1e5, impdiff=imp, tol=1e-13, dt_f=1e-5)
        O = oracle_mod.OracleDomain(case)
        try:
            s0 = cases.dhc_initial_scalar(case, lambda ib: O.grid(ib, 0, oracle_mod.G_XC))
            O.field(0, capi.S0)[...] = s0[0]
            O.bounduvw(False)
            O.boundp(capi.P)
            O.boundp(capi.S0)
            O.step(10)
            out[imp] = {k: O.field(0, k)[1:-1, 1:-1, 1:-1].copy() for k in (capi.U, capi.W, capi.S0)}
        finally:
            O.close()
    for k in out[0]:
        a, b = out[0][k], out[1][k]
        assert np.max(np.abs(a)) > 0
        assert np.max(np.abs(a - b)) <= 1e-6 * np.max(np.abs(a)), k


@pytest.mark.parametrize("which", ["duct", "kovasznay"])
def test_oracle_inflow_planes(oracle_mod, which):
    """init_inflow (initflow.f90:369-429) and inflow (bound.f90:438-477), restated in numpy: the normal
    component on the inflow face, the tangential ones mirrored about the inflow value into the ghost."""
    from snac_gb300 import capi
    case = cases.developing_duct() if which == "duct" else cases.kovasznay()
    O = oracle_mod.OracleDomain(case)
    try:
        rng = np.random.default_rng(4)
        for k in (capi.U, capi.V, capi.W):
            O.field(0, k)[...] = rng.standard_normal(O.field(0, k).shape)
        O.bounduvw(False)
        O.inflow(False)
        b = case.blocks[0]
        yc = O.grid(0, 1, oracle_mod.G_XC)
        zc, zf = O.grid(0, 2, oracle_mod.G_XC), O.grid(0, 2, oracle_mod.G_XF)
        if which == "duct":
            def pois(r, l0, l1):
                rr = (r - l0) / (l1 - l0)
                return 6.0 * (rr * (1.0 - rr))
            un = (1.0 * pois(yc, b.lmin[1], b.lmax[1]))[:, None] * pois(zc, b.lmin[2], b.lmax[2])[None, :]
            vt = np.zeros_like(un)
            wt = np.zeros_like(un)
        else:
            reb = 1.0 * 1.0 / (1.0 / case.visci)
            lam = reb / 2 - np.sqrt(reb * reb / 4 + 4 * (np.pi * np.pi))
            un = np.broadcast_to(1.0 - np.exp(lam * -0.5) * np.cos(2 * np.pi * zc)[None, :], (len(yc), len(zc)))
            vt = np.zeros_like(un)
            wt = np.broadcast_to(lam / (2 * np.pi) * np.exp(lam * -0.5) * np.sin(2 * np.pi * zf)[None, :], un.shape)
        u, v, w = (O.field(0, k) for k in (capi.U, capi.V, capi.W))
        np.testing.assert_allclose(u[0], un, rtol=1e-14, atol=1e-14)
        np.testing.assert_allclose(v[0], -v[1] + 2.0 * vt, rtol=1e-14, atol=1e-14)
        np.testing.assert_allclose(w[0], -w[1] + 2.0 * wt, rtol=1e-14, atol=1e-14)
        # is_correc leaves the normal component alone
        u[0] = 7.0
        O.inflow(True)
        assert np.all(u[0] == 7.0)
    finally:
        O.close()


@pytest.mark.parametrize("which", ["ldc_x", "channel_z"])
def test_oracle_impdiff_fft_matches_3d(oracle_mod, which):
    """solve_impdiff_field_fft and solve_impdiff_field_3d solve the same discrete Helmholtz problems where
    the transform axis is uniform: the field's own transform (the staggered kinds and eigenvalues along a
    wall-bounded axis for LDC along x, the periodic ones for the channel along z) diagonalises it exactly,
    so whole IMPDIFF steps agree to the solver tolerance."""
    import dataclasses
    from snac_gb300 import capi

    def run(case):
        O = oracle_mod.OracleDomain(case)
        try:
            rng = np.random.default_rng(3)
            for ib in range(len(case.blocks)):
                for k in (capi.U, capi.V, capi.W, capi.P):
                    f = O.field(ib, k)
                    f[...] = 0.1 * rng.standard_normal(f.shape)
            O.bounduvw(False)
            O.boundp(capi.P)
            O.step(3)
            return [[O.field(ib, k)[1:-1, 1:-1, 1:-1].copy() for k in (capi.U, capi.V, capi.W)]
                    for ib in range(len(case.blocks))]
        finally:
            O.close()

    if which == "ldc_x":
        mk = lambda fa: cases.ldc_reference_test(fft_axis=fa)
        fa = 1
    else:
        mk = lambda fa: dataclasses.replace(cases.channel_4block(nx=(16, 32), ny=(8, 16), nz=16), fft_axis=fa)
        fa = 3
    a = run(dataclasses.replace(mk(0), impdiff=1, dt_f=2e-3, tol=1e-13))
    b = run(dataclasses.replace(mk(fa), impdiff=1, dt_f=2e-3, tol=1e-13))
    for fa_, fb_ in zip(a, b):
        for x, y in zip(fa_, fb_):
            assert np.max(np.abs(x - y)) <= 1e-11 * np.max(np.abs(x))


def test_oracle_checkpoint_format(oracle_mod, tmp_path):
    """load_one (load.f90:92-160): each file is the block's interior in Fortran order followed by
    [time, istep] in FP64; loading restores the interiors exactly and rejects a file of the wrong size."""
    from snac_gb300 import capi
    case = cases.channel_4block_scalar()
    O = oracle_mod.OracleDomain(case)
    O2 = oracle_mod.OracleDomain(case)
    try:
        rng = np.random.default_rng(12)
        for ib in range(len(case.blocks)):
            for k in (capi.U, capi.V, capi.W, capi.P, capi.S0):
                O.field(ib, k)[...] = rng.standard_normal(O.field(ib, k).shape)
        O.bounduvw(False)
        O.step(1)
        prefix = str(tmp_path / "fld")
        O.checkpoint_save(prefix)
        t, istep = O.time_istep
        assert istep == 1
        for ib, b in enumerate(case.blocks):
            for k, tag in ((capi.U, "u"), (capi.V, "v"), (capi.W, "w"), (capi.P, "p"), (capi.S0, "s_001")):
                raw = np.fromfile(f"{prefix}_b_{ib + 1:03d}_{tag}.bin", dtype=np.float64)
                n = int(np.prod(b.ng))
                assert raw.size == n + 2
                interior = O.field(ib, k)[1:-1, 1:-1, 1:-1]
                np.testing.assert_array_equal(raw[:n].reshape(tuple(b.ng), order="F"), interior)
                assert raw[n] == t and raw[n + 1] == float(istep)
        O2.checkpoint_load(prefix)
        assert O2.time_istep == (t, istep)
        for ib in range(len(case.blocks)):
            for k in (capi.U, capi.V, capi.W, capi.P, capi.S0):
                np.testing.assert_array_equal(O2.field(ib, k)[1:-1, 1:-1, 1:-1], O.field(ib, k)[1:-1, 1:-1, 1:-1])
        with open(f"{prefix}_b_002_v.bin", "ab") as f:
            f.write(b"\0" * 8)
        with pytest.raises(IOError):
            O2.checkpoint_load(prefix)
    finally:
        O.close()
        O2.close()


def test_fortran_e15_7_format(oracle_mod):
    """output.f90 writes profiles with '(2E15.7)': 0.ddddddd mantissa, E+ee exponent, 15 columns."""
    f = oracle_mod.fortran_e15_7
    assert f(1.0) == "  0.1000000E+01"
    assert f(-2.5e-3) == " -0.2500000E-02"
    assert f(0.0) == "  0.0000000E+00"
    assert f(123456789.0) == "  0.1234568E+09"
    assert f(9.99999996) == "  0.1000000E+02"   # rounding carries into the exponent
    assert f(1.5e-120) == "  0.1500000-119"   # three exponent digits drop the E
    rng = np.random.default_rng(0)
    for v in rng.standard_normal(200) * 10.0 ** rng.integers(-30, 30, 200):
        s = f(v)
        assert len(s) == 15
        assert abs(float(s.replace("E", "e")) - v) <= 5.1e-7 * abs(v)  # 7 significant digits


def test_oracle_out1d_matches_numpy(oracle_mod, tmp_path):
    """out1d (output.f90:34-125): plane averages with the field's spacings (out1d.h90) over the block
    lengths, against a numpy restatement, and the text file they are written to."""
    from snac_gb300 import capi
    case = cases.channel_4block(nx=(16, 32), ny=(8, 16), nz=16)
    O = oracle_mod.OracleDomain(case)
    try:
        rng = np.random.default_rng(14)
        for k in (capi.U, capi.V, capi.W, capi.P):
            O.field(1, k)[...] = rng.standard_normal(O.field(1, k).shape)
        b = case.blocks[1]
        l = [b.lmax[a] - b.lmin[a] for a in range(3)]
        for k in (capi.U, capi.V, capi.W, capi.P):
            stag = [k - capi.U == a if k <= capi.W else False for a in range(3)]
            dl = [O.grid(1, a, oracle_mod.G_DXC if stag[a] else oracle_mod.G_DXF)[1:-1] for a in range(3)]
            xg = [O.grid(1, a, oracle_mod.G_XF if stag[a] else oracle_mod.G_XC)[1:-1] for a in range(3)]
            f = O.field(1, k)[1:-1, 1:-1, 1:-1]
            for idir in (1, 2, 3):
                x, p = O.out1d(1, k, idir, fname=tmp_path / f"p{k}{idir}.out")
                t = [a for a in range(3) if a != idir - 1]
                wa = dl[t[0]].reshape([-1 if a == t[0] else 1 for a in range(3)])
                wb = dl[t[1]].reshape([-1 if a == t[1] else 1 for a in range(3)])
                ref = (f * wa * wb / (l[t[0]] * l[t[1]])).sum(axis=tuple(t))
                np.testing.assert_allclose(p, ref, rtol=1e-12, atol=1e-14)
                np.testing.assert_array_equal(x, xg[idir - 1])
                lines = open(tmp_path / f"p{k}{idir}.out").read().splitlines()
                assert len(lines) == len(p) and all(len(s) == 30 for s in lines)
                vals = np.array([[float(s[:15]), float(s[15:])] for s in lines])
                np.testing.assert_allclose(vals[:, 1], p, rtol=1e-6, atol=1e-7 * np.max(np.abs(p)))
    finally:
        O.close()
