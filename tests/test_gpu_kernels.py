"""Per-routine parity of the CUDA kernels (reference-signature C ABI) against the oracle.

Random fields on one block with an uneven, non-unit-based index range and
random positive stretched spacings; every routine runs once on the oracle
and once through libsnac_gb300 on copies of the same arrays.  FP64 results
agree to rounding: the kernels replace divisions by reciprocal tables and use
FMAs, so the tolerance is a few ulps of the largest term (rtol 1e-12 of the
field's max magnitude).
"""
import ctypes as C

import numpy as np
import pytest

from snac_gb300 import capi, hotpath

pytestmark = pytest.mark.gpu

LO = (3, 5, 7)
N = (13, 9, 11)
HI = tuple(LO[a] + N[a] - 1 for a in range(3))


def P(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def I3(v):
    return (C.c_int * 3)(*v)


def metrics(rng):
    """dxc,dxf,dyc,dyf,dzc,dzf as (n+2) arrays of positive spacings (dc consistent with df as initgrid makes it)."""
    out = []
    for a in range(3):
        df = 0.5 + rng.random(N[a] + 2)
        dc = np.empty_like(df)
        dc[:-1] = 0.5 * (df[:-1] + df[1:])
        dc[-1] = dc[-2]
        out += [dc, df]
    return out


def field(rng, halo=True):
    shape = tuple(n + 2 for n in N) if halo else N
    return np.asfortranarray(rng.standard_normal(shape))


def close(a, b, rtol=1e-12):
    scale = max(np.max(np.abs(b)), 1e-300)
    np.testing.assert_allclose(a, b, rtol=0, atol=rtol * scale)


@pytest.mark.parametrize("impdiff,bouss", [(0, 0), (1, 0), (0, 1)])
def test_rk_mom(snac_lib, oracle_mod, impdiff, bouss):
    rng = np.random.default_rng(10 + impdiff + 2 * bouss)
    m = metrics(rng)
    u, v, w, p, s = (field(rng) for _ in range(5))
    ro = [field(rng, False) for _ in range(3)]
    rk = (25.0 / 60.0, -17.0 / 60.0)
    args = dict(dt=0.013, bforce=(0.3, -0.1, 0.2), gacc=(0.0, 0.5, -1.0), beta=0.7, visc=0.01)
    ref = [x.copy(order="F") for x in (u, v, w, *ro)]
    oracle_mod.lib().or_rk_mom(capi.darr(rk), I3(LO), I3(HI), *[P(x) for x in m], args["dt"], capi.darr(args["bforce"]),
                               capi.darr(args["gacc"]), args["beta"], P(s), args["visc"], *[P(x) for x in ref[:3]], P(p),
                               *[P(x) for x in ref[3:]], impdiff, bouss)
    got = [x.copy(order="F") for x in (u, v, w, *ro)]
    hotpath.rk_mom(rk, LO, HI, *m, args["dt"], args["bforce"], args["gacc"], args["beta"], s, args["visc"], *got[:3], p,
                   *got[3:], impdiff=impdiff, boussinesq=bouss)
    for g, r in zip(got, ref):
        close(g, r)


@pytest.mark.parametrize("impdiff", [0, 1])
def test_rk_scal(snac_lib, oracle_mod, impdiff):
    rng = np.random.default_rng(20 + impdiff)
    m = metrics(rng)
    u, v, w, s = (field(rng) for _ in range(4))
    ro = field(rng, False)
    rk = (32.0 / 60.0, 0.0)
    s_ref, ro_ref, f_ref = s.copy(order="F"), ro.copy(order="F"), C.c_double()
    oracle_mod.lib().or_rk_scal(capi.darr(rk), I3(LO), I3(HI), *[P(x) for x in m], 0.02, 0.003, 7.5, P(u), P(v), P(w), 1,
                                0.4, 0.05, P(ro_ref), P(s_ref), C.byref(f_ref), impdiff)
    s_got, ro_got = s.copy(order="F"), ro.copy(order="F")
    f = hotpath.rk_scal(rk, LO, HI, *m, 0.02, 0.003, 7.5, u, v, w, True, 0.4, 0.05, ro_got, s_got, impdiff=impdiff)
    close(s_got, s_ref)
    close(ro_got, ro_ref)
    assert abs(f - f_ref.value) <= 1e-12 * max(1.0, abs(f_ref.value))


@pytest.mark.parametrize("fft_axis", [0, 1, 2, 3])
def test_fillps(snac_lib, oracle_mod, fft_axis):
    rng = np.random.default_rng(30 + fft_axis)
    m = metrics(rng)
    u, v, w, pp = (field(rng) for _ in range(4))
    ref, got = pp.copy(order="F"), pp.copy(order="F")
    oracle_mod.lib().or_fillps(I3(LO), I3(HI), P(m[1]), P(m[3]), P(m[5]), 0.07, P(u), P(v), P(w), P(ref), fft_axis)
    hotpath.fillps(LO, HI, m[1], m[3], m[5], 0.07, u, v, w, got, fft_axis)
    close(got, ref)


def test_correc(snac_lib, oracle_mod):
    rng = np.random.default_rng(40)
    m = metrics(rng)
    u, v, w, pp = (field(rng) for _ in range(4))
    ref = [x.copy(order="F") for x in (u, v, w)]
    got = [x.copy(order="F") for x in (u, v, w)]
    oracle_mod.lib().or_correc(I3(LO), I3(HI), P(m[0]), P(m[2]), P(m[4]), 0.05, P(pp), *[P(x) for x in ref])
    hotpath.correc(LO, HI, m[0], m[2], m[4], 0.05, pp, *got)
    for g, r in zip(got, ref):
        close(g, r)


@pytest.mark.parametrize("impdiff", [0, 1])
def test_updt_pressure(snac_lib, oracle_mod, impdiff):
    rng = np.random.default_rng(50 + impdiff)
    m = metrics(rng)
    p, pp = field(rng), field(rng)
    ref, got = p.copy(order="F"), p.copy(order="F")
    oracle_mod.lib().or_updt_pressure(I3(LO), I3(HI), *[P(x) for x in m], -0.004, P(pp), P(ref), impdiff)
    hotpath.updt_pressure(LO, HI, *m, -0.004, pp, got, impdiff=impdiff)
    close(got, ref)


def test_updt_rhs(snac_lib, oracle_mod):
    rng = np.random.default_rng(60)
    p = field(rng)
    rx = np.asfortranarray(rng.standard_normal((N[1], N[2], 2)))
    ry = np.asfortranarray(rng.standard_normal((N[0], N[2], 2)))
    rz = np.asfortranarray(rng.standard_normal((N[0], N[1], 2)))
    isb = [[1, 0], [1, 1], [0, 1]]
    ref, got = p.copy(order="F"), p.copy(order="F")
    oracle_mod.lib().or_updt_rhs(I3(LO), I3(HI), (C.c_int * 6)(*[isb[a][s] for a in range(3) for s in range(2)]),
                                 P(rx), P(ry), P(rz), P(ref))
    hotpath.updt_rhs(LO, HI, isb, rx, ry, rz, got)
    close(got, ref, 1e-15)


def test_chkdt_chkdiv(snac_lib, oracle_mod):
    rng = np.random.default_rng(70)
    m = metrics(rng)
    u, v, w = (field(rng) for _ in range(3))
    dti, dlmin = C.c_double(), C.c_double()
    oracle_mod.lib().or_chkdt_local(I3(LO), I3(HI), *[P(x) for x in m], P(u), P(v), P(w), C.byref(dti), C.byref(dlmin))
    visc = 0.003
    dt_ref = min(np.sqrt(3.0) / dti.value, 1.65 / 12.0 / visc * dlmin.value ** 2)
    dt_got = hotpath.chkdt(LO, HI, *m, visc, u, v, w)
    assert abs(dt_got - dt_ref) <= 1e-13 * dt_ref
    tot, mx = C.c_double(), C.c_double()
    oracle_mod.lib().or_chkdiv_local(I3(LO), I3(HI), P(m[1]), P(m[3]), P(m[5]), P(u), P(v), P(w), 3.3, C.byref(tot),
                                     C.byref(mx))
    gt, gm = hotpath.chkdiv(LO, HI, m[1], m[3], m[5], u, v, w, 3.3)
    assert abs(gm - mx.value) <= 1e-13 * mx.value
    # the total is a sum of O(1) terms; compare against the sum of magnitudes
    assert abs(gt - tot.value) <= 1e-13 * np.prod(N)


@pytest.mark.parametrize("ctype,centered", [("D", 1), ("N", 1), ("D", 0), ("N", 0)])
@pytest.mark.parametrize("idir", [1, 2, 3])
@pytest.mark.parametrize("ib", [0, 1])
def test_set_bc(snac_lib, oracle_mod, ctype, centered, idir, ib):
    rng = np.random.default_rng(80 + idir)
    p = field(rng)
    ref, got = p.copy(order="F"), p.copy(order="F")
    oracle_mod.lib().or_set_bc(ctype.encode(), ib, I3(LO), I3(HI), idir, centered, 0.37, 0.11, P(ref))
    hotpath.set_bc(ctype, ib, LO, HI, idir, centered, 0.37, 0.11, got)
    np.testing.assert_array_equal(got, ref)


# bounduvw / boundp with the reference's argument lists: walls on some faces (D and N, both centrings), periodic
# self-neighbour directions exchanged on the device, and a face whose neighbour is another rank left alone
BOUND_CASES = {
    "walls_x_periodic_yz": dict(is_bound=[[1, 1], [0, 0], [0, 0]], nb=[[-1, -1], [0, 0], [0, 0]]),
    "walls_y_periodic_x_rank_z": dict(is_bound=[[0, 0], [1, 1], [0, 0]], nb=[[0, 0], [-1, -1], [3, 5]]),
    "box_walls": dict(is_bound=[[1, 1], [1, 1], [1, 1]], nb=[[-1, -1], [-1, -1], [-1, -1]]),
}


@pytest.mark.parametrize("case", sorted(BOUND_CASES))
@pytest.mark.parametrize("is_correc", [0, 1])
def test_bounduvw_boundp_block(snac_lib, oracle_mod, case, is_correc):
    rng = np.random.default_rng(170 + is_correc)
    cfg = BOUND_CASES[case]
    dxc, dxf, dyc, dyf, dzc, dzf = metrics(rng)
    kinds = "DN"
    cbc = [[[kinds[(c + d + s_) % 2] for s_ in range(2)] for d in range(3)] for c in range(3)]
    bc = rng.standard_normal((3, 3, 2))
    is_bound = np.array(cfg["is_bound"], dtype=np.int32)
    nb = np.array(cfg["nb"], dtype=np.int32)
    u, v, w = field(rng), field(rng), field(rng)
    ref = [a.copy(order="F") for a in (u, v, w)]
    got = [a.copy(order="F") for a in (u, v, w)]
    cb = hotpath._cbc(cbc)
    IP = C.POINTER(C.c_int)
    oracle_mod.lib().or_bounduvw_block(cb, I3(LO), I3(HI), P(np.ascontiguousarray(bc)), is_correc,
                                       is_bound.ctypes.data_as(IP), nb.ctypes.data_as(IP), 0, P(dxc), P(dxf),
                                       P(dyc), P(dyf), P(dzc), P(dzf), *(P(a) for a in ref))
    hotpath.bounduvw(cbc, LO, HI, bc, is_correc, is_bound, nb, 0, dxc, dxf, dyc, dyf, dzc, dzf, *got)
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g, r)
    # a face exchanged with another rank is untouched (the caller's MPI exchange)
    if nb[2][0] > 0:
        np.testing.assert_array_equal(got[0][1:-1, 1:-1, 0], u[1:-1, 1:-1, 0])
    p = field(rng)
    pref, pgot = p.copy(order="F"), p.copy(order="F")
    cbp = [row[:] for row in cbc[0]]
    bcp = np.ascontiguousarray(bc[0])
    oracle_mod.lib().or_boundp_block(hotpath._cbc(cbp), I3(LO), I3(HI), P(bcp), is_bound.ctypes.data_as(IP),
                                     nb.ctypes.data_as(IP), 0, P(dxc), P(dyc), P(dzc), P(pref))
    hotpath.boundp(cbp, LO, HI, bcp, is_bound, nb, 0, dxc, dyc, dzc, pgot)
    np.testing.assert_array_equal(pgot, pref)


def test_post_vorticity_strain_rotation_q(snac_lib, oracle_mod):
    """post.f90:8-156 on the device against the oracle: vorticity, strain and rotation rates, the Q criterion
    from the two rates and the one-pass Q criterion (the same expressions, so agreement to rounding)."""
    rng = np.random.default_rng(140)
    m = metrics(rng)  # dxc, dxf, dyc, dyf, dzc, dzf
    dxc, dxf, dyc, dyf, dzc, dzf = m
    u, v, w = (field(rng) for _ in range(3))
    n = I3(N)
    L, O = capi.lib(), oracle_mod.lib()
    ref = [np.zeros(N, order="F") for _ in range(6)]
    got = [np.zeros(N, order="F") for _ in range(7)]
    O.or_cmpt_vorticity(n, P(dxc), P(dyc), P(dzc), P(u), P(v), P(w), P(ref[0]), P(ref[1]), P(ref[2]))
    O.or_cmpt_strain_rate(n, P(dxc), P(dyc), P(dzc), P(dxf), P(dyf), P(dzf), P(u), P(v), P(w), P(ref[3]))
    O.or_cmpt_rotation_rate(n, P(dxc), P(dyc), P(dzc), P(u), P(v), P(w), P(ref[4]))
    O.or_cmpt_q_criterion(n, P(ref[4]), P(ref[3]), P(ref[5]))
    capi.check(L.snac_cmpt_vorticity(n, P(dxc), P(dyc), P(dzc), P(u), P(v), P(w), P(got[0]), P(got[1]), P(got[2])))
    capi.check(L.snac_cmpt_strain_rate(n, P(dxc), P(dyc), P(dzc), P(dxf), P(dyf), P(dzf), P(u), P(v), P(w),
                                       P(got[3])))
    capi.check(L.snac_cmpt_rotation_rate(n, P(dxc), P(dyc), P(dzc), P(u), P(v), P(w), P(got[4])))
    capi.check(L.snac_cmpt_q_criterion(n, P(got[4]), P(got[3]), P(got[5])))
    capi.check(L.snac_q_criterion(n, P(dxc), P(dyc), P(dzc), P(dxf), P(dyf), P(dzf), P(u), P(v), P(w), P(got[6])))
    for g, r in zip(got[:6], ref):
        close(g, r)
    close(got[6], ref[5])


@pytest.mark.parametrize("kind", ["R2HC", "HC2R", "REDFT10", "REDFT01", "REDFT11", "RODFT10", "RODFT01", "RODFT11",
                                  "REDFT00", "RODFT00"])
@pytest.mark.parametrize("idir,n", [(1, 8), (2, 12), (3, 16), (3, 128), (3, 2), (1, 96), (2, 160), (3, 256),
                                    (1, 15), (2, 7)])
def test_fft_kinds(snac_lib, oracle_mod, kind, idir, n):
    """fft.f90:85-94: every FFTW kind along every axis against the oracle's FFTW definitions: the radix-2 path
    (power-of-two R2HC/HC2R), the mixed-radix path (every kind whose complex length factors into 2, 3, 5:
    the DCTs and DSTs through symmetric extensions, odd and non-power-of-two lengths), and the dense path
    (n = 7: lengths 7 and 14 have a prime factor 7)."""
    if n == 2 and kind in ("REDFT00", "RODFT00"):
        pytest.skip("FFTW's REDFT00 needs n >= 2 points; covered at other sizes")
    rng = np.random.default_rng(90 + n + idir)
    shape = [5, 6, 7]
    shape[idir - 1] = n
    a = np.asfortranarray(rng.standard_normal(shape))
    ref = a.copy(order="F")
    O = oracle_mod
    st = [1, shape[0], shape[0] * shape[1]]
    t1, t2 = [x for x in range(3) if x != idir - 1]
    for l2 in range(shape[t2]):
        for l1 in range(shape[t1]):
            base = ref.reshape(-1, order="F")[l1 * st[t1] + l2 * st[t2]::st[idir - 1]][:n].copy()
            out = O.r2r(getattr(O, kind), base)
            flat = ref.reshape(-1, order="F")
            idx = l1 * st[t1] + l2 * st[t2] + np.arange(n) * st[idir - 1]
            flat[idx] = out
    got = a.copy(order="F")
    hotpath.fft(getattr(capi, kind), idir, got)
    close(got, ref, 1e-12 * n)


def test_find_fft_and_eigenvalues(snac_lib, oracle_mod):
    for bc in ("FF", "NN", "DD", "ND", "DN"):
        for cen in (0, 1):
            kf, kb, norm = hotpath.find_fft(bc, cen)
            okf, okb, onorm = oracle_mod.find_fft(bc, cen)
            assert (kf, kb) == (okf, okb) and np.array_equal(norm, onorm)
    for bc in ("FF", "NN", "DD", "ND"):
        np.testing.assert_allclose(hotpath.eigenvalues(16, bc, 1), oracle_mod.eigenvalues(16, bc, True), rtol=0, atol=1e-15)


def test_registered_mirrors(snac_lib, oracle_mod):
    """Registered arrays are used in place on the device; the host copy changes only on snac_update_host."""
    rng = np.random.default_rng(100)
    m = metrics(rng)
    p, pp = field(rng), field(rng)
    L = capi.lib()
    capi.check(L.snac_register(p.ctypes.data, p.nbytes))
    try:
        before = p.copy(order="F")
        hotpath.updt_pressure(LO, HI, *m, 0.0, pp, p)
        np.testing.assert_array_equal(p, before)     # host untouched
        capi.check(L.snac_update_host(p.ctypes.data))
        ref = before.copy(order="F")
        oracle_mod.lib().or_updt_pressure(I3(LO), I3(HI), *[P(x) for x in m], 0.0, P(pp), P(ref), 0)
        close(p, ref)
    finally:
        capi.check(L.snac_unregister(p.ctypes.data))


def test_open_and_outflow_bcs(snac_lib, oracle_mod):
    """bound.f90:250-541 on the device against the oracle: every face of the estimated-traction and zero-traction
    open BC on the wall-normal velocity, the traction estimate alone, the traction BC on the correction pressure,
    and the outflow / outflow_p drivers over all six faces (the same operations in the same order, no FMA
    contraction on either side: bit-identical)."""
    rng = np.random.default_rng(210)
    L, O = capi.lib(), oracle_mod.lib()
    IP = C.POINTER(C.c_int)
    nh = [n + 2 for n in N]

    def planes(ax):
        t1, t2 = [q for q in range(3) if q != ax]
        return np.asfortranarray(rng.standard_normal((nh[t1], nh[t2], 2)))

    for idir in (1, 2, 3):
        for ib in (0, 1):
            u, v, w, p = field(rng), field(rng), field(rng), field(rng)
            tr = planes(idir - 1)
            ref = [a.copy(order="F") for a in (u, v, w, tr)]
            got = [a.copy(order="F") for a in (u, v, w, tr)]
            O.or_set_open_bc_uvw(ib, I3(LO), I3(HI), idir, 1e-3, 0.3, *(P(a) for a in ref[:3]), P(p), P(ref[3]))
            assert L.snac_set_open_bc_uvw(ib, I3(LO), I3(HI), idir, 1e-3, 0.3, *(P(a) for a in got[:3]), P(p),
                                          P(got[3])) == 0, L.snac_last_error()
            for g, r in zip(got, ref):
                np.testing.assert_array_equal(g, r)
            t_ref, t_got = tr.copy(order="F"), tr.copy(order="F")
            O.or_cmpt_estimated_traction(ib, I3(LO), I3(HI), idir, 2e-3, 0.7, P(u), P(v), P(w), P(p), P(t_ref))
            assert L.snac_cmpt_estimated_traction(ib, I3(LO), I3(HI), idir, 2e-3, 0.7, P(u), P(v), P(w), P(p),
                                                  P(t_got)) == 0, L.snac_last_error()
            np.testing.assert_array_equal(t_got, t_ref)
            drc = np.array([0.4, 0.55])
            p_ref, p_got = p.copy(order="F"), p.copy(order="F")
            O.or_set_open_bc_p(ib, I3(LO), I3(HI), idir, P(drc), 0.45, 3.0, P(p_ref))
            assert L.snac_set_open_bc_p(ib, I3(LO), I3(HI), idir, P(drc), 0.45, 3.0, P(p_got)) == 0
            np.testing.assert_array_equal(p_got, p_ref)
    mask = np.array([[1, 1], [0, 1], [1, 0]], dtype=np.int32)
    est = np.array([[1, 0], [0, 1], [1, 1]], dtype=np.int32)
    dl, dl_h = rng.random((3, 2)) + 0.1, rng.random((3, 2)) + 0.1
    dlc, dlf = rng.random((3, 2, 2)) + 0.1, rng.random((3, 2)) + 0.1
    u, v, w, p = field(rng), field(rng), field(rng), field(rng)
    trs = [planes(ax) for ax in range(3)]
    ref = [a.copy(order="F") for a in (u, v, w, p, *trs)]
    got = [a.copy(order="F") for a in (u, v, w, p, *trs)]
    O.or_outflow(mask.ctypes.data_as(IP), est.ctypes.data_as(IP), I3(LO), I3(HI), P(dl), P(dl_h), 1.5e-3,
                 *(P(a) for a in ref))
    assert L.snac_outflow(mask.ctypes.data_as(IP), est.ctypes.data_as(IP), I3(LO), I3(HI), P(dl), P(dl_h), 1.5e-3,
                          *(P(a) for a in got)) == 0, L.snac_last_error()
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g, r)
    O.or_outflow_p(mask.ctypes.data_as(IP), I3(LO), I3(HI), P(dlc), P(dlf), 2.0, P(ref[3]))
    assert L.snac_outflow_p(mask.ctypes.data_as(IP), I3(LO), I3(HI), P(dlc), P(dlf), 2.0, P(got[3])) == 0
    np.testing.assert_array_equal(got[3], ref[3])
