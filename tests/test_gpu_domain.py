"""Domain-level parity on the GPU: every block resident in HBM against the oracle.

Covers the multi-block halo exchange and boundary conditions (bit-identical
copies), the Poisson solve (FP64 and FP32-in-FP64), and whole RK3 steps on
the reference's LDC test layout (3-D solve and FFT along x), the Taylor-Green
vortex (FFT along z) and the uneven four-block channel.  The reference's own
golden vector is checked with the reference's tolerance.
"""
import ctypes as C
import dataclasses
import os

import numpy as np
import pytest

from snac_gb300 import capi, cases
from snac_gb300.domain import Domain

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ldc_re1000_profile.txt")


def seed_fields(case, oracle_dom, dom, seed=0, amp=1.0):
    """Same random velocity/pressure on both sides (then the reference's initial bounduvw/boundp)."""
    O = oracle_dom
    rng = np.random.default_rng(seed)
    for ib in range(len(case.blocks)):
        for k in (capi.U, capi.V, capi.W, capi.P):
            f = O.field(ib, k)
            f[...] = amp * rng.standard_normal(f.shape)
            dom.set(ib, k, f)


def weighted_mean_free(p, ib, grid):
    dxf, dyf, dzf = (grid(ib, a)[1:-1] for a in range(3))
    w = dxf[:, None, None] * dyf[None, :, None] * dzf[None, None, :]
    return w


def compare_fields(case, O, dom, kinds, rtol, mean_free_p=False):
    worst = 0.0
    if mean_free_p:
        num = den = 0.0
        numo = 0.0
        for ib in range(len(case.blocks)):
            w = weighted_mean_free(None, ib, lambda b, a: O.grid(b, a, 1))
            num += np.sum(w * dom.get(ib, capi.P)[1:-1, 1:-1, 1:-1])
            numo += np.sum(w * O.field(ib, capi.P)[1:-1, 1:-1, 1:-1])
            den += np.sum(w)
        mg, mo = num / den, numo / den
    for ib in range(len(case.blocks)):
        for k in kinds:
            g = dom.get(ib, k)[1:-1, 1:-1, 1:-1] if k != capi.DUDTRKO else dom.get(ib, k)
            r = O.field(ib, k)[1:-1, 1:-1, 1:-1] if k != capi.DUDTRKO else O.field(ib, k)
            if k == capi.P and mean_free_p:
                g = g - mg
                r = r - mo
            scale = max(np.max(np.abs(r)), 1e-300)
            err = np.max(np.abs(g - r)) / scale
            worst = max(worst, err)
            assert err <= rtol, (ib, k, err)
    return worst


@pytest.fixture
def ldc3d(snac_lib, oracle_mod):
    case = cases.ldc_reference_test(fft_axis=0)
    O = oracle_mod.OracleDomain(case)
    d = Domain(case)
    yield case, O, d
    d.close()


def test_geometry_matches_oracle(ldc3d):
    case, O, d = ldc3d
    for ib in range(len(case.blocks)):
        assert d.geom[ib] == O.geom[ib]
        for a in range(3):
            for w in range(4):
                np.testing.assert_array_equal(d.grid(ib, a, w), O.grid(ib, a, w))


def test_bound_exchange_and_bc_bitwise(ldc3d):
    """bound.f90:8-106 on four blocks: ghost planes, edges and corners equal the oracle's exactly."""
    case, O, d = ldc3d
    seed_fields(case, O, d, seed=1)
    for is_correc in (False, True):
        O.bounduvw(is_correc)
        d.bounduvw(is_correc)
        for ib in range(4):
            for k in (capi.U, capi.V, capi.W):
                np.testing.assert_array_equal(d.get(ib, k), O.field(ib, k))
    O.boundp(capi.P)
    d.boundp(capi.P)
    for ib in range(4):
        np.testing.assert_array_equal(d.get(ib, capi.P), O.field(ib, capi.P))


@pytest.mark.parametrize("precision", [0, 1])
def test_solve_pressure_matches_oracle(snac_lib, oracle_mod, precision):
    """fillps + updt_rhs + solve + boundp on the four-block channel (FFT along z, stretched y)."""
    case = cases.channel_4block(nx=(16, 32), ny=(8, 16), nz=16)
    O = oracle_mod.OracleDomain(case)
    d = Domain(case, precision=precision)
    try:
        seed_fields(case, O, d, seed=2)
        O.bounduvw(False)
        d.bounduvw(False)
        L = oracle_mod.lib()
        L.or_fillps_all(O.h, 0.01)
        L.or_updt_rhs_all(O.h)
        d.fillps(0.01)
        d.updt_rhs()
        for ib in range(4):
            np.testing.assert_allclose(d.get(ib, capi.PP), O.field(ib, capi.PP), rtol=0,
                                       atol=1e-12 * np.max(np.abs(O.field(ib, capi.PP))))
        L.or_solve_pressure(O.h)
        rc = d.solve_pressure()
        assert rc == 0, capi.lib().snac_last_error()
        O.boundp(capi.PP)
        d.boundp(capi.PP)
        # x periodic, y walls with N pressure, z periodic -> wavenumber 0 singular: compare mean-free
        for ib in range(4):
            g = d.get(ib, capi.PP)[1:-1, 1:-1, 1:-1]
            r = O.field(ib, capi.PP)[1:-1, 1:-1, 1:-1]
            scale = np.max(np.abs(r))
            assert np.max(np.abs((g - g.mean()) - (r - r.mean()))) <= 2e-9 * scale
    finally:
        d.close()


@pytest.mark.parametrize("nu_coarse", [0, 2])
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("which", ["channel", "ldc3d"])
def test_fused_vcycle_matches_unfused(snac_lib, precision, which, nu_coarse):
    """The tiled smoother / one-CTA coarse tail give the same solves as one kernel per sweep, with the
    default smoothing counts (one sweep per side on levels 2 and coarser with a transform axis) and with
    two sweeps everywhere.

    The V-cycles agree term by term; r.z is summed in a different order (tile partials against
    flat partials), so the two converged solutions agree to the solver tolerance, not bitwise.
    """
    case = (cases.channel_4block(nx=(32, 64), ny=(32, 48), nz=8) if which == "channel"
            else cases.lid_driven_cavity(32))
    out = {}
    for mode in ("1", "0"):
        # "1": one kernel per sweep; "0": every fused kernel of both precisions (mask 15)
        d = Domain(case, precision=precision, nu_coarse=nu_coarse, mg_fuse=-1 if mode == "1" else 15)
        try:
            rng = np.random.default_rng(11)
            for ib in range(len(case.blocks)):
                for k in (capi.U, capi.V, capi.W):
                    d.set(ib, k, rng.standard_normal(d.shape(ib, k)))
            d.bounduvw(False)
            d.fillps(0.01)
            d.updt_rhs()
            assert d.solve_pressure() == 0
            out[mode] = [d.get(ib, capi.PP) for ib in range(len(case.blocks))]
        finally:
            d.close()
    for a, b in zip(out["1"], out["0"]):
        a, b = a[1:-1, 1:-1, 1:-1], b[1:-1, 1:-1, 1:-1]
        a, b = a - a.mean(), b - b.mean()  # both cases have a singular (mean-free) wavenumber
        scale = np.max(np.abs(a))
        assert np.max(np.abs(a - b)) <= 1e-9 * scale


def test_tile_smoother_inverse_diagonal_in_registers_is_bitwise(snac_lib):
    """mg_inv = 1 makes the FP32 tiled smoother form 1 / diagonal from the cell's coefficients and the system's
    shift instead of reading the per-system table; the table holds exactly those values, so the solves are
    bit for bit the same (levels 0 and 1 tiled: mg_cta_level = 2)."""
    case = cases.channel_4block(nx=(32, 64), ny=(32, 48), nz=8)
    out = {}
    for inv in (0, 1):
        d = Domain(case, precision=1, mg_inv=inv, mg_cta_level=2)
        try:
            rng = np.random.default_rng(12)
            for ib in range(len(case.blocks)):
                for k in (capi.U, capi.V, capi.W):
                    d.set(ib, k, rng.standard_normal(d.shape(ib, k)))
            d.bounduvw(False)
            d.fillps(0.01)
            d.updt_rhs()
            assert d.solve_pressure() == 0
            out[inv] = [d.get(ib, capi.PP) for ib in range(len(case.blocks))]
        finally:
            d.close()
    for a, b in zip(out[0], out[1]):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("which,tile", [("channel", 0), ("ldc_fft_x", 0), ("tgv", 0), ("lbox_fft_z", 0),
                                        ("channel", 1), ("channel", 2), ("channel", 4), ("channel", 5),
                                        ("channel", 6), ("lbox_fft_z", 2)])
def test_restricting_pre_smoother_is_bitwise(snac_lib, which, tile):
    """The FP32 tiled pre-smoother that restricts its own residual (the default) and the pre-smoother followed by
    the separate restriction pass (mg_restrict = -1) give bit-identical solves and steps: y-only coarsening with
    periodic x (channel), both axes halved between walls (the reference's cavity along x, four blocks), triperiodic
    (Taylor-Green), and inactive cells in the plane (the L-shaped box along z), with the default tile shape and
    every other one the autotuner may choose (mg_tile 1..6).  Levels 0 and 1 run the tiled smoothers
    (mg_cta_level = 2: these small layouts would otherwise fit the one-CTA V-cycle whole).  The fused form
    launches fewer kernels per solve."""
    case = {"channel": lambda: cases.channel_4block(nx=(32, 64), ny=(32, 48), nz=8),
            "ldc_fft_x": lambda: cases.ldc_reference_test(fft_axis=1),
            "tgv": lambda: cases.taylor_green(32),
            "lbox_fft_z": lambda: dataclasses.replace(cases.l_shaped_box(32, 16), fft_axis=3)}[which]()
    out, launches = {}, {}
    for mode in (-1, 0):
        d = Domain(case, precision=1, use_graph=0, mg_restrict=mode, mg_cta_level=2, mg_tile=tile)
        try:
            rng = np.random.default_rng(13)
            for ib in range(len(case.blocks)):
                for k in (capi.U, capi.V, capi.W):
                    d.set(ib, k, rng.standard_normal(d.shape(ib, k)))
            d.bounduvw(False)
            d.fillps(0.01)
            d.updt_rhs()
            n0, n1 = C.c_longlong(), C.c_longlong()
            capi.check(capi.lib().snac_launch_count(C.byref(n0)))
            assert d.solve_pressure() == 0
            capi.check(capi.lib().snac_launch_count(C.byref(n1)))
            launches[mode] = n1.value - n0.value
            pp = [d.get(ib, capi.PP) for ib in range(len(case.blocks))]
            d.bounduvw(False)
            assert d.step(2) == 0
            out[mode] = (pp, [d.get(ib, k) for ib in range(len(case.blocks)) for k in (capi.U, capi.V, capi.W, capi.P)],
                         d.kinetic_energy())
        finally:
            d.close()
    for a, b in zip(out[-1][0] + out[-1][1], out[0][0] + out[0][1]):
        np.testing.assert_array_equal(a, b)
    assert out[-1][2] == out[0][2]
    assert launches[0] < launches[-1], launches


@pytest.mark.parametrize("precision", [0, 1])
def test_fused_vcycle_iterations_multiwave(snac_lib, precision):
    """Fused and unfused V-cycles are the same preconditioner, also when the tiled kernels run in
    several waves (tiles of one launch then read and write neighbouring cells at different times)."""
    case = cases.channel_4block(nx=(96, 160), ny=(64, 80), nz=32)
    res = {}
    for mode in ("1", "0"):
        d = Domain(case, precision=precision, mg_fuse=-1 if mode == "1" else 15)
        try:
            ic = cases.channel_initial_condition(case, lambda ib: d.grid(ib, 1, capi.G_XC))
            for ib, (u, v, w) in ic.items():
                d.set(ib, capi.U, u)
                d.set(ib, capi.V, v)
                d.set(ib, capi.W, w)
            d.bounduvw(False)
            d.fillps(1e-3)
            d.updt_rhs()
            assert d.solve_pressure() == 0
            st = d.stats()
            res[mode] = (st["iters"], [d.get(ib, capi.PP)[1:-1, 1:-1, 1:-1] for ib in range(len(case.blocks))])
        finally:
            d.close()
    assert res["0"][0] == res["1"][0], (res["0"][0], res["1"][0])
    for a, b in zip(res["0"][1], res["1"][1]):
        a, b = a - a.mean(), b - b.mean()
        assert np.max(np.abs(a - b)) <= 1e-9 * np.max(np.abs(a))


def _run_both(case, oracle_mod, nsteps, precision=0, seed=3, amp=0.1):
    O = oracle_mod.OracleDomain(case)
    d = Domain(case, precision=precision)
    seed_fields(case, O, d, seed=seed, amp=amp)
    O.bounduvw(False)
    O.boundp(capi.P)
    d.bounduvw(False)
    d.boundp(capi.P)
    O.step(nsteps)
    d.step(nsteps)
    return O, d


@pytest.mark.parametrize("fft_axis", [0, 1])
def test_steps_ldc_layout(snac_lib, oracle_mod, fft_axis):
    case = cases.ldc_reference_test(fft_axis=fft_axis)
    O, d = _run_both(case, oracle_mod, 5)
    try:
        assert abs(d.dt - O.dt) <= 1e-15 * O.dt
        compare_fields(case, O, d, (capi.U, capi.V, capi.W), 1e-10)
        compare_fields(case, O, d, (capi.P,), 1e-9, mean_free_p=True)
        assert d.chkdiv()[1] < 1e-10
    finally:
        d.close()


def test_steps_tgv(snac_lib, oracle_mod):
    case = cases.taylor_green(16)
    O, d = _run_both(case, oracle_mod, 3, amp=0.5)
    try:
        compare_fields(case, O, d, (capi.U, capi.V, capi.W), 1e-10)
        compare_fields(case, O, d, (capi.P,), 1e-9, mean_free_p=True)
    finally:
        d.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_steps_channel(snac_lib, oracle_mod, precision):
    case = cases.channel_4block(nx=(16, 32), ny=(8, 16), nz=16)
    O, d = _run_both(case, oracle_mod, 3, precision=precision, amp=0.2)
    try:
        compare_fields(case, O, d, (capi.U, capi.V, capi.W), 1e-10)
        compare_fields(case, O, d, (capi.P,), 1e-9, mean_free_p=True)
        ke_o, ke_g = O.kinetic_energy(), d.kinetic_energy()
        assert abs(ke_g - ke_o) <= 1e-12 * ke_o
    finally:
        d.close()


def test_steps_dhc_scalar_buoyancy(snac_lib, oracle_mod):
    """The reference's differentially-heated-cavity layout (tests/differentially_heated_cavity): one
    scalar advected and diffused by rk_scal, Boussinesq buoyancy in rk_mom, FFT along y, fixed dt."""
    case = cases.dhc_reference_test()
    O = oracle_mod.OracleDomain(case)
    d = Domain(case)
    try:
        s0 = cases.dhc_initial_scalar(case, lambda ib: O.grid(ib, 0, oracle_mod.G_XC))
        rng = np.random.default_rng(5)
        for ib in range(len(case.blocks)):
            O.field(ib, capi.S0)[...] = s0[ib] + 1e-3 * rng.standard_normal(s0[ib].shape)
            d.set(ib, capi.S0, O.field(ib, capi.S0))
        for X in (O, d):
            X.bounduvw(False)
            X.boundp(capi.P)
            X.boundp(capi.S0)
        O.step(20)
        d.step(20)
        compare_fields(case, O, d, (capi.U, capi.V, capi.W, capi.S0), 1e-10)
        compare_fields(case, O, d, (capi.P,), 1e-9, mean_free_p=True)
        assert np.max(np.abs(d.get(0, capi.W))) > 1e-6  # buoyancy has set the fluid in motion
    finally:
        d.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_steps_dhc_impdiff(snac_lib, oracle_mod, precision):
    """IMPDIFF on the stretched heated cavity: the Helmholtz solves of u, v, w (staggered along their own
    axis, hif = hi - 1 at a wall) and of the scalar, with the 3-D pressure solve."""
    case = cases.heated_cavity(n=(16, 16, 8), stretch=1.2, ra=1e5, impdiff=1, tol=1e-12, dt_f=2e-3)
    O = oracle_mod.OracleDomain(case)
    d = Domain(case, precision=precision)
    try:
        s0 = cases.dhc_initial_scalar(case, lambda ib: O.grid(ib, 0, oracle_mod.G_XC))
        rng = np.random.default_rng(11)
        O.field(0, capi.S0)[...] = s0[0] + 1e-2 * rng.standard_normal(s0[0].shape)
        d.set(0, capi.S0, O.field(0, capi.S0))
        for X in (O, d):
            X.bounduvw(False)
            X.boundp(capi.P)
            X.boundp(capi.S0)
        O.step(5)
        d.step(5)
        st = d.stats()
        assert 0 < st["helm_iters"] and st["helm_residual"] <= case.tol
        compare_fields(case, O, d, (capi.U, capi.V, capi.W, capi.S0), 1e-9)
        compare_fields(case, O, d, (capi.P,), 1e-8, mean_free_p=True)
        assert np.max(np.abs(d.get(0, capi.V))) > 1e-8
    finally:
        d.close()


@pytest.mark.parametrize("which,precision", [("ldc_x", 0), ("ldc_x", 1), ("channel_z", 0), ("channel_z", 1),
                                             ("dhc_y", 0)])
def test_steps_impdiff_fft(snac_lib, oracle_mod, which, precision):
    """IMPDIFF with a transform axis (solve_impdiff_field_fft): each field's own transform, per-wavenumber
    Helmholtz solves with the shift lambda_k + alphai.  LDC along x has walls on the transform axis (u is
    staggered there: the transform drops its wall face), the channel is periodic along z, the heated cavity
    (FFT along y) adds the scalar's Helmholtz solve and buoyancy."""
    import dataclasses
    if which == "ldc_x":
        case = dataclasses.replace(cases.ldc_reference_test(fft_axis=1), impdiff=1, dt_f=2e-3)
    elif which == "channel_z":
        case = dataclasses.replace(cases.channel_4block(nx=(16, 32), ny=(8, 16), nz=16), impdiff=1, dt_f=2e-3)
    else:
        case = dataclasses.replace(cases.dhc_reference_test(), impdiff=1, dt_f=5e-3)
    O = oracle_mod.OracleDomain(case)
    d = Domain(case, precision=precision)
    try:
        seed_fields(case, O, d, seed=8, amp=0.1)
        if which == "dhc_y":
            s0 = cases.dhc_initial_scalar(case, lambda ib: O.grid(ib, 0, oracle_mod.G_XC))
            O.field(0, capi.S0)[...] = s0[0]
            d.set(0, capi.S0, s0[0])
        for X in (O, d):
            X.bounduvw(False)
            X.boundp(capi.P)
            if which == "dhc_y":
                X.boundp(capi.S0)
        O.step(3)
        d.step(3)
        st = d.stats()
        assert st["helm_iters"] > 0 and st["helm_residual"] <= case.tol
        kinds = (capi.U, capi.V, capi.W) + ((capi.S0,) if which == "dhc_y" else ())
        compare_fields(case, O, d, kinds, 1e-9)
        compare_fields(case, O, d, (capi.P,), 1e-8, mean_free_p=True)
    finally:
        d.close()


def test_steps_lshape_impdiff(snac_lib, oracle_mod):
    """IMPDIFF across block interfaces: the L-shaped box of three blocks, where a velocity component's
    Helmholtz box runs through the friend faces (hif = hi there) and stops short of the walls."""
    import dataclasses
    case = dataclasses.replace(cases.l_shaped_box(n=16, nz=8), impdiff=1, dt_f=1e-3)
    O, d = _run_both(case, oracle_mod, 3, amp=0.2)
    try:
        compare_fields(case, O, d, (capi.U, capi.V, capi.W), 1e-9)
        compare_fields(case, O, d, (capi.P,), 1e-8, mean_free_p=True)
    finally:
        d.close()


@pytest.mark.parametrize("fft_axis", [0, 3])
def test_fillps_tma_matches_plain(snac_lib, fft_axis):
    """fillps through TMA-staged tiles (the uneven four-block channel: every tile kind, partial tiles at the
    block ends) gives the same bits as the kernel that reads the fields directly."""
    import dataclasses
    case = dataclasses.replace(cases.channel_4block(nx=(48, 64), ny=(24, 40), nz=14), fft_axis=fft_axis)
    out = {}
    for tma in (0, -1):
        d = Domain(case, tma=tma)
        try:
            rng = np.random.default_rng(12)
            for ib in range(len(case.blocks)):
                for k in (capi.U, capi.V, capi.W):
                    d.set(ib, k, rng.standard_normal(d.shape(ib, k)))
            d.fillps(0.37)
            out[tma] = [d.get(ib, capi.PP) for ib in range(len(case.blocks))]
        finally:
            d.close()
    for a, b in zip(out[0], out[-1]):
        np.testing.assert_array_equal(a[1:-1, 1:-1, 1:-1], b[1:-1, 1:-1, 1:-1])


@pytest.mark.parametrize("which", ["cavity_3d", "channel_z"])
def test_impdiff_solve_entry(snac_lib, oracle_mod, which):
    """snac_impdiff_solve (solve_impdiff_field with the reference's arguments) on each field of a domain: the
    heated cavity's 3-D Helmholtz solves of u, v, w and T, and the channel's per-wavenumber solves along z,
    against the oracle's solve of the same field from the same state."""
    import dataclasses
    if which == "cavity_3d":
        case = cases.heated_cavity(n=(16, 16, 8), stretch=1.5, ra=1e6, impdiff=1, tol=1e-12, dt_f=2e-3)
        fields = (capi.U, capi.V, capi.W, capi.S0)
    else:
        case = dataclasses.replace(cases.channel_4block(nx=(16, 32), ny=(8, 16), nz=16), impdiff=1, dt_f=1e-3)
        fields = (capi.U, capi.V, capi.W)
    O = oracle_mod.OracleDomain(case)
    d = Domain(case)
    try:
        seed_fields(case, O, d, seed=9, amp=0.3)
        if capi.S0 in fields:
            rng = np.random.default_rng(10)
            t = rng.standard_normal(O.field(0, capi.S0).shape)
            O.field(0, capi.S0)[...] = t
            d.set(0, capi.S0, t)
        for X in (O, d):
            X.bounduvw(False)
        alphai = -2.0 * case.visci / 1e-3
        L = capi.lib()
        for f in fields:
            fo = 3 + (f - capi.S0) if f >= capi.S0 else f - capi.U
            assert oracle_mod.lib().or_impdiff_solve(O.h, fo, alphai) == 0
            assert L.snac_impdiff_solve(f, alphai, 0.0) == 0, L.snac_last_error()
            compare_fields(case, O, d, (f,), 1e-10)
        with pytest.raises(AssertionError):
            assert L.snac_impdiff_solve(capi.P, alphai, 0.0) == 0
    finally:
        d.close()


@pytest.mark.parametrize("which", ["duct", "kovasznay"])
def test_inflow_bitwise(snac_lib, oracle_mod, which):
    """inflow (bound.f90:438-477) after bounduvw: the inflow planes and mirrored ghosts equal the oracle's."""
    case = cases.developing_duct() if which == "duct" else cases.kovasznay()
    O = oracle_mod.OracleDomain(case)
    d = Domain(case)
    try:
        seed_fields(case, O, d, seed=6)
        for is_correc in (False, True):
            for X in (O, d):
                X.bounduvw(is_correc)
                X.inflow(is_correc)
            for k in (capi.U, capi.V, capi.W):
                np.testing.assert_array_equal(d.get(0, k), O.field(0, k))
    finally:
        d.close()


@pytest.mark.parametrize("which,impdiff", [("duct", 0), ("duct", 1), ("kovasznay", 0), ("kovasznay", 1)])
def test_steps_inflow(snac_lib, oracle_mod, which, impdiff):
    """Whole steps with an inflow face (explicit and implicit diffusion; under IMPDIFF the inflow planes are
    the boundary values of the velocity Helmholtz problems)."""
    case = (cases.developing_duct(impdiff=impdiff, dt_f=5e-3) if which == "duct"
            else cases.kovasznay(impdiff=impdiff, dt_f=1e-4 if not impdiff else 2e-3))
    O = oracle_mod.OracleDomain(case)
    d = Domain(case)
    try:
        for X in (O, d):
            X.bounduvw(False)
            X.inflow(False)
            X.boundp(capi.P)
        O.step(5)
        d.step(5)
        # the Kovasznay flow has no v: there v is rounding noise, compared against the scale of u
        vel = (capi.U, capi.V, capi.W) if which == "duct" else (capi.U, capi.W)
        compare_fields(case, O, d, vel, 1e-9)
        if which == "kovasznay":
            umax = np.max(np.abs(O.field(0, capi.U)))
            assert np.max(np.abs(d.get(0, capi.V) - O.field(0, capi.V))) <= 1e-9 * umax
        compare_fields(case, O, d, (capi.P,), 1e-8)
        assert d.chkdiv()[1] < 1e-10
    finally:
        d.close()


def test_steps_channel_forced_scalar(snac_lib, oracle_mod):
    """Four uneven blocks with a bulk-forced scalar: the bulk mean of rk_scal is taken over all blocks and
    the scalar's ghost planes come through the friend links."""
    case = cases.channel_4block_scalar()
    O = oracle_mod.OracleDomain(case)
    d = Domain(case)
    try:
        seed_fields(case, O, d, seed=3, amp=0.2)
        for X in (O, d):
            X.bounduvw(False)
            X.boundp(capi.P)
        rng = np.random.default_rng(9)
        for ib in range(len(case.blocks)):
            f = O.field(ib, capi.S0)
            f[...] = 0.5 + 0.1 * rng.standard_normal(f.shape)
            d.set(ib, capi.S0, f)
        O.boundp(capi.S0)
        d.boundp(capi.S0)
        O.step(3)
        d.step(3)
        compare_fields(case, O, d, (capi.U, capi.V, capi.W, capi.S0), 1e-10)
        compare_fields(case, O, d, (capi.P,), 1e-9, mean_free_p=True)
    finally:
        d.close()


@pytest.mark.parametrize("fft_axis", [0, 1])
def test_gpu_ldc_golden(snac_lib, fft_axis):
    """The reference's regression (tests/lid_driven_cavity/test.py) on the GPU path, with its tolerance."""
    from test_oracle_golden import ldc_profile
    case = cases.ldc_reference_test(fft_axis=fft_axis)
    d = Domain(case)
    try:
        d.bounduvw(False)
        d.boundp(capi.P)
        d.step(1500)
        prof = ldc_profile(lambda ib: d.get(ib, capi.V))
        ref = np.loadtxt(GOLDEN)
        np.testing.assert_allclose(prof, ref[:, 1], rtol=1e-7, atol=5e-8)
    finally:
        d.close()


def test_checkpoint_bytes_match_oracle(snac_lib, oracle_mod, tmp_path):
    """Checkpoints written from device state are byte-identical to the oracle's load_one files of the same
    fields, and loading the oracle's files restores the device interiors exactly (with time and istep)."""
    case = cases.channel_4block_scalar()
    O = oracle_mod.OracleDomain(case)
    d = Domain(case)
    try:
        rng = np.random.default_rng(13)
        for ib in range(len(case.blocks)):
            for k in (capi.U, capi.V, capi.W, capi.P, capi.S0):
                f = O.field(ib, k)
                f[...] = rng.standard_normal(f.shape)
                d.set(ib, k, f)
        pg, po = str(tmp_path / "gpu"), str(tmp_path / "orc")
        d.checkpoint_save(pg)
        O.checkpoint_save(po)
        for ib in range(len(case.blocks)):
            for tag in ("u", "v", "w", "p", "s_001"):
                a = open(f"{pg}_b_{ib + 1:03d}_{tag}.bin", "rb").read()
                b = open(f"{po}_b_{ib + 1:03d}_{tag}.bin", "rb").read()
                assert a == b, (ib, tag)
        # the oracle advances one step and writes; the device loads the oracle's files
        O.bounduvw(False)
        O.boundp(capi.P)
        O.step(1)
        O.checkpoint_save(po)
        d.checkpoint_load(po)
        st = d.stats()
        assert (st["time"], st["istep"]) == O.time_istep
        for ib in range(len(case.blocks)):
            for k in (capi.U, capi.V, capi.W, capi.P, capi.S0):
                np.testing.assert_array_equal(d.get(ib, k)[1:-1, 1:-1, 1:-1], O.field(ib, k)[1:-1, 1:-1, 1:-1])
        with open(f"{po}_b_001_u.bin", "ab") as f:
            f.write(b"\0" * 8)
        assert capi.lib().snac_checkpoint_load(po.encode()) == capi.ERR_IO
    finally:
        d.close()


def test_out1d_out3d_match_oracle(snac_lib, oracle_mod, tmp_path):
    """out1d profiles reduced on the device agree with the oracle's serial sums (their order differs: 1e-13),
    the text files carry the same coordinates and 7-digit values, and out3d dumps are byte-identical."""
    case = cases.channel_4block(nx=(16, 32), ny=(8, 16), nz=16)
    O = oracle_mod.OracleDomain(case)
    d = Domain(case)
    try:
        seed_fields(case, O, d, seed=15)
        for ib in range(len(case.blocks)):
            for k in (capi.U, capi.V, capi.W, capi.P):
                for idir in (1, 2, 3):
                    xg, pg = d.out1d(ib, k, idir)
                    xo, po = O.out1d(ib, k, idir, fname=tmp_path / "o.out")
                    np.testing.assert_array_equal(xg, xo)
                    np.testing.assert_allclose(pg, po, rtol=1e-13, atol=1e-13 * np.max(np.abs(po)))
                    assert capi.lib().snac_out1d_write(str(tmp_path / "g.out").encode(), ib, k, idir) == 0
                    lg = open(tmp_path / "g.out").read().splitlines()
                    lo = open(tmp_path / "o.out").read().splitlines()
                    assert len(lg) == len(lo)
                    for a, b in zip(lg, lo):
                        assert a[:15] == b[:15]
                        assert abs(float(a[15:]) - float(b[15:])) <= 1e-6 * max(abs(float(b[15:])), 1e-30)
            assert capi.lib().snac_out3d_write(str(tmp_path / "f.bin").encode(), ib, capi.W) == 0
            raw = np.fromfile(tmp_path / "f.bin", dtype=np.float64)
            interior = O.field(ib, capi.W)[1:-1, 1:-1, 1:-1]
            np.testing.assert_array_equal(raw, interior.ravel(order="F"))
    finally:
        d.close()


def test_graph_replay_bitwise(snac_lib):
    """The mixed path's refinement steps replayed as CUDA graphs give the same bits as launched one by one."""
    case = cases.channel_4block(nx=(32, 64), ny=(32, 48), nz=16)
    out = {}
    for g in (0, 1):
        d = Domain(case, precision=1, use_graph=g)
        try:
            ic = cases.channel_initial_condition(case, lambda ib: d.grid(ib, 1, capi.G_XC))
            for ib, (u, v, w) in ic.items():
                d.set(ib, capi.U, u)
                d.set(ib, capi.V, v)
                d.set(ib, capi.W, w)
            d.bounduvw(False)
            d.step(3)
            out[g] = [d.get(ib, k) for ib in range(len(case.blocks)) for k in (capi.U, capi.V, capi.W, capi.P)]
        finally:
            d.close()
    for a, b in zip(out[0], out[1]):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("precision", [0, 1])
def test_100_steps_channel_against_oracle(snac_lib, oracle_mod, precision):
    """The acceptance criteria on the uneven four-block channel layout (FFT along z, stretched walls):
    after 100 RK3 steps the velocity and pressure fields are within 1e-10 relative of the oracle's,
    max|div u| <= 1e-10, and the kinetic energy within 1e-8 relative; for the mixed path (FP32 V-cycles
    in FP64 refinement) this also states its error against the FP64 path."""
    case = cases.channel_4block(nx=(16, 32), ny=(8, 16), nz=16)
    O = oracle_mod.OracleDomain(case)
    d = Domain(case, precision=precision, use_graph=precision)
    try:
        ic = cases.channel_initial_condition(case, lambda ib: O.grid(ib, 1, oracle_mod.G_XC))
        for ib, (u, v, w) in ic.items():
            for k, f in ((capi.U, u), (capi.V, v), (capi.W, w)):
                O.field(ib, k)[...] = f
                d.set(ib, k, f)
        for X in (O, d):
            X.bounduvw(False)
            X.boundp(capi.P)
        O.step(100)
        d.step(100)
        err_v = compare_fields(case, O, d, (capi.U, capi.V, capi.W), 1e-10)
        err_p = compare_fields(case, O, d, (capi.P,), 1e-10, mean_free_p=True)
        assert d.chkdiv()[1] <= 1e-10
        ke_o, ke_g = O.kinetic_energy(), d.kinetic_energy()
        assert abs(ke_g - ke_o) <= 1e-8 * ke_o
        print(f"precision {precision}: max rel. error velocity {err_v:.2e}, pressure {err_p:.2e}")
    finally:
        d.close()


def test_100_steps_heated_cavity_impdiff_against_oracle(snac_lib, oracle_mod):
    """100 steps of the stretched heated cavity with IMPDIFF, Boussinesq buoyancy and the 3-D solves
    (the layout of the 512x512x256 configuration at 16x16x8): fields within 1e-10, divergence <= 1e-10."""
    case = cases.heated_cavity(n=(16, 16, 8), stretch=1.5, ra=1e6, impdiff=1, tol=1e-12, dt_f=2e-3)
    O = oracle_mod.OracleDomain(case)
    d = Domain(case)
    try:
        s0 = cases.dhc_initial_scalar(case, lambda ib: O.grid(ib, 0, oracle_mod.G_XC))
        rng = np.random.default_rng(21)
        O.field(0, capi.S0)[...] = s0[0] + 1e-3 * rng.uniform(-1, 1, s0[0].shape)
        d.set(0, capi.S0, O.field(0, capi.S0))
        for X in (O, d):
            X.bounduvw(False)
            X.boundp(capi.P)
            X.boundp(capi.S0)
        O.step(100)
        d.step(100)
        compare_fields(case, O, d, (capi.U, capi.V, capi.W, capi.S0), 1e-10)
        compare_fields(case, O, d, (capi.P,), 1e-10, mean_free_p=True)
        assert d.chkdiv()[1] <= 1e-10
    finally:
        d.close()


@pytest.mark.parametrize("fft_axis", [0, 3])
def test_steps_one_cell_periodic_axis(snac_lib, oracle_mod, fft_axis):
    """A one-cell periodic z (a 2-D flow run in 3-D): the self-couplings of that axis cancel in the 3-D
    operator (as HYPRE's periodic wrap makes them), and the transform along it is one mode."""
    import dataclasses
    case = dataclasses.replace(cases.taylor_green(16), fft_axis=fft_axis)
    case = dataclasses.replace(case, blocks=[dataclasses.replace(case.blocks[0], ng=(16, 16, 1))])
    O, d = _run_both(case, oracle_mod, 3, amp=0.5)
    try:
        compare_fields(case, O, d, (capi.U, capi.V), 1e-10)
        compare_fields(case, O, d, (capi.P,), 1e-9, mean_free_p=True)
        assert d.chkdiv()[1] < 1e-10
    finally:
        d.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_autotune_restores_state(snac_lib, precision):
    """snac_autotune times its candidates from a snapshot and then restores the state: the fields, time and
    step count after the call are those before it, bit for bit, and stepping on with the chosen settings
    converges to the same tolerance.  Against the same steps without tuning, the fields differ only by
    what the solver tolerance allows."""
    case = cases.channel_4block(nx=(16, 32), ny=(8, 16), nz=16)
    runs = {}
    for tune in (0, 1):
        d = Domain(case, precision=precision, use_graph=precision)
        try:
            ic = cases.channel_initial_condition(case, lambda ib: d.grid(ib, 1, capi.G_XC))
            for ib, (u, v, w) in ic.items():
                d.set(ib, capi.U, u)
                d.set(ib, capi.V, v)
                d.set(ib, capi.W, w)
            d.bounduvw(False)
            d.step(3)
            before = [d.get(ib, k) for ib in range(len(case.blocks)) for k in (capi.U, capi.V, capi.W, capi.P)]
            st0 = d.stats()
            if tune:
                r = d.autotune(2)
                # (mixed with 5, 6, 7 inner iterations, plain) x (1, 2 sweeps), 6 tile shapes, 3 waves, up to 2
                # coarse-cycle levels, and for the mixed solve 2 refinement strategies
                assert 17 <= r["candidates"] <= 21, r
                assert r["precision"] in (0, 1) and r["inner_iters"] in (5, 6, 7) and r["nu_coarse"] in (1, 2), r
                assert r["mg_tile"] in (1, 2, 3, 4, 5, 6) and r["mg_waves"] in (1, 2, 4), r
                assert 0.0 < r["ms_per_step"] <= r["ms_before"] * 1.5, r
                after = [d.get(ib, k) for ib in range(len(case.blocks)) for k in (capi.U, capi.V, capi.W, capi.P)]
                for a, b in zip(before, after):
                    np.testing.assert_array_equal(a, b)
                st1 = d.stats()
                assert st1["istep"] == st0["istep"] and st1["time"] == st0["time"] and st1["dt"] == st0["dt"]
            assert d.step(3) == 0
            assert d.stats()["residual"] <= case.tol and d.chkdiv()[1] < 1e-10
            runs[tune] = [d.get(ib, k) for ib in range(len(case.blocks)) for k in (capi.U, capi.V, capi.W)]
        finally:
            d.close()
    for a, b in zip(runs[0], runs[1]):
        assert np.max(np.abs(a - b)) <= 1e-9 * np.max(np.abs(a))


def test_autotune_3d_solve_searches_the_coarse_level(snac_lib):
    """With the 3-D solve snac_autotune times the solve group (mixed with 5, 6, 7 inner iterations, plain), the
    level where the one-CTA coarse V-cycle starts (default, one coarser, one finer) and, for the mixed solve, the
    two refinement strategies; the state after the call is the state before it, bit for bit."""
    import dataclasses
    case = dataclasses.replace(cases.l_shaped_box(16, 8), dt_f=4e-3)
    d = Domain(case, precision=1, use_graph=1)
    try:
        d.bounduvw(False)
        d.step(2)
        before = [d.get(ib, k) for ib in range(len(case.blocks)) for k in (capi.U, capi.V, capi.W, capi.P)]
        r = d.autotune(1)
        assert 4 <= r["candidates"] <= 9, r
        assert r["mg_cta_level"] >= 1, r
        after = [d.get(ib, k) for ib in range(len(case.blocks)) for k in (capi.U, capi.V, capi.W, capi.P)]
        for a, b in zip(before, after):
            np.testing.assert_array_equal(a, b)
        assert d.step(2) == 0
        assert d.stats()["residual"] <= case.tol and d.chkdiv()[1] < 1e-10
    finally:
        d.close()


@pytest.mark.parametrize("fail_at", [0, 3])
def test_autotune_error_restores_settings_and_state(snac_lib, fail_at):
    """A candidate that fails part-way (a host-side injected error after its solvers are rebuilt) makes
    snac_autotune return that error with the original settings, rebuilt solvers and the snapshot's state:
    the fields, time and step count are unchanged bit for bit and the next steps run as without the call."""
    case = cases.channel_4block(nx=(16, 32), ny=(8, 16), nz=16)
    d = Domain(case, precision=1, use_graph=1)
    try:
        ic = cases.channel_initial_condition(case, lambda ib: d.grid(ib, 1, capi.G_XC))
        for ib, (u, v, w) in ic.items():
            d.set(ib, capi.U, u)
            d.set(ib, capi.V, v)
            d.set(ib, capi.W, w)
        d.bounduvw(False)
        d.step(2)
        keys = (capi.U, capi.V, capi.W, capi.P)
        before = [d.get(ib, k) for ib in range(len(case.blocks)) for k in keys]
        st0 = d.stats()
        assert capi.lib().snac_tune_inject_failure(fail_at) == 0
        with pytest.raises(capi.SnacError) as ei:
            d.autotune(1)
        assert ei.value.code == capi.ERR_STATE and "injected" in str(ei.value)
        after = [d.get(ib, k) for ib in range(len(case.blocks)) for k in keys]
        for a, b in zip(before, after):
            np.testing.assert_array_equal(a, b)
        st1 = d.stats()
        assert (st1["istep"], st1["time"], st1["dt"]) == (st0["istep"], st0["time"], st0["dt"])
        assert d.step(2) == 0
        assert d.stats()["residual"] <= case.tol
        # the reference run: the same two steps without the failed tuning call, same settings
        d2 = Domain(case, precision=1, use_graph=1)
        try:
            for ib, (u, v, w) in ic.items():
                d2.set(ib, capi.U, u)
                d2.set(ib, capi.V, v)
                d2.set(ib, capi.W, w)
            d2.bounduvw(False)
            d2.step(4)
            for ib in range(len(case.blocks)):
                for k in keys[:3]:
                    a, b = d.get(ib, k), d2.get(ib, k)
                    assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))
        finally:
            d2.close()
    finally:
        capi.lib().snac_tune_inject_failure(-1)
        d.close()


def test_batched_field_copies(snac_lib):
    """snac_set_fields / snac_get_fields move the same bytes as the one-field calls (two streams, one
    synchronisation)."""
    case = cases.channel_4block(nx=(16, 32), ny=(8, 16), nz=16)
    d = Domain(case, precision=1)
    try:
        rng = np.random.default_rng(5)
        items = []
        for ib in range(len(case.blocks)):
            for k in (capi.U, capi.V, capi.W, capi.P):
                items.append((ib, k, np.asfortranarray(rng.standard_normal(d.shape(ib, k)))))
        d.set_many(items)
        for ib, k, a in items:
            np.testing.assert_array_equal(d.get(ib, k), a)
        outs = [(ib, k, np.zeros(a.shape, order="F")) for ib, k, a in items]
        d.get_many(outs)
        for (_, _, a), (_, _, b) in zip(items, outs):
            np.testing.assert_array_equal(a, b)
        with pytest.raises(capi.SnacError):
            d.set_many([(99, capi.U, items[0][2])])
    finally:
        d.close()
