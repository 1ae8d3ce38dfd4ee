"""Parity at the configurations' full sizes: the GPU paths against the oracle after many RK3 steps.

The acceptance bars of the hot path (velocity and mean-free pressure within 1e-10 relative of the oracle,
kinetic energy within 1e-8, max|div u| <= 1e-10) on the layouts the benchmarks run, at their full sizes:

* the four-block channel 256x144x128 (uneven blocks 96|160 x 64|80, tanh-stretched walls, FFT along z),
  100 steps, with the plain FP64 solve and with FP32 V-cycles inside FP64 refinement (graph replay);
* the triperiodic Taylor-Green vortex 128^3 (FFT along z, 128 systems of 128x128) from its analytic
  velocity and pressure, 50 steps;
* the lid-driven cavity 64^3 (3-D multigrid, Re = 1000, CFL 0.5) from rest, 100 steps;
* the L-shaped closed box, three 144x144x96 blocks (3-D multigrid on a solver box a third inactive), from
  rest, 10 steps;
* the differentially heated cavity 512x512x256 (IMPDIFF u, v, w, T Helmholtz solves, Boussinesq buoyancy,
  3-D pressure multigrid), 2 steps.

The oracle (C restatement with OpenMP on all host cores) runs each case once; the GPU paths are compared
against it.  Each test prints the measured errors.  These sizes exercise what the small layouts of the
other tests cannot: the full multigrid hierarchies (the channel's seven levels down to a 16x9 dense level),
the one-CTA coarse V-cycle's shared-memory plan, the tiled smoother's full grids and the multi-wave
reductions.
"""
import numpy as np
import pytest

from snac_gb300 import capi, cases
from snac_gb300.domain import Domain

from test_gpu_domain import compare_fields

pytestmark = pytest.mark.gpu

_ORACLE = {}


def _oracle_run(oracle_mod, key, case, init, nsteps):
    """Oracle state after nsteps from init (run once per case and reused by the GPU paths)."""
    if key not in _ORACLE:
        O = oracle_mod.OracleDomain(case)
        fields = init(lambda ib, a, which: O.grid(ib, a, which))
        for ib, fs in fields.items():
            for k, f in fs:
                O.field(ib, k)[...] = f
        O.bounduvw(False)
        O.boundp(capi.P)
        O.step(nsteps)
        _ORACLE[key] = (O, fields)
    return _ORACLE[key]


def _gpu_run(case, fields, nsteps, precision):
    d = Domain(case, precision=precision, use_graph=precision)
    for ib, fs in fields.items():
        for k, f in fs:
            d.set(ib, k, f)
    d.bounduvw(False)
    d.boundp(capi.P)
    assert d.step(nsteps) == 0
    return d


def _check(case, O, d, label, vel_tol=1e-10, p_tol=1e-10):
    err_v = compare_fields(case, O, d, (capi.U, capi.V, capi.W), vel_tol)
    err_p = compare_fields(case, O, d, (capi.P,), p_tol, mean_free_p=True)
    div_g, div_o = d.chkdiv()[1], O.chkdiv()[1]
    ke_g, ke_o = d.kinetic_energy(), O.kinetic_energy()
    st = d.stats()
    print(f"{label}: step {st['istep']} t={st['time']:.6e} max rel. error velocity {err_v:.2e}, pressure "
          f"{err_p:.2e}; |KE-KE_o|/KE_o {abs(ke_g - ke_o) / ke_o:.2e}; max|div u| GPU {div_g:.2e} oracle "
          f"{div_o:.2e}")
    assert st["istep"] == O.istep
    assert div_g <= 1e-10
    assert abs(ke_g - ke_o) <= 1e-8 * ke_o
    return err_v, err_p


def _channel_init(case):
    def init(grid):
        ic = cases.channel_initial_condition(case, lambda ib: grid(ib, 1, capi.G_XC))
        return {ib: ((capi.U, u), (capi.V, v), (capi.W, w)) for ib, (u, v, w) in ic.items()}
    return init


@pytest.mark.parametrize("precision", [0, 1])
def test_channel_256x144x128_100_steps(snac_lib, oracle_mod, precision):
    case = cases.channel_4block()
    O, fields = _oracle_run(oracle_mod, "channel", case, _channel_init(case), 100)
    d = _gpu_run(case, fields, 100, precision)
    try:
        _check(case, O, d, f"channel 256x144x128, precision {precision}")
    finally:
        d.close()


def test_taylor_green_128_50_steps(snac_lib, oracle_mod):
    case = cases.taylor_green(128)

    def init(grid):
        ic = cases.tgv_initial_condition(case, grid)
        return {ib: ((capi.U, u), (capi.V, v), (capi.W, w), (capi.P, p)) for ib, (u, v, w, p) in ic.items()}

    O, fields = _oracle_run(oracle_mod, "tgv", case, init, 50)
    for precision in (0, 1):
        d = _gpu_run(case, fields, 50, precision)
        try:
            _check(case, O, d, f"Taylor-Green 128^3, precision {precision}")
        finally:
            d.close()


def test_lid_driven_cavity_64_100_steps(snac_lib, oracle_mod):
    case = cases.lid_driven_cavity(64)

    def init(grid):
        z = np.zeros((66, 66, 66), order="F")
        return {0: ((capi.U, z), (capi.V, z), (capi.W, z), (capi.P, z))}

    O, fields = _oracle_run(oracle_mod, "ldc", case, init, 100)
    for precision in (0, 1):
        d = _gpu_run(case, fields, 100, precision)
        try:
            _check(case, O, d, f"lid-driven cavity 64^3, precision {precision}")
        finally:
            d.close()


def test_l_shaped_box_3x144x144x96_10_steps(snac_lib, oracle_mod):
    """The L-shaped closed box at its benchmark size (three 144x144x96 blocks, 5.97 M cells, 3-D multigrid on
    the 288x288x96 solver box with a third of it inactive), lid-driven from rest: 10 steps (the oracle's 3-D
    solve takes about 15 s per step on 16 host cores)."""
    case = cases.l_shaped_box(144, 96)

    def init(grid):
        z = np.zeros((146, 146, 98), order="F")
        return {ib: ((capi.U, z), (capi.V, z), (capi.W, z), (capi.P, z)) for ib in range(3)}

    O, fields = _oracle_run(oracle_mod, "lbox", case, init, 10)
    for precision in (0, 1):
        d = _gpu_run(case, fields, 10, precision)
        try:
            _check(case, O, d, f"L-shaped box 3x144x144x96, precision {precision}")
        finally:
            d.close()


def test_heated_cavity_512x512x256_2_steps(snac_lib, oracle_mod):
    """The differentially heated cavity at its benchmark size (512x512x256 = 67 M cells, stretched 1.5 toward every
    wall, Ra = 1e8, Pr = 0.71, Boussinesq buoyancy, IMPDIFF: u, v, w and T Helmholtz solves plus the 3-D pressure
    solve every stage), from rest with seeded temperature noise of 1e-3, at the reference test's fixed dt = 1e-3:
    2 steps (the oracle's step takes about a minute on 16 host cores).  The temperature is compared too."""
    case = cases.heated_cavity((512, 512, 256), dt_f=1e-3)

    def init(grid):
        n = [int(x) for x in case.blocks[0].ng]
        z = np.zeros([x + 2 for x in n], order="F")
        t = np.zeros_like(z)
        r = cases.splitmix64_uniform_fast(0x5EED, n[0] * n[1] * n[2]).reshape(n, order="F")
        t[1:-1, 1:-1, 1:-1] = 2e-3 * (r - 0.5)
        return {0: ((capi.U, z), (capi.V, z), (capi.W, z), (capi.P, z), (capi.S0, t))}

    if "dhc" not in _ORACLE:
        O = oracle_mod.OracleDomain(case)
        fields = init(None)
        for k, f in fields[0]:
            O.field(0, k)[...] = f
        O.bounduvw(False)
        O.boundp(capi.P)
        O.boundp(capi.S0)
        O.step(2)
        _ORACLE["dhc"] = (O, fields)
    O, fields = _ORACLE["dhc"]
    for precision in (0, 1):
        d = Domain(case, precision=precision, use_graph=precision)
        try:
            for k, f in fields[0]:
                d.set(0, k, f)
            d.bounduvw(False)
            d.boundp(capi.P)
            d.boundp(capi.S0)
            assert d.step(2) == 0
            err_t = compare_fields(case, O, d, (capi.S0,), 1e-10)
            _check(case, O, d, f"heated cavity 512x512x256, precision {precision} (temperature {err_t:.2e})")
        finally:
            d.close()
