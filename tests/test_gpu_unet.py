"""The three-level U-Net of the 3-D pressure solve's learned guess: its tensor-core forward pass and its
gradients against the float64 oracle (oracle/unet.py, same BF16 rounding points), the bounded accumulator
wait, and the guess end to end in the 3-D solve of an L-shaped box."""
import ctypes as C

import numpy as np
import pytest

import unet
from snac_gb300 import capi

pytestmark = pytest.mark.gpu


def _inputs(rng, nb, shape, dead=0.1):
    x2 = np.zeros((nb, 2) + shape, dtype=np.float32)
    x2[:, 0] = rng.standard_normal((nb,) + shape)
    x2[:, 1] = rng.random((nb,) + shape) > dead
    return x2


def _params(seed):
    rng = np.random.default_rng(seed)
    p = unet.init_params(seed)
    for l in range(5):
        o = unet.woff(l) + unet.CIN[l] * unet.COUT[l] * 27
        p[o:o + unet.COUT[l]] = 0.1 * rng.standard_normal(unet.COUT[l])
    p[unet.HEAD + 16] = 0.05
    return p.astype(np.float32)


def _forward(x2, p):
    nb, _, n2, n1, n0 = x2.shape
    out = np.zeros((nb, n2, n1, n0), dtype=np.float32)
    rc = capi.lib().snac_unet_forward(x2.ctypes.data_as(capi.FP), nb, n0, n1, n2, p.ctypes.data_as(capi.FP),
                                      out.ctypes.data_as(capi.FP))
    return rc, out


@pytest.mark.parametrize("nb,shape", [(2, (6, 10, 40)), (1, (5, 6, 130)), (1, (9, 7, 33)), (3, (4, 4, 4))])
def test_unet_forward_matches_oracle(snac_lib, nb, shape):
    """tcgen05 forward (row segments of 128 cells, ragged x extents, odd extents that pool to partial windows,
    several volumes) against the oracle with the same BF16 operands."""
    assert capi.lib().snac_unet_nparams() == unet.NPAR
    rng = np.random.default_rng(sum(shape) + nb)
    x2 = _inputs(rng, nb, shape)
    p = _params(nb + shape[2])
    rc, out = _forward(x2, p)
    assert rc == 0, capi.lib().snac_last_error()
    ref, _ = unet.forward(x2.astype(np.float64), p.astype(np.float64))
    err = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    assert err < 2e-3, err
    assert np.max(np.abs(out - ref)) < 2e-2 * np.max(np.abs(ref))


def test_unet_gradients_match_oracle(snac_lib):
    """Loss and gradient of every layer (input gradients through the transposed tcgen05 convolutions, weight
    gradients as FP32 reductions on the CUDA cores) against the oracle's backward pass."""
    rng = np.random.default_rng(17)
    nb, shape = 2, (8, 6, 20)
    x2 = _inputs(rng, nb, shape)
    t = rng.standard_normal((nb,) + shape).astype(np.float32)
    p = _params(23)
    g = np.zeros(unet.NPAR, dtype=np.float32)
    loss = C.c_double()
    rc = capi.lib().snac_unet_grad(x2.ctypes.data_as(capi.FP), t.ctypes.data_as(capi.FP), nb, shape[2], shape[1],
                                   shape[0], p.ctypes.data_as(capi.FP), g.ctypes.data_as(capi.FP), C.byref(loss))
    assert rc == 0, capi.lib().snac_last_error()
    lo, go = unet.loss_and_grad(x2.astype(np.float64), t.astype(np.float64), p.astype(np.float64))
    assert abs(loss.value - lo) <= 1e-3 * lo, (loss.value, lo)
    for l in range(5):
        o, n = unet.woff(l), unet.CIN[l] * unet.COUT[l] * 27
        for a, b, what in ((g[o:o + n], go[o:o + n], "w"), (g[o + n:o + n + unet.COUT[l]], go[o + n:o + n + unet.COUT[l]], "b")):
            assert np.linalg.norm(a - b) <= 2e-2 * np.linalg.norm(b), (l, what, np.linalg.norm(a - b) / np.linalg.norm(b))
    h = slice(unet.HEAD, unet.NPAR)
    assert np.linalg.norm(g[h] - go[h]) <= 2e-2 * np.linalg.norm(go[h])


def test_unet_accumulator_wait_runs_out(snac_lib):
    """With the poll bound at zero every accumulator wait of the U-Net's convolutions runs out: the call reports
    SNAC_ERR_TIMEOUT after the kernels let their MMAs finish and free their tensor memory; the next call, with
    the default bound, gives the right answer on the same context."""
    L = capi.lib()
    rng = np.random.default_rng(8)
    x2 = _inputs(rng, 1, (4, 6, 20))
    p = _params(3)
    try:
        assert L.snac_unet_set_poll_limit(0) == 0
        rc, _ = _forward(x2, p)
        assert rc == capi.ERR_TIMEOUT
        assert b"timed out" in L.snac_last_error()
    finally:
        L.snac_unet_set_poll_limit(-1)
    rc, out = _forward(x2, p)
    assert rc == 0, L.snac_last_error()
    ref, _ = unet.forward(x2.astype(np.float64), p.astype(np.float64))
    assert np.linalg.norm(out - ref) <= 2e-3 * np.linalg.norm(ref)


def test_unet_guess_in_the_3d_solve(snac_lib):
    """The learned guess of the 3-D solve end to end on a lid-driven L-shaped box: crops of (residual of the
    previous solution, diagonally scaled correction) recorded from the solver's own solves, the U-Net trained on
    the GPU, then guided solves.  The multigrid iterates to the same tolerance; the minimal-residual step keeps
    the residual the guess leaves at or below the previous solution's, and the test prints what it gains."""
    import dataclasses
    from snac_gb300 import cases
    from snac_gb300.domain import Domain
    L = capi.lib()
    # fixed dt: from rest the CFL limit sees no velocity, and the viscous one alone is too large at this size
    case = dataclasses.replace(cases.l_shaped_box(24, 16), dt_f=4e-3)
    d = Domain(case, precision=1)
    try:
        d.step(4)
        assert L.snac_guess_mode(1) == 0
        d.step(8)
        lf, ll, npairs = C.c_double(), C.c_double(), C.c_int()
        assert L.snac_guess_train(150, 2e-3, C.byref(lf), C.byref(ll), C.byref(npairs)) == 0, L.snac_last_error()
        assert npairs.value == 8 * 3 * 4
        assert ll.value < lf.value, (lf.value, ll.value)
        assert L.snac_guess_mode(0) == 0
        d.step(2)
        plain = d.stats()
        assert L.snac_guess_mode(2) == 0
        assert L.snac_guess_measure(1, None, None) == 0
        d.step(2)
        guided = d.stats()
        med, mx = C.c_double(), C.c_double()
        assert L.snac_guess_measure(1, C.byref(med), C.byref(mx)) == 0
        assert guided["residual"] <= case.tol and d.chkdiv()[1] < 1e-10
        assert 0.0 < med.value <= 1.0 + 1e-12, med.value
        print(f"U-Net loss {lf.value:.3f} -> {ll.value:.3f}; residual after the guess / before {med.value:.3f}; "
              f"refinement steps plain {plain['iters']} guided {guided['iters']}")
    finally:
        L.snac_guess_mode(0)
        d.close()
