"""The tensor-core (tcgen05) 3x3 convolution of the learned initial guess against a float64 reference of
the same BF16-rounded inputs."""
import ctypes as C

import numpy as np
import pytest

from snac_gb300 import capi

pytestmark = pytest.mark.gpu


def bf16(a):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def conv_ref(x, w, b, relu):
    n, c, h, wd = x.shape
    xp = np.zeros((n, c, h + 2, wd + 2))
    xp[:, :, 1:-1, 1:-1] = bf16(x)
    wb = bf16(w)
    y = np.zeros((n, 16, h, wd))
    for dy in range(3):
        for dx in range(3):
            y += np.einsum("oc,nchw->nohw", wb[:, :, dy, dx], xp[:, :, dy:dy + h, dx:dx + wd])
    y += b[None, :, None, None]
    return np.maximum(y, 0.0) if relu else y


@pytest.mark.parametrize("shape,relu", [((1, 16, 3, 128), 0), ((2, 16, 5, 200), 1), ((3, 16, 7, 37), 0)])
def test_conv3x3_tcgen05(snac_lib, shape, relu):
    rng = np.random.default_rng(sum(shape))
    x = rng.standard_normal(shape).astype(np.float32)
    w = (0.2 * rng.standard_normal((16, 16, 3, 3))).astype(np.float32)
    b = rng.standard_normal(16).astype(np.float32)
    y = np.zeros(shape, dtype=np.float32)
    rc = capi.lib().snac_cnn_conv3x3(x.ctypes.data_as(capi.FP), shape[0], shape[2], shape[3],
                                     w.ctypes.data_as(capi.FP), b.ctypes.data_as(capi.FP), relu, y.ctypes.data_as(capi.FP))
    assert rc == 0, capi.lib().snac_last_error()
    ref = conv_ref(x, w, b.astype(np.float64), relu)
    np.testing.assert_allclose(y, ref, rtol=1e-5, atol=1e-5 * np.max(np.abs(ref)))


def test_conv3x3_accumulator_wait_runs_out(snac_lib):
    """The convolution's wait for its tensor-core accumulator is bounded.  With the bound set to zero polls every
    wait runs out at once: the call reports SNAC_ERR_TIMEOUT, having let the MMAs in flight finish and freed the
    tensor memory, and the next call (default bound) on the same context gives the right answer -- which it
    could not if the tensor memory had not been released."""
    L = capi.lib()
    shape = (2, 16, 5, 200)
    rng = np.random.default_rng(77)
    x = rng.standard_normal(shape).astype(np.float32)
    w = (0.2 * rng.standard_normal((16, 16, 3, 3))).astype(np.float32)
    b = rng.standard_normal(16).astype(np.float32)
    y = np.zeros(shape, dtype=np.float32)
    args = (x.ctypes.data_as(capi.FP), shape[0], shape[2], shape[3], w.ctypes.data_as(capi.FP),
            b.ctypes.data_as(capi.FP), 1, y.ctypes.data_as(capi.FP))
    try:
        assert L.snac_cnn_set_poll_limit(0) == 0
        assert L.snac_cnn_conv3x3(*args) == capi.ERR_TIMEOUT
        assert b"timed out" in L.snac_last_error()
    finally:
        L.snac_cnn_set_poll_limit(-1)
    assert L.snac_cnn_conv3x3(*args) == 0, L.snac_last_error()
    ref = conv_ref(x, w, b.astype(np.float64), 1)
    np.testing.assert_allclose(y, ref, rtol=1e-5, atol=1e-5 * np.max(np.abs(ref)))


NPAR = 3 * (16 * 16 * 9 + 16)


def unpack(params):
    out, o = [], 0
    for _ in range(3):
        w = params[o:o + 2304].reshape(16, 16, 3, 3).astype(np.float64)
        b = params[o + 2304:o + 2320].astype(np.float64)
        out.append((w, b))
        o += 2320
    return out


def conv(x, w):  # x (n, 16, h, wd) already rounded as the forward rounds it; w (16, 16, 3, 3)
    n, c, h, wd = x.shape
    xp = np.zeros((n, c, h + 2, wd + 2))
    xp[:, :, 1:-1, 1:-1] = x
    y = np.zeros((n, 16, h, wd))
    for dy in range(3):
        for dx in range(3):
            y += np.einsum("oc,nchw->nohw", w[:, :, dy, dx], xp[:, :, dy:dy + h, dx:dx + wd])
    return y


def net_oracle(x, t, params):
    """The network in float64 with the tensor-core forward's BF16 roundings (inputs and weights of every
    layer), its loss, and the gradients by backpropagation (straight through the roundings)."""
    layers = unpack(params)
    xs, ys = [bf16(x)], []
    for l, (w, b) in enumerate(layers):
        y = conv(xs[l], bf16(w)) + b[None, :, None, None]
        if l < 2:
            y = np.maximum(y, 0.0)
            xs.append(bf16(y))
        ys.append(y)
    nb = x.shape[0]
    tn = (t.astype(np.float64) ** 2).sum(axis=(1, 2))
    e = ys[2][:, 0] - t
    loss = float(((e ** 2).sum(axis=(1, 2)) / tn).sum() / nb)
    d = np.zeros_like(ys[2])
    d[:, 0] = 2.0 * e / (nb * tn[:, None, None])
    grads = []
    for l in (2, 1, 0):
        w, b = layers[l]
        if l < 2:
            d = d * (ys[l] > 0)
        n, c, h, wd = xs[l].shape
        xp = np.zeros((n, c, h + 2, wd + 2))
        xp[:, :, 1:-1, 1:-1] = xs[l]
        gw = np.zeros((16, 16, 3, 3))
        for dy in range(3):
            for dx in range(3):
                gw[:, :, dy, dx] = np.einsum("nohw,nchw->oc", d, xp[:, :, dy:dy + h, dx:dx + wd])
        gb = d.sum(axis=(0, 2, 3))
        grads.append((l, gw, gb))
        if l > 0:  # input gradient: correlation with the flipped BF16 kernel
            dp = np.zeros((n, 16, h + 2, wd + 2))
            dp[:, :, 1:-1, 1:-1] = d
            wb = bf16(w)
            dn = np.zeros((n, 16, h, wd))
            for dy in range(3):
                for dx in range(3):
                    dn += np.einsum("oc,nohw->nchw", wb[:, :, dy, dx], dp[:, :, 2 - dy:2 - dy + h, 2 - dx:2 - dx + wd])
            d = dn
    flat = np.zeros(NPAR)
    for l, gw, gb in grads:
        flat[l * 2320:l * 2320 + 2304] = gw.ravel()
        flat[l * 2320 + 2304:(l + 1) * 2320] = gb
    return loss, flat


def test_guess_network_gradients_match_oracle(snac_lib):
    """Forward on the tensor cores and backward on the GPU give the loss and the gradient of every parameter
    of the learned-guess network as the float64 oracle does (up to FP32 accumulation)."""
    rng = np.random.default_rng(31)
    nb, h, wd = 2, 6, 150
    x = np.zeros((nb, 16, h, wd), dtype=np.float32)
    x[:, 0] = rng.standard_normal((nb, h, wd))
    x[:, 1] = 0.3
    t = rng.standard_normal((nb, h, wd)).astype(np.float32)
    params = np.zeros(NPAR, dtype=np.float32)
    for l in range(3):
        params[l * 2320:l * 2320 + 2304] = 0.3 * rng.standard_normal(2304)
        params[l * 2320 + 2304:(l + 1) * 2320] = 0.05 * rng.standard_normal(16)
    grads = np.zeros(NPAR, dtype=np.float32)
    loss = C.c_double()
    rc = capi.lib().snac_guess_grad(x.ctypes.data_as(capi.FP), t.ctypes.data_as(capi.FP), nb, h, wd,
                                    params.ctypes.data_as(capi.FP), grads.ctypes.data_as(capi.FP), C.byref(loss))
    assert rc == 0, capi.lib().snac_last_error()
    lo, go = net_oracle(x.astype(np.float64), t.astype(np.float64), params)
    assert abs(loss.value - lo) <= 1e-4 * lo
    for l in range(3):
        a, b = grads[l * 2320:(l + 1) * 2320], go[l * 2320:(l + 1) * 2320]
        assert np.linalg.norm(a - b) <= 2e-3 * np.linalg.norm(b), l


def test_learned_guess_trains_and_reports_gain(snac_lib):
    """The learned initial guess end to end on a four-block channel: pairs recorded from the solver's own
    solves, training on the GPU (tensor-core forward, FP32 backward, Adam), then guided solves.  The
    multigrid still iterates to the same tolerance; the test states what the network gains: the residual
    its correction leaves relative to the previous solution's residual, per wavenumber system (the
    minimal-residual step keeps that ratio at or below 1 for every system)."""
    from snac_gb300 import cases
    from snac_gb300.domain import Domain
    L = capi.lib()
    case = cases.channel_4block(nx=(32, 64), ny=(32, 48), nz=16)
    d = Domain(case, precision=1)
    try:
        ic = cases.channel_initial_condition(case, lambda ib: d.grid(ib, 1, capi.G_XC))
        for ib, (u, v, w) in ic.items():
            d.set(ib, capi.U, u)
            d.set(ib, capi.V, v)
            d.set(ib, capi.W, w)
        d.bounduvw(False)
        d.step(3)
        assert L.snac_guess_mode(1) == 0
        d.step(6)
        lf, ll, npairs = C.c_double(), C.c_double(), C.c_int()
        assert L.snac_guess_train(400, 2e-3, C.byref(lf), C.byref(ll), C.byref(npairs)) == 0, L.snac_last_error()
        assert npairs.value == 6 * 3 * 16
        assert ll.value < 0.5 * lf.value, (lf.value, ll.value)  # the network learns the corrections
        assert L.snac_guess_mode(0) == 0
        d.step(2)
        plain = d.stats()
        assert L.snac_guess_mode(2) == 0
        med, mx = C.c_double(), C.c_double()
        assert L.snac_guess_measure(1, None, None) == 0
        d.step(2)
        guided = d.stats()
        assert L.snac_guess_measure(1, C.byref(med), C.byref(mx)) == 0
        assert guided["residual"] <= case.tol and d.chkdiv()[1] < 1e-10  # same tolerance, same projection
        assert 0.0 < med.value < 0.9, med.value  # the correction reduces the typical system's residual
        assert mx.value <= 1.0 + 1e-12, mx.value  # and no system's
        print(f"loss {lf.value:.3f} -> {ll.value:.3f}; residual after the guess / before: median {med.value:.3f}, "
              f"largest {mx.value:.3f}; refinement steps plain {plain['iters']} guided {guided['iters']}")
    finally:
        L.snac_guess_mode(0)
        d.close()
