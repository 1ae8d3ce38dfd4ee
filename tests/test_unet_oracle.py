"""The U-Net oracle (float64 restatement of the 3-D learned guess's network) against finite differences and
the adjoint identities its backward pass relies on.  CPU only."""
import numpy as np

import unet


def test_pool_and_upsample_adjoints():
    rng = np.random.default_rng(3)
    for shape in ((4, 6, 8), (5, 3, 7)):
        a = rng.standard_normal((2, 3) + shape)
        cs = unet.coarse_shape(shape)
        g = rng.standard_normal((2, 3) + cs)
        # <pool(a), g> = <a, unpool(g)> and <upsample(g), a> = <g, sum_children(a)>
        assert np.isclose(np.sum(unet.pool(a) * g), np.sum(a * unet.unpool(g, shape)))
        assert np.isclose(np.sum(unet.upsample(g, shape) * a), np.sum(g * unet.sum_children(a, cs)))


def test_conv_input_grad_is_the_adjoint():
    rng = np.random.default_rng(4)
    x = rng.standard_normal((2, 16, 5, 4, 6))
    w = rng.standard_normal((32, 16, 27))
    dz = rng.standard_normal((2, 32, 5, 4, 6))
    assert np.isclose(np.sum(unet.conv(x, w) * dz), np.sum(x * unet.conv_input_grad(dz, w)))
    assert np.isclose(np.sum(unet.conv(x, w) * dz), np.sum(w * unet.weight_grad(dz, x)))


def test_gradient_matches_finite_differences():
    """Without BF16 rounding the network is a float64 function: central differences of the loss agree with
    the analytic gradient for parameters of every layer, the biases and the head."""
    rng = np.random.default_rng(5)
    shape = (6, 5, 7)
    x2 = np.zeros((2, 2) + shape)
    x2[:, 0] = rng.standard_normal((2,) + shape)
    x2[:, 1] = rng.random((2,) + shape) > 0.15
    t = rng.standard_normal((2,) + shape)
    p = unet.init_params(2)
    for l in range(5):  # non-zero biases, so that the bias gradients are exercised off the ReLU kinks
        o = unet.woff(l) + unet.CIN[l] * unet.COUT[l] * 27
        p[o:o + unet.COUT[l]] = 0.1 * rng.standard_normal(unet.COUT[l])
    L, g = unet.loss_and_grad(x2, t, p, rnd=False)
    assert unet.NPAR == 179889 and L > 0
    idx = []
    for l in range(5):
        o = unet.woff(l)
        n = unet.CIN[l] * unet.COUT[l] * 27
        live_w = [i for i in range(n) if (i // 27) % unet.CIN[l] < (2 if l == 0 else unet.CIN[l])]
        idx += list(rng.choice(live_w, 6, replace=False) + o)
        idx += [o + n + int(rng.integers(unet.COUT[l]))]
    idx += [unet.HEAD + 3, unet.HEAD + 16]
    eps = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fd = (unet.loss_and_grad(x2, t, pp, rnd=False)[0] - unet.loss_and_grad(x2, t, pm, rnd=False)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(g[i])) + 1e-7, (i, fd, g[i])
