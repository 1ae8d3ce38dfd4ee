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
