"""snac_chkdiv_noalloc: the divergence check for callers that cannot allocate device memory.

A driver that placed its fields on the GPU once and checks the divergence
inside its time loop cannot afford a cudaMalloc/cudaFree per check (they
synchronise the device and fail on a full GPU).  This entry point takes the
caller's device arrays and uses only a fixed scratch array owned by the
library.  The test gives it device copies of the same fields that the regular
snac_chkdiv receives as host arrays and requires the same results, twice in a
row (the second call reuses the scratch the first one left behind).
This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from snac_gb300 import capi, hotpath

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    flat = np.ascontiguousarray(a.reshape(-1, order="F"))
    return torch.from_numpy(flat).to("cuda")


def _oracle_chkdiv(oracle_mod, lo, hi, dxf, dyf, dzf, u, v, w, vol):
    tot, mx = C.c_double(), C.c_double()
    p = oracle_mod._ptr
    oracle_mod.lib().or_chkdiv_local(capi.iarr(lo), capi.iarr(hi), p(dxf), p(dyf), p(dzf), p(u), p(v), p(w), vol,
                                     C.byref(tot), C.byref(mx))
    return tot.value, mx.value


# (13, 9, 11): ragged tiles at an offset; (96, 64, 40): 960 tiles, one per CTA; (256, 144, 128): the largest
# block of the four-block channel layout's solver box, 18,432 tiles, so every CTA walks several of them
@pytest.mark.parametrize("shape,lo,stream", [((13, 9, 11), (3, 5, 7), False), ((96, 64, 40), (1, 1, 1), False),
                                             ((256, 144, 128), (1, 1, 1), True)])
def test_chkdiv_noalloc_matches_chkdiv(snac_lib, oracle_mod, shape, lo, stream):
    import torch
    rng = np.random.default_rng(7)
    hi = tuple(lo[a] + shape[a] - 1 for a in range(3))
    u, v, w = (np.asfortranarray(rng.standard_normal(tuple(n + 2 for n in shape))) for _ in range(3))
    dxf, dyf, dzf = (0.5 + rng.random(n + 2) for n in shape)
    vol = 3.7
    ref_tot, ref_max = hotpath.chkdiv(lo, hi, dxf, dyf, dzf, u, v, w, vol)
    or_tot, or_max = _oracle_chkdiv(oracle_mod, lo, hi, dxf, dyf, dzf, u, v, w, vol)
    du, dv, dw, gx, gy, gz = (_dev(a) for a in (u, v, w, dxf, dyf, dzf))
    torch.cuda.synchronize()
    # a caller's own stream (the documented contract: the kernels run on it and the call waits for them)
    s = torch.cuda.Stream() if stream else None
    handle = s.cuda_stream if s is not None else None
    L = capi.lib()
    for _ in range(2):
        tot, mx = C.c_double(), C.c_double()
        capi.check(L.snac_chkdiv_noalloc(capi.iarr(lo), capi.iarr(hi), gx.data_ptr(), gy.data_ptr(), gz.data_ptr(),
                                         du.data_ptr(), dv.data_ptr(), dw.data_ptr(), vol, handle, C.byref(tot),
                                         C.byref(mx)))
        assert abs(mx.value - ref_max) <= 1e-13 * ref_max
        assert abs(mx.value - or_max) <= 1e-13 * or_max
        # the total is a signed sum of O(1) terms summed in another order: compare against the number of terms
        assert abs(tot.value - ref_tot) <= 1e-13 * np.prod(shape)
        assert abs(tot.value - or_tot) <= 1e-13 * np.prod(shape)


def test_chkdiv_noalloc_rejects_oversized_block(snac_lib):
    lo, hi = (1, 1, 1), (65536, 65536, 1)
    tot, mx = C.c_double(), C.c_double()
    rc = capi.lib().snac_chkdiv_noalloc(capi.iarr(lo), capi.iarr(hi), 1, 1, 1, 1, 1, 1, 1.0, None, C.byref(tot),
                                        C.byref(mx))
    assert rc == capi.ERR_ARG
    assert b"exceeds" in capi.lib().snac_last_error()
