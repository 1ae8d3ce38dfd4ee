"""The oracle against the reference's own golden vector.

tests/lid_driven_cavity of the reference runs four 2x32x32 blocks for 1500
steps (HYPRE PFMG, FFT_AXIS=0 and FFT_AXIS=1) and checks the v profile at the
cavity mid-plane against data_ldc_re1000.txt with rtol=1e-7, atol=5e-8
(tests/lid_driven_cavity/test.py:15).  The oracle must pass the same check.
"""
import os

import numpy as np
import pytest

from snac_gb300 import cases

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ldc_re1000_profile.txt")


def ldc_profile(get_v):
    """test.py:4-15: np.block([[d1,d3],[d2,d4]]) of v(x=1,:,:) per block, row 32 (0-based)."""
    blk = lambda ib: get_v(ib)[1, 1:-1, 1:-1]
    data = np.block([[blk(0), blk(2)], [blk(1), blk(3)]])
    return data[data.shape[1] // 2, :]


@pytest.mark.parametrize("fft_axis", [1, 0])
def test_oracle_ldc_golden(oracle_mod, fft_axis):
    O = oracle_mod
    d = O.OracleDomain(cases.ldc_reference_test(fft_axis=fft_axis, tol=1e-12))
    d.bounduvw(False)
    d.boundp(O.P)
    d.step(1500)
    prof = ldc_profile(lambda ib: d.field(ib, O.V))
    ref = np.loadtxt(GOLDEN)
    np.testing.assert_allclose(prof, ref[:, 1], rtol=1e-7, atol=5e-8)
    divtot, divmax = d.chkdiv()
    assert divmax < 1e-10
