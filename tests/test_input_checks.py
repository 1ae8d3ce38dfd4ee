"""Host-side input validation of snac_init's set-up (snac_check_case: placement, grids, operator
assembly, hierarchy), without a device: the reference's fatal input errors become SNAC_ERR_* codes."""
import ctypes as C
import dataclasses

import pytest

from snac_gb300 import capi, cases


def check(case):
    c, arr, keep = capi.fill_descs(case)
    lev = C.c_int()
    coarse = C.c_long()
    rc = capi.lib().snac_check_case(C.byref(c), arr, C.byref(lev), C.byref(coarse))
    return rc, lev.value, coarse.value


def test_valid_cases_accepted():
    for case in (cases.ldc_reference_test(0), cases.ldc_reference_test(1), cases.taylor_green(16),
                 cases.channel_4block(), cases.l_shaped_box(16, 8), cases.heated_cavity(n=(16, 16, 8)),
                 cases.kovasznay(), cases.developing_duct(), cases.dhc_reference_test()):
        rc, lev, coarse = check(case)
        assert rc == 0, (case.name, capi.lib().snac_last_error())
        assert lev >= 1 and coarse >= 1


def test_channel_hierarchy():
    """The semicoarsened hierarchy of the benchmark channel ends in a 16 x 9 dense level (7 levels)."""
    rc, lev, coarse = check(cases.channel_4block())
    assert rc == 0 and lev == 7 and coarse == 16 * 9


def test_no_blocks_rejected():
    case = dataclasses.replace(cases.ldc_reference_test(0), blocks=[])
    c, arr, keep = capi.fill_descs(cases.ldc_reference_test(0))
    c.nblocks = 0
    assert capi.lib().snac_check_case(C.byref(c), arr, None, None) == capi.ERR_ARG


def test_inconsistent_friend_rejected():
    """A friend face whose neighbour does not point back (initmpi.f90 connectivity) is an input error."""
    case = cases.channel_4block(nx=(16, 32), ny=(8, 16), nz=16)
    b0 = case.blocks[0]
    bad = dataclasses.replace(b0, ng=(b0.ng[0], b0.ng[1] + 2, b0.ng[2]))  # no longer matches its friends
    case = dataclasses.replace(case, blocks=[bad] + list(case.blocks[1:]))
    rc, _, _ = check(case)
    assert rc == capi.ERR_ARG


def test_inflow_on_periodic_axis_rejected():
    """chk_inflow (sanity.f90:173-189): periodicity and inflow BCs cannot be combined."""
    case = cases.kovasznay()
    b = case.blocks[0]
    bad = dataclasses.replace(b, inflow_type=[[0, 0], [1, 0], [0, 0]])  # y is periodic
    rc, _, _ = check(dataclasses.replace(case, blocks=[bad]))
    assert rc == capi.ERR_ARG
    assert b"periodicity" in capi.lib().snac_last_error()


def test_dn_transform_pair_rejected():
    """fft.f90 defines no eigenvalues for a 'DN' pressure pair along the transform axis."""
    case = cases.ldc_reference_test(1)
    blocks = []
    for b in case.blocks:
        cp = [list(r) for r in b.cbcpre]
        cp[0] = ["D", "N"]
        blocks.append(dataclasses.replace(b, cbcpre=cp))
    rc, _, _ = check(dataclasses.replace(case, blocks=blocks))
    assert rc in (capi.ERR_ARG, capi.ERR_UNSUPPORTED)


def test_one_cell_periodic_axis_accepted():
    """A one-cell periodic direction (a 2-D problem run in 3-D) is a valid layout for both solves."""
    for fa in (0, 3):
        case = dataclasses.replace(cases.taylor_green(16), fft_axis=fa)
        b = case.blocks[0]
        case = dataclasses.replace(case, blocks=[dataclasses.replace(b, ng=(16, 16, 1))])
        rc, lev, _ = check(case)
        assert rc == 0, capi.lib().snac_last_error()


@pytest.mark.parametrize("hi", [(65536, 65536, 1), (2147483647 - 63, 1, 1), (1, 1, 2147483647)])
def test_chkdiv_noalloc_rejects_oversized_block(hi):
    """The allocation-free divergence check rejects, on the host and before any device work, a block above
    2^31 - 1 cells or one whose extent along an axis leaves no room for the (n + 2)-long metric arrays in
    32-bit indices; the placeholder device pointers passed here are never dereferenced."""
    tot, mx = C.c_double(), C.c_double()
    L = capi.lib()
    rc = L.snac_chkdiv_noalloc(capi.iarr((1, 1, 1)), capi.iarr(hi), 8, 8, 8, 8, 8, 8, 1.0, None, C.byref(tot),
                               C.byref(mx))
    assert rc == capi.ERR_ARG
    assert b"exceeds" in L.snac_last_error()
