"""The C ABI library loads and exports every function declared in include/snac_gpu.h (no GPU needed)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "snac_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(snac_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_hot_path():
    names = declared_functions()
    for n in ("snac_rk_mom", "snac_fillps", "snac_correc", "snac_updt_pressure", "snac_updt_rhs", "snac_chkdt",
              "snac_chkdiv", "snac_set_bc", "snac_fft", "snac_init", "snac_step", "snac_solve_pressure",
              "snac_bounduvw_all", "snac_boundp_all"):
        assert n in names


def test_library_exports_every_declared_symbol():
    from snac_gb300 import capi, _build
    path = _build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # the Python prototypes cover the whole header too
    assert sorted(capi.PROTOTYPES) == declared_functions()


def test_fortran_module_binds_declared_functions():
    """fortran/mod_snac_gpu.f90 binds only entry points the header declares, one interface each, and covers the
    reference-signature and per-block boundary calls (the module is not compiled here: no Fortran compiler)."""
    src = open(os.path.join(ROOT, "fortran", "mod_snac_gpu.f90")).read()
    bound = re.findall(r"bind\(C,name='(snac_[a-z0-9_]+)'\)", src)
    assert len(bound) == len(set(bound))
    assert set(bound) <= set(declared_functions())
    for n in ("snac_rk_mom", "snac_fillps", "snac_correc", "snac_updt_pressure", "snac_chkdt", "snac_chkdiv",
              "snac_bounduvw", "snac_boundp", "snac_impdiff_solve", "snac_fft"):
        assert n in bound, n


def test_calls_fail_cleanly_without_device():
    """Without a CUDA device the library reports SNAC_ERR_CUDA instead of computing anything on the CPU."""
    from snac_gb300 import capi
    if capi.device_count() > 0:
        return
    import numpy as np
    from snac_gb300 import cases
    from snac_gb300.domain import Domain
    try:
        Domain(cases.lid_driven_cavity(8))
    except capi.SnacError as e:
        assert e.code == capi.ERR_CUDA
    else:
        raise AssertionError("snac_init succeeded without a device")
