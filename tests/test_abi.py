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


def _fortran_types():
    """Members of every `type, bind(C)` of the Fortran module: [(name, kind, element count)] in order."""
    src = open(os.path.join(ROOT, "fortran", "mod_snac_gpu.f90")).read()
    params = {m.group(1).lower(): int(m.group(2))
              for m in re.finditer(r"\b(\w+)\s*=\s*(\d+)\b", re.sub(r"!.*", "", src)) if m.group(1).isupper()}
    types = {}
    for m in re.finditer(r"type, bind\(C\) :: (\w+)\n(.*?)\n\s*end type", src, flags=re.S):
        members = []
        for line in m.group(2).splitlines():
            line = re.sub(r"!.*", "", line).strip()
            if not line:
                continue
            decl, names = line.split("::")
            kind = re.search(r"(c_int|c_double|c_char|c_ptr)", decl).group(1)
            for item in re.findall(r"(\w+)(\([^)]*\))?(?:\s*=\s*[^,]+)?", names):
                name, dims = item
                count = 1
                for d in (dims.strip("()").split(",") if dims else []):
                    d = d.strip()
                    count *= int(d) if d.isdigit() else params[d.lower()]
                members.append((name.lower(), kind, count))
        types[m.group(1)] = members
    return types


def _ctypes_members(struct):
    import ctypes as C
    out = []
    for name, t in struct._fields_:
        count = 1
        while hasattr(t, "_length_"):
            count *= t._length_
            t = t._type_
        kind = {C.c_int: "c_int", C.c_double: "c_double", C.c_char: "c_char"}.get(t, "c_ptr")
        out.append((name, kind, count))
    return out


def test_fortran_types_match_the_c_structs():
    """The module's bind(C) types for snac_init carry the members of snac_case, snac_block_desc and snac_options
    in the same order, with the same interoperable kinds and element counts as the C structs (through the
    ctypes mirrors the tests drive), so a Fortran driver passes the layout the library reads."""
    from snac_gb300 import capi
    types = _fortran_types()
    for ftype, struct in (("snac_case", capi.CaseDesc), ("snac_block_desc", capi.BlockDesc),
                          ("snac_options", capi.Options)):
        assert types[ftype] == _ctypes_members(struct), ftype


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
