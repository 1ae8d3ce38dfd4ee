"""The bounds-check build (-DSNAC_BOUNDS_CHECK) compiles, exports the whole C ABI and reports itself; the normal
build reports no checks.  CPU only (no kernel runs)."""
import ctypes as C
import re

from snac_gb300 import _build, capi


def test_checked_library_builds_and_reports_itself():
    path = _build.build_checked()
    L = C.CDLL(path)
    L.snac_bounds_checked.restype = C.c_int
    assert L.snac_bounds_checked() == 1
    with open(_build.os.path.join(_build.ROOT, "include", "snac_gpu.h")) as f:
        names = set(re.findall(r"\b(snac_\w+)\s*\(", f.read()))
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert capi.lib().snac_bounds_checked() == 0
