"""The bounds-check build on the GPU: cases step through it with every check passing and the same results as
the normal build, and a check that fails by design (the probe addresses nothing) comes back as SNAC_ERR_BOUNDS
naming the kernel and the cell, after which the library keeps working."""
import json
import os
import subprocess
import sys

import pytest

from snac_gb300 import capi

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import dataclasses, json, sys
sys.path.insert(0, %(root)r)
from snac_gb300 import capi, cases
from snac_gb300.domain import Domain
L = capi.lib()
out = {"checked": L.snac_bounds_checked()}
def run(name, case, init, steps):
    d = Domain(case, precision=1)
    try:
        init(d, case)
        d.step(steps)
        out[name] = {"ke": d.kinetic_energy(), "div": d.chkdiv()[1]}
    finally:
        d.close()
def init_channel(d, case):
    ic = cases.channel_initial_condition(case, lambda ib: d.grid(ib, 1, capi.G_XC))
    for ib, (u, v, w) in ic.items():
        d.set(ib, capi.U, u); d.set(ib, capi.V, v); d.set(ib, capi.W, w)
    d.bounduvw(False)
def init_rest(d, case):
    d.bounduvw(False)
run("channel", cases.channel_4block(nx=(32, 64), ny=(32, 48), nz=16), init_channel, 3)
run("lbox", dataclasses.replace(cases.l_shaped_box(16, 8), dt_f=4e-3), init_rest, 3)
rc = L.snac_bounds_selftest()
out["selftest"] = [rc, L.snac_last_error().decode()]
run("after", dataclasses.replace(cases.l_shaped_box(16, 8), dt_f=4e-3), init_rest, 1)
print(json.dumps(out))
"""


def test_bounds_checked_build_runs_clean_and_reports_a_failure(snac_lib):
    env = dict(os.environ, SNAC_BOUNDS_CHECK="1")
    r = subprocess.run([sys.executable, "-c", SCRIPT % {"root": ROOT}], env=env, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["checked"] == 1
    rc, msg = out["selftest"]
    assert rc == capi.ERR_BOUNDS and "probe" in msg and "(9, 0, 0)" in msg, (rc, msg)
    assert out["after"]["div"] < 1e-10
    # the same cases on the normal build give the same results (the checks change no arithmetic)
    import dataclasses
    from snac_gb300 import cases
    from snac_gb300.domain import Domain
    assert capi.lib().snac_bounds_selftest() == capi.ERR_UNSUPPORTED
    for name, case in (("channel", cases.channel_4block(nx=(32, 64), ny=(32, 48), nz=16)),
                       ("lbox", dataclasses.replace(cases.l_shaped_box(16, 8), dt_f=4e-3))):
        d = Domain(case, precision=1)
        try:
            if name == "channel":
                ic = cases.channel_initial_condition(case, lambda ib: d.grid(ib, 1, capi.G_XC))
                for ib, (u, v, w) in ic.items():
                    d.set(ib, capi.U, u)
                    d.set(ib, capi.V, v)
                    d.set(ib, capi.W, w)
            d.bounduvw(False)
            d.step(3)
            assert d.kinetic_energy() == out[name]["ke"], name
        finally:
            d.close()
