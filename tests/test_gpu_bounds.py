"""The bounds-checked debug build (libglobe_gb300_bounds.so, -DGLOBE_CHECK_BOUNDS):
every main operation runs through it with no failed index check, and the same
results as the production library.  It runs in a child process (the library is
chosen when globe_gb300 is imported)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from helpers import ROOT

pytestmark = pytest.mark.gpu

SCRIPT = r"""
import ctypes as C, json, sys
sys.path.insert(0, %(root)r); sys.path.insert(0, %(tests)r)
import numpy as np
import globe_gb300 as G
from globe_gb300 import synth
from helpers import VC_F, golden_case, cohort
L = G._lib.lib()
code = C.c_uint32(0)
out = {"status0": L.globe_debug_bounds(C.byref(code))}
c = golden_case("geno_small")
res = {}
with G.Context(0) as ctx:
    ctx.load_records(c["indiv"], c["X"], c["y"], c["N"])
    ctx.load_bed(c["packed"])
    ctx.set_vc(VC_F)
    Z = np.random.default_rng(1).standard_normal((c["N"], 4))
    B = np.column_stack([c["X"], c["y"]])
    for prec in (G.PREC_FP64, G.PREC_MIXED):
        ctx.set_precision(prec)
        res["grm%%d" %% prec] = ctx.grm_apply(Z).tolist()
        res["vx%%d" %% prec] = ctx.vx(B).tolist()
    ctx.set_precision(G.PREC_FP64)
    res["pcg"] = ctx.pcg(B, tol=1e-10, rule=G.RULE_AIREML)[0].tolist()
    res["pcg_mask"] = ctx.pcg(B, tol=1e-10, rule=G.RULE_AIREML, mask=True)[0].tolist()
    res["mme"] = ctx.mme(tol=1e-10, rule=G.RULE_PCGSOLVER, precision=G.PREC_MIXED)["uhat"].tolist()
    g = ctx.aireml_eval(4, seed=3, tol=1e-8, precision=G.PREC_MIXED)
    res["grad"] = g["grad"].tolist()
    res["ai"] = ctx.aireml_ai(tol=1e-8).tolist()
    gx = G.Context(0)
    gx.set_individuals(c["N"]); gx.set_precision(G.PREC_MIXED); gx.load_bed(c["packed"])
    res["lt"] = gx.grm_build()[:500].tolist()
    gx.close()
# long blocks (a warp per individual) and the dense product
coh = cohort(8, 300, 400, recs=("uniform", 40, 60), miss=0.02)
with G.Context(0) as ctx:
    ctx.load_records(coh["indiv"].astype(np.int32), coh["X"], coh["y"], 300)
    ctx.load_grm(synth.grm_from_packed(coh["packed"], 300), 300)
    ctx.set_vc(VC_F)
    Bl = np.column_stack([coh["X"], coh["y"]])
    res["long_pcg"] = ctx.pcg(Bl, tol=1e-10, rule=G.RULE_AIREML, precision=G.PREC_MIXED)[0].tolist()
out["status"] = L.globe_debug_bounds(C.byref(code))
out["code"] = code.value
out["res"] = res
print(json.dumps(out))
"""


def _run(lib):
    env = dict(os.environ, GLOBE_LIB=lib)
    r = subprocess.run([sys.executable, "-c", SCRIPT % {"root": ROOT, "tests": os.path.join(ROOT, "tests")}],
                       capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_checked_build_runs_clean():
    lib = os.path.join(ROOT, "globe_gb300", "libglobe_gb300_bounds.so")
    assert os.path.exists(lib), "build() makes the checked library beside the production one"
    chk = _run(lib)
    assert chk["status0"] == 0 and chk["status"] == 0, hex(chk["code"])
    prod = _run(os.path.join(ROOT, "globe_gb300", "libglobe_gb300.so"))
    assert prod["status"] < 0                      # production build: the checks are compiled out
    for key, val in prod["res"].items():           # and the checks change no result (two compiles
        a, b = np.asarray(val), np.asarray(chk["res"][key])   # may contract FMAs differently)
        assert np.abs(a - b).max() <= 1e-12 * max(np.abs(a).max(), 1e-300), key
