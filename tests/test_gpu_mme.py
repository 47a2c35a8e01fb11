"""Fixed and random effects on the GPU vs the reference's FP64 program
(golden) and the oracle: the plain FP64 drop-in, relative error <= 1e-8."""
import numpy as np
import pytest

import globe_gb300 as G
from helpers import VC_F, golden_case, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["geno_small", "tiny"])
@pytest.mark.parametrize("src", ["geno", "grm"])
def test_mme_matches_reference_fp64(gctx, orc, name, src):
    c = golden_case(name)
    gctx.load_records(c["indiv"], c["X"], c["y"], c["N"])
    if src == "geno":
        gctx.load_bed(c["packed"])
        s = orc.Solver(c["indiv"], c["X"], c["y"], c["N"], VC_F, packed=c["packed"])
    else:
        gctx.load_grm(c["grm"], c["N"])
        s = orc.Solver(c["indiv"], c["X"], c["y"], c["N"], VC_F, grm_lt=c["grm"])
    gctx.set_vc(VC_F)
    r = gctx.mme(tol=1e-13, rule=G.RULE_PCGSOLVER)
    o = s.mme(1e-13, rule=0)
    for v in ("beta", "uhat", "bhat"):
        assert rel(r[v], o[v]) < 1e-8, v                          # oracle, same algorithm
        assert rel(r[v], c["ref"]["%s64_%s" % (src, v)]) < 2e-8, v  # the reference program


def test_mme_aireml_start_matches_oracle(gctx, orc):
    c = golden_case("aireml_small")
    th0 = c["ref"]["theta0"]
    gctx.load_records(c["indiv"], c["X"], c["y"], c["N"])
    gctx.load_grm(c["grm"], c["N"])
    gctx.set_vc(th0)
    r = gctx.mme(tol=1e-12, rule=G.RULE_AIREML, x0mode=G.X0_PRECOND)
    s = orc.Solver(c["indiv"], c["X"], c["y"], c["N"], th0, grm_lt=c["grm"])
    o = s.mme(1e-12, rule=1, x0mode=1)
    for v in ("beta", "uhat", "bhat", "vinv_r"):
        assert rel(r[v], o[v]) < 1e-8, v
