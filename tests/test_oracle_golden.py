"""Pin the C oracle to the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from the upstream programs)."""
import numpy as np
import pytest

from helpers import VC_F, aireml_probes, golden_case, rel


@pytest.mark.parametrize("name", ["geno_small", "tiny"])
def test_bed_stats_bit_exact(orc, name):
    c = golden_case(name)
    alt, miss, maf, mr, keep = orc.bed_stats(c["packed"], c["N"])
    r = c["ref"]
    assert np.array_equal(alt, r["stats_alt"])
    assert np.array_equal(miss, r["stats_miss"])
    assert np.array_equal(maf.view(np.uint32), r["stats_maf"].view(np.uint32))
    assert np.array_equal(mr.view(np.uint32), r["stats_miss_rate"].view(np.uint32))
    assert np.array_equal(keep, r["stats_keep"].astype(bool))


@pytest.mark.parametrize("name", ["geno_small", "tiny"])
@pytest.mark.parametrize("src", ["geno", "grm"])
def test_mme_vs_fp64_reference(orc, name, src):
    c = golden_case(name)
    kw = dict(packed=c["packed"]) if src == "geno" else dict(grm_lt=c["grm"])
    s = orc.Solver(c["indiv"], c["X"], c["y"], c["N"], VC_F, **kw)
    res = s.mme(1e-13)
    for v in ("beta", "uhat", "bhat"):
        # both sides stop at relative residual 1e-13; the residual vector
        # V^-1 r = V^-1 y - V^-1 X beta loses a few digits to cancellation
        assert rel(res[v], c["ref"]["%s64_%s" % (src, v)]) < 2e-8, v


def test_fp32_reference_accuracy(orc):
    """The shipped FP32 program is ~1e-5..1e-4 from the FP64 solution."""
    c = golden_case("geno_small")
    for v in ("beta", "uhat", "bhat"):
        assert rel(c["ref"]["f32_" + v], c["ref"]["geno64_" + v]) < 1e-3


def test_aireml_first_evaluation(orc):
    """Gradient and AI at theta0 and at the first trial point, with the
    reference's probe draws injected (varCompEst.cpp:980-1041)."""
    c = golden_case("aireml_small")
    ref = c["ref"]
    probes, per = aireml_probes(c, 2)
    th0 = np.array(ref["theta0"])
    s = orc.Solver(c["indiv"], c["X"], c["y"], c["N"], th0, grm_lt=c["grm"])
    s.mme(ref["pcg_tol"], rule=1, x0mode=1)
    g = s.aireml_grad(probes[:per], ref["numMC"], ref["pcg_tol"])
    it1 = ref["iterations"][0]
    assert rel(g["grad"], it1["gradients"][0]) < 1e-8
    ai = s.aireml_ai(g["f_theta"], ref["pcg_tol"])
    assert rel(ai, np.array(it1["ai"][0])) < 1e-8
    # first trial point theta0 + step, second probe batch
    th1 = th0 + np.array(it1["steps"][0])
    s.set_vc(th1)
    s.mme(ref["pcg_tol"], rule=1, x0mode=1)
    g1 = s.aireml_grad(probes[per:2 * per], ref["numMC"], ref["pcg_tol"])
    assert rel(g1["grad"], it1["gradients"][1]) < 1e-7
