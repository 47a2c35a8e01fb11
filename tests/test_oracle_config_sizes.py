"""Pin the C oracle to the reference's own outputs at a benchmark configuration's
size: runPCGsolver --geno at N=2,000 individuals, M=10,000 SNPs (MAF U(0.05,0.5),
1% missing, 3-10 records each).  The inputs are regenerated byte for byte
(globe_gb300.synth.portable_cohort, SHA-256 checked); the fixture holds the
outputs of the reference programs built from their sources."""
import numpy as np
import pytest

from helpers import VC_F, portable_case, rel


@pytest.fixture(scope="module")
def c1(tmp_path_factory):
    return portable_case("geno_2k_10k", str(tmp_path_factory.mktemp("geno_2k_10k")))


def test_bed_stats_bit_exact(orc, c1):
    alt, miss, maf, mr, keep = orc.bed_stats(c1["packed"], c1["N"])
    r = c1["ref"]
    assert np.array_equal(alt, r["stats_alt"])
    assert np.array_equal(miss, r["stats_miss"])
    assert np.array_equal(maf.view(np.uint32), r["stats_maf"].view(np.uint32))
    assert np.array_equal(mr.view(np.uint32), r["stats_miss_rate"].view(np.uint32))
    assert np.array_equal(keep, r["stats_keep"].astype(bool))


def test_mme_vs_fp64_reference(orc, c1):
    s = orc.Solver(c1["indiv"], c1["X"], c1["y"], c1["N"], VC_F, packed=c1["packed"])
    res = s.mme(1e-13)
    for v in ("beta", "uhat", "bhat"):
        assert rel(res[v], c1["ref"]["geno64_" + v]) < 1e-8, v


def test_fp32_reference_accuracy(c1):
    """The shipped FP32 program (PCG tolerance 1e-5) against its FP64 build."""
    for v in ("beta", "uhat", "bhat"):
        assert rel(c1["ref"]["f32_" + v], c1["ref"]["geno64_" + v]) < 1e-3, v


@pytest.fixture(scope="module")
def c2s(tmp_path_factory):
    return portable_case("aireml_dense_2k", str(tmp_path_factory.mktemp("aireml_dense_2k")))


def test_aireml_dense_2k_first_evaluation(orc, c2s):
    """runAIREML's structure on a dense .grm.bin at N=2,000 (Poisson(5)+1 records,
    numMC=15): gradient and AI matrix at theta0 with the reference's probe draws."""
    from globe_gb300 import synth
    ref = c2s["ref"]
    per = ref["numMC"] * (3 * c2s["N"] + c2s["Nrec"])
    probes = synth.normal_stream(ref["probe_seed"], per)
    s = orc.Solver(c2s["indiv"], c2s["X"], c2s["y"], c2s["N"], ref["theta0"], grm_lt=c2s["grm"])
    s.mme(ref["pcg_tol"], rule=1, x0mode=1)
    g = s.aireml_grad(probes, ref["numMC"], ref["pcg_tol"])
    it1 = ref["iterations"][0]
    assert rel(g["grad"], it1["gradients"][0]) < 1e-8
    ai = s.aireml_ai(g["f_theta"], ref["pcg_tol"])
    assert rel(ai, np.array(it1["ai"][0])) < 1e-8
