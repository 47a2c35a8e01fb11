"""The CUDA path against the reference's own outputs at the benchmark
configurations' sizes.

* runPCGsolver --geno at N=2,000 individuals, M=10,000 SNPs (MAF U(0.05,0.5),
  1% missing, 3-10 records each, ~13k records): per-SNP statistics bit-exact,
  beta / u-hat / b-hat in FP64 and on the tensor cores against the reference's
  FP64 build, and the drop-in program's output files.
* runAIREML on a dense .grm.bin at N=2,000 with the structure of the dense
  benchmark (Poisson(5)+1 records, numMC=15): first-evaluation gradient and AI
  matrix, and the trajectory, in FP64 and on the tensor cores, against the
  reference's FP64 build with the same probe draws injected.

Inputs are regenerated byte for byte (SHA-256 checked against the inputs the
reference ran on)."""
import os
import subprocess

import numpy as np
import pytest

import globe_gb300 as G
from globe_gb300 import synth
from helpers import ROOT, VC_F, portable_case, rel

pytestmark = pytest.mark.gpu
BIN = os.path.join(ROOT, "globe_gb300", "bin")
VCARGS = ["--sig2e", "0.6", "--sig2g", "0.4", "--sig2b0", "0.4", "--sigb01", "0.2", "--sig2b1", "0.2"]


@pytest.fixture(scope="module")
def c1(tmp_path_factory):
    return portable_case("geno_2k_10k", str(tmp_path_factory.mktemp("geno_2k_10k")))


@pytest.fixture(scope="module")
def c1ctx(c1):
    with G.Context(0) as ctx:
        ctx.load_records(c1["indiv"], c1["X"], c1["y"], c1["N"])
        ctx.stats = ctx.load_bed(c1["packed"])
        ctx.set_vc(VC_F)
        yield ctx


def test_geno_2k_10k_stats_bit_exact(c1, c1ctx):
    st, r = c1ctx.stats, c1["ref"]
    assert np.array_equal(st["alt"], r["stats_alt"])
    assert np.array_equal(st["miss"], r["stats_miss"])
    assert np.array_equal(st["maf"].view(np.uint32), r["stats_maf"].view(np.uint32))
    assert np.array_equal(st["miss_rate"].view(np.uint32), r["stats_miss_rate"].view(np.uint32))
    assert np.array_equal(st["keep"], r["stats_keep"].astype(bool))


@pytest.mark.parametrize("prec", [G.PREC_FP64, G.PREC_MIXED], ids=["fp64", "mixed"])
def test_geno_2k_10k_mme_vs_fp64_reference(c1, c1ctx, prec):
    r = c1ctx.mme(tol=1e-13, rule=G.RULE_PCGSOLVER, precision=prec)
    for v in ("beta", "uhat", "bhat"):
        assert rel(r[v], c1["ref"]["geno64_" + v]) < 1e-8, v


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_geno_2k_10k_runpcgsolver_outputs(c1, tmp_path, prec):
    out = os.path.join(str(tmp_path), "o")
    r = subprocess.run([os.path.join(BIN, "runPCGsolver"), "--input", c1["prefix"] + ".txt", "--output", out,
                        "--geno", c1["prefix"], "--save64", "--pcgTol", "1e-13", "--precision", prec] + VCARGS,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for v, n in (("beta", 4), ("uhat", c1["N"]), ("bhat", 2 * c1["N"])):
        f32 = G.read_vector("%s_%s.bin" % (out, v))
        f64 = G.read_vector("%s_%s.f64.bin" % (out, v))
        assert f32.dtype == np.float32 and f32.size == n
        assert rel(f64, c1["ref"]["geno64_" + v]) < 1e-8, v
        assert np.array_equal(f32, f64.astype(np.float32))


def test_geno_2k_10k_default_tolerance_like_fp32_reference(c1, tmp_path):
    """At the reference's own tolerance (1e-5) the program's float32 outputs sit as
    close to the FP64 solution as the reference's FP32 program does."""
    out = os.path.join(str(tmp_path), "o")
    r = subprocess.run([os.path.join(BIN, "runPCGsolver"), "--input", c1["prefix"] + ".txt", "--output", out,
                        "--geno", c1["prefix"]] + VCARGS, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for v in ("beta", "uhat", "bhat"):
        ours = rel(G.read_vector("%s_%s.bin" % (out, v)), c1["ref"]["geno64_" + v])
        theirs = rel(c1["ref"]["f32_" + v], c1["ref"]["geno64_" + v])
        assert ours < max(3 * theirs, 1e-5), (v, ours, theirs)


# ---- dense-GRM AIREML, numMC = 15 -------------------------------------------------

@pytest.fixture(scope="module")
def c2s(tmp_path_factory):
    if not os.path.exists(os.path.join(ROOT, "tests", "golden", "aireml_dense_2k_ref.json")):
        pytest.fail("fixture aireml_dense_2k_ref.json missing")
    return portable_case("aireml_dense_2k", str(tmp_path_factory.mktemp("aireml_dense_2k")))


def _probes(c, n_evals):
    ref = c["ref"]
    per = ref["numMC"] * (3 * c["N"] + c["Nrec"])
    return synth.normal_stream(ref["probe_seed"], per * n_evals), per


@pytest.mark.parametrize("prec", [G.PREC_FP64, G.PREC_MIXED], ids=["fp64", "mixed"])
def test_aireml_dense_2k_first_evaluation(c2s, prec):
    ref = c2s["ref"]
    probes, per = _probes(c2s, 1)
    tol = ref["pcg_tol"]
    with G.Context(0) as ctx:
        ctx.load_records(c2s["indiv"], c2s["X"], c2s["y"], c2s["N"])
        ctx.load_grm(c2s["grm"], c2s["N"])
        ctx.set_vc(ref["theta0"])
        ctx.set_precision(prec)
        ctx.mme(tol=tol, rule=G.RULE_AIREML, x0mode=G.X0_PRECOND)
        g = ctx.aireml_grad(ref["numMC"], probes=probes, tol=tol)
        ai = ctx.aireml_ai(tol=tol)
    it1 = ref["iterations"][0]
    assert rel(g["grad"], it1["gradients"][0]) < 1e-8
    assert rel(ai, np.array(it1["ai"][0])) < 1e-8


def _log_thetas(path):
    """The accepted components of each iteration from a runAIREML-layout log."""
    out = []
    for line in open(path):
        if line.startswith("Estimated variance components:"):
            out.append([float(x.split("=")[1]) for x in line.split(":", 1)[1].split(",")])
    return np.array(out)


@pytest.mark.parametrize("prec", [G.PREC_FP64, G.PREC_MIXED], ids=["fp64", "mixed"])
def test_aireml_dense_2k_trajectory(c2s, prec, tmp_path):
    """Iterations 1-5 of the run (gradients, trust-region steps while the radius is
    infinite, one rejected step and its halving, the radius update): every accepted
    theta within 1e-7 of the reference's, in FP64 and on the tensor cores.  The
    reference's sixth step is NLopt's inexact solution of a subproblem with a binding
    trust-region constraint (test_trust_region.py shows ours is the exact optimum), so
    the runs part there."""
    ref = c2s["ref"]
    probes, per = _probes(c2s, 12)
    log = os.path.join(str(tmp_path), "a.log")
    with G.Context(0) as ctx:
        ctx.load_records(c2s["indiv"], c2s["X"], c2s["y"], c2s["N"])
        ctx.load_grm(c2s["grm"], c2s["N"])
        r = ctx.aireml_run(theta0=ref["theta0"], maxiter=5, numMC=ref["numMC"], pcg_tol=ref["pcg_tol"],
                           probes=probes, precision=prec, log_path=log)
    assert r["iterations"] == 5
    got = _log_thetas(log)
    want = np.array([it["theta"] for it in ref["iterations"][:5]])
    assert got.shape == want.shape
    for i in range(5):
        assert rel(got[i], want[i]) < 1e-7, i
    assert rel(r["theta"], want[4]) < 1e-7
