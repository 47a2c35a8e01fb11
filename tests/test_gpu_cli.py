"""The drop-in command-line programs on the golden inputs."""
import os
import subprocess

import numpy as np
import pytest

import globe_gb300 as G
from helpers import GOLDEN, ROOT, aireml_probes, golden_case, rel

pytestmark = pytest.mark.gpu
BIN = os.path.join(ROOT, "globe_gb300", "bin")
VCARGS = ["--sig2e", "0.6", "--sig2g", "0.4", "--sig2b0", "0.4", "--sigb01", "0.2", "--sig2b1", "0.2"]


def _run(args, **kw):
    return subprocess.run(args, capture_output=True, text=True, **kw)


@pytest.mark.parametrize("src", ["geno", "grm"])
def test_runpcgsolver_outputs(tmp_path, src):
    c = golden_case("geno_small")
    out = os.path.join(str(tmp_path), "o")
    r = _run([os.path.join(BIN, "runPCGsolver"), "--input", c["prefix"] + ".txt", "--output", out,
              "--" + src, c["prefix"], "--save64", "--pcgTol", "1e-13"] + VCARGS)
    assert r.returncode == 0, r.stderr
    for v, n in (("beta", 4), ("uhat", c["N"]), ("bhat", 2 * c["N"])):
        f32 = G.read_vector("%s_%s.bin" % (out, v))
        f64 = G.read_vector("%s_%s.f64.bin" % (out, v))
        assert f32.dtype == np.float32 and f32.size == n
        assert rel(f64, c["ref"]["%s64_%s" % (src, v)]) < 2e-8
        assert np.array_equal(f32, f64.astype(np.float32))
    # default tolerance (1e-5, as the reference) stays within the reference FP32 program's accuracy
    r = _run([os.path.join(BIN, "runPCGsolver"), "--input", c["prefix"] + ".txt", "--output", out, "--geno",
              c["prefix"]] + VCARGS)
    assert r.returncode == 0, r.stderr
    for v in ("beta", "uhat", "bhat"):
        assert rel(G.read_vector("%s_%s.bin" % (out, v)), c["ref"]["geno64_" + v]) < 1e-3


def test_runpcgsolver_argument_errors(tmp_path):
    c = golden_case("tiny")
    exe = os.path.join(BIN, "runPCGsolver")
    base = [exe, "--input", c["prefix"] + ".txt", "--output", os.path.join(str(tmp_path), "o")]
    assert _run([exe]).returncode != 0
    r = _run(base + ["--geno", c["prefix"], "--grm", c["prefix"]] + VCARGS)
    assert r.returncode != 0 and "exactly one" in r.stderr
    r = _run(base + ["--geno", c["prefix"]] + VCARGS[:-2])
    assert r.returncode != 0 and "Missing required" in r.stderr
    r = _run(base + ["--geno", c["prefix"], "--bogus"] + VCARGS)
    assert r.returncode != 0 and "Unknown flag" in r.stderr
    r = _run(base + ["--geno", c["prefix"], "--minMAF", "0.7"] + VCARGS)
    assert r.returncode != 0 and "thresholds" in r.stderr


def test_runaireml_with_injected_probes(tmp_path):
    c = golden_case("aireml_small")
    ref = c["ref"]
    probes, _ = aireml_probes(c, 60)
    pf = os.path.join(str(tmp_path), "probes.bin")
    probes.tofile(pf)
    out = os.path.join(str(tmp_path), "res")
    r = _run([os.path.join(BIN, "runAIREML"), c["prefix"] + ".txt", c["prefix"], out, "--numMC",
              str(ref["numMC"]), "--maxiter", str(ref["maxiter"]), "--probes", pf, "--pcgTol", "1e-12"])
    assert r.returncode == 0, r.stderr
    log = open(out + ".log").read()
    assert "Final variance components" in log
    line = [l for l in log.splitlines() if l.startswith("Estimated variance components")][-1]
    th = [float(x.split("=")[1]) for x in line.split(":", 1)[1].split(",")]
    assert rel(th, ref["iterations"][-1]["theta"]) < 1e-5


def _final_theta(log_path):
    log = open(log_path).read()
    line = [l for l in log.splitlines() if l.startswith("Estimated variance components")][-1]
    return [float(x.split("=")[1]) for x in line.split(":", 1)[1].split(",")]


def test_runaireml_geno_matches_grm_input(tmp_path):
    """runAIREML --geno (genetic relationships from the PLINK genotypes, on the fly)
    against runAIREML on the .grm.bin built from the same genotypes; FP64 and mixed
    (the dense mixed run takes the tensor-core digit-plane product)."""
    c = golden_case("geno_small")
    common = ["--numMC", "5", "--maxiter", "6", "--seed", "5", "--pcgTol", "1e-10"]
    th = {}
    for name, extra in (("dense", []), ("dense_mixed", ["--precision", "mixed"]), ("geno", ["--geno", c["prefix"]]),
                        ("geno_mixed", ["--geno", c["prefix"], "--precision", "mixed"])):
        out = os.path.join(str(tmp_path), name)
        grm_arg = c["prefix"] if name.startswith("dense") else "-"
        r = _run([os.path.join(BIN, "runAIREML"), c["prefix"] + ".txt", grm_arg, out] + common + extra)
        assert r.returncode == 0, r.stderr
        th[name] = _final_theta(out + ".log")
    assert rel(th["geno"], th["dense"]) < 1e-4          # float32 rounding of the .grm.bin
    assert rel(th["geno_mixed"], th["geno"]) < 1e-6
    assert rel(th["dense_mixed"], th["dense"]) < 1e-6


def test_runpcgsolver_digits_flag(tmp_path):
    """--precision mixed --digits 6: the solve matches the FP64 reference to the product's
    ~5e-9 rounding (amplified by the solve), well inside the FP32 program's accuracy."""
    c = golden_case("geno_small")
    out = os.path.join(str(tmp_path), "d")
    exe = os.path.join(BIN, "runPCGsolver")
    base = [exe, "--input", c["prefix"] + ".txt", "--output", out, "--geno", c["prefix"], "--save64",
            "--pcgTol", "1e-13", "--precision", "mixed"] + VCARGS
    r = _run(base + ["--digits", "6"])
    assert r.returncode == 0, r.stderr
    for v in ("beta", "uhat", "bhat"):
        assert rel(G.read_vector("%s_%s.f64.bin" % (out, v)), c["ref"]["geno64_" + v]) < 1e-6, v
    r = _run(base + ["--digits", "12"])
    assert r.returncode != 0 and "digits" in r.stderr


@pytest.mark.parametrize("prog", ["runAIREML", "runAIREML_reducedModel"])
def test_aireml_on_built_grm_matches_geno(tmp_path, prog):
    """The .grm.bin that buildGRM writes is the matrix --geno applies: AIREML on it follows
    AIREML on the genotypes to the float32 rounding of the file, for both models."""
    c = golden_case("geno_small")
    g = os.path.join(str(tmp_path), "g")
    r = _run([os.path.join(BIN, "buildGRM"), c["prefix"], g])
    assert r.returncode == 0, r.stderr
    common = ["--numMC", "5", "--maxiter", "6", "--seed", "5", "--pcgTol", "1e-10"]
    th = {}
    for name, grm_arg, extra in (("built", g, []), ("geno", "-", ["--geno", c["prefix"]])):
        out = os.path.join(str(tmp_path), name)
        r = _run([os.path.join(BIN, prog), c["prefix"] + ".txt", grm_arg, out] + common + extra)
        assert r.returncode == 0, r.stderr
        th[name] = _final_theta(out + ".log")
    assert len(th["geno"]) == (5 if prog == "runAIREML" else 2)
    assert rel(th["built"], th["geno"]) < 1e-5
