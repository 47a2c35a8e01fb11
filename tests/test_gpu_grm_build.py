"""globe_grm_build: the GRM of the loaded genotypes on the GPU (tensor-core
and FP64 paths) against the oracle's orc_grm_build and the .grm.bin fixtures,
the buildGRM program, and its error paths."""
import os
import subprocess

import numpy as np
import pytest

import globe_gb300 as G
from globe_gb300 import synth
from helpers import ROOT, VC_F, f32_ulps, golden_case, rel

pytestmark = pytest.mark.gpu
BIN = os.path.join(ROOT, "globe_gb300", "bin")
PRECS = [G.PREC_MIXED, G.PREC_FP64]


def _geno(seed, N, M, miss=0.02, edge=False, maf_lo=0.01):
    rng = np.random.default_rng(seed)
    return synth.pack_genotypes(synth.simulate_genotypes(rng, M, N, maf_lo, 0.5, miss, extra_edge_snps=edge))


def _build(packed, N, prec, min_maf=0.01, max_miss=0.2):
    with G.Context(0) as ctx:
        ctx.set_individuals(N)
        ctx.set_precision(prec)
        ctx.load_bed(packed, min_maf, max_miss)
        return ctx.grm_build()


def _close(lt, ref):
    """Each value is one float32 rounding of a sum that is exact to a small
    absolute error: the FP64 paths to ~1e-16 relative, the tensor-core path to
    2^(e-40) with 2^e >= max |inv_std zs| / 16 (the digit range), ~1e-11 of
    max |A| here.  So values agree to one ulp plus that error -- entries far
    below max |A| can differ by more than one of their own ulps -- and nearly
    all are equal."""
    lt = np.asarray(lt, np.float64)
    ref32 = np.asarray(ref, np.float32)
    ref = ref32.astype(np.float64)
    ulp = np.spacing(np.abs(ref32)).astype(np.float64)
    assert (np.abs(lt - ref) <= ulp + 1e-10 * np.abs(ref).max()).all(), np.abs(lt - ref).max()
    assert (f32_ulps(lt.astype(np.float32), ref32) == 0).mean() > 0.999


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("N,M", [(1, 200), (37, 300), (333, 1200), (1030, 2500)])
def test_matches_oracle(orc, prec, N, M):
    packed = _geno(N + M, N, M)
    _close(_build(packed, N, prec), orc.grm_build(packed, N))


@pytest.mark.parametrize("prec", PRECS)
def test_edge_snps_and_no_filter(orc, prec):
    """Monomorphic, all-missing and near-monomorphic SNPs with the filters off
    (inv_std = 1 where 2f(1-f) <= 1e-12; rare SNPs widen the digit range)."""
    N, M = 300, 900
    packed = _geno(5, N, M, miss=0.05, edge=True, maf_lo=0.0)
    _close(_build(packed, N, prec, 0.0, 1.0), orc.grm_build(packed, N, 0.0, 1.0))


@pytest.mark.parametrize("name", ["geno_small", "tiny"])
def test_matches_fixture(name):
    """Against the .grm.bin the reference programs were run on (built with the
    FP32 program's float allele frequency; this builder uses the double one)."""
    c = golden_case(name)
    lt = _build(c["packed"], c["N"], G.PREC_MIXED)
    assert np.abs(lt - c["grm"]).max() <= 5e-7 * np.abs(c["grm"]).max()


def test_many_launches_tc_vs_fp64():
    """N large enough that the tensor-core build needs several launches (groups
    of 21 columns, ~2 GB of digits + partials per launch): both paths agree."""
    N, M = 6000, 30000
    packed = _geno(77, N, M)
    _close(_build(packed, N, G.PREC_MIXED), _build(packed, N, G.PREC_FP64))


def test_same_matrix_as_the_genotype_product(gctx):
    """The dense path on the built GRM applies the matrix the --geno path applies."""
    c = golden_case("geno_small")
    N = c["N"]
    lt = _build(c["packed"], N, G.PREC_MIXED)
    Z = np.random.default_rng(3).standard_normal((N, 3))
    gctx.load_records(c["indiv"], c["X"], c["y"], N)
    gctx.set_vc(VC_F)
    gctx.load_bed(c["packed"])
    g_geno = gctx.grm_apply(Z)
    gctx.load_grm(lt, N)
    g_dense = gctx.grm_apply(Z)
    assert rel(g_dense, g_geno) < 1e-6


def test_errors():
    with G.Context(0) as ctx:
        out = np.empty(1, np.float32)
        with pytest.raises(G.GlobeError) as e:
            ctx.grm_build()
        assert e.value.code == -3
        packed = _geno(1, 50, 40)
        ctx.set_individuals(50)
        ctx.load_bed(packed, 0.5, 0.0)   # no SNP passes
        with pytest.raises(G.GlobeError) as e:
            ctx.grm_build()
        assert "no SNP" in str(e.value)
        # a genotype-only context has no record table for the solver
        ctx.load_bed(packed)
        ctx.set_vc(VC_F)
        with pytest.raises(G.GlobeError) as e:
            ctx.grm_apply(np.ones((50, 1)))
        assert "record table" in str(e.value)
        with pytest.raises(G.GlobeError):
            ctx.set_individuals(0)
        del out


def test_buildgrm_program(tmp_path):
    c = golden_case("geno_small")
    out = os.path.join(str(tmp_path), "g")
    r = subprocess.run([os.path.join(BIN, "buildGRM"), c["prefix"], out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lt = np.fromfile(out + ".grm.bin", np.float32)
    assert lt.size == c["N"] * (c["N"] + 1) // 2
    assert np.abs(lt - c["grm"]).max() <= 5e-7 * np.abs(c["grm"]).max()
    ids = open(out + ".grm.id").read().split("\n")
    assert len([l for l in ids if l]) == c["N"]
    fam = [l.split()[:2] for l in open(c["prefix"] + ".fam") if l.split()]
    assert ids[0].split("\t") == fam[0]
    # FP64 path through the program, and the Python helper
    r = subprocess.run([os.path.join(BIN, "buildGRM"), c["prefix"], out + "64", "--precision", "fp64"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    _close(np.fromfile(out + "64.grm.bin", np.float32), lt)
    lt2 = G.build_grm(c["prefix"], out + "py")
    assert np.array_equal(lt2, lt)
    assert np.array_equal(G.read_grm(out + "py", c["N"]), lt)
    # the built file is a drop-in --grm input of runPCGsolver
    o2 = os.path.join(str(tmp_path), "o")
    vc = ["--sig2e", "0.6", "--sig2g", "0.4", "--sig2b0", "0.4", "--sigb01", "0.2", "--sig2b1", "0.2"]
    r = subprocess.run([os.path.join(BIN, "runPCGsolver"), "--input", c["prefix"] + ".txt", "--output", o2,
                        "--grm", out, "--save64", "--pcgTol", "1e-13"] + vc, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for v in ("beta", "uhat", "bhat"):
        assert rel(G.read_vector("%s_%s.f64.bin" % (o2, v)), c["ref"]["geno64_" + v]) < 1e-5, v


def test_buildgrm_program_errors(tmp_path):
    c = golden_case("tiny")
    exe = os.path.join(BIN, "buildGRM")
    assert subprocess.run([exe], capture_output=True).returncode != 0
    r = subprocess.run([exe, c["prefix"], os.path.join(str(tmp_path), "x"), "--bogus"], capture_output=True,
                       text=True)
    assert r.returncode != 0 and "unknown argument" in r.stderr
    r = subprocess.run([exe, os.path.join(str(tmp_path), "missing"), os.path.join(str(tmp_path), "x")],
                       capture_output=True, text=True)
    assert r.returncode != 0 and ".fam" in r.stderr


def test_built_grm_solve_matches_reference_run(gctx):
    """The MME on the GPU-built GRM matches the reference's FP64 runPCGsolver --grm on the
    oracle-built GRM (tests/golden/geno_small_grmf64_ref.npz): the two matrices are the
    same to float32 rounding ties."""
    c = golden_case("geno_small")
    d = np.load(os.path.join(ROOT, "tests", "golden", "geno_small_grmf64_ref.npz"))
    lt = _build(c["packed"], c["N"], G.PREC_MIXED)
    gctx.load_records(c["indiv"], c["X"], c["y"], c["N"])
    gctx.load_grm(lt, c["N"])
    gctx.set_vc(VC_F)
    r = gctx.mme(tol=1e-13, rule=G.RULE_PCGSOLVER)
    for v in ("beta", "uhat", "bhat"):
        assert rel(r[v], d[v]) < 2e-8, v
