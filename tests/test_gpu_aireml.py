"""AIREML terms and loop on the GPU vs the reference run (golden, probes
injected) and the oracle."""
import os

import numpy as np
import pytest

import globe_gb300 as G
from helpers import aireml_probes, golden_case, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case(gctx):
    c = golden_case("aireml_small")
    gctx.load_records(c["indiv"], c["X"], c["y"], c["N"])
    gctx.load_grm(c["grm"], c["N"])
    return c


def test_first_evaluation_matches_reference(gctx, orc, case):
    ref = case["ref"]
    probes, per = aireml_probes(case, 1)
    gctx.set_vc(ref["theta0"])
    tol = ref["pcg_tol"]
    gctx.mme(tol=tol, rule=G.RULE_AIREML, x0mode=G.X0_PRECOND)
    g = gctx.aireml_grad(ref["numMC"], probes=probes, tol=tol)
    ai = gctx.aireml_ai(tol=tol)
    it1 = ref["iterations"][0]
    assert rel(g["grad"], it1["gradients"][0]) < 1e-8
    assert rel(ai, np.array(it1["ai"][0])) < 1e-8
    s = orc.Solver(case["indiv"], case["X"], case["y"], case["N"], ref["theta0"], grm_lt=case["grm"])
    s.mme(tol, rule=1, x0mode=1)
    og = s.aireml_grad(probes, ref["numMC"], tol)
    assert rel(g["first"], og["first"]) < 1e-9 and rel(g["trace"], og["trace"]) < 1e-9
    assert rel(g["f_theta"], og["f_theta"]) < 1e-9


def test_device_probes_are_reproducible(gctx, case):
    th = case["ref"]["theta0"]
    gctx.set_vc(th)
    gctx.mme(tol=1e-10, rule=G.RULE_AIREML, x0mode=G.X0_PRECOND)
    a = gctx.aireml_grad(8, seed=77, tol=1e-10)["grad"]
    b = gctx.aireml_grad(8, seed=77, tol=1e-10)["grad"]
    c = gctx.aireml_grad(8, seed=78, tol=1e-10)["grad"]
    assert np.array_equal(a, b) and not np.array_equal(a, c)


def _device_stream_normals(seed, n):
    """The device probe stream, restated: normal m = Box-Muller on the splitmix hashes of
    pair m // 2 (cosine half for even m, sine half for odd m)."""
    M64 = np.uint64(0xFFFFFFFFFFFFFFFF)

    def pmix(z):
        with np.errstate(over="ignore"):
            z = z + np.uint64(0x9E3779B97F4A7C15)
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            return (z ^ (z >> np.uint64(31))) & M64

    idx = np.arange(n, dtype=np.uint64)
    pair = idx >> np.uint64(1)
    s = np.uint64(seed)
    with np.errstate(over="ignore"):
        h1 = pmix(s ^ pmix(np.uint64(2) * pair + np.uint64(1)))
        h2 = pmix(s ^ pmix(np.uint64(2) * pair + np.uint64(2)))
    u1 = ((h1 >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)
    u2 = ((h2 >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)
    rad = np.sqrt(-2.0 * np.log(u1))
    return np.where((idx & np.uint64(1)) == 1, rad * np.sin(2.0 * np.pi * u2), rad * np.cos(2.0 * np.pi * u2))


def test_device_probes_are_the_stream_injected(gctx, case):
    """Probes drawn on the device from a seed (per-individual normals once, Box-Muller pairs)
    equal the same stream's normals passed in as injected draws, at their draw positions."""
    th = case["ref"]["theta0"]
    gctx.set_vc(th)
    gctx.mme(tol=1e-10, rule=G.RULE_AIREML, x0mode=G.X0_PRECOND)
    numMC, seed = 6, 1234567
    per = 3 * case["N"] + len(case["indiv"])
    gen = gctx.aireml_grad(numMC, seed=seed, tol=1e-10)
    inj = gctx.aireml_grad(numMC, probes=_device_stream_normals(seed, numMC * per), tol=1e-10)
    for key in ("grad", "trace", "first"):
        assert rel(gen[key], inj[key]) < 1e-11, key


def test_loop_follows_reference_trajectory(gctx, case, tmp_path):
    ref = case["ref"]
    probes, per = aireml_probes(case, 60)
    log = os.path.join(str(tmp_path), "a.log")
    r = gctx.aireml_run(theta0=ref["theta0"], maxiter=ref["maxiter"], numMC=ref["numMC"], pcg_tol=ref["pcg_tol"],
                        probes=probes, log_path=log)
    assert r["iterations"] == ref["maxiter"]
    assert rel(r["theta"], ref["iterations"][-1]["theta"]) < 1e-5
    assert rel(r["se"], [f[1] for f in ref["final"]]) < 1e-4
    text = open(log).read()
    assert "Final variance components" in text and text.count("Rho:") == sum(len(i["rho"]) for i in ref["iterations"])


def test_fused_evaluation_matches_separate_solves(gctx, case):
    """globe_aireml_eval (one block solve of [X y | probes]) against globe_mme followed
    by globe_aireml_grad on the same probes; the AI matrix after either."""
    ref = case["ref"]
    probes, per = aireml_probes(case, 1)
    tol = 1e-12
    gctx.set_vc(ref["theta0"])
    gctx.mme(tol=tol, rule=G.RULE_AIREML, x0mode=G.X0_PRECOND)
    g = gctx.aireml_grad(ref["numMC"], probes=probes, tol=tol)
    ai = gctx.aireml_ai(tol=tol)
    gctx.set_vc(ref["theta0"])
    f = gctx.aireml_eval(ref["numMC"], probes=probes, tol=tol)
    ai_f = gctx.aireml_ai(tol=tol)
    for v in ("first", "trace", "grad"):
        assert rel(f[v], g[v]) < 1e-9, v
    assert rel(ai_f, ai) < 1e-9
    assert rel(f["grad"], ref["iterations"][0]["gradients"][0]) < 1e-8


def test_loop_fused_and_separate_agree(gctx, case):
    ref = case["ref"]
    probes, per = aireml_probes(case, 60)
    kw = dict(theta0=ref["theta0"], maxiter=ref["maxiter"], numMC=ref["numMC"], pcg_tol=ref["pcg_tol"], probes=probes)
    a = gctx.aireml_run(fuse=True, **kw)
    b = gctx.aireml_run(fuse=False, **kw)
    assert a["iterations"] == b["iterations"]
    assert rel(a["theta"], b["theta"]) < 1e-6


def test_loop_with_fewer_digits(orc):
    """AIREML on genotypes with 6 base-32 digits per column (GLOBE_PREC_MIXED) follows the
    9-digit and the FP64 runs to well inside the estimate's Monte-Carlo accuracy, and
    leaves the context's own digit setting alone."""
    from helpers import cohort
    coh = cohort(41, 400, 1500, recs=("uniform", 2, 8), miss=0.02)
    th0 = (0.5, 0.3, 0.2, 0.1, 0.1)
    out = {}
    with G.Context(0) as ctx:
        ctx.load_records(coh["indiv"].astype(np.int32), coh["X"], coh["y"], coh["N"])
        ctx.load_bed(coh["packed"])
        for name, prec, nd in (("fp64", G.PREC_FP64, 0), ("d9", G.PREC_MIXED, 0), ("d6", G.PREC_MIXED, 6)):
            out[name] = ctx.aireml_run(theta0=th0, maxiter=8, numMC=5, precision=prec, seed=7, digits=nd)
            assert ctx.get_digits() == 9
    for name in ("d9", "d6"):
        assert out[name]["iterations"] == out["fp64"]["iterations"]
        assert rel(out[name]["theta"], out["fp64"]["theta"]) < 1e-5, name
