"""The model without time effects (the reference's runAIREML_reducedModel,
varCompEst_reducedModel_noTime.cpp): V = sig2g A + sig2e I with components
(sig2e, sig2g).  CPU part: the 2-component step against the steps NLopt took in
the reference run and against SLSQP, and the record-table reader.  GPU part:
first-evaluation score and AI, the AIREML loop and the drop-in program against
the reference run with injected probes (tests/golden/reduced_small_ref.json)."""
import json
import os
import subprocess

import numpy as np
import pytest

import globe_gb300 as G
from globe_gb300 import synth, trust_region_step_no_time
from helpers import GOLDEN, ROOT, rel

PRE = os.path.join(GOLDEN, "reduced_small")


def _ref():
    with open(PRE + "_ref.json") as f:
        return json.load(f)


def _probes(ref, n_evals):
    per = ref["numMC"] * 2 * ref["N"]          # Z1 (individuals) then Z3 (records) per probe
    return synth.normal_stream(ref["probe_seed"], per * n_evals), per


def test_steps_match_reference_run():
    ref = _ref()
    theta = np.array(ref["theta0"])
    it0 = ref["iterations"][0]
    g_cur, A_cur = np.array(it0["gradients"][0]), np.array(it0["ai"][0])
    for it in ref["iterations"]:
        if not it["steps"]:
            continue
        p, st = trust_region_step_no_time(theta, g_cur, A_cur, 1e20)
        assert st == 0
        assert rel(p, it["steps"][0]) < 1e-5      # MMA stops at its xtol
        if it["rho"] and it["rho"][-1] > 0.25:          # step accepted: its gradient and AI carry over
            theta = np.array(it["theta"])
            g_cur, A_cur = np.array(it["gradients"][-1]), np.array(it["ai"][-1])


@pytest.mark.parametrize("seed", range(16))
def test_constrained_steps_vs_slsqp(seed):
    sp = pytest.importorskip("scipy.optimize")
    rng = np.random.default_rng(seed)
    Q = rng.standard_normal((2, 2))
    A = (Q @ Q.T + 0.3 * np.eye(2)) * 10 ** rng.uniform(0, 3)
    theta = np.array([0.6, 0.3]) * rng.uniform(0.05, 2, 2)
    g = A @ (rng.standard_normal(2) * 0.8)
    delta = [1e20, 3.0, 0.3, -0.5][seed % 4]
    p, st = trust_region_step_no_time(theta, g, A, delta)
    m = lambda q: g @ q - 0.5 * q @ A @ q
    cons = [{"type": "ineq", "fun": lambda q, k=k: theta[k] + q[k] - 1e-5} for k in (0, 1)]
    cons.append({"type": "ineq", "fun": lambda q: delta - np.dot(np.diag(A), q)})
    best = None
    for x0 in (np.zeros(2), -0.5 * theta, np.array([5.0, -5.0])):
        r = sp.minimize(lambda q: -m(q), x0, bounds=[(-10, 10)] * 2, constraints=cons, method="SLSQP",
                        options=dict(ftol=1e-15, maxiter=1000))
        if r.success and (best is None or r.fun < best.fun):
            best = r
    if best is None:
        return
    assert st == 0
    x = theta + p
    assert np.all(np.abs(p) <= 10 + 1e-9) and np.all(x >= 1e-5 - 1e-9)
    assert np.dot(np.diag(A), p) <= delta + 1e-9 * max(1.0, abs(delta))
    assert m(p) >= -best.fun - 1e-7 * max(1.0, abs(best.fun))      # exact: never worse than SLSQP


def test_reader():
    indiv, X, y, N = G.read_records_no_time(PRE + ".txt")
    assert N == 300 and X.shape == (300, 3) and np.array_equal(indiv, np.arange(300))
    assert np.all(X[:, 0] == 1.0)


def _load(gctx):
    indiv, X, y, N = G.read_records_no_time(PRE + ".txt")
    gctx.set_model(G.MODEL_NO_TIME)
    gctx.load_records(indiv, X, y, N)              # last covariate takes time's place (unused)
    gctx.load_grm(G.read_grm(PRE, N), N)
    return N


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol_ref", [(G.PREC_FP64, 1e-8), (G.PREC_MIXED, 1e-7)], ids=["fp64", "mixed"])
def test_first_evaluation_matches_reference(gctx, prec, tol_ref):
    """Score and AI of the reduced model against the FP64 reference run; mixed precision runs
    the tensor-core dense product and the double-float record kernels (sig2b* = 0)."""
    ref = _ref()
    try:
        _load(gctx)
        probes, per = _probes(ref, 1)
        gctx.set_vc(list(ref["theta0"]) + [0.0, 0.0, 0.0])
        tol = ref["pcg_tol"]
        gctx.mme(tol=tol, rule=G.RULE_AIREML, x0mode=G.X0_PRECOND, precision=prec)
        n0 = gctx.record_df_solves()
        g = gctx.aireml_grad(ref["numMC"], probes=probes, tol=tol, precision=prec)
        ai = gctx.aireml_ai(tol=tol, precision=prec)
        assert (gctx.record_df_solves() > n0) == (prec == G.PREC_MIXED)
        it1 = ref["iterations"][0]
        assert rel(g["grad"][:2], it1["gradients"][0]) < tol_ref
        assert np.all(g["grad"][2:] == 0)
        assert rel(ai[:2, :2], np.array(it1["ai"][0])) < tol_ref
        f = gctx.aireml_eval(ref["numMC"], probes=probes, tol=tol, precision=prec)   # one block solve: same score
        assert rel(f["grad"][:2], it1["gradients"][0]) < tol_ref
    finally:
        gctx.set_model(G.MODEL_FULL)


@pytest.mark.gpu
def test_loop_follows_reference(gctx):
    ref = _ref()
    try:
        _load(gctx)
        probes, per = _probes(ref, 60)
        r = gctx.aireml_run(theta0=list(ref["theta0"]) + [0, 0, 0], maxiter=ref["maxiter"], numMC=ref["numMC"],
                            pcg_tol=ref["pcg_tol"], probes=probes)
        assert r["iterations"] == len(ref["iterations"])
        assert rel(r["theta"][:2], ref["iterations"][-1]["theta"]) < 1e-5
        assert rel(r["se"][:2], [f[1] for f in ref["final"]]) < 1e-4
        assert np.all(r["theta"][2:] == 0)
    finally:
        gctx.set_model(G.MODEL_FULL)


@pytest.mark.gpu
def test_program(tmp_path):
    ref = _ref()
    probes, per = _probes(ref, 60)
    pf = os.path.join(str(tmp_path), "probes.bin")
    probes.tofile(pf)
    out = os.path.join(str(tmp_path), "red")
    exe = os.path.join(ROOT, "globe_gb300", "bin", "runAIREML_reducedModel")
    r = subprocess.run([exe, PRE + ".txt", PRE, out, "--numMC", str(ref["numMC"]), "--maxiter", str(ref["maxiter"]),
                        "--probes", pf, "--pcgTol", "1e-12"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    log = open(out + ".log", encoding="utf-8").read()
    line = [ln for ln in log.splitlines() if ln.startswith("Estimated variance components")][-1]
    th = [float(x.split("=")[1]) for x in line.split(":", 1)[1].split(",")]
    assert len(th) == 2 and rel(th, ref["iterations"][-1]["theta"]) < 1e-5
    assert "sig2e" in log and "sig2b0" not in log.split("Final variance components")[1]
    assert subprocess.run([exe], capture_output=True, text=True).returncode != 0
