"""The AIREML step subproblem (oneIter_AIREML, varCompEst.cpp:1148-1199):
our interior-point solver against the steps NLopt's MMA took in the
reference run, and against scipy SLSQP on constrained cases."""
import json
import os

import numpy as np
import pytest

from globe_gb300 import trust_region_step
from helpers import GOLDEN, golden_case, rel


def test_steps_match_reference_run():
    ref = golden_case("aireml_small")["ref"]
    theta = np.array(ref["theta0"])
    it0 = ref["iterations"][0]
    g_cur, A_cur = np.array(it0["gradients"][0]), np.array(it0["ai"][0])
    for it in ref["iterations"]:
        assert it["nlopt"] == [4]           # MMA converged (xtol) in this run
        p, st = trust_region_step(theta, g_cur, A_cur, 1e20)
        assert st == 0
        # MMA stops at its xtol; the exact optimum differs from it by ~1e-7
        assert rel(p, it["steps"][0]) < 1e-5
        # the accepted trial is the last one evaluated in the block
        theta = np.array(it["theta"])
        g_cur, A_cur = np.array(it["gradients"][-1]), np.array(it["ai"][-1])


def _scipy_step(theta, g, A, delta):
    from scipy.optimize import minimize
    cons = [{"type": "ineq", "fun": lambda p, k=k: theta[k] + p[k] - 1e-5} for k in (0, 1, 2, 4)]
    cons.append({"type": "ineq", "fun": lambda p: (theta[2] + p[2]) * (theta[4] + p[4]) - 1e-3 -
                 (theta[3] + p[3]) ** 2})
    cons.append({"type": "ineq", "fun": lambda p: delta - np.dot(np.diag(A), p)})
    f = lambda p: -(g @ p - 0.5 * p @ A @ p)
    best = None
    for x0 in (np.zeros(5), -0.5 * theta, np.full(5, 0.01)):
        r = minimize(f, x0, jac=lambda p: -(g - A @ p), bounds=[(-10, 10)] * 5, constraints=cons, method="SLSQP",
                     options=dict(ftol=1e-15, maxiter=1000))
        if r.success and (best is None or r.fun < best.fun):
            best = r
    return best


@pytest.mark.parametrize("seed", range(12))
def test_constrained_cases_vs_slsqp(seed):
    pytest.importorskip("scipy")
    rng = np.random.default_rng(seed)
    Q = rng.standard_normal((5, 5))
    A = Q @ Q.T + 0.5 * np.eye(5)
    A *= 10 ** rng.uniform(0, 3)
    theta = np.array([0.6, 0.3, 0.3, 0.1, 0.2]) * rng.uniform(0.2, 2, 5)
    theta[3] = 0.9 * np.sqrt(theta[2] * theta[4] - 1e-3) if theta[2] * theta[4] > 1e-3 else 0.0
    g = A @ (rng.standard_normal(5) * 0.5)   # unconstrained optimum far away: constraints bind
    delta = [1e20, 5.0, 0.5][seed % 3]
    p, st = trust_region_step(theta, g, A, delta)
    assert st == 0
    x = theta + p
    assert np.all(np.abs(p) <= 10 + 1e-9)
    assert all(x[k] >= 1e-5 - 1e-9 for k in (0, 1, 2, 4))
    assert x[3] ** 2 <= x[2] * x[4] - 1e-3 + 1e-9
    assert np.dot(np.diag(A), p) <= delta + 1e-7 * max(1.0, abs(delta))
    m = lambda q: g @ q - 0.5 * q @ A @ q
    r = _scipy_step(theta, g, A, delta)
    if r is not None:
        # the problem is convex: ours is at least as good as SLSQP's, and close
        assert m(p) >= m(r.x) - 1e-7 * max(1.0, abs(m(r.x)))
        assert abs(m(p) - m(r.x)) <= 1e-5 * max(1.0, abs(m(r.x)))


def _feasible(theta, A, delta, p, slack=1e-9):
    x = theta + p
    return (np.all(np.abs(p) <= 10 + slack) and all(x[k] >= 1e-5 - slack for k in (0, 1, 2, 4))
            and x[3] ** 2 <= x[2] * x[4] - 1e-3 + slack and np.dot(np.diag(A), p) <= delta + 1e-7 * abs(delta))


def test_active_trust_region_beats_the_reference_step():
    """Where the trust-region constraint binds, NLopt's MMA stops short of the
    subproblem's optimum.  The reference's constraint function is the signed sum
    sum_k AI_kk p_k - Delta but the gradient it hands MMA is 2 AI_kk^2 p_k
    (varCompEst.cpp:1068-1089), so MMA's local models of the constraint are wrong and
    it stops on its x tolerance (result 4) at a point that is feasible but not
    stationary.  Seen in the dense N=2,000, numMC=15 run at iteration 6, the first
    step taken with Delta finite (10.93, after the rejection of iteration 5): the
    reference's step has model value 0.039, ours (the exact optimum, equal to
    SLSQP's) 0.147, and both lie on the constraint.  So the two runs agree through
    iteration 5 and part from there."""
    pytest.importorskip("scipy")
    ref = json.load(open(os.path.join(GOLDEN, "aireml_dense_2k_ref.json")))
    it5, it6 = ref["iterations"][4], ref["iterations"][5]
    theta = np.array(it5["theta"])
    g, A = np.array(it5["gradients"][-1]), np.array(it5["ai"][-1])
    delta = it5["delta_after"][0]
    p_ref = np.array(it6["steps"][0])
    assert it6["nlopt"] == [4]

    def q(p):
        return g @ p - 0.5 * p @ A @ p
    p, st = trust_region_step(theta, g, A, delta)
    assert st == 0
    assert _feasible(theta, A, delta, p) and _feasible(theta, A, delta, p_ref)
    assert abs(np.dot(np.diag(A), p) - delta) < 1e-6 * delta              # the constraint binds
    assert abs(np.dot(np.diag(A), p_ref) - delta) < 1e-6 * delta
    assert q(p) > 3.0 * q(p_ref) > 0
    r = _scipy_step(theta, g, A, delta)
    assert rel(p, r.x) < 1e-5 and abs(q(p) - (-r.fun)) < 1e-9 * abs(q(p))
