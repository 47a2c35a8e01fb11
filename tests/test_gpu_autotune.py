"""The autotuner of the tensor-core genotype product: split-K counts and column
groupings change speed only -- every choice gives the same bits -- and its
decisions are logged."""
import numpy as np
import pytest

import globe_gb300 as G
from helpers import VC_F, cohort

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tctx():
    coh = cohort(61, 3000, 9000, recs=("uniform", 1, 4), miss=0.02)
    with G.Context(0) as ctx:
        ctx.load_records(coh["indiv"].astype(np.int32), coh["X"], coh["y"], coh["N"])
        ctx.load_bed(coh["packed"])
        ctx.set_vc(VC_F)
        ctx.set_precision(G.PREC_MIXED)
        yield ctx, coh["N"]


@pytest.mark.parametrize("k", [5, 20])
def test_choices_give_identical_bits(tctx, k):
    ctx, N = tctx
    Z = np.random.default_rng(k).standard_normal((N, k)) * np.logspace(-2, 2, k)
    ctx.set_autotune(False)
    ref = ctx.grm_apply(Z)                         # the cost model's split counts and grouping
    try:
        for s in (1, 2, 3, 7):
            ctx.debug_force_splits(s)
            assert np.array_equal(ctx.grm_apply(Z), ref), s
    finally:
        ctx.debug_force_splits(0)
    ctx.set_autotune(True)
    tuned = ctx.grm_apply(Z)                       # first use: times the candidates
    assert np.array_equal(tuned, ref)
    assert np.array_equal(ctx.grm_apply(Z), ref)   # cached choice
    log = ctx.autotune_log()
    kinds = {(d["kind"], d.get("columns")) for d in log}
    assert ("splits", None) in kinds
    if k >= 9:
        assert ("groups", k) in kinds
    for d in log:
        assert str(d["choice"]) in d["ms"] and str(d["model"]) in d["ms"]


def test_pcg_with_tuning_matches_without(tctx):
    ctx, N = tctx
    B = np.random.default_rng(3).standard_normal((ctx.Nrec, 6))
    ctx.set_autotune(False)
    Xa, ia = ctx.pcg(B, tol=1e-10, rule=G.RULE_AIREML, precision=G.PREC_MIXED)
    ctx.set_autotune(True)
    Xb, ib = ctx.pcg(B, tol=1e-10, rule=G.RULE_AIREML, precision=G.PREC_MIXED)
    assert np.array_equal(Xa, Xb) and ia["iters"] == ib["iters"]
