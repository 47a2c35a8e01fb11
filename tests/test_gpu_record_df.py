"""Double-float record kernels of mixed-precision block PCG (k_records_df.cu) against the
FP64 record kernels and the oracle."""
import numpy as np
import pytest

import globe_gb300 as G
from helpers import VC_F, cohort, rel

pytestmark = pytest.mark.gpu


def _solve(ctx, B, df, **kw):
    ctx.set_record_df(df)
    try:
        n0 = ctx.record_df_solves()
        X, info = ctx.pcg(B, **kw)
        return X, info, ctx.record_df_solves() - n0
    finally:
        ctx.set_record_df(True)


@pytest.fixture(scope="module")
def blocks(orc):
    """Blocks of 1-150 records (the thread and the warp layouts), genotype GRM, a context of
    its own."""
    coh = cohort(23, 300, 400, recs=("geometric", 0.04, 1, 150), T=10.0, miss=0.02)
    counts = np.bincount(coh["indiv"])
    assert counts.max() > 48 and counts.min() <= 48
    indiv = coh["indiv"].astype(np.int32)
    with G.Context(0) as ctx:
        ctx.load_records(indiv, coh["X"], coh["y"], 300)
        ctx.load_bed(coh["packed"])
        ctx.set_vc(VC_F)
        s = orc.Solver(indiv, coh["X"], coh["y"], 300, VC_F, packed=coh["packed"])
        s.precond_build()
        rng = np.random.default_rng(5)
        B = np.column_stack([coh["X"], coh["y"], rng.standard_normal((len(indiv), 3))])
        yield ctx, s, B


@pytest.mark.parametrize("rule,tol", [(G.RULE_PCGSOLVER, 1e-12), (G.RULE_AIREML, 1e-11)])
def test_df_records_match_fp64_records_and_oracle(blocks, rule, tol):
    ctx, s, B = blocks
    assert ctx.get_record_df()
    Xd, idf, nd = _solve(ctx, B, True, tol=tol, rule=rule, precision=G.PREC_MIXED)
    Xf, iff, nf = _solve(ctx, B, False, tol=tol, rule=rule, precision=G.PREC_MIXED)
    assert nd == 1 and nf == 0
    assert idf["converged"] and abs(idf["iters"] - iff["iters"]) <= 1
    assert rel(Xd, Xf) < 1e-9
    Xo, _ = s.pcg(B, tol, rule=0 if rule == G.RULE_PCGSOLVER else 1)
    assert rel(Xd, Xo) < 1e-9
    # FP64 solves never take the double-float kernels
    _, _, n64 = _solve(ctx, B, True, tol=tol, rule=rule, precision=G.PREC_FP64)
    assert n64 == 0


@pytest.mark.parametrize("x0mode", [G.X0_PRECOND, G.X0_GIVEN])
def test_df_records_from_other_start_points(blocks, x0mode):
    """From a start point other than 0 the set-up runs in FP64 and x, r, z, p are converted
    to double-float in place."""
    ctx, s, B = blocks
    kw = dict(tol=1e-11, rule=G.RULE_AIREML, precision=G.PREC_MIXED, x0mode=x0mode)
    if x0mode == G.X0_GIVEN:
        kw["X0"], _ = ctx.pcg(B, tol=1e-3, rule=G.RULE_AIREML)
    Xd, idf, nd = _solve(ctx, B, True, **kw)
    Xf, iff, nf = _solve(ctx, B, False, **kw)
    assert nd == 1 and nf == 0 and idf["converged"]
    assert rel(Xd, Xf) < 1e-9
    Xo, _ = s.pcg(B, 1e-11, rule=1, x0mode=1 if x0mode == G.X0_PRECOND else 2, X0=kw.get("X0"))
    assert rel(Xd, Xo) < 1e-9


def test_power_of_two_scaling_is_exact(blocks):
    """Each column runs scaled to a unit-size right-hand side: a right-hand side 2^40 or
    2^-40 times larger gives the solution times 2^40 or 2^-40, bit for bit, and the same
    iterations."""
    ctx, _, B = blocks
    kw = dict(tol=1e-10, rule=G.RULE_AIREML, precision=G.PREC_MIXED)
    X1, i1, n1 = _solve(ctx, B, True, **kw)
    assert n1 == 1
    for e in (40, -40):
        sc = 2.0 ** e
        Xs, isc, ns = _solve(ctx, B * sc, True, **kw)
        assert ns == 1
        assert np.array_equal(Xs, X1 * sc)
        assert isc == i1


def test_range_guard_keeps_fp64_records(blocks):
    """With sig2e above 2^30 a mixed solve keeps the FP64 record kernels: the same bits as
    with the double-float kernels switched off."""
    ctx, _, B = blocks
    vc = (2.0 ** 31,) + tuple(VC_F[1:])
    ctx.set_vc(vc)
    try:
        kw = dict(tol=1e-8, rule=G.RULE_AIREML, precision=G.PREC_MIXED, maxit=200)
        Xg, ig, ng = _solve(ctx, B, True, **kw)
        Xo, io, no = _solve(ctx, B, False, **kw)
    finally:
        ctx.set_vc(VC_F)
    assert ng == 0 and no == 0
    assert np.array_equal(Xg, Xo) and ig == io


@pytest.mark.parametrize("precision", [G.PREC_FP64, G.PREC_MIXED])
def test_many_columns_with_long_blocks(blocks, precision):
    """390 right-hand sides with blocks of more than 48 records: the warp-per-block kernels
    stage their per-warp sums 32 columns at a time (390 columns once needed 50 KB of shared
    memory per CTA)."""
    ctx, s, B = blocks
    rng = np.random.default_rng(11)
    Bw = rng.standard_normal((B.shape[0], 390))
    X, info = ctx.pcg(Bw, tol=1e-10, rule=G.RULE_AIREML, precision=precision)
    assert info["converged"]
    Xo, _ = s.pcg(Bw, 1e-10, rule=1)
    assert rel(X, Xo) < 1e-8
