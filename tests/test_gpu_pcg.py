"""Block PCG on the GPU (runPCG_multi / runPCG_multi_VC) vs the oracle."""
import numpy as np
import pytest

import globe_gb300 as G
from helpers import VC_F, cohort, golden_case, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(gctx, orc):
    c = golden_case("geno_small")
    gctx.load_records(c["indiv"], c["X"], c["y"], c["N"])
    gctx.load_bed(c["packed"])
    gctx.set_vc(VC_F)
    s = orc.Solver(c["indiv"], c["X"], c["y"], c["N"], VC_F, packed=c["packed"])
    s.precond_build()
    B = np.column_stack([c["X"], c["y"]])
    return gctx, s, B


def test_rule_pcgsolver_matches_oracle(setup):
    ctx, s, B = setup
    X, info = ctx.pcg(B, tol=1e-12, rule=G.RULE_PCGSOLVER)
    Xo, it = s.pcg(B, 1e-12, rule=0)
    assert abs(info["iters"] - it) <= 1
    assert rel(X, Xo) < 1e-9
    assert info["converged"] and info["rhs_iters"] == B.shape[1] * info["iters"]


@pytest.mark.parametrize("x0mode", [G.X0_ZERO, G.X0_PRECOND])
def test_rule_aireml_x0_modes(setup, x0mode):
    ctx, s, B = setup
    X, info = ctx.pcg(B, tol=1e-11, rule=G.RULE_AIREML, x0mode=x0mode)
    Xo, it = s.pcg(B, 1e-11, rule=1, x0mode=x0mode)
    assert abs(info["iters"] - it) <= 1
    assert rel(X, Xo) < 1e-8
    r = B - ctx.vx(X)
    assert np.all(np.linalg.norm(r, axis=0) < 1.01e-11 * np.linalg.norm(B, axis=0))


def test_given_start_point(setup):
    ctx, s, B = setup
    X1, _ = ctx.pcg(B, tol=1e-4, rule=G.RULE_AIREML)
    X2, info = ctx.pcg(B, X0=X1, tol=1e-11, rule=G.RULE_AIREML)
    Xo, _ = s.pcg(B, 1e-11, rule=1, x0mode=2, X0=X1)
    assert rel(X2, Xo) < 1e-8


def test_masking_freezes_converged_columns(setup):
    ctx, s, B = setup
    B2 = B.copy()
    B2[:, 0] *= 1e-3      # columns converge at different iterations
    X, info = ctx.pcg(B2, tol=1e-10, rule=G.RULE_AIREML, mask=True)
    Xf, info_f = ctx.pcg(B2, tol=1e-10, rule=G.RULE_AIREML, mask=False)
    assert info["rhs_iters"] <= info_f["rhs_iters"]
    r = B2 - ctx.vx(X)
    assert np.all(np.linalg.norm(r, axis=0) < 1.01e-10 * np.linalg.norm(B2, axis=0))
    assert rel(X, Xf) < 1e-7


def test_zero_rhs_column_and_cap(setup):
    ctx, s, B = setup
    B2 = B.copy()
    B2[:, 2] = 0.0
    X, info = ctx.pcg(B2, tol=1e-10, rule=G.RULE_AIREML)
    assert np.all(X[:, 2] == 0.0) and np.all(np.isfinite(X))
    X3, info3 = ctx.pcg(B, tol=1e-14, maxit=3, rule=G.RULE_AIREML)
    assert info3["iters"] == 3 and not info3["converged"]


@pytest.mark.parametrize("precision,tol_o", [(G.PREC_FP64, 1e-9), (G.PREC_MIXED, 1e-8)], ids=["fp64", "mixed"])
def test_dense_and_odd_sizes(gctx, orc, precision, tol_o):
    """Dense GRM, N = 131 individuals of 1-6 records; mixed precision runs the tensor-core
    dense product (A to 2^-34 max|A|) and the double-float record kernels."""
    from globe_gb300 import synth
    coh = cohort(21, 131, 257, recs=("uniform", 1, 6), miss=0.03)
    grm = synth.grm_from_packed(coh["packed"], 131)
    gctx.load_records(coh["indiv"], coh["X"], coh["y"], 131)
    gctx.load_grm(grm, 131)
    gctx.set_vc(VC_F)
    s = orc.Solver(coh["indiv"], coh["X"], coh["y"], 131, VC_F, grm_lt=grm)
    s.precond_build()
    B = np.column_stack([coh["X"], coh["y"]])
    X, info = gctx.pcg(B, tol=1e-12, rule=G.RULE_PCGSOLVER, precision=precision)
    Xo, it = s.pcg(B, 1e-12, rule=0)
    assert info["converged"] and rel(X, Xo) < tol_o


@pytest.mark.parametrize("precision", [G.PREC_FP64, G.PREC_MIXED])
def test_mixed_block_lengths(gctx, orc, precision):
    """Record blocks of 1-150 records: one thread per block of <= 48 records and one
    warp per longer block, side by side in every record kernel."""
    coh = cohort(23, 300, 400, recs=("geometric", 0.04, 1, 150), T=10.0, miss=0.02)
    counts = np.bincount(coh["indiv"])
    assert counts.max() > 48 and counts.min() <= 48
    indiv = coh["indiv"].astype(np.int32)
    gctx.load_records(indiv, coh["X"], coh["y"], 300)
    gctx.load_bed(coh["packed"])
    gctx.set_vc(VC_F)
    s = orc.Solver(indiv, coh["X"], coh["y"], 300, VC_F, packed=coh["packed"])
    s.precond_build()
    rng = np.random.default_rng(3)
    x = rng.standard_normal((len(indiv), 4))
    assert rel(gctx.vx(x), s.vx(x)) < 1e-11
    assert rel(gctx.precond_apply(x), s.precond_apply(x)) < 1e-12
    B = np.column_stack([coh["X"], coh["y"]])
    X, info = gctx.pcg(B, tol=1e-12, rule=G.RULE_PCGSOLVER, precision=precision)
    Xo, it = s.pcg(B, 1e-12, rule=0)
    assert rel(X, Xo) < 1e-9


@pytest.mark.parametrize("src,prec", [("geno", G.PREC_MIXED), ("geno", G.PREC_FP64), ("grm", G.PREC_MIXED)])
def test_graph_replay_matches_direct_launches(gctx, src, prec):
    """The block PCG with its iteration body replayed as CUDA graphs is bit-identical to
    direct launches (the same kernels in the same order, deterministic reductions), also
    when masking shrinks the column set mid-solve, and it counts the replayed kernels."""
    from globe_gb300 import synth
    coh = cohort(41, 400, 700, recs=("uniform", 1, 5), miss=0.02)
    indiv = coh["indiv"].astype(np.int32)
    gctx.load_records(indiv, coh["X"], coh["y"], 400)
    if src == "geno":
        gctx.load_bed(coh["packed"])
    else:
        gctx.load_grm(synth.grm_from_packed(coh["packed"], 400), 400)
    gctx.set_vc(VC_F)
    rng = np.random.default_rng(2)
    # columns of very different scale converge at different iterations under masking
    B = np.column_stack([coh["X"], coh["y"], rng.standard_normal((len(indiv), 3)) * [1e-3, 1.0, 1e3]])
    out = {}
    try:
        # a first direct solve builds what the context makes once (preconditioner, copies);
        # the second graph run updates the cached graphs in place
        for on in (False, False, True, True):
            gctx.set_graphs(on)
            assert gctx.get_graphs() == on
            l0 = gctx.kernel_launches()
            X, info = gctx.pcg(B, tol=1e-9, rule=G.RULE_AIREML, mask=True, precision=prec)
            out.setdefault(on, []).append((X, info, gctx.kernel_launches() - l0))
    finally:
        gctx.set_graphs(True)
    Xd, infod, nd_ = out[False][1]
    assert np.array_equal(out[False][0][0], Xd)
    assert infod["converged"] and infod["iters"] > 3
    for Xg, infog, ng in out[True]:
        assert np.array_equal(Xg, Xd)
        assert infog == infod
        assert ng == nd_
    with pytest.raises(G.GlobeError):
        gctx.set_graphs(2)


def _solve(ctx, B, device_loop, **kw):
    ctx.set_device_loop(device_loop)
    try:
        runs0 = ctx.device_loop_runs()
        X, info = ctx.pcg(B, **kw)
        return X, info, ctx.device_loop_runs() - runs0
    finally:
        ctx.set_device_loop(True)


@pytest.fixture(scope="module")
def own(orc):
    """A context of its own (the shared one is reloaded by other tests of this module)."""
    c = golden_case("geno_small")
    with G.Context(0) as ctx:
        ctx.load_records(c["indiv"], c["X"], c["y"], c["N"])
        ctx.load_bed(c["packed"])
        ctx.set_vc(VC_F)
        s = orc.Solver(c["indiv"], c["X"], c["y"], c["N"], VC_F, packed=c["packed"])
        s.precond_build()
        yield ctx, s, np.column_stack([c["X"], c["y"]])


CASES = [dict(tol=1e-12, rule=G.RULE_PCGSOLVER), dict(tol=1e-11, rule=G.RULE_AIREML),
         dict(tol=1e-11, rule=G.RULE_AIREML, x0mode=G.X0_PRECOND), dict(tol=1e-14, rule=G.RULE_AIREML, maxit=4),
         dict(tol=1e-12, rule=G.RULE_PCGSOLVER, precision=G.PREC_MIXED)]


@pytest.mark.parametrize("kw", CASES, ids=["pcgsolver", "aireml", "aireml-x0", "cap", "mixed"])
def test_device_loop_matches_host_loop(own, kw):
    """The device-side loop (WHILE graph node, stopping rule checked on the device) gives
    the host-checked loop's solution bit for bit and the same iteration counts."""
    ctx, s, B = own
    assert ctx.get_graphs()
    Xh, ih, nh = _solve(ctx, B, False, **kw)
    Xd, idv, nd = _solve(ctx, B, True, **kw)
    assert nh == 0 and nd == 1
    assert np.array_equal(Xd, Xh)
    for key in ("iters", "rhs_iters", "converged", "stagnated"):
        assert idv[key] == ih[key], key
    assert idv["max_rel_res"] == ih["max_rel_res"]


def _ill_conditioned(seed=1, N=1500):
    """A dense GRM with eigenvalues spaced evenly in [1e-9, 1] and every other variance
    component 1e-10: kappa(V) ~ 1e9, so after its fast start CG gains well under 0.5% per
    iteration on the slowest column."""
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((N, N)))
    A = (Q * np.linspace(1e-9, 1.0, N)) @ Q.T
    lt = ((A + A.T) / 2)[np.tril_indices(N)].astype(np.float32)
    t = rng.uniform(0, 5, N)
    X = np.asfortranarray(np.column_stack([np.ones(N), rng.standard_normal(N), t]))
    return np.arange(N, dtype=np.int32), X, rng.standard_normal(N), N, (1e-10, 1.0, 1e-10, 0.0, 1e-10), lt


def test_stagnation_stop(orc):
    """runPCGsolver's stagnation stop (PCGsolver.cpp:1373-1415): 10 iterations in a row
    with < 0.5% improvement of the largest relative residual end the solve unconverged --
    on the device loop and the host loop alike (same iterations, same bits), where the
    oracle stops."""
    indiv, X, y, N, vc, lt = _ill_conditioned()
    B = np.column_stack([X, y])
    s = orc.Solver(indiv, X, y, N, vc, grm_lt=lt)
    s.precond_build()
    _, it8 = s.pcg(B, 1e-8, rule=0)
    _, it11 = s.pcg(B, 1e-11, rule=0)
    assert it8 == it11 < 200            # the oracle stagnates too (the tolerance plays no part)
    with G.Context(0) as ctx:
        ctx.load_records(indiv, X, y, N)
        ctx.load_grm(lt, N)
        ctx.set_vc(vc)
        Xh, ih, _ = _solve(ctx, B, False, tol=1e-8, rule=G.RULE_PCGSOLVER)
        Xd, idv, nd = _solve(ctx, B, True, tol=1e-8, rule=G.RULE_PCGSOLVER)
    assert nd == 1 and ih["stagnated"] and idv["stagnated"] and not idv["converged"]
    assert idv["iters"] == ih["iters"] and np.array_equal(Xd, Xh)
    assert abs(idv["iters"] - it8) <= 2
