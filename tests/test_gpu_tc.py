"""Tensor-core genotype GRM product (GLOBE_PREC_MIXED) vs the FP64 oracle."""
import numpy as np
import pytest

import globe_gb300 as G
from globe_gb300 import synth
from helpers import VC_F, cohort, golden_case, rel

pytestmark = pytest.mark.gpu


def _load(gctx, orc, indiv, X, y, N, packed):
    gctx.load_records(indiv, X, y, N)
    gctx.load_bed(packed)
    gctx.set_vc(VC_F)
    return orc.Solver(indiv, X, y, N, VC_F, packed=packed)


CASES = [("tiny", None), ("geno_small", None), ("odd", (9, 131, 257, ("uniform", 1, 6), 0.03)),
         ("wide", (12, 300, 4500, ("uniform", 1, 3), 0.02)), ("tall", (13, 2500, 400, ("uniform", 1, 2), 0.02))]


def _case(name, spec):
    if spec is None:
        c = golden_case(name)
        return c["indiv"], c["X"], c["y"], c["N"], c["packed"]
    seed, N, M, recs, miss = spec
    c = cohort(seed, N, M, recs=recs, miss=miss, edge=True)
    return c["indiv"].astype(np.int32), c["X"], c["y"], N, c["packed"]


@pytest.mark.parametrize("name,spec", CASES, ids=[c[0] for c in CASES])
def test_grm_apply_tc_matches_fp64(gctx, orc, name, spec):
    s = _load(gctx, orc, *_case(name, spec))
    N = s.N
    rng = np.random.default_rng(N)
    try:
        gctx.set_precision(G.PREC_MIXED)
        for k in (1, 4, 5, 9, 22, 30, 65):   # widths 16..256, a two-group split (30 -> 15 + 15), and the
                                             # 65-column batching shape (17 + 16 + 16 + 16)
            Z = rng.standard_normal((N, k)) * np.logspace(-3, 2, k)
            got, ref = gctx.grm_apply(Z), s.grm_apply(Z)
            assert max(rel(got[:, c], ref[:, c]) for c in range(k)) < 1e-11, k
        x = rng.standard_normal((s.Nrec, 3))
        assert rel(gctx.vx(x), s.vx(x)) < 1e-11
    finally:
        gctx.set_precision(G.PREC_FP64)


def test_mme_mixed_matches_reference(gctx, orc):
    c = golden_case("geno_small")
    _load(gctx, orc, c["indiv"], c["X"], c["y"], c["N"], c["packed"])
    r = gctx.mme(tol=1e-13, rule=G.RULE_PCGSOLVER, precision=G.PREC_MIXED)
    for v in ("beta", "uhat", "bhat"):
        assert rel(r[v], c["ref"]["geno64_" + v]) < 2e-8, v


def test_pcg_mixed_masked_block(gctx, orc):
    s = _load(gctx, orc, *_case("wide", CASES[3][1]))
    B = np.column_stack([s.grm_apply(np.ones((s.N, 1)))[:, 0][np.asarray(s._keep[0])],
                         np.random.default_rng(1).standard_normal((s.Nrec, 6))])
    X, info = gctx.pcg(B, tol=1e-10, rule=G.RULE_AIREML, mask=True, precision=G.PREC_MIXED)
    s.precond_build()
    Xo, _ = s.pcg(B, 1e-10, rule=1)
    assert rel(X, Xo) < 1e-7


def test_mixed_precision_covers_every_grm_product(gctx, orc):
    """With precision MIXED every GRM product of the call (PCG, u-hat, the probes' u-hat)
    runs on the tensor cores: the context's own precision stays FP64 and is restored,
    and the AIREML loop on genotypes matches the FP64 loop (same probes)."""
    coh = cohort(21, 400, 700, recs=("uniform", 1, 4), miss=0.02)
    indiv, N = coh["indiv"].astype(np.int32), coh["N"]
    s = _load(gctx, orc, indiv, coh["X"], coh["y"], N, coh["packed"])
    gctx.set_precision(G.PREC_FP64)
    gctx.prof_enable(True)
    grm0, tc0 = gctx.prof_query(G._lib.PROF_GRM)[0], gctx.prof_query(G._lib.PROF_GRM_PASS1)[0]
    gctx.mme(tol=1e-10, rule=G.RULE_AIREML, precision=G.PREC_MIXED)
    gctx.aireml_grad(5, seed=3, tol=1e-10, rule=G.RULE_AIREML, precision=G.PREC_MIXED)
    grm1, tc1 = gctx.prof_query(G._lib.PROF_GRM)[0], gctx.prof_query(G._lib.PROF_GRM_PASS1)[0]
    gctx.prof_enable(False)
    assert grm1 > grm0 and tc1 - tc0 == grm1 - grm0        # every GRM product ran one tensor-core pass 1
    res = {}
    for prec in (G.PREC_FP64, G.PREC_MIXED):
        gctx.set_vc(VC_F)
        res[prec] = gctx.aireml_run(theta0=(0.5, 0.3, 0.2, 0.1, 0.1), maxiter=8, tol=1e-3, numMC=5,
                                    pcg_tol=1e-10, precision=prec, seed=7)
    assert res[G.PREC_MIXED]["iterations"] == res[G.PREC_FP64]["iterations"]
    assert rel(res[G.PREC_MIXED]["theta"], res[G.PREC_FP64]["theta"]) < 1e-6


def _dense(gctx, orc, N, seed):
    coh = cohort(seed, N, 600, recs=("uniform", 1, 3), miss=0.02)
    grm = synth.grm_from_packed(coh["packed"], N)
    indiv = coh["indiv"].astype(np.int32)
    gctx.load_records(indiv, coh["X"], coh["y"], N)
    gctx.load_grm(grm, N)
    gctx.set_vc(VC_F)
    return grm, orc.Solver(indiv, coh["X"], coh["y"], N, VC_F, grm_lt=grm)


@pytest.mark.parametrize("N", [129, 203, 2000])
def test_dense_mixed_matches_emulation(gctx, orc, N):
    """Dense GRM under GLOBE_PREC_MIXED (tensor cores): the product of A rounded to its 7
    digit planes (within 2^-34 max|A|) and each column of Z rounded to 9 base-32 digits,
    equal to that product evaluated in FP64 (the MMA sums are exact integers); and within
    ~1e-10 of the FP64 oracle (the rounding of A).  N = 129, 203 pad the last row tile
    and K chunk; k = 40 runs two column groups (MMA widths 16 .. 192)."""
    from helpers import dense_tc_emulation, lt_to_full
    grm, s = _dense(gctx, orc, N, 31 + N)
    A = lt_to_full(grm, N)
    rng = np.random.default_rng(N)
    try:
        gctx.set_precision(G.PREC_MIXED)
        for k in (1, 5, 16, 21, 40):
            Z = rng.standard_normal((N, k)) * np.logspace(-3, 3, k)
            got, ref = gctx.grm_apply(Z), s.grm_apply(Z)
            emu = dense_tc_emulation(A, Z, VC_F[1], 9)
            assert max(rel(got[:, c], emu[:, c]) for c in range(k)) < 1e-13, k
            assert max(rel(got[:, c], ref[:, c]) for c in range(k)) < 1e-9, k
    finally:
        gctx.set_precision(G.PREC_FP64)


def test_dense_mixed_digit_count(gctx, orc):
    """The digit count sets the planes of A too (min(7, digits)); changing it rebuilds them."""
    from helpers import dense_tc_emulation, lt_to_full
    N = 300
    grm, s = _dense(gctx, orc, N, 5)
    A = lt_to_full(grm, N)
    Z = np.random.default_rng(2).standard_normal((N, 6))
    try:
        gctx.set_precision(G.PREC_MIXED)
        for nd in (4, 9, 2, 6):
            gctx.set_digits(nd)
            got = gctx.grm_apply(Z)
            emu = dense_tc_emulation(A, Z, VC_F[1], nd)
            assert max(rel(got[:, c], emu[:, c]) for c in range(6)) < 1e-13, nd
    finally:
        gctx.set_digits(9)
        gctx.set_precision(G.PREC_FP64)


def test_dense_mixed_nonfinite_entry(gctx, orc):
    """A non-finite GRM entry has no digit planes: the product propagates it (double-float
    kernel), into the rows of both of its indices, as the FP64 product does."""
    N = 150
    grm, _ = _dense(gctx, orc, N, 8)
    grm = grm.copy()
    i0, j0 = 40, 7
    grm[i0 * (i0 + 1) // 2 + j0] = np.nan
    gctx.load_grm(grm, N)
    Z = np.random.default_rng(1).standard_normal((N, 3))
    out = {}
    try:
        for prec in (G.PREC_MIXED, G.PREC_FP64):
            gctx.set_precision(prec)
            out[prec] = gctx.grm_apply(Z)
    finally:
        gctx.set_precision(G.PREC_FP64)
    for o in out.values():
        bad = ~np.isfinite(o).all(axis=1)
        assert set(np.flatnonzero(bad)) == {i0, j0}
    ok = np.isfinite(out[G.PREC_FP64])
    assert rel(out[G.PREC_MIXED][ok], out[G.PREC_FP64][ok]) < 1e-11


@pytest.mark.parametrize("nd", [2, 3, 4, 5, 6, 7, 8, 9])
def test_digit_count_matches_exact_emulation(gctx, orc, nd):
    """With nd digits per column the product is the exact product of the nd-digit-rounded
    columns: equal to its CPU emulation up to FP64 rounding, for one group of 20 columns
    (MMA width round16(20 nd)) and for a width that splits into groups."""
    from helpers import tc_product_emulation
    indiv, X, y, N, packed = _case("odd", (9, 131, 257, ("uniform", 1, 6), 0.03))
    s = _load(gctx, orc, indiv, X, y, N, packed)
    alt, miss, maf, _, keep = orc.bed_stats(packed, N)
    Gk = synth.unpack_genotypes(packed[keep], N)
    Gk = np.where(Gk < 0, 0, Gk)
    rng = np.random.default_rng(nd)
    assert gctx.get_digits() == 9
    try:
        gctx.set_precision(G.PREC_MIXED)
        gctx.set_digits(nd)
        for k in (20, 256 // nd + 3):
            Z = rng.standard_normal((N, k)) * np.logspace(-2, 2, k)
            got = gctx.grm_apply(Z)
            emu = tc_product_emulation(Gk, s.f, s.inv_std, Z, VC_F[1] / keep.sum(), nd)
            assert max(rel(got[:, c], emu[:, c]) for c in range(k)) < 1e-11, k
            # and the error against the exact product is the digit rounding's
            ref = s.grm_apply(Z)
            assert max(rel(got[:, c], ref[:, c]) for c in range(k)) < 16 * 2.0 ** -(5 * (nd - 1) + 4) + 1e-12
    finally:
        gctx.set_digits(9)
        gctx.set_precision(G.PREC_FP64)


def test_digit_count_arguments(gctx):
    for bad in (0, 1, 10):
        with pytest.raises(G.GlobeError):
            gctx.set_digits(bad)
    assert gctx.get_digits() == 9


def _synth_cohort(gctx, N, M, seed):
    """Genotypes from the device generator (copied back for the oracle) and a one-record-
    per-individual table; returns (indiv, X, y, packed)."""
    torch = pytest.importorskip("torch")
    bps = (N + 3) // 4
    stride = (bps + 15) // 16 * 16
    raw = torch.empty((M, stride), dtype=torch.uint8, device="cuda")
    gctx.synth_bed_dev(raw.data_ptr(), M, N, stride, seed, 0.01, 0.5, 0.02)
    packed = raw[:, :bps].cpu().numpy()
    del raw
    rng = np.random.default_rng(seed)
    indiv = np.arange(N, dtype=np.int32)
    X = np.asfortranarray(np.column_stack([np.ones(N), rng.standard_normal(N), rng.uniform(0, 5, N)]))
    return indiv, X, rng.standard_normal(N), packed


def test_k_range_split_beyond_one_cta(gctx, orc):
    """M = 600k SNPs: pass 2 sums over 600k SNPs, more than the 2^19 products one CTA may
    accumulate exactly in FP32, so its K range is split across CTAs; the product stays exact."""
    N, M = 1000, 600_000
    indiv, X, y, packed = _synth_cohort(gctx, N, M, 123)
    s = _load(gctx, orc, indiv, X, y, N, packed)
    Z = np.random.default_rng(1).standard_normal((N, 3)) * np.array([1.0, 1e-2, 1e2])
    try:
        gctx.set_precision(G.PREC_MIXED)
        got = gctx.grm_apply(Z)
    finally:
        gctx.set_precision(G.PREC_FP64)
    ref = s.grm_apply(Z)
    assert max(rel(got[:, c], ref[:, c]) for c in range(3)) < 1e-11


def test_mid_size_properties(gctx):
    """N = 20k, M = 40k (12 K-stages per CTA, hundreds of CTAs): the mixed product is symmetric
    and linear to FP64 rounding and matches the FP64 GPU product."""
    N, M = 20_000, 40_000
    indiv, X, y, packed = _synth_cohort(gctx, N, M, 321)
    gctx.load_records(indiv, X, y, N)
    gctx.load_bed(packed)
    gctx.set_vc(VC_F)
    rng = np.random.default_rng(2)
    Z = rng.standard_normal((N, 5))
    try:
        gctx.set_precision(G.PREC_MIXED)
        AZ = gctx.grm_apply(Z)
        # symmetry: x'(A y) = (A x)'y for every pair of columns
        S = Z.T @ AZ
        assert np.abs(S - S.T).max() < 1e-11 * np.abs(S).max()
        # linearity: A(2 z0 - z1) = 2 A z0 - A z1
        comb = gctx.grm_apply(np.column_stack([2 * Z[:, 0] - Z[:, 1]]))[:, 0]
        assert rel(comb, 2 * AZ[:, 0] - AZ[:, 1]) < 1e-11
        gctx.set_precision(G.PREC_FP64)
        ref = gctx.grm_apply(Z)
    finally:
        gctx.set_precision(G.PREC_FP64)
    assert max(rel(AZ[:, c], ref[:, c]) for c in range(5)) < 1e-11
