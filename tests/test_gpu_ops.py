"""Operators on the GPU vs the oracle: GRM product (genotype and dense),
genetic diagonal, V x and the block preconditioner."""
import numpy as np
import pytest

from helpers import VC_F, cohort, golden_case, rel

pytestmark = pytest.mark.gpu


def _cases():
    odd = cohort(9, 131, 257, recs=("uniform", 1, 6), miss=0.03, edge=True)   # N not /4 /8 /128, 1-record indivs
    big = cohort(11, 1000, 700, recs=("poisson", 4), T=10.0)
    out = []
    for nm in ("geno_small", "tiny"):
        c = golden_case(nm)
        out.append((nm, c["indiv"], c["X"], c["y"], c["N"], c["packed"], c["grm"]))
    for nm, c in (("odd", odd), ("big", big)):
        from globe_gb300 import synth
        out.append((nm, c["indiv"].astype(np.int32), c["X"], c["y"], c["N"], c["packed"],
                    synth.grm_from_packed(c["packed"], c["N"])))
    return out


CASES = _cases()


def _setup(gctx, orc, case, src, vc=VC_F):
    nm, indiv, X, y, N, packed, grm = case
    gctx.load_records(indiv, X, y, N)
    if src == "geno":
        gctx.load_bed(packed)
        s = orc.Solver(indiv, X, y, N, vc, packed=packed)
    else:
        gctx.load_grm(grm, N)
        s = orc.Solver(indiv, X, y, N, vc, grm_lt=grm)
    gctx.set_vc(vc)
    return s


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("src", ["geno", "grm"])
def test_operators_match_oracle(gctx, orc, case, src):
    s = _setup(gctx, orc, case, src)
    N, Nrec = case[4], len(case[1])
    rng = np.random.default_rng(N)
    for k in (1, 3, 9):
        Z = rng.standard_normal((N, k))
        assert rel(gctx.grm_apply(Z), s.grm_apply(Z)) < 1e-12, k
        x = rng.standard_normal((Nrec, k))
        assert rel(gctx.vx(x), s.vx(x)) < 1e-12, k
    assert rel(gctx.genetic_diag(), s.genetic_diag()) < 1e-12
    s.precond_build()
    r = rng.standard_normal((Nrec, 4))
    assert rel(gctx.precond_apply(r), s.precond_apply(r)) < 1e-10


def test_vx_is_symmetric_positive(gctx, orc):
    s = _setup(gctx, orc, CASES[2], "geno")
    rng = np.random.default_rng(3)
    a = rng.standard_normal(len(CASES[2][1]))
    b = rng.standard_normal(len(CASES[2][1]))
    Va, Vb = gctx.vx(a)[:, 0], gctx.vx(b)[:, 0]
    assert abs(a @ Vb - b @ Va) < 1e-10 * abs(a @ Vb)
    assert a @ Va > 0
