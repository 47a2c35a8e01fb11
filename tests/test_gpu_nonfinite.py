"""Non-finite right-hand sides on the tensor-core products (GLOBE_PREC_MIXED).

The reference's FP32 loops carry a NaN or an infinity of the input through every
sum it enters (computeVx_multi, PCGsolver.cpp:1151-1213), and so does the FP64
path here.  The mixed products scale and split each column into integer digits,
which cannot hold a NaN; a column holding one is marked when its scale is taken
and its output is NaN.  Every other column of the same call is unchanged."""
import numpy as np
import pytest

import globe_gb300 as G
from helpers import VC_F, golden_case, rel

pytestmark = pytest.mark.gpu

# mixed vs FP64 on finite columns: the genotype product is exact up to the 45-bit rounding
# of each column; the dense one also holds A to 2^-34 max|A| (its 7 digit planes)
TOL = {"genotypes": 1e-11, "dense": 1e-9}
BAD = (("nan", 1, 3, np.nan), ("inf", 2, 7, np.inf), ("-inf", 4, 0, -np.inf))


def _poison(Z):
    Z = Z.copy()
    for _, c, r, v in BAD:
        Z[r, c] = v
    Z[:, 5] = np.nan                    # a column of NaN only
    return Z


def _both(gctx, fn, Z):
    out = {}
    try:
        for prec in (G.PREC_FP64, G.PREC_MIXED):
            gctx.set_precision(prec)
            out[prec] = fn(Z)
    finally:
        gctx.set_precision(G.PREC_FP64)
    return out[G.PREC_FP64], out[G.PREC_MIXED]


def _check(f64, mixed, clean, poisoned, tol):
    # the FP64 path: every entry of a poisoned column is non-finite, the rest finite
    assert np.isfinite(f64[:, clean]).all()
    assert not np.isfinite(f64[:, poisoned]).any()
    # the mixed path: the same pattern; its poisoned columns are NaN
    assert np.array_equal(np.isfinite(mixed), np.isfinite(f64))
    assert np.isnan(mixed[:, poisoned]).all()
    for c in clean:
        assert rel(mixed[:, c], f64[:, c]) < tol, c


def _setup(gctx, source):
    c = golden_case("geno_small")
    gctx.load_records(c["indiv"], c["X"], c["y"], c["N"])
    if source == "genotypes":
        gctx.load_bed(c["packed"])
    else:
        gctx.load_grm(c["grm"], c["N"])
    gctx.set_vc(VC_F)
    return c


@pytest.mark.parametrize("source", ["genotypes", "dense"])
def test_grm_apply_propagates_nonfinite(gctx, source):
    c = _setup(gctx, source)
    Z = _poison(np.random.default_rng(3).standard_normal((c["N"], 7)))
    f64, mixed = _both(gctx, gctx.grm_apply, Z)
    _check(f64, mixed, clean=[0, 3, 6], poisoned=[1, 2, 4, 5], tol=TOL[source])


@pytest.mark.parametrize("source", ["genotypes", "dense"])
def test_vx_propagates_nonfinite(gctx, source):
    """V x: a non-finite record enters its individual's J'x, so the GRM term spreads it
    to every record; the mixed path gives the FP64 path's pattern."""
    c = _setup(gctx, source)
    x = _poison(np.random.default_rng(4).standard_normal((c["Nrec"], 7)))
    f64, mixed = _both(gctx, gctx.vx, x)
    _check(f64, mixed, clean=[0, 3, 6], poisoned=[1, 2, 4, 5], tol=TOL[source])


def test_clean_call_after_nonfinite(gctx):
    """A poisoned call leaves nothing behind: the next product equals the FP64 one."""
    c = _setup(gctx, "genotypes")
    rng = np.random.default_rng(5)
    Z = rng.standard_normal((c["N"], 7))
    _both(gctx, gctx.grm_apply, _poison(Z))
    f64, mixed = _both(gctx, gctx.grm_apply, Z)
    assert rel(mixed, f64) < 1e-11
