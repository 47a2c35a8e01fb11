"""Failure paths return status codes (no GPU fault is provoked)."""
import numpy as np
import pytest

import globe_gb300 as G
from globe_gb300 import synth
from helpers import VC_F, cohort

pytestmark = pytest.mark.gpu


def test_state_and_argument_errors():
    with G.Context(0) as ctx:
        z = np.zeros(3)
        rc = ctx._L.globe_grm_apply(ctx.h, G.api._p(z), G.api._p(z), 1)
        assert rc == -3   # GLOBE_ERR_STATE: nothing loaded
        with pytest.raises(G.GlobeError, match="record table"):
            ctx.load_bed(np.zeros((2, 1), np.uint8))
        coh = cohort(1, 20, 30)
        ctx.load_records(coh["indiv"], coh["X"], coh["y"], 20)
        with pytest.raises(G.GlobeError, match="GRM has N"):
            ctx.load_grm(np.zeros(21 * 22 // 2, np.float32), 21)
        ctx.load_bed(coh["packed"])
        with pytest.raises(G.GlobeError, match="not set"):
            ctx.vx(np.zeros(len(coh["indiv"])))
        with pytest.raises(G.GlobeError, match="sig2e"):
            ctx.set_vc((0.0, 0.4, 0.4, 0.2, 0.2))
        ctx.set_vc(VC_F)
        with pytest.raises(G.GlobeError, match="globe_mme"):
            ctx.aireml_grad(2, seed=1)


def test_record_table_errors():
    with G.Context(0) as ctx:
        X = np.ones((4, 2))
        y = np.zeros(4)
        with pytest.raises(G.GlobeError, match="contiguous"):
            ctx.load_records(np.array([0, 1, 0, 1]), X, y, 2)
        with pytest.raises(G.GlobeError, match="outside"):
            ctx.load_records(np.array([0, 0, 1, 5]), X, y, 2)
        with pytest.raises(G.GlobeError, match="individuals have records"):
            ctx.load_records(np.array([0, 0, 1, 1]), X, y, 3)
        X[1, 0] = np.nan
        with pytest.raises(G.GlobeError, match="non-finite"):
            ctx.load_records(np.array([0, 0, 1, 1]), X, y, 2)


def test_tensor_core_wait_timeout_is_reported_and_recovered(orc):
    """A tensor-core launch whose first digit stage never arrives (test hook): its bounded
    waits run out (~2 s), the kernel aborts cleanly and the call reports the timeout; the
    same context then computes the product correctly."""
    import time
    from helpers import rel
    c = cohort(23, 200, 300, recs=("uniform", 1, 3), miss=0.02)     # one CTA per pass
    N = c["N"]
    Z = np.random.default_rng(4).standard_normal((N, 3))
    with G.Context(0) as ctx:
        ctx.load_records(c["indiv"].astype(np.int32), c["X"], c["y"], N)
        ctx.load_bed(c["packed"])
        ctx.set_vc(VC_F)
        ctx.set_precision(G.PREC_MIXED)
        assert ctx._L.globe_debug_stall_next_gemm(ctx.h) == 0
        t0 = time.perf_counter()
        with pytest.raises(G.GlobeError) as e:
            ctx.grm_apply(Z)
        assert time.perf_counter() - t0 < 30
        assert e.value.code == -2 and "timed out" in str(e.value)   # GLOBE_ERR_CUDA
        got = ctx.grm_apply(Z)                  # the context is still usable
        s = orc.Solver(c["indiv"].astype(np.int32), c["X"], c["y"], N, VC_F, packed=c["packed"])
        assert rel(got, s.grm_apply(Z)) < 1e-11


def test_dense_tensor_core_wait_timeout_is_reported_and_recovered(orc):
    """The same for the dense GRM's tensor-core kernel: its first stage (digit planes and
    digit tiles) never arrives, the MMA issuers' bounded waits run out, the call reports
    the timeout, and the context then computes the dense product correctly."""
    import time
    from helpers import rel
    c = cohort(29, 200, 300, recs=("uniform", 1, 3), miss=0.02)
    N = c["N"]
    grm = synth.grm_from_packed(c["packed"], N)
    Z = np.random.default_rng(5).standard_normal((N, 3))
    with G.Context(0) as ctx:
        ctx.load_records(c["indiv"].astype(np.int32), c["X"], c["y"], N)
        ctx.load_grm(grm, N)
        ctx.set_vc(VC_F)
        ctx.set_precision(G.PREC_MIXED)
        assert ctx._L.globe_debug_stall_next_gemm(ctx.h) == 0
        t0 = time.perf_counter()
        with pytest.raises(G.GlobeError) as e:
            ctx.grm_apply(Z)
        assert time.perf_counter() - t0 < 30
        assert e.value.code == -2 and "timed out" in str(e.value)   # GLOBE_ERR_CUDA
        got = ctx.grm_apply(Z)
        s = orc.Solver(c["indiv"].astype(np.int32), c["X"], c["y"], N, VC_F, grm_lt=grm)
        assert rel(got, s.grm_apply(Z)) < 1e-9


def test_timeout_inside_a_solve_is_reported_at_its_end(orc):
    """A bounded-wait timeout in the first GRM product of a block PCG is reported when the
    solve returns, although the later products (and the graph replays) ran without one:
    the kernels only set bits in the error word, and the solve's final check reads and
    clears it.  The next solve on the context is correct."""
    from helpers import rel
    c = cohort(23, 200, 300, recs=("uniform", 1, 3), miss=0.02)
    N = c["N"]
    indiv = c["indiv"].astype(np.int32)
    B = np.column_stack([c["X"], c["y"]])
    with G.Context(0) as ctx:
        ctx.load_records(indiv, c["X"], c["y"], N)
        ctx.load_bed(c["packed"])
        ctx.set_vc(VC_F)
        assert ctx._L.globe_debug_stall_next_gemm(ctx.h) == 0
        with pytest.raises(G.GlobeError) as e:
            ctx.pcg(B, tol=1e-10, maxit=6, rule=G.RULE_PCGSOLVER, precision=G.PREC_MIXED)
        assert e.value.code == -2 and "timed out" in str(e.value)
        X, info = ctx.pcg(B, tol=1e-10, rule=G.RULE_PCGSOLVER, precision=G.PREC_MIXED)
        assert info["converged"]
    s = orc.Solver(indiv, c["X"], c["y"], N, VC_F, packed=c["packed"])
    s.precond_build()
    Xo, _ = s.pcg(B, 1e-10, rule=0)
    assert rel(X, Xo) < 1e-8
