"""Failure paths return status codes (no GPU fault is provoked)."""
import numpy as np
import pytest

import globe_gb300 as G
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
