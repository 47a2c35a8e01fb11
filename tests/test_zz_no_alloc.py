"""globe_precond_apply_dev_noalloc: the block preconditioner on device buffers,
with its r'z partials in a static device buffer (no device allocation),
against globe_precond_apply on the same inputs.  Collected last, and passes
alone as well."""
import ctypes as C

import numpy as np
import pytest

import globe_gb300 as G
from globe_gb300 import synth
from helpers import VC_F, rel

pytestmark = pytest.mark.gpu

PART_DOUBLES = 1 << 18          # size of the static partials buffer (globe.h)
GLOBE_ERR_ARG, GLOBE_ERR_STATE = -1, -3


def _counts(layout, rng):
    if layout == "short_blocks":             # every block <= 48 records: one thread per (block, column)
        return rng.integers(1, 11, size=3000)
    if layout == "all_long":                 # every block > 48 records: one warp per block
        return np.full(2000, 49)
    c = rng.integers(1, 6, size=2000)          # a few blocks > 48 records get a warp each, the rest a thread
    c[[5, 777, 1999]] = (60, 49, 120)
    return c


def _partial_slots(counts):
    """CTAs writing r'z partials per column: one per 256 blocks (thread layout) plus one
    per 8 blocks longer than 48 records (warp layout)."""
    nlong = int((np.asarray(counts) > 48).sum())
    return (len(counts) + 255) // 256 + (nlong + 7) // 8


def _setup(ctx, layout, seed):
    rng = np.random.default_rng(seed)
    counts = _counts(layout, rng)
    N = len(counts)
    indiv = np.repeat(np.arange(N, dtype=np.int32), counts)
    Nrec = len(indiv)
    t = rng.uniform(0.0, 10.0, Nrec)
    X = np.asfortranarray(np.column_stack([np.ones(Nrec), rng.standard_normal(Nrec), t]))
    y = rng.standard_normal(Nrec)
    ctx.load_records(indiv, X, y, N)
    ctx.load_bed(synth.pack_genotypes(synth.simulate_genotypes(rng, 64, N, 0.05, 0.5, 0.01)))
    ctx.set_vc(VC_F)
    return N, Nrec, rng


def _noalloc(ctx, dr, dz, k, drz):
    return ctx._L.globe_precond_apply_dev_noalloc(ctx.h, C.c_void_p(dr), C.c_void_p(dz), k,
                                                  C.c_void_p(drz) if drz else None)


def _dev(torch, a):
    """Nrec x k float64 -> device tensor (k, Nrec): the column-major layout of the C ABI."""
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).cuda()


@pytest.mark.parametrize("layout", ["short_blocks", "long_blocks"])
def test_matches_precond_apply_on_two_calls(layout):
    torch = pytest.importorskip("torch")
    with G.Context(0) as ctx:
        N, Nrec, rng = _setup(ctx, layout, 11)
        k = 7
        r = rng.standard_normal((Nrec, k)) * np.logspace(-2, 2, k)
        z_ref = ctx.precond_apply(r)           # existing entry point; builds the preconditioner
        rz_ref = (r * z_ref).sum(axis=0)
        dr = _dev(torch, r)
        dz = torch.empty_like(dr)
        drz = torch.empty(k, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        bytes0 = ctx.device_bytes()
        for _ in range(2):
            dz.fill_(float("nan"))
            drz.fill_(float("nan"))
            torch.cuda.synchronize()
            rc = _noalloc(ctx, dr.data_ptr(), dz.data_ptr(), k, drz.data_ptr())
            assert rc == 0, ctx._L.globe_last_error(ctx.h)
            ctx.synchronize()
            z = dz.cpu().numpy().T
            assert rel(z, z_ref) < 1e-13
            assert rel(drz.cpu().numpy(), rz_ref) < 1e-12
        assert ctx.device_bytes() == bytes0      # the context allocated nothing


def test_rejects_sizes_beyond_static_buffer():
    torch = pytest.importorskip("torch")
    with G.Context(0) as ctx:
        N, Nrec, rng = _setup(ctx, "all_long", 12)
        k = PART_DOUBLES // _partial_slots(np.full(N, 49)) + 1    # first width whose partials do not fit
        r = np.zeros((Nrec, k))
        r[:, :2] = rng.standard_normal((Nrec, 2))
        z_ref = ctx.precond_apply(r[:, :2])
        dr = _dev(torch, r)
        dz = torch.zeros_like(dr)
        drz = torch.zeros(k, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = _noalloc(ctx, dr.data_ptr(), dz.data_ptr(), k, drz.data_ptr())
        assert rc == GLOBE_ERR_ARG
        assert b"static buffer" in ctx._L.globe_last_error(ctx.h)
        ctx.synchronize()
        assert float(dz.abs().max()) == 0.0    # rejected before any launch
        # without r'z no partials are needed: widths up to 65535 are accepted
        rc = _noalloc(ctx, dr.data_ptr(), dz.data_ptr(), k, 0)
        assert rc == 0, ctx._L.globe_last_error(ctx.h)
        ctx.synchronize()
        assert rel(dz[:2].cpu().numpy().T, z_ref) < 1e-13


def test_needs_a_built_preconditioner():
    torch = pytest.importorskip("torch")
    with G.Context(0) as ctx:
        N, Nrec, rng = _setup(ctx, "short_blocks", 13)
        dr = _dev(torch, rng.standard_normal((Nrec, 1)))
        dz = torch.empty_like(dr)
        rc = _noalloc(ctx, dr.data_ptr(), dz.data_ptr(), 1, 0)
        assert rc == GLOBE_ERR_STATE
        assert b"preconditioner" in ctx._L.globe_last_error(ctx.h)


def _setup_widths(ctx, seed):
    """88 records: one individual of 49 records (warp layout) and 39 of one record."""
    rng = np.random.default_rng(seed)
    counts = np.ones(40, dtype=np.int64)
    counts[17] = 49
    indiv = np.repeat(np.arange(40, dtype=np.int32), counts)
    Nrec = len(indiv)
    t = rng.uniform(0.0, 10.0, Nrec)
    X = np.asfortranarray(np.column_stack([np.ones(Nrec), rng.standard_normal(Nrec), t]))
    ctx.load_records(indiv, X, rng.standard_normal(Nrec), 40)
    ctx.load_bed(synth.pack_genotypes(synth.simulate_genotypes(rng, 64, 40, 0.2, 0.5, 0.0)))
    ctx.set_vc(VC_F)
    return Nrec, rng


def test_width_limits_checked_before_launch():
    """Widths whose launch could not start are rejected up front: more than 65535
    columns, and more than 768 columns with r'z when a block is longer than 48 records
    (the warp-per-block kernel's shared-memory partials at the default 48 KB)."""
    torch = pytest.importorskip("torch")
    with G.Context(0) as ctx:
        Nrec, rng = _setup_widths(ctx, 14)
        r = rng.standard_normal((Nrec, 768))
        z_ref = ctx.precond_apply(r)
        rz_ref = (r * z_ref).sum(axis=0)
        for k, with_rz, ok in ((768, True, True), (769, True, False), (65535, False, True), (65536, False, False)):
            dr = torch.zeros((k, Nrec), dtype=torch.float64, device="cuda")
            dr[:768] = _dev(torch, r)
            dz = torch.zeros_like(dr)
            drz = torch.zeros(k, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            rc = _noalloc(ctx, dr.data_ptr(), dz.data_ptr(), k, drz.data_ptr() if with_rz else 0)
            ctx.synchronize()
            if ok:
                assert rc == 0, ctx._L.globe_last_error(ctx.h)
                assert rel(dz[:768].cpu().numpy().T, z_ref) < 1e-13
                if with_rz:
                    assert rel(drz.cpu().numpy(), rz_ref) < 1e-12
            else:
                assert rc == GLOBE_ERR_ARG
                assert b"at most" in ctx._L.globe_last_error(ctx.h)
                assert float(dz.abs().max()) == 0.0      # rejected before any launch
