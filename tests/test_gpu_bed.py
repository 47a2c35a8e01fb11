"""PLINK statistics and filter on the GPU: bit-exact with the reference."""
import numpy as np
import pytest

from globe_gb300 import Context
from helpers import cohort, golden_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["geno_small", "tiny"])
def test_stats_bit_exact_vs_reference(gctx, name):
    c = golden_case(name)
    gctx.load_records(c["indiv"], c["X"], c["y"], c["N"])
    st = gctx.load_bed(c["packed"])
    r = c["ref"]
    assert np.array_equal(st["alt"], r["stats_alt"])
    assert np.array_equal(st["miss"], r["stats_miss"])
    assert np.array_equal(st["maf"].view(np.uint32), r["stats_maf"].view(np.uint32))
    assert np.array_equal(st["miss_rate"].view(np.uint32), r["stats_miss_rate"].view(np.uint32))
    assert np.array_equal(st["keep"], r["stats_keep"].astype(bool))
    assert st["kept"] == int(r["stats_keep"].sum())


@pytest.mark.parametrize("N", [61, 62, 63, 64, 65, 131])
@pytest.mark.parametrize("thr", [(0.01, 0.2), (0.0, 1.0), (0.2, 0.05), (0.5, 0.0)])
def test_stats_vs_oracle_all_phantom_counts(gctx, orc, N, thr):
    coh = cohort(100 + N, N, 203, recs=("uniform", 1, 3), miss=0.08, edge=True)
    gctx.load_records(coh["indiv"], coh["X"], coh["y"], N)
    st = gctx.load_bed(coh["packed"], *thr)
    alt, miss, maf, mr, keep = orc.bed_stats(coh["packed"], N, *thr)
    assert np.array_equal(st["alt"], alt) and np.array_equal(st["miss"], miss)
    assert np.array_equal(st["maf"].view(np.uint32), maf.view(np.uint32))
    assert np.array_equal(st["miss_rate"].view(np.uint32), mr.view(np.uint32))
    assert np.array_equal(st["keep"], keep)


def test_no_snp_passes(gctx):
    coh = cohort(5, 40, 16, miss=0.0)
    gctx.load_records(coh["indiv"], coh["X"], coh["y"], 40)
    st = gctx.load_bed(coh["packed"], 0.5, 0.0)   # maf must be exactly 0.5
    assert st["kept"] == int(st["keep"].sum())


@pytest.mark.parametrize("chunk", [0, 1, 3 * 13, 1000])
def test_streamed_file_matches_in_memory(gctx, tmp_path, chunk):
    """globe_load_bed_file (chunked reads through pinned buffers, 2-D copies into padded
    device rows) gives the in-memory load's statistics and the same genetic source;
    chunk sizes of one row, a few rows with a ragged tail, and the default."""
    from globe_gb300 import synth
    coh = cohort(71, 51, 211, recs=("uniform", 1, 3), miss=0.05, edge=True)
    pre = synth.write_cohort(str(tmp_path), "s", coh)
    gctx.load_records(coh["indiv"], coh["X"], coh["y"], 51)
    ref = gctx.load_bed(coh["packed"])
    z = np.random.default_rng(1).standard_normal((51, 3))
    g_ref = gctx.grm_apply(z)
    st = gctx.load_bed_file(pre, chunk_bytes=chunk)
    for k in ("alt", "miss", "keep"):
        assert np.array_equal(st[k], ref[k]), k
    assert np.array_equal(st["maf"].view(np.uint32), ref["maf"].view(np.uint32))
    assert st["kept"] == ref["kept"]
    assert np.array_equal(gctx.grm_apply(z), g_ref)


def test_streamed_file_errors(gctx, tmp_path):
    import globe_gb300 as G
    from globe_gb300 import synth
    coh = cohort(72, 40, 30, recs=("uniform", 1, 2))
    pre = synth.write_cohort(str(tmp_path), "e", coh)
    gctx.load_records(coh["indiv"], coh["X"], coh["y"], 40)
    with open(pre + ".bed", "r+b") as f:                 # drop the last SNP row
        f.truncate(3 + 29 * 10)
    with pytest.raises(G.GlobeError) as e:
        gctx.load_bed_file(pre)
    assert e.value.code == -5
    with pytest.raises(G.GlobeError) as e:
        gctx.load_bed_file(str(tmp_path / "missing"))
    assert e.value.code == -4


def test_resident_genotype_copies():
    """After loading, the genotypes are held as the SNP-major tile-blocked copy only (the
    compacted rows and the staging buffers are gone); the first tensor-core product adds
    the individual-major copy, and FP64 work never needs it."""
    c = cohort(17, 2000, 10000, recs=("uniform", 3, 10), miss=0.01)
    N = c["N"]
    with Context(0) as ctx:
        ctx.load_records(c["indiv"].astype(np.int32), c["X"], c["y"], N)
        before = ctx.device_bytes()
        st = ctx.load_bed(c["packed"])
        grew = ctx.device_bytes() - before
        Mk = int(st["kept"])
        # tiles of 128 rows x 32 bytes, row counts rounded to 512 (a CTA's four tiles)
        blk1 = -(-Mk // 512) * 512 * (-(-((N + 3) // 4) // 32) * 32)
        blk2 = -(-N // 512) * 512 * (-(-((Mk + 3) // 4) // 32) * 32)
        tables = Mk * 8 * 6 + N * 8          # zs (4), f, inv per SNP; genetic diagonal
        assert blk1 <= grew <= blk1 + tables + (1 << 20)
        ctx.set_vc((0.6, 0.4, 0.4, 0.2, 0.2))
        ctx.grm_apply(np.ones((N, 1)))        # FP64: no second copy
        assert ctx.device_bytes() - before - grew < blk2 // 2
        from globe_gb300 import PREC_MIXED
        ctx.set_precision(PREC_MIXED)
        ctx.grm_apply(np.ones((N, 1)))        # tensor cores: the individual-major copy appears
        assert ctx.device_bytes() - before >= blk1 + blk2
