"""The oracle's GRM builder (orc_grm_build) against the .grm.bin fixtures.
Those are the matrices the reference programs were run on
(tests/golden/make_golden.py), whose --grm solutions agree with the
reference's own --geno solutions (test_oracle_golden.py), so this pins the
builder's arithmetic and convention to the reference's standardisation."""
import os

import numpy as np
import pytest

from helpers import GOLDEN, VC_F, f32_ulps, golden_case, rel


@pytest.mark.parametrize("name", ["geno_small", "tiny"])
def test_oracle_grm_matches_fixture(orc, name):
    c = golden_case(name)
    # the fixtures take the FP32 program's float allele frequency: bit-exact
    lt = orc.grm_build(c["packed"], c["N"], freq="f32")
    assert lt.size == c["grm"].size
    u = f32_ulps(lt, c["grm"])
    assert u.max() <= 1
    assert (u == 0).mean() > 0.999
    # with the double frequency of the FP64 build (the product path's), the
    # matrices differ by the float rounding of f: a few 1e-7 of max |A|
    lt64 = orc.grm_build(c["packed"], c["N"])
    assert np.abs(lt64 - c["grm"]).max() <= 5e-7 * np.abs(c["grm"]).max()


def test_oracle_grm_definition(orc):
    """All entries from the definition, in numpy."""
    c = golden_case("tiny")
    N = c["N"]
    lt = orc.grm_build(c["packed"], N)
    alt, miss, maf, _, keep = orc.bed_stats(c["packed"], N)
    f, inv = orc.std_params(alt[keep], miss[keep], N)
    codes = np.unpackbits(c["packed"][keep][:, :, None], axis=2, bitorder="little").reshape(keep.sum(), -1)
    codes = (codes[:, 0::2] + 2 * codes[:, 1::2])[:, :N]
    g = np.choose(codes, [2, 0, 1, 0]).astype(np.float64)
    Z = (g - 2 * f[:, None]) * inv[:, None]
    A = Z.T @ Z / keep.sum()
    il = np.tril_indices(N)
    assert np.abs(lt - A[il]).max() <= 2 * np.abs(A).max() * 2.0 ** -24


def test_reference_on_built_grm_reproduces_geno(orc):
    """The reference's own FP64 runPCGsolver, run with --grm on the GRM this builder's
    convention gives (oracle build; tests/golden/geno_small_grmf64_ref.npz), reproduces its
    --geno solution to the float32 rounding of the file; the oracle's solve on that GRM
    matches the reference run."""
    c = golden_case("geno_small")
    d = np.load(os.path.join(GOLDEN, "geno_small_grmf64_ref.npz"))
    for v in ("beta", "uhat", "bhat"):
        assert rel(d[v], c["ref"]["geno64_" + v]) < 5e-8, v
    lt = orc.grm_build(c["packed"], c["N"])
    s = orc.Solver(c["indiv"], c["X"], c["y"], c["N"], VC_F, grm_lt=lt)
    res = s.mme(1e-13)
    for v in ("beta", "uhat", "bhat"):
        assert rel(res[v], d[v]) < 2e-8, v
