"""Host-side restatements that the kernels rely on, checked on the CPU."""
import numpy as np
import pytest

from globe_gb300 import synth
from helpers import cohort


def test_pack_unpack_roundtrip():
    rng = np.random.default_rng(0)
    for N in (1, 2, 3, 4, 5, 37, 128, 129):
        G = rng.integers(-1, 3, size=(7, N)).astype(np.int8)
        assert np.array_equal(synth.unpack_genotypes(synth.pack_genotypes(G), N), G)


def test_normal_stream_is_deterministic():
    a = synth.normal_stream(9, 100001)
    assert np.array_equal(a, synth.normal_stream(9, 100001))
    assert abs(a.mean()) < 0.02 and abs(a.std() - 1) < 0.02


def test_numpy_stats_equal_oracle(orc):
    coh = cohort(4, 203, 300, edge=True)
    a, m, f, k = synth.ref_allele_stats(coh["packed"], 203)
    a2, m2, f2, _, k2 = orc.bed_stats(coh["packed"], 203)
    assert np.array_equal(a, a2) and np.array_equal(m, m2) and np.array_equal(k, k2)
    assert np.array_equal(f.view(np.uint32), f2.view(np.uint32))


@pytest.mark.parametrize("n", [1, 2, 3, 7, 40])
def test_woodbury_block_inverse(n):
    """Q = s2e I + W C W' (W = [1 t], C = D + diag(g, 0)) inverted as
    (r - W H W'r)/s2e, H = (s2e I + C W'W)^-1 C -- the form k_build_H /
    k_precond_apply evaluate -- equals the dense inverse of the
    reference's block (PCGsolver.cpp:1014-1049)."""
    rng = np.random.default_rng(n)
    s2e, s2g, s2b0, sb01, s2b1, aii = 0.6, 0.4, 0.4, 0.2, 0.2, 1.07
    t = np.sort(rng.uniform(0, 10, n))
    g = s2g * aii
    Q = g + s2b0 + sb01 * (t[:, None] + t[None, :]) + s2b1 * np.outer(t, t) + s2e * np.eye(n)
    W = np.column_stack([np.ones(n), t])
    Cm = np.array([[s2b0 + g, sb01], [sb01, s2b1]])
    G2 = W.T @ W
    H = np.linalg.solve(s2e * np.eye(2) + Cm @ G2, Cm)
    r = rng.standard_normal(n)
    z = (r - W @ (H @ (W.T @ r))) / s2e
    assert np.allclose(z, np.linalg.solve(Q, r), rtol=1e-10, atol=1e-12)


def test_time_block_rank2_form():
    """U D U' x over one block = (D00 s0 + D01 s1) + t (D01 s0 + D11 s1)."""
    rng = np.random.default_rng(1)
    t = rng.uniform(0, 5, 9)
    x = rng.standard_normal(9)
    b0, b01, b1 = 0.4, 0.2, 0.2
    full = (b0 + b01 * (t[:, None] + t[None, :]) + b1 * np.outer(t, t)) @ x
    s0, s1 = x.sum(), (t * x).sum()
    assert np.allclose(full, (b0 * s0 + b01 * s1) + t * (b01 * s0 + b1 * s1))
