"""Seeded synthetic cohorts in GLOBE's file formats.

Writes the three inputs the ``runPCGsolver`` / ``runAIREML`` command lines
read:

* the record table: whitespace separated, header ``INDIV PHENO TIMES <cov...>``
  with the three named columns first (``PCGsolver.cpp:529-587``), individual
  IDs 1..N in ``.fam`` order, records grouped by individual;
* PLINK ``.bed/.bim/.fam``, SNP-major (magic ``6C 1B 01``), sample ``j`` of a
  SNP at bits ``2*(j%4)`` of byte ``j//4`` (``PCGsolver.cpp:811-826``), codes
  00 = two A1 alleles, 10 = one, 11 = none, 01 = missing;
* ``<prefix>.grm.bin``: float32 packed lower triangle, row major, with the
  diagonal, no header (``PCGsolver.cpp:778-809``).

The model simulated is the longitudinal genomic mixed model
``y = X b + J u + U b_i + e`` with ``u ~ N(0, s2g A)``, ``b_i ~ N(0, D)``.
Values written to the record table are quantised to short binary fractions so
that a float32 parse and a float64 parse of the same text give the same
number.
"""
import os

import numpy as np

VC_DEFAULT = (0.6, 0.4, 0.4, 0.2, 0.2)   # sig2e, sig2g, sig2b0, sigb01, sig2b1
CODE_OF_GENOTYPE = np.array([0b11, 0b10, 0b00], dtype=np.uint8)   # g = 0, 1, 2
CODE_MISSING = 0b01


def _q(x, step):
    return np.round(np.asarray(x, dtype=np.float64) / step) * step


def record_counts(rng, N, dist):
    """Records per individual.  ``dist``: ("uniform", lo, hi) | ("poisson", lam)
    (Poisson(lam)+1) | ("fixed", n) | ("geometric", p, lo, hi)."""
    kind = dist[0]
    if kind == "uniform":
        return rng.integers(dist[1], dist[2] + 1, size=N)
    if kind == "poisson":
        return rng.poisson(dist[1], size=N) + 1
    if kind == "fixed":
        return np.full(N, int(dist[1]))
    if kind == "geometric":
        c = rng.geometric(dist[1], size=N)
        return np.clip(c, dist[2], dist[3])
    raise ValueError(dist)


def pack_genotypes(G):
    """G: (M, N) int8 with values 0/1/2 (count of A1) or -1 (missing).
    Returns (M, ceil(N/4)) uint8 in PLINK SNP-major order; padding pairs are 00."""
    M, N = G.shape
    bps = (N + 3) // 4
    codes = np.where(G < 0, CODE_MISSING, CODE_OF_GENOTYPE[np.clip(G, 0, 2)]).astype(np.uint8)
    pad = bps * 4 - N
    if pad:
        codes = np.concatenate([codes, np.zeros((M, pad), np.uint8)], axis=1)
    c = codes.reshape(M, bps, 4)
    return (c[:, :, 0] | (c[:, :, 1] << 2) | (c[:, :, 2] << 4) | (c[:, :, 3] << 6)).astype(np.uint8)


def unpack_genotypes(packed, N):
    """Inverse of :func:`pack_genotypes` (missing -> -1)."""
    M, bps = packed.shape
    sh = np.array([0, 2, 4, 6], dtype=np.uint8)
    codes = ((packed[:, :, None] >> sh[None, None, :]) & 3).reshape(M, bps * 4)[:, :N]
    lut = np.array([2, -1, 1, 0], dtype=np.int8)
    return lut[codes]


def simulate_genotypes(rng, M, N, maf_lo, maf_hi, miss_rate, extra_edge_snps=False):
    p = rng.uniform(maf_lo, maf_hi, size=M)
    # A1 is the counted allele; flip half the SNPs so A1 frequency > 0.5 occurs
    flip = rng.random(M) < 0.5
    pa1 = np.where(flip, 1.0 - p, p)
    G = rng.binomial(2, pa1[:, None], size=(M, N)).astype(np.int8)
    if miss_rate > 0:
        G[rng.random((M, N)) < miss_rate] = -1
    if extra_edge_snps and M >= 8:
        G[0, :] = 2                         # monomorphic -> filtered (maf=1)
        G[1, :] = 0                         # monomorphic -> filtered (maf=0)
        G[2, :] = -1                        # all missing -> n_obs=0, maf=0
        G[3, rng.random(N) < 0.5] = -1      # ~50% missing -> filtered
        G[4, :] = 0
        G[4, : max(1, N // 200)] = 1        # maf ~ 0.0025 -> filtered at 0.01
    return G


def simulate_cohort(seed, N, M, recs, T, maf_lo=0.05, maf_hi=0.5, miss_rate=0.01,
                    vc=VC_DEFAULT, n_cov=2, edge_snps=False, exact_genetic=True):
    """Returns a dict with the record table columns (0-based ``indiv``), the
    SNP-major genotype matrix ``G`` (M x N int8, -1 missing) and the packed bytes."""
    rng = np.random.default_rng(seed)
    counts = record_counts(rng, N, recs)
    Nrec = int(counts.sum())
    indiv = np.repeat(np.arange(N, dtype=np.int64), counts)
    times = np.empty(Nrec)
    off = 0
    for n in counts:
        times[off:off + n] = np.sort(rng.uniform(0.0, T, size=n))
        off += n
    times = _q(times, 1.0 / 256)
    cov = np.column_stack([np.ones(Nrec)] + [_q(rng.standard_normal(Nrec), 1.0 / 1024) for _ in range(n_cov)])
    G = simulate_genotypes(rng, M, N, maf_lo, maf_hi, miss_rate, extra_edge_snps=edge_snps) if M > 0 else None
    s2e, s2g, s2b0, sb01, s2b1 = vc
    if G is not None and exact_genetic:
        Gf = np.where(G < 0, 0, G).astype(np.float64)
        f = np.clip(Gf.mean(axis=1) / 2.0, 1e-3, 1 - 1e-3)
        Zs = (Gf - 2 * f[:, None]) / np.sqrt(2 * f * (1 - f))[:, None]
        u = Zs.T @ rng.standard_normal(M) * np.sqrt(s2g / M)
    else:
        u = rng.standard_normal(N) * np.sqrt(s2g)
    Dm = np.array([[s2b0, sb01], [sb01, s2b1]])
    L = np.linalg.cholesky(Dm)
    b = rng.standard_normal((N, 2)) @ L.T
    beta = np.array([1.0, 0.5, -0.3][: n_cov + 1] + [0.1])
    X = np.column_stack([cov, times])
    y = X @ beta + u[indiv] + b[indiv, 0] + b[indiv, 1] * times + rng.standard_normal(Nrec) * np.sqrt(s2e)
    y = _q(y, 1.0 / 4096)
    out = dict(N=N, Nrec=Nrec, p=n_cov + 1, indiv=indiv, times=times, cov=cov, y=y, counts=counts)
    if G is not None:
        out["G"] = G
        out["packed"] = pack_genotypes(G)
    return out


def write_record_table(path, coh):
    """Header ``INDIV PHENO TIMES c0 c1 ...``; INDIV is 1-based."""
    n_cov = coh["cov"].shape[1]
    hdr = ["INDIV", "PHENO", "TIMES"] + ["COV%d" % j for j in range(n_cov)]
    cols = [coh["indiv"] + 1, coh["y"], coh["times"]] + [coh["cov"][:, j] for j in range(n_cov)]
    with open(path, "w") as f:
        f.write(" ".join(hdr) + "\n")
        rows = np.column_stack([c.astype(np.float64) for c in cols])
        for r in rows:
            f.write("%d %.10g %.10g " % (int(r[0]), r[1], r[2]) + " ".join("%.10g" % v for v in r[3:]) + "\n")


def write_plink(prefix, packed, N):
    M = packed.shape[0]
    with open(prefix + ".bed", "wb") as f:
        f.write(bytes([0x6C, 0x1B, 0x01]))
        f.write(np.ascontiguousarray(packed).tobytes())
    with open(prefix + ".bim", "w") as f:
        for s in range(M):
            f.write("1\tsnp%d\t0\t%d\tA\tG\n" % (s + 1, 1000 + s))
    with open(prefix + ".fam", "w") as f:
        for i in range(N):
            f.write("%d %d 0 0 0 -9\n" % (i + 1, i + 1))


def ref_allele_stats(packed, N, min_maf=0.01, max_miss=0.2):
    """Per-SNP counts, float32 maf and keep mask with the reference's float
    arithmetic (``PCGsolver.cpp:700-743``).  Vectorised numpy; the C oracle
    restates the same per SNP."""
    G = unpack_genotypes(packed, N)
    miss = (G < 0).sum(axis=1).astype(np.int64)
    alt = np.where(G < 0, 0, G).astype(np.int64).sum(axis=1)
    n_obs = N - miss
    with np.errstate(divide="ignore", invalid="ignore"):
        maf = np.where(n_obs > 0, alt.astype(np.float32) / (np.float32(2.0) * n_obs.astype(np.float32)),
                       np.float32(0.0)).astype(np.float32)
    miss_rate = (miss.astype(np.float32) / np.float32(N)).astype(np.float32)
    mm = np.float32(min_maf)
    keep = (maf >= mm) & (maf <= np.float32(1.0) - mm) & (miss_rate <= np.float32(max_miss))
    return alt, miss, maf, keep


def grm_from_packed(packed, N, min_maf=0.01, max_miss=0.2):
    """GRM with the on-the-fly convention of ``PCGsolver.cpp:826-842``:
    A = Zs' Zs / M_kept, zs = (g - 2f) / sqrt(2f(1-f)), missing g -> 0,
    f the float32 A1 frequency.  Returns the float32 packed lower triangle."""
    alt, miss, maf, keep = ref_allele_stats(packed, N, min_maf, max_miss)
    G = unpack_genotypes(packed[keep], N)
    f = maf[keep].astype(np.float64)
    g = np.where(G < 0, 0, G).astype(np.float64)
    den = 2 * f * (1 - f)
    inv = np.where(den > 1e-12, 1.0 / np.sqrt(np.where(den > 0, den, 1.0)), 1.0)
    Zs = (g - 2 * f[:, None]) * inv[:, None]
    A = (Zs.T @ Zs) / max(int(keep.sum()), 1)
    il = np.tril_indices(N)
    return A[il].astype(np.float32)


def write_grm_bin(prefix, A_lt):
    with open(prefix + ".grm.bin", "wb") as f:
        f.write(np.ascontiguousarray(A_lt, dtype=np.float32).tobytes())


def write_cohort(dirpath, name, coh, grm=False, min_maf=0.01, max_miss=0.2):
    """Write ``<name>.txt`` (+ PLINK trio, + ``.grm.bin`` if ``grm``).
    Returns the path prefix."""
    os.makedirs(dirpath, exist_ok=True)
    pre = os.path.join(dirpath, name)
    write_record_table(pre + ".txt", coh)
    if "packed" in coh:
        write_plink(pre, coh["packed"], coh["N"])
        if grm:
            write_grm_bin(pre, grm_from_packed(coh["packed"], coh["N"], min_maf, max_miss))
    return pre


def _splitmix64(state, n):
    """n successive splitmix64 outputs starting after ``state`` (uint64 array math)."""
    with np.errstate(over="ignore"):
        k = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(state) + k * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def normal_stream(seed, n):
    """Standard normal draws from a splitmix64 stream by Box-Muller; the same
    on every platform and numpy version (used for injected AIREML probes)."""
    m = (n + 1) // 2
    with np.errstate(over="ignore"):
        st = np.uint64(seed) * np.uint64(0x2545F4914F6CDD1D)
    u = _splitmix64(st, 2 * m)
    u = ((u >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)
    r = np.sqrt(-2.0 * np.log(u[0::2]))
    th = 2.0 * np.pi * u[1::2]
    out = np.empty(2 * m)
    out[0::2] = r * np.cos(th)
    out[1::2] = r * np.sin(th)
    return out[:n]


# ---- portable cohorts ---------------------------------------------------------
# Inputs that must come out bit-identical on every platform and numpy version (so a
# fixture can hold the reference's outputs and a checksum of its inputs instead of
# the inputs): every draw is a splitmix64 hash of (seed, stream, index) in uint64
# arithmetic, and every value is formed by IEEE additions, multiplications,
# divisions and square roots applied elementwise in a fixed order -- no library
# random streams, no transcendental functions, no reductions whose order a BLAS or
# SIMD loop may choose.

_GOLD = np.uint64(0x9E3779B97F4A7C15)


def _mix64(z):
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def hash_u64(seed, stream, idx):
    """splitmix64 output for (seed, stream) at each index of ``idx`` (uint64 array)."""
    with np.errstate(over="ignore"):
        key = _mix64(np.uint64(seed) * _GOLD + np.uint64(stream) * np.uint64(0xD1B54A32D192ED03))
        return _mix64(key + (np.asarray(idx, dtype=np.uint64) + np.uint64(1)) * _GOLD)


def hash_uniform(seed, stream, idx):
    """Uniform [0, 1) doubles with 53 random bits (exact conversions)."""
    return (hash_u64(seed, stream, idx) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def hash_normal(seed, stream, idx):
    """Approximately standard normal draws: the Irwin-Hall sum of 12 uniforms minus 6,
    each uniform 24 bits, summed exactly in int64 (mean 0, variance 1, |x| <= 6)."""
    s = np.zeros(np.shape(idx), dtype=np.int64)
    for j in range(12):
        s += (hash_u64(seed, 16 * stream + j, idx) >> np.uint64(40)).astype(np.int64)
    return (s - 12 * (1 << 23)).astype(np.float64) * (1.0 / (1 << 24))


def _poisson_plus1(u, lam):
    """Poisson(lam) + 1 by inverse CDF.  exp(-lam) is summed as an exact rational
    series and rounded once, so the CDF table is the same everywhere."""
    from fractions import Fraction
    x, term, e = Fraction(lam).limit_denominator(1 << 20), Fraction(1), Fraction(0)
    for k in range(1, 400):
        e += term
        term = term * (-x) / k
    p = float(e + term)
    cdf, k, out = p, 0, np.ones(u.shape, dtype=np.int64)
    while cdf < 1.0 - 1e-15 and k < 200:
        out += (u >= cdf)
        k += 1
        p = p * lam / k
        cdf += p
    return out


def portable_cohort(seed, N, M, recs, T, maf_lo=0.05, maf_hi=0.5, miss_rate=0.01, vc=VC_DEFAULT,
                    freq_levels=0):
    """The cohort of :func:`simulate_cohort` (same model, same distributions; the
    normal draws are Irwin-Hall) with hash draws, so the record table text and the
    PLINK bytes are identical wherever this runs.  ``recs``: ("uniform", lo, hi) or
    ("poisson", lam) (Poisson(lam)+1).  ``freq_levels`` > 0 draws each SNP's allele
    frequency from that many equally spaced values in [maf_lo, maf_hi] (the exact
    GRM of :func:`portable_grm` groups SNPs by it); the frequency is also returned
    as ``p_a1``."""
    ind = np.arange(N, dtype=np.uint64)
    if recs[0] == "uniform":
        lo, hi = int(recs[1]), int(recs[2])
        counts = lo + (hash_u64(seed, 1, ind) % np.uint64(hi - lo + 1)).astype(np.int64)
    elif recs[0] == "poisson":
        counts = _poisson_plus1(hash_uniform(seed, 1, ind), float(recs[1]))
    else:
        raise ValueError(recs)
    Nrec = int(counts.sum())
    indiv = np.repeat(np.arange(N, dtype=np.int64), counts)
    ridx = np.arange(Nrec, dtype=np.uint64)
    tq = int(round(T * 256))
    tint = (hash_u64(seed, 2, ridx) % np.uint64(tq + 1)).astype(np.int64)
    tint = tint[np.lexsort((tint, indiv))]            # sorted within each individual
    times = tint.astype(np.float64) / 256.0
    cov = np.column_stack([np.ones(Nrec)] + [np.round(hash_normal(seed, 3 + j, ridx) * 1024.0) / 1024.0
                                             for j in range(2)])
    # genotypes, SNP blocks of 512: g = [u1 < p] + [u2 < p], missing if u3 < miss_rate
    sidx = np.arange(M, dtype=np.uint64)
    if freq_levels > 0:
        lev = (hash_u64(seed, 5, sidx) % np.uint64(freq_levels)).astype(np.float64)
        p = maf_lo + (maf_hi - maf_lo) * (lev / max(freq_levels - 1, 1))
    else:
        p = maf_lo + (maf_hi - maf_lo) * hash_uniform(seed, 5, sidx)
    flip = (hash_u64(seed, 6, sidx) >> np.uint64(63)) == np.uint64(1)
    pa1 = np.where(flip, 1.0 - p, p)
    G = np.empty((M, N), dtype=np.int8)
    for s0 in range(0, M, 512):
        s1 = min(M, s0 + 512)
        e = (np.arange(s0, s1, dtype=np.uint64)[:, None] * np.uint64(N) + ind[None, :])
        pp = pa1[s0:s1, None]
        g = (hash_uniform(seed, 7, e) < pp).astype(np.int8) + (hash_uniform(seed, 8, e) < pp).astype(np.int8)
        if miss_rate > 0:
            g[hash_uniform(seed, 9, e) < miss_rate] = -1
        G[s0:s1] = g
    s2e, s2g, s2b0, sb01, s2b1 = vc
    # genetic values u = Zs' w sqrt(s2g / M), summed SNP by SNP
    w = hash_normal(seed, 10, sidx)
    gsum = np.zeros(N)
    sc = np.sqrt(s2g / M)
    for s in range(M):
        gs = np.where(G[s] < 0, 0, G[s]).astype(np.float64)
        f = min(max(float(int(gs.sum())) / (2.0 * N), 1e-3), 1.0 - 1e-3)   # an integer sum: exact
        gsum += (gs - 2.0 * f) * (w[s] / np.sqrt(2.0 * f * (1.0 - f)))
    u = gsum * sc
    # b_i ~ N(0, D) through the 2x2 Cholesky factor of D
    l00 = np.sqrt(s2b0)
    l10 = sb01 / l00
    l11 = np.sqrt(s2b1 - l10 * l10)
    z0, z1 = hash_normal(seed, 11, ind), hash_normal(seed, 12, ind)
    b0, b1 = l00 * z0, l10 * z0 + l11 * z1
    beta = (1.0, 0.5, -0.3, 0.1)
    y = beta[0] * cov[:, 0]
    y = y + beta[1] * cov[:, 1]
    y = y + beta[2] * cov[:, 2]
    y = y + beta[3] * times
    y = y + u[indiv]
    y = y + b0[indiv]
    y = y + b1[indiv] * times
    y = y + hash_normal(seed, 13, ridx) * np.sqrt(s2e)
    y = np.round(y * 4096.0) / 4096.0
    return dict(N=N, Nrec=Nrec, p=3, indiv=indiv, times=times, cov=cov, y=y, counts=counts, G=G,
                packed=pack_genotypes(G), p_a1=pa1)


def portable_grm(G, p_a1):
    """A = Zs' Zs / M with zs = (g - 2p)/sqrt(2p(1-p)), p the generating A1 frequency
    (missing g -> 0), as a float32 packed lower triangle.  SNPs are grouped by their
    frequency (a few discrete levels, ``portable_cohort(freq_levels=...)``); within a
    group A gets w (G'G - 2p (r 1' + 1 r') + 4 p^2 n) with G'G and r integer sums (a
    float64 product of small integers is exact in any order), and the groups are added
    in a fixed order -- so every platform writes the same bytes."""
    M, N = G.shape
    g = np.where(G < 0, 0, G).astype(np.float64)
    A = np.zeros((N, N))
    for pv in np.unique(p_a1):
        sel = p_a1 == pv
        Gg = g[sel]
        T = Gg.T @ Gg
        r = Gg.sum(axis=0)                  # integers: exact in any order
        n = float(sel.sum())
        wv = 1.0 / (2.0 * pv * (1.0 - pv))
        A += wv * ((T - 2.0 * pv * (r[:, None] + r[None, :])) + 4.0 * pv * pv * n)
    A = A / M
    return A[np.tril_indices(N)].astype(np.float32)


def file_sha256(path):
    import hashlib
    h = hashlib.sha256()
    with open(path, "rb") as f:
        for chunk in iter(lambda: f.read(1 << 20), b""):
            h.update(chunk)
    return h.hexdigest()
