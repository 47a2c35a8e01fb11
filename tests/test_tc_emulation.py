"""CPU emulation of the tensor-core genotype product's data layout
(globe_gb300/csrc/k_tc_geno.cu): the 2-bit -> e4m3 byte-permute decode, the
K permutation it induces, base-16 digit slicing of the right-hand sides, the
exact integer accumulation and the FP64 recombination -- checked against the
oracle's FP64 GRM product.  Runs without a GPU."""
import numpy as np

from helpers import cohort, rel

LUT_G = 0x00380040
E4M3 = {0x00: 0.0, 0x38: 1.0, 0x40: 2.0}
NDIG = 9      # balanced base-32 digits
DBITS = 5


def byte_perm(x, s):
    """__byte_perm(x, 0, s) for selector nibbles 0..3 (bytes of x)."""
    out = 0
    for i in range(4):
        sel = (s >> (4 * i)) & 0x7
        b = (x >> (8 * sel)) & 0xFF if sel < 4 else 0
        out |= b << (8 * i)
    return out


def decode_word(w):
    e = w & 0x33333333
    o = (w >> 2) & 0x33333333
    return [byte_perm(LUT_G, e & 0xFFFF), byte_perm(LUT_G, (e >> 16) & 0xFFFF),
            byte_perm(LUT_G, o & 0xFFFF), byte_perm(LUT_G, (o >> 16) & 0xFFFF)]


def kpos(i):
    q = i & 15
    return (i & ~15) + (8 + (q >> 1) if q & 1 else q >> 1)


def decode_row(packed_row):
    """Packed bytes of one row -> e4m3 values in the kernel's K order."""
    b = np.asarray(packed_row, np.uint8)
    pad = (-len(b)) % 4
    b = np.concatenate([b, np.zeros(pad, np.uint8)])
    words = b.view("<u4")
    out = []
    for w in words:
        for r in decode_word(int(w)):
            out += [E4M3[(r >> (8 * i)) & 0xFF] for i in range(4)]
    return np.array(out)


def digits(col):
    """Balanced base-32 digits as k_digits forms them: I = round(x 2^-e 32^(NDIG-1)),
    digits peeled from the least significant end, the leading one what remains."""
    mx = np.abs(col).max()
    e = (np.frexp(mx)[1] - (DBITS - 1)) if mx > 0 else -(DBITS - 1)
    I = np.rint(np.ldexp(col, DBITS * (NDIG - 1) - e)).astype(np.int64)
    assert np.all(np.abs(I) < 2 ** 44)
    D = np.zeros((NDIG, len(col)))
    for j in range(NDIG - 1, 0, -1):
        d = ((I + 16) & 31) - 16
        D[j] = d
        I = (I - d) >> DBITS
    assert np.all(np.abs(I) <= 16)
    D[0] = I
    return D, e


def test_decode_permutation_matches_kpos():
    rng = np.random.default_rng(0)
    G = rng.integers(-1, 3, size=(1, 64)).astype(np.int8)
    from globe_gb300 import synth
    row = synth.pack_genotypes(G)[0]
    dec = decode_row(row)
    g = np.where(G[0] < 0, 0, G[0]).astype(float)
    for i in range(64):
        assert dec[kpos(i)] == g[i]


def test_product_emulation_matches_oracle(orc):
    from globe_gb300 import synth
    coh = cohort(31, 77, 150, recs=("uniform", 1, 3), miss=0.05, edge=True)
    N = coh["N"]
    s = orc.Solver(coh["indiv"], coh["X"], coh["y"], N, (0.6, 0.4, 0.4, 0.2, 0.2), packed=coh["packed"])
    alt, miss, maf, _, keep = orc.bed_stats(coh["packed"], N)
    f, inv = s.f, s.inv_std
    kept = coh["packed"][keep]
    Mk = kept.shape[0]
    rng = np.random.default_rng(5)
    Z = rng.standard_normal((N, 3)) * np.array([1.0, 1e-3, 40.0])
    # pass 1: rows = SNPs, K = individuals in kpos order
    K1 = ((N + 127) // 128) * 128
    A1 = np.zeros((Mk, K1))
    for sidx in range(Mk):
        d = decode_row(kept[sidx])
        A1[sidx, :len(d)] = d[:K1]
    U = np.zeros((Mk, 3))
    for c in range(3):
        D, e = digits(Z[:, c])
        B = np.zeros((NDIG, K1))
        for i in range(N):
            B[:, kpos(i)] = D[:, i]
        P = A1 @ B.T                       # exact integers
        assert np.all(P == np.rint(P)) and np.abs(P).max() < 2 ** 24
        gv = np.ldexp(P @ (32.0 ** -np.arange(NDIG)), e)
        U[:, c] = inv ** 2 * (gv - 2 * f * Z[:, c].sum())
    # pass 2: rows = individuals, K = SNPs (individual-major codes)
    Gk = synth.unpack_genotypes(kept, N)              # Mk x N, -1 missing
    Gt = np.where(Gk < 0, 0, Gk).T                    # N x Mk
    out = np.zeros((N, 3))
    for c in range(3):
        D, e = digits(U[:, c])
        P2 = Gt @ D.T
        out[:, c] = np.ldexp(P2 @ (32.0 ** -np.arange(NDIG)), e) - 2 * (f * U[:, c]).sum()
    out *= 0.4 / Mk
    assert rel(out, s.grm_apply(Z)) < 1e-12
