"""CPU emulation of the tensor-core genotype product's data layout
(globe_gb300/csrc/k_tc_geno.cu): the PLINK -> tile-code recoding, the 2-bit ->
e4m3 decode by masks (subnormal bytes 2^-9 g and 2^-7 g), the K permutation it
induces and the 4x digits at even genotypes that equalise the products, base-32
digit slicing of the right-hand sides, the exact accumulation (multiples of 2^-7)
and the FP64 recombination -- checked against the oracle's FP64 GRM product.
Runs without a GPU."""
import numpy as np

from helpers import cohort, rel

# e4m3 bytes the decode produces: subnormals m 2^-9 (m = 1, 2, 4) and the smallest normal
E4M3 = {0x00: 0.0, 0x01: 2.0 ** -9, 0x02: 2.0 ** -8, 0x04: 2.0 ** -7, 0x08: 2.0 ** -6}
NDIG = 9      # balanced base-32 digits
DBITS = 5


def e4m3_value(byte):
    """OCP e4m3 (no infinities): sign, 4 exponent bits (bias 7), 3 mantissa bits."""
    sgn = -1.0 if byte & 0x80 else 1.0
    e, m = (byte >> 3) & 15, byte & 7
    return sgn * (m * 2.0 ** -9 if e == 0 else (1 + m / 8) * 2.0 ** (e - 7))


def recode_tile(w):
    """PLINK codes -> tile codes (00 = genotype 0 or missing, 01 = 1, 10 = 2)."""
    lo, hi = w & 0x55555555, (w >> 1) & 0x55555555
    return (((~hi & ~lo & 0x55555555) << 1) | (hi & ~lo)) & 0xFFFFFFFF


def decode_word(w):
    h = w >> 4
    return [w & 0x03030303, w & 0x0C0C0C0C, h & 0x03030303, h & 0x0C0C0C0C]


def kpos_g(i):
    q = i & 15
    return (i & ~15) + 4 * (q & 3) + (q >> 2)


def unit(i):
    """Value of genotype 1 at genotype position i after the decode."""
    return 2.0 ** -9 if i % 2 == 0 else 2.0 ** -7


def mult(i):
    """Digit multiplier at genotype position i: every product becomes g d 2^-7."""
    return 4.0 if i % 2 == 0 else 1.0


def decode_row(packed_row):
    """Packed bytes of one row -> e4m3 values in the kernel's K order."""
    b = np.asarray(packed_row, np.uint8)
    pad = (-len(b)) % 4
    b = np.concatenate([b, np.zeros(pad, np.uint8)])
    words = b.view("<u4")
    out = []
    for w in words:
        for r in decode_word(recode_tile(int(w))):
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
        assert dec[kpos_g(i)] == g[i] * unit(i)
    assert sorted(kpos_g(i) for i in range(64)) == list(range(64))
    assert all(kpos_g(kpos_g(i)) == i for i in range(64))     # its own inverse


def test_decoded_bytes_are_e4m3_multiples():
    """The masked fields are e4m3 bytes whose values are 0, 1, 2 times one unit."""
    for off, u in ((0, 2.0 ** -9), (2, 2.0 ** -7)):
        for code in (0, 1, 2):
            assert e4m3_value(code << off) == code * u
    for d in range(-16, 17):     # digits and 4x digits are exact in e4m3 (3 mantissa bits, max 448)
        for m in (1, 4):
            v = m * d
            e = np.frexp(abs(v))[1] if v else 0
            assert v == 0 or (abs(v) <= 448 and float(np.ldexp(np.rint(np.ldexp(v, 4 - e)), e - 4)) == v)


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
    # pass 1: rows = SNPs, K = individuals in kpos_g order
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
            B[:, kpos_g(i)] = D[:, i] * mult(i)
        P = (A1 @ B.T) * 128.0               # exact integers (multiples of 2^-7 before scaling)
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


def test_tile_code_decode_all_words():
    """Every PLINK code in every position of a word decodes to its genotype (missing -> 0)."""
    g_of = {0: 2.0, 1: 0.0, 2: 1.0, 3: 0.0}
    rng = np.random.default_rng(0)
    for w in [0, 0xFFFFFFFF, 0x55555555, 0xAAAAAAAA] + [int(x) for x in rng.integers(0, 2 ** 32, 2000)]:
        out = decode_word(recode_tile(w))
        vals = [E4M3[(r >> (8 * i)) & 0xFF] for r in out for i in range(4)]
        # output order: r0 = genotypes 0,4,8,12; r1 = 1,5,9,13; r2 = 2,6,10,14; r3 = 3,7,11,15
        order = [0, 4, 8, 12, 1, 5, 9, 13, 2, 6, 10, 14, 3, 7, 11, 15]
        want = [g_of[(w >> (2 * q)) & 3] * unit(q) for q in order]
        assert vals == want
        assert [kpos_g(q) for q in order] == list(range(16))


def test_digit_count_error_bound(orc):
    """The product with nd digits per column (CPU emulation) is within a few times the
    rounding unit 2^-(5(nd-1)+4) of the exact product, column by column."""
    from globe_gb300 import synth
    from helpers import tc_product_emulation
    coh = cohort(31, 77, 150, recs=("uniform", 1, 3), miss=0.05, edge=True)
    N = coh["N"]
    s = orc.Solver(coh["indiv"], coh["X"], coh["y"], N, (0.6, 0.4, 0.4, 0.2, 0.2), packed=coh["packed"])
    alt, miss, maf, _, keep = orc.bed_stats(coh["packed"], N)
    Gk = synth.unpack_genotypes(coh["packed"][keep], N)
    Gk = np.where(Gk < 0, 0, Gk)
    Z = np.random.default_rng(5).standard_normal((N, 3)) * np.array([1.0, 1e-3, 40.0])
    ref = s.grm_apply(Z)
    for nd in range(2, 10):
        out = tc_product_emulation(Gk, s.f, s.inv_std, Z, 0.4 / keep.sum(), nd)
        assert max(rel(out[:, c], ref[:, c]) for c in range(3)) < 8 * 2.0 ** -(5 * (nd - 1) + 4), nd


def _dense_plane_digits(A, da):
    """k_dense_digits on the CPU: the da balanced base-32 digit planes of A (plane 0 most
    significant) and the exponent e, max|A| 2^-e in [8, 16)."""
    mx = np.abs(A).max()
    e = (np.frexp(mx)[1] - 4) if mx > 0 else -4
    I = np.rint(np.ldexp(A, 5 * (da - 1) - e)).astype(np.int64)
    P = np.zeros((da,) + A.shape, np.int64)
    for d in range(da - 1, 0, -1):
        dg = ((I + 16) & 31) - 16
        P[d] = dg
        I = (I - dg) >> 5
    P[0] = I
    return P, e


def test_dense_digit_planes_and_bound(orc):
    """The dense tensor-core product (globe_gb300/csrc/k_tc_dense.cu) on the CPU: A's digit
    planes are integers in [-16, 16], they rebuild A to within 2^-34 max|A| (7 planes), every
    plane-by-digit partial sum is an exact FP32 integer (|sum| <= 256 K), and the
    recombination sum_d 32^-d R_d matches the FP64 oracle product to ~1e-10."""
    from globe_gb300 import synth
    from helpers import lt_to_full, tc_digits
    N = 333
    c = cohort(3, N, 500, recs=("uniform", 1, 2), miss=0.02)
    lt = synth.grm_from_packed(c["packed"], N)
    A = lt_to_full(lt, N)
    P, e = _dense_plane_digits(A, 7)
    assert np.abs(P).max() <= 16
    Ar = np.ldexp(np.tensordot(32.0 ** -np.arange(7), P.astype(np.float64), 1), e)
    assert np.abs(Ar - A).max() <= 2.0 ** -34 * np.abs(A).max()
    z = np.random.default_rng(1).standard_normal(N)
    D, ez = tc_digits(z, NDIG)
    R = np.einsum("dij,kj->dik", P.astype(np.float64), D)      # plane x row x z digit
    assert np.abs(R).max() <= 256 * N and np.array_equal(R, np.rint(R))
    assert np.array_equal(R.astype(np.float32).astype(np.float64), R)
    y = np.ldexp(np.einsum("dik,d,k->i", R, 32.0 ** -np.arange(7), 32.0 ** -np.arange(NDIG)), e + ez)
    indiv = c["indiv"].astype(np.int32)
    s = orc.Solver(indiv, c["X"], c["y"], N, (0.6, 1.0, 0.4, 0.2, 0.2), grm_lt=lt)
    assert rel(y, s.grm_apply(z[:, None])[:, 0]) < 1e-9


def _fold_chunks(P, da, nd):
    """k_dense_combine's recombination of the plane-by-digit sums P[d, j] (exact integers):
    sums T_s by total weight s = d + j, three int64 chunks of five weights, then FP64."""
    NT = 7 + nd - 1
    T = [0] * NT
    for d in range(da):
        for j in range(nd):
            T[d + j] += int(P[d, j])
    C = [0, 0, 0]
    for q in range(3):
        for m in range(5):
            C[q] = C[q] * 32 + (T[5 * q + m] if 5 * q + m < NT else 0)
    assert all(abs(c) < 2 ** 63 for c in C)       # the int64 chunks cannot overflow
    return 2.0 ** -20 * (float(C[0]) + np.ldexp(float(C[1]), -25) + np.ldexp(float(C[2]), -50))


def test_dense_combine_chunks_are_exact():
    """The three-chunk int64 fold of k_dense_combine equals sum_{d,j} 32^-(d+j) P[d, j]
    evaluated in exact integer arithmetic, to FP64 rounding, at every digit count and with
    partial sums at their bound (|P| <= 256 K, K = 2^20 individuals)."""
    from fractions import Fraction
    rng = np.random.default_rng(5)
    K = 1 << 20
    for nd in range(2, NDIG + 1):
        for da in range(2, min(7, nd) + 1):
            for trial in range(3):
                P = rng.integers(-256 * K, 256 * K + 1, size=(da, nd), dtype=np.int64)
                if trial == 0:
                    P[:] = 256 * K                          # every partial at its bound
                exact = sum(Fraction(int(P[d, j]), 32 ** (d + j)) for d in range(da) for j in range(nd))
                got = _fold_chunks(P, da, nd)
                assert abs(got - float(exact)) <= 4 * np.spacing(abs(float(exact))), (nd, da, trial)
