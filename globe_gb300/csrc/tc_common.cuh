// tc_common.cuh -- what the tensor-core genotype kernels share: the tile and
// digit constants, the K permutation of the decoded operand, the e4m3 digit
// encoding, the exact recombination of split partials, and the host launch
// of k_tc_gemm (defined in k_tc_geno.cu).
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp8.h>

#include <algorithm>
#include <atomic>
#include <cmath>

#include "internal.cuh"

namespace globe {
namespace tc {

constexpr int BM = 128;           // rows per MMA tile (TMEM lanes)
constexpr int BK = 128;           // K elements per stage (one 128-byte swizzle panel of e4m3)
constexpr int PKB = BK / 4;       // packed bytes per row per stage
constexpr int DBITS = 5;          // digit base 32
constexpr int DHALF = 1 << (DBITS - 1);   // 16: digits in [-16, 16]
constexpr int NDIG = 9;           // digits per right-hand-side column by default (45 bits)
constexpr int MIN_DIG = 2;        // fewest digits a context may ask for (globe_set_digits)

// The tile-blocked genotype copies hold "tile codes", 2 bits per genotype like the PLINK
// codes they are made from (re-encoded once, by recode_tile), equal to the genotype:
//   00 = genotype 0 or missing, 01 = genotype 1, 10 = genotype 2 (11 is not produced).
// A field masked in place is then an e4m3 byte proportional to its genotype: at bit offset 0
// of a byte 0x00 / 0x01 / 0x02 = 0, 2^-9, 2^-8 (subnormals); at offset 2 0x00 / 0x04 / 0x08 =
// 0, 2^-7, 2^-6.  So the decode is four masks and one shift (decode_word in k_tc_geno.cu).
__host__ __device__ __forceinline__ uint32_t recode_tile(uint32_t w) {
    const uint32_t lo = w & 0x55555555u, hi = (w >> 1) & 0x55555555u;   // PLINK bit 0 / bit 1 of each code
    // PLINK 00 (g=2) -> 10, 10 (g=1) -> 01, 11 (g=0) and 01 (missing) -> 00
    return ((~hi & ~lo & 0x55555555u) << 1) | (hi & ~lo);
}
// the PLINK code each tile code stands for (missing and genotype 0 share tile code 00)
__host__ __device__ constexpr int tile_to_plink(int t) { return t == 1 ? 2 : (t == 2 ? 0 : 3); }

// (sh, sl) += (h, l) in double-float: Knuth's two-sum of the high parts, the rounding error and
// the low parts into sl (GB300's FP32 pipe is many times its FP64 pipe)
__device__ __forceinline__ void df_add(float& sh, float& sl, float h, float l) {
    const float s = __fadd_rn(sh, h);
    const float bp = __fsub_rn(s, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bp)), __fsub_rn(h, bp));
    sl = __fadd_rn(sl, __fadd_rn(err, l));
    sh = s;
}

// Byte b of row `row` in a tile-blocked copy with nch 32-byte chunks per row: block (row / 128,
// b / 32) of 128 rows x 32 bytes, the two 16-byte halves of a row swapped when bit 2 of the row
// (within its tile) is set.
__host__ __device__ __forceinline__ int64_t blk_offset(int64_t row, int64_t b, int nch) {
    const int64_t t = row >> 7;
    const int r = (int)(row & 127);
    const int w = (int)(b & 31);
    const int h = (w >> 4) ^ ((r >> 2) & 1);
    return (((t * nch + (b >> 5)) * 128 + r) * 32) + h * 16 + (w & 15);
}

__device__ __forceinline__ int kpos(int64_t i) {
    // K position of element i within groups of 16 in the dense product's operands (digit planes
    // of A and digits of Z): evens first, then odds
    const int q = (int)(i & 15);
    return (int)(i & ~15ll) + ((q & 1) ? 8 + (q >> 1) : (q >> 1));
}
// K position of genotype i of a 16-genotype word after decode_word (k_tc_geno.cu): word r holds
// the genotypes at field r of the word's four bytes, so position 4 (i % 4) + i / 4.  Its own
// inverse.  Even genotypes (fields 0 and 2) decode to 2^-9 g, odd ones to 2^-7 g, so the digit
// operand of the genotype products carries 4 d at even genotypes (geno_digit_mult): every
// product is then g d 2^-7.
__host__ __device__ __forceinline__ int kpos_g(int64_t i) {
    const int q = (int)(i & 15);
    return (int)(i & ~15ll) + 4 * (q & 3) + (q >> 2);
}
__host__ __device__ constexpr int geno_digit_mult(int64_t i) { return (i & 1) ? 1 : 4; }
constexpr float GENO_UNIT_INV = 128.0f;   // genotype-product partials are multiples of 2^-7

__device__ __forceinline__ uint32_t e4m3_int(int d) {   // d in [-16, 16], or 4x that: exact in e4m3
    return (uint32_t)__nv_cvt_float_to_fp8((float)d, __NV_SATFINITE, __NV_E4M3);
}

// Exact int64 -> FP64 conversion scaled by a power of two, from the bits: GB300's FP64 pipe,
// which also runs its int64 -> FP64 conversion instruction, is small, and the recombinations
// convert two or three integers per value.  It gives the bits of the FP64 route it replaces.
// (The digit kernels' FP64 -> int64 rounding stays on the conversion instruction: an integer
// form of it measured slower there.)

// v s for |v| < 2^53 and s a power of two: (double)v * s, built from the bits when the result
// is a normal double (both the conversion and the product are exact then), else computed so
__device__ __forceinline__ double ll_times_pow2(long long v, double s) {
    if (v == 0) return 0.0;
    const int es = (int)((__double_as_longlong(s) >> 52) & 0x7ff);
    const unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
    const int msb = 63 - __clzll((long long)a);
    const int ex = es + msb;   // biased exponent of v s
    if (es == 0 || msb > 52 || ex <= 0 || ex >= 2047) return (double)v * s;
    const unsigned long long mant = (a << (52 - msb)) & 0xfffffffffffffull;
    return __longlong_as_double((long long)((v < 0 ? 0x8000000000000000ull : 0ull) | ((unsigned long long)ex << 52) |
                                            mant));
}

// max(m, |v|) for m >= 0 by comparing bits (non-negative doubles order as integers; a NaN v
// wins, where fmax would drop it -- the column sums carry NaN either way)
__device__ __forceinline__ double absmax_bits(double m, double v) {
    const long long a = __double_as_longlong(m), b = __double_as_longlong(v) & 0x7fffffffffffffffll;
    return __longlong_as_double(a > b ? a : b);
}

// 2^e sum_j 32^-j P_j of one row of a genotype product, ND digits per column (rows c*ND + j
// of the partials).  Every FP32 partial is an exact multiple of 2^-7 (|P| < 2^17), so it is
// scaled to an integer, the split partials are summed in int64 and the digits combined in two
// exact int64 halves (hi = digits 0..ND_HI-1, lo = the rest); the only rounding is the final
// FP64 addition.
// With YU > 1, YU splits' ND loads issue together: k_combine2 reads 10 splits and waits on
// them; k_combine1 reads 2, holds more registers, and runs faster one split at a time.
template <int ND, int YU = 1>
__device__ __forceinline__ double recombine(const float* __restrict__ part, int nsplit, int nmma, int64_t ldp, int c,
                                           int64_t row, double s_hi, double s_lo) {
    constexpr int NH = (ND + 1) / 2;
    long long pj[ND];
    if constexpr (YU == 1) {
#pragma unroll
        for (int j = 0; j < ND; ++j)
            pj[j] = (long long)__float2int_rn(part[((int64_t)c * ND + j) * ldp + row] * GENO_UNIT_INV);
        for (int y = 1; y < nsplit; ++y) {
#pragma unroll
            for (int j = 0; j < ND; ++j)
                pj[j] += (long long)__float2int_rn(part[((int64_t)y * nmma + c * ND + j) * ldp + row] * GENO_UNIT_INV);
        }
    } else {
#pragma unroll
        for (int j = 0; j < ND; ++j) pj[j] = 0;
        for (int y0 = 0; y0 < nsplit; y0 += YU) {
            float v[YU][ND];
#pragma unroll
            for (int u = 0; u < YU; ++u)
                if (y0 + u < nsplit) {
#pragma unroll
                    for (int j = 0; j < ND; ++j) v[u][j] = part[((int64_t)(y0 + u) * nmma + c * ND + j) * ldp + row];
                }
#pragma unroll
            for (int u = 0; u < YU; ++u)
                if (y0 + u < nsplit) {
#pragma unroll
                    for (int j = 0; j < ND; ++j) pj[j] += (long long)__float2int_rn(v[u][j] * GENO_UNIT_INV);
                }
        }
    }
    long long hi = 0, lo = 0;
#pragma unroll
    for (int j = 0; j < NH; ++j) hi = hi * (1 << DBITS) + pj[j];
#pragma unroll
    for (int j = NH; j < ND; ++j) lo = lo * (1 << DBITS) + pj[j];
    return ll_times_pow2(hi, s_hi) + ll_times_pow2(lo, s_lo);
}

// scale factors of recombine<ND> for exponent e: 2^(e - 5 (ND_HI - 1)) and 2^(e - 5 (ND - 1))
template <int ND>
__device__ __forceinline__ void recombine_scales(int e, double& s_hi, double& s_lo) {
    s_hi = ldexp(1.0, e - DBITS * ((ND + 1) / 2 - 1));
    s_lo = ldexp(1.0, e - DBITS * (ND - 1));
}

// CTAs per column of k_col_maxsum for n rows: ~8 values per thread (its FP64 reduction runs
// on GB300's small FP64 pipe, so surplus CTAs cost more than they hide), at most 304
__host__ __forceinline__ int col_parts(int64_t n) {
    const int64_t p = (n + 2047) / 2048;
    return (int)(p < 1 ? 1 : (p > 304 ? 304 : p));
}

// per-column max |x| and sum over n rows (partials per CTA); colinfo[c] = {exponent e with
// max |x 2^-e| < 16, column sum} from those partials, or {0, NaN} for a column holding a
// NaN or an infinity (k_tc_geno.cu).  k_col_maxsum forms colinfo itself when given it and
// zeroed per-column counts cnt (tc_counters), in its last CTA per column; else k_col_finish.
__global__ void k_col_maxsum(const double* __restrict__ X, int64_t n, int64_t ld, double* __restrict__ pmax,
                             double* __restrict__ psum, unsigned* __restrict__ cnt, double* __restrict__ colinfo);
__global__ void k_col_finish(const double* __restrict__ pmax, const double* __restrict__ psum, int nparts, int k,
                             double* __restrict__ colinfo);

// ND digits of X (n x k, FP64) into D[(c*ND + j) * kpad + pos(r)]  (e4m3); every position
// in [0, kpad) of the column's digit rows is written (rows >= n give digit 0).  One thread
// fills 4 consecutive positions P..P+3 (a 32-bit word).  GENO: the operand of a genotype
// product -- pos = kpos_g (position P + q of a group of 16 holds row 4 q + P/4) and digits
// times geno_digit_mult(row); otherwise the dense product's kpos (position P < 8 holds row
// 2P, P >= 8 row 2(P-8)+1).
// x 2^-e is rounded once to the integer I = round(x 2^-e 32^(ND-1)), |I| <= 2^(5 ND - 1); its
// balanced base-32 digits are peeled off from the least significant end in integer
// arithmetic (d = ((I + 16) mod 32) - 16, in [-16, 15]); the leading digit is what
// remains, in [-16, 16].  sum_j d_j 32^-j equals x 2^-e rounded to 5 (ND-1) fraction bits.
template <int ND, bool GENO>
__global__ void k_digits(const double* __restrict__ X, int64_t n, int64_t ld, int k, const double* __restrict__ colinfo,
                         uint8_t* __restrict__ D, int64_t kpad) {
    const int c = blockIdx.y;
    const double sc = ldexp(1.0, DBITS * (ND - 1) - (int)colinfo[2 * c]);   // a power of two: x * sc is exact
    const bool bad = isnan(colinfo[2 * c + 1]);   // non-finite column (k_col_finish): zero digits
    const int64_t nw = kpad >> 2;
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += (int64_t)gridDim.x * blockDim.x) {
        const int64_t P = w << 2, base = P & ~(int64_t)15;
        const int pl = (int)(P & 15);
        const int mult = GENO ? geno_digit_mult(pl >> 2) : 1;   // GENO: rows 4 q + pl/4 share its parity
        long long I[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int pq = pl + q;
            const int64_t src = base + (GENO ? 4 * q + (pl >> 2) : (pq < 8 ? 2 * pq : 2 * (pq - 8) + 1));
            I[q] = (src < n && !bad) ? __double2ll_rn(X[src + c * ld] * sc) : 0ll;
        }
        uint32_t word[ND];
#pragma unroll
        for (int j = 0; j < ND; ++j) word[j] = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
#pragma unroll
            for (int j = ND - 1; j > 0; --j) {
                const int d = (int)((I[q] + DHALF) & (2 * DHALF - 1)) - DHALF;
                I[q] = (I[q] - d) >> DBITS;   // exact: I - d is a multiple of 32
                word[j] |= e4m3_int(mult * d) << (8 * q);
            }
            word[0] |= e4m3_int(mult * (int)I[q]) << (8 * q);
        }
#pragma unroll
        for (int j = 0; j < ND; ++j) *reinterpret_cast<uint32_t*>(D + ((int64_t)c * ND + j) * kpad + P) = word[j];
    }
}

}  // namespace tc

// Extra launch dimension of k_tc_gemm: gridDim.z = nz independent digit
// operands stacked in one tensor map (operand z = map rows z*NMMA ..), partials
// of operand z at part + z * pz.  A CTA whose rows all lie below
// skip0 + z * skipz does nothing (the lower-triangle GRM build uses this).
struct ZGrid {
    int nz = 1;
    int64_t pz = 0;
    int skip0 = 0, skipz = 0;
    int stall = 0;   // test hook (globe_debug_stall_next_gemm): leave the first digit stage unloaded
};

int make_map(globe_ctx* ctx, CUtensorMap* m, const void* base, uint64_t inner, uint64_t outer, uint32_t box_in,
             uint32_t box_out, bool sw128);
// Tile-blocked genotype copies hold a multiple of TILE_PAD row tiles of 128, so that CTAs of
// 1, 2, 3 or 4 tiles never run past them; gemm_dispatch checks it for each launch (ntiles:
// the row tiles of blk).
constexpr int TILE_PAD = 12;
int gemm_dispatch(globe_ctx* ctx, int nmma, const uint8_t* blk, int ntiles, const CUtensorMap& mB, int rows, int nchunks,
                  int splits, float* part, int64_t ldp, unsigned* err, const ZGrid& zg);
int rows_per_cta(int nmma);
int eff_splits(int nchunks, int splits);

}  // namespace globe
