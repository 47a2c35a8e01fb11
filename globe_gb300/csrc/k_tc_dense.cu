// k_tc_dense.cu -- dense GRM product on the 5th-generation tensor cores
// (GLOBE_PREC_MIXED).
//
//   out (N x k) = scale * A Z,  A(i,j) = lt[max(i,j)(max(i,j)+1)/2 + min(i,j)]
//   (PCGsolver.cpp:1202-1213, varCompEst.cpp:531-558)
//
// A is held a second time on the device as DA planes of balanced base-32 digits of
// one fixed-point grid: A(i,j) ~ 2^eA sum_d a_d(i,j) 32^-d, integer a_d in [-16,16]
// (exact in e4m3), eA fixed by max|A| (max|A| 2^-eA in [8,16)).  That is A rounded
// once to a step of 2^(eA - 5(DA-1)) <= 2^(-3 - 5(DA-1)) max|A|; with the default
// DA = 7 every entry within 2^-34 max|A|, i.e. within half a float32 ulp for every
// |A(i,j)| >= max|A| / 2^10.  DA = min(7, the context's digit count).
// The right-hand sides are split into ND digits per column exactly as in the
// genotype product.  Every MMA multiplies two digits (|a z| <= 256), so an FP32
// sum over up to 2^16 of them is an exact integer: the tensor-core accumulation
// carries no rounding; the DA x ND digit products are recombined in int64 / FP64.
//
// Layout: plane d, row i, K position P at adig[(d*NP + i) * NP + P] with
// NP = N rounded up to 128 and K permuted within groups of 16 like the digit
// tiles of the right-hand sides (kpos), rows padded to a multiple of 256.
// The planes are full squares (both triangles), 7 N^2 bytes at DA = 7.
//
// Kernel (one CTA = 2 x 128 rows x one K range, M=128 x N=NMMA MMAs per row tile):
//   warp 0     TMA of both operands per stage: two 128 x 128-byte tiles of the
//              digit planes (HBM) and the NMMA x 128-byte digit tile of Z (L2)
//   warps 1-2  one tcgen05.mma issue stream per row tile (kind::f8f6f4, E4M3 x
//              E4M3 -> F32, both operands from 128B-swizzled shared memory)
//   warp 3     TMEM allocation
//   warps 4-7  epilogue (tcgen05.ld of TMEM lane quadrant warp % 4 -> FP32 partials)
// Every mbarrier wait is bounded; on timeout the CTA records an error bit, waits
// (bounded) for its issued copies / MMAs and frees TMEM.
#include <cstring>
#include <vector>

#include "tc_ptx.cuh"

namespace globe {
namespace tc {

constexpr int DA_MAX = 7;        // digit planes of A at most
constexpr int DMT = 2;           // row tiles per CTA
constexpr int DROWS = DMT * BM;  // rows per CTA
constexpr int DK_MAX_CHUNKS = 512;   // K <= 2^16 per CTA: |sum| <= 256 * 2^16 = 2^24, exact in FP32

template <int NMMA>
struct DGeo {
    static constexpr int ABYTES = DMT * BM * BK;      // digit-plane bytes per stage (HBM)
    static constexpr int BBYTES = NMMA * BK;          // Z digit bytes per stage (L2)
    static constexpr int ST0 = (210 * 1024) / (ABYTES + BBYTES);
    static constexpr int STAGES = ST0 > 6 ? 6 : ST0;
    static_assert(STAGES >= 3, "stages");
};

template <int NMMA>
struct __align__(1024) DSmem {
    uint8_t a[DGeo<NMMA>::STAGES][DMT][BM * BK];   // 1024-aligned 16 KB tiles
    uint8_t b[DGeo<NMMA>::STAGES][NMMA * BK];      // NMMA * 128 B, a multiple of 2 KB
    uint64_t full[DGeo<NMMA>::STAGES], empty[DGeo<NMMA>::STAGES], accfull[DMT];
    uint32_t tmem_base;
    int abort;
};

template <int NMMA>
__global__ void __launch_bounds__(256, 1)
    k_tc_dense(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int rows,
               int nchunks, int cps, float* __restrict__ part, int64_t ldp, unsigned* __restrict__ err, int stall) {
    constexpr int ST = DGeo<NMMA>::STAGES;
    static_assert(NMMA % 16 == 0 && NMMA >= 16 && NMMA <= 256, "NMMA");
    constexpr uint32_t NCOLS = ncols_alloc(DMT * NMMA);
    extern __shared__ uint8_t smraw[];
    DSmem<NMMA>& S = *reinterpret_cast<DSmem<NMMA>*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row0 = blockIdx.x * DROWS, split = blockIdx.y;
    const int c0 = split * cps;
    const int nloc = min(nchunks, c0 + cps) - c0;

    if (threadIdx.x == 0) {
        for (int s = 0; s < ST; ++s) {
            mbar_init(&S.full[s], 1);
            mbar_init(&S.empty[s], DMT);
        }
        for (int m = 0; m < DMT; ++m) mbar_init(&S.accfull[m], 1);
        S.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 3) tmem_alloc(&S.tmem_base, NCOLS);
    tc_before();
    __syncthreads();
    tc_after();
    const uint32_t tmem = S.tmem_base;
    int* abort = &S.abort;

    if (warp == 0) {
        if (lane == 0 && nloc > 0) {
            int issued = 0;
            for (int it = 0; it < nloc; ++it) {
                const int s = it % ST, n = it / ST;
                if (n > 0 && !mbar_wait(&S.empty[s], (n - 1) & 1, abort, err, 1u)) break;
                if (stall && it == 0) {   // test hook: the stage is never loaded, so its waits run out
                    issued = 1;
                    continue;
                }
                mbar_expect_tx(&S.full[s], DGeo<NMMA>::ABYTES + DGeo<NMMA>::BBYTES);
                const int x = (c0 + it) * BK;
                tma_load_2d(S.a[s][0], &tmA, x, row0, &S.full[s]);
                tma_load_2d(S.a[s][1], &tmA, x, row0 + BM, &S.full[s]);
                tma_load_2d(S.b[s], &tmB, x, 0, &S.full[s]);
                issued = it + 1;
            }
            for (int it = issued - 1; it >= 0 && it >= issued - ST; --it) mbar_drain(&S.full[it % ST], (it / ST) & 1);
        }
    } else if (warp == 1 || warp == 2) {
        const int m = warp - 1;
        if (lane == 0 && nloc > 0) {
            const uint32_t idesc = (1u << 4) | ((uint32_t)(NMMA >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
            const uint32_t dcol = tmem + (uint32_t)(m * NMMA);
            for (int it = 0; it < nloc; ++it) {
                const int s = it % ST;
                if (!mbar_wait(&S.full[s], (it / ST) & 1, abort, err, 2u)) break;
                tc_after();
                const uint64_t ad = desc_sw128(saddr(S.a[s][m])), bd = desc_sw128(saddr(S.b[s]));
#pragma unroll
                for (int kk = 0; kk < BK / 32; ++kk)
                    mma_f8(dcol, ad + (uint64_t)(2 * kk), bd + (uint64_t)(2 * kk), idesc, (it | kk) != 0);
                mma_commit(&S.empty[s]);
            }
            mma_commit(&S.accfull[m]);   // tracks every MMA this thread issued
        }
    } else if (warp >= 4) {
        const int quad = warp & 3;   // a warp reaches TMEM lanes 32 (warp % 4) ..
        const uint32_t lane_addr = (uint32_t)(quad * 32) << 16;
#pragma unroll 1
        for (int m = 0; m < DMT; ++m) {
            bool go = nloc > 0 && mbar_wait(&S.accfull[m], 0, abort, err, 4u);
            go = __all_sync(0xffffffffu, go);   // tcgen05.ld is warp-collective
            if (!go) continue;
            tc_after();
            const int rr = row0 + m * BM + quad * 32 + lane;
#pragma unroll 1
            for (int cb = 0; cb < NMMA; cb += 16) {
                uint32_t acc[16];
                tmem_ld16(tmem + lane_addr + (uint32_t)(m * NMMA + cb), acc);
                if (rr < rows) {
#pragma unroll
                    for (int jj = 0; jj < 16; ++jj)
                        part[((int64_t)split * NMMA + cb + jj) * ldp + rr] = __uint_as_float(acc[jj]);
                }
            }
        }
    }
    // leave: MMAs that were issued must finish before TMEM is released
    if ((warp == 1 || warp == 2) && nloc > 0) mbar_drain(&S.accfull[warp - 1], 0);
    tc_before();
    __syncthreads();
    if (warp == 3) {
        tc_after();
        tmem_dealloc(tmem, NCOLS);
    }
}

// max |A| over the packed triangle as float bits (non-negative floats order like their bits),
// and whether any entry is not finite
__global__ void k_dense_absmax(const float* __restrict__ lt, int64_t n, unsigned* __restrict__ out) {
    unsigned mx = 0, bad = 0;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const float v = lt[e];
        if (!isfinite(v)) bad = 1;
        else mx = max(mx, __float_as_uint(fabsf(v)));
    }
    for (int o = 16; o > 0; o >>= 1) {
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        bad |= __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out, mx);
        if (bad) atomicOr(out + 1, 1u);
    }
}

// The DA digit planes of one 64 x 64 block (I0, J0) of the full square: the block is staged
// through shared memory (rows of the triangle left of the diagonal, columns of it right of
// the diagonal: coalesced either way), then each thread writes 4 words of 4 K positions per
// plane.  Position P of a group of 16 holds column 2P (P < 8) or 2(P-8)+1 (the inverse of
// kpos).  x 2^-eA is rounded once to I = round(x 2^-eA 32^(DA-1)); its balanced base-32
// digits are peeled off from the least significant end (d = ((I + 16) mod 32) - 16); the
// leading digit is what remains, in [-16, 16].
template <int DA>
__global__ void __launch_bounds__(256) k_dense_digits(const float* __restrict__ lt, int32_t N, int eA,
                                                      uint8_t* __restrict__ D, int64_t np) {
    constexpr int DT = 64;
    __shared__ float At[DT][DT + 1];
    const int tid = threadIdx.x;
    const int64_t I0 = (int64_t)blockIdx.y * DT, J0 = (int64_t)blockIdx.x * DT;
    if (J0 + DT <= I0) {
        const int jj = tid & (DT - 1);
        for (int m = tid >> 6; m < DT; m += 4) {
            const int64_t i = I0 + m, j = J0 + jj;
            At[m][jj] = (i < N) ? lt[i * (i + 1) / 2 + j] : 0.0f;
        }
    } else if (J0 >= I0 + DT) {
        const int ii = tid & (DT - 1);
        for (int m = tid >> 6; m < DT; m += 4) {
            const int64_t i = I0 + ii, j = J0 + m;
            At[ii][m] = (i < N && j < N) ? lt[j * (j + 1) / 2 + i] : 0.0f;
        }
    } else {
        const int jj = tid & (DT - 1);
        for (int m = tid >> 6; m < DT; m += 4) {
            const int64_t i = I0 + m, j = J0 + jj;
            float v = 0.0f;
            if (i < N && j < N) v = (i >= j) ? lt[i * (i + 1) / 2 + j] : lt[j * (j + 1) / 2 + i];
            At[m][jj] = v;
        }
    }
    __syncthreads();
    const double sc = ldexp(1.0, DBITS * (DA - 1) - eA);   // a power of two: x * sc is exact
#pragma unroll 1
    for (int w = tid; w < DT * (DT / 4); w += 256) {
        const int m = w >> 4, pl = (w & 15) * 4;   // row in the block, first K position in the block
        long long I[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int p = pl + q, base = p & ~15, pp = p & 15;
            const int jl = base + (pp < 8 ? 2 * pp : 2 * (pp - 8) + 1);
            I[q] = __double2ll_rn((double)At[m][jl] * sc);
        }
        uint32_t word[DA];
#pragma unroll
        for (int d = 0; d < DA; ++d) word[d] = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
#pragma unroll
            for (int d = DA - 1; d > 0; --d) {
                const int dg = (int)((I[q] + DHALF) & (2 * DHALF - 1)) - DHALF;
                I[q] = (I[q] - dg) >> DBITS;   // exact: I - dg is a multiple of 32
                word[d] |= e4m3_int(dg) << (8 * q);
            }
            word[0] |= e4m3_int((int)I[q]) << (8 * q);
        }
#pragma unroll
        for (int d = 0; d < DA; ++d)
            *reinterpret_cast<uint32_t*>(D + ((int64_t)d * np + I0 + m) * np + J0 + pl) = word[d];
    }
}

// out[i,c] = sA 2^e_c sum_{d,j} 32^-(d+j) P[plane d, digit j](i,c), sA = scale 2^eA.  Each
// split partial is an exact integer in FP32; they are summed in int64 by total weight
// s = d + j (T_s, |T_s| <= 7 * 256 N), and the weights folded in three exact int64 chunks of
// five (C_q = sum_{s=5q}^{5q+4} 32^(5q+4-s) T_s, |C_q| < 2^31 N): three conversions and two
// FP64 additions per value instead of a recombination per plane.
template <int ND>
__global__ void k_dense_combine(const float* __restrict__ part, int nsplit, int nmma, int64_t ldp, int32_t N,
                                int64_t np, int da, const double* __restrict__ colinfo, double sA,
                                double* __restrict__ out, int64_t ldo) {
    constexpr int NT = DA_MAX + ND - 1;
    static_assert(NT <= 15, "three chunks of five weights");
    const int c = blockIdx.y;
    const double s0 = sA * ldexp(1.0, (int)colinfo[2 * c] - 20);   // 2^(e_c - 5*4) for chunk 0
    const bool bad = isnan(colinfo[2 * c + 1]);   // a non-finite column (k_col_finish): NaN out
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        long long T[NT];
#pragma unroll
        for (int q = 0; q < NT; ++q) T[q] = 0;
        // per plane: the ND digit loads of split 0 issued together, further splits after
#pragma unroll
        for (int d = 0; d < DA_MAX; ++d) {
            if (d < da) {
                const float* src = part + (int64_t)c * ND * ldp + (int64_t)d * np + i;
                long long pj[ND];
#pragma unroll
                for (int j = 0; j < ND; ++j) pj[j] = (long long)__float2int_rn(src[(int64_t)j * ldp]);
                for (int y = 1; y < nsplit; ++y) {
#pragma unroll
                    for (int j = 0; j < ND; ++j)
                        pj[j] += (long long)__float2int_rn(src[((int64_t)y * nmma + j) * ldp]);
                }
#pragma unroll
                for (int j = 0; j < ND; ++j) T[d + j] += pj[j];
            }
        }
        long long C[3] = {0, 0, 0};
#pragma unroll
        for (int q = 0; q < 3; ++q)
#pragma unroll
            for (int m = 0; m < 5; ++m) C[q] = C[q] * 32 + (5 * q + m < NT ? T[5 * q + m] : 0);
        const double v = s0 * (ll_times_pow2(C[0], 1.0) + ll_times_pow2(C[1], 0x1p-25) + ll_times_pow2(C[2], 0x1p-50));
        out[i + c * ldo] = bad ? colinfo[2 * c + 1] : v;
    }
}

}  // namespace tc

// ---- host side ---------------------------------------------------------------

using namespace tc;

int dense_digit_planes(globe_ctx* ctx) {
    auto& g = ctx->gen;
    const int da = std::min(DA_MAX, ctx->digits);
    if (g.adig_state != 0 && g.adig_da == da) return GLOBE_OK;
    dfree(ctx, g.adig);
    g.adig = nullptr;
    g.adig_state = -1;   // until the planes are complete
    const int32_t N = ctx->coh.N;
    const int64_t np = ((int64_t)N + BM - 1) / BM * BM;
    const int64_t rows = ((int64_t)da * np + DROWS - 1) / DROWS * DROWS;
    const size_t bytes = (size_t)rows * (size_t)np;
    // the planes must fit beside what is resident; otherwise the double-float kernel stays in use
    size_t fr = 0, tot = 0;
    GLOBE_CK(ctx, cudaMemGetInfo(&fr, &tot));
    if (bytes + ((size_t)2 << 30) > fr || rows > INT32_MAX) {
        g.adig_da = da;
        return GLOBE_OK;
    }
    unsigned* mx;   // words 1-2 of the error-flag slot (word 0 is the kernels' flag): max |A| bits, non-finite
    GLOBE_RET(tc_err_word(ctx, &mx));
    GLOBE_CK(ctx, cudaMemsetAsync(mx + 1, 0, 2 * sizeof(unsigned), ctx->stream));
    const int64_t nelt = (int64_t)N * (N + 1) / 2;
    k_dense_absmax<<<(unsigned)std::min<int64_t>(div_up(nelt, 256), 152 * 8), 256, 0, ctx->stream>>>(g.grm, nelt,
                                                                                                    mx + 1);
    GLOBE_LAUNCHED(ctx, "k_dense_absmax");
    unsigned h[2] = {0, 0};
    GLOBE_CK(ctx, cudaMemcpyAsync(h, mx + 1, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    GLOBE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    g.adig_da = da;
    if (h[1]) return GLOBE_OK;   // a non-finite entry: the double-float kernel propagates it
    float amax;
    std::memcpy(&amax, &h[0], sizeof(float));
    int E = 0;
    if (amax > 0.0f) std::frexp((double)amax, &E);
    g.adig_e = E - (DBITS - 1);   // max|A| 2^-eA in [8, 16)
    GLOBE_RET(dalloc(ctx, &g.adig, bytes));
    if (rows > da * np)
        GLOBE_CK(ctx, cudaMemsetAsync(g.adig + (size_t)da * np * np, 0, (size_t)(rows - da * np) * np, ctx->stream));
    const dim3 grid((unsigned)(np / 64), (unsigned)(np / 64));
    switch (da) {
        case 2: k_dense_digits<2><<<grid, 256, 0, ctx->stream>>>(g.grm, N, g.adig_e, g.adig, np); break;
        case 3: k_dense_digits<3><<<grid, 256, 0, ctx->stream>>>(g.grm, N, g.adig_e, g.adig, np); break;
        case 4: k_dense_digits<4><<<grid, 256, 0, ctx->stream>>>(g.grm, N, g.adig_e, g.adig, np); break;
        case 5: k_dense_digits<5><<<grid, 256, 0, ctx->stream>>>(g.grm, N, g.adig_e, g.adig, np); break;
        case 6: k_dense_digits<6><<<grid, 256, 0, ctx->stream>>>(g.grm, N, g.adig_e, g.adig, np); break;
        default: k_dense_digits<7><<<grid, 256, 0, ctx->stream>>>(g.grm, N, g.adig_e, g.adig, np); break;
    }
    GLOBE_LAUNCHED(ctx, "k_dense_digits");
    GLOBE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    g.adig_np = np;
    g.adig_rows = rows;
    g.adig_state = 1;
    return GLOBE_OK;
}

template <int NMMA>
static int launch_dense(globe_ctx* ctx, const CUtensorMap& mA, const CUtensorMap& mB, int rows, int nchunks,
                        int cps, float* part, int64_t ldp, unsigned* err, int stall) {
    const size_t smem = sizeof(DSmem<NMMA>) + 1024;
    static std::atomic<uint64_t> attr_set{0};   // the shared-memory opt-in is per device
    const uint64_t bit = 1ull << (ctx->device & 63);
    if (!(attr_set.load() & bit)) {
        GLOBE_CK(ctx, cudaFuncSetAttribute(k_tc_dense<NMMA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set.fetch_or(bit);
    }
    const int splits = (nchunks + cps - 1) / cps;
    const dim3 grid((unsigned)(rows / DROWS), (unsigned)splits);
    k_tc_dense<NMMA><<<grid, 256, smem, ctx->stream>>>(mA, mB, rows, nchunks, cps, part, ldp, err, stall);
    GLOBE_LAUNCHED(ctx, "k_tc_dense");
    return GLOBE_OK;
}

static int dense_dispatch(globe_ctx* ctx, int nmma, const CUtensorMap& mA, const CUtensorMap& mB, int rows,
                          int nchunks, int cps, float* part, int64_t ldp, unsigned* err, int stall) {
    switch (nmma) {
#define GLOBE_DENSE_CASE(n) \
    case n: return launch_dense<n>(ctx, mA, mB, rows, nchunks, cps, part, ldp, err, stall);
        GLOBE_DENSE_CASE(16) GLOBE_DENSE_CASE(32) GLOBE_DENSE_CASE(48) GLOBE_DENSE_CASE(64)
        GLOBE_DENSE_CASE(80) GLOBE_DENSE_CASE(96) GLOBE_DENSE_CASE(112) GLOBE_DENSE_CASE(128)
        GLOBE_DENSE_CASE(144) GLOBE_DENSE_CASE(160) GLOBE_DENSE_CASE(176) GLOBE_DENSE_CASE(192)
        GLOBE_DENSE_CASE(208) GLOBE_DENSE_CASE(224) GLOBE_DENSE_CASE(240) GLOBE_DENSE_CASE(256)
#undef GLOBE_DENSE_CASE
    }
    return set_err(ctx, GLOBE_ERR_ARG, "unsupported MMA width %d", nmma);
}

// K stages per CTA.  One CTA runs per SM; the product takes about ceil(CTAs / SMs) waves of
// (stages per CTA + a fixed cost: setup, pipeline fill, and the epilogue's partials, written
// here and read again by the combine: 8 NMMA bytes per row, in units of a 128-byte stage).
// Fewest waves-weighted stages win, within K <= 2^16 per CTA (exact FP32 sums).
static int dense_cps(globe_ctx* ctx, int tiles, int nchunks, int nmma) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess || sms < 1) sms = 152;
    const double fixed = 4.0 + 8.0 * nmma / BK;
    const int lo = std::max(1, (nchunks + DK_MAX_CHUNKS - 1) / DK_MAX_CHUNKS);
    const int hi = std::max(lo, std::min(64, nchunks / 8));
    int best = (nchunks + lo - 1) / lo;
    double best_cost = 1e300;
    for (int s = lo; s <= hi; ++s) {
        const int cps = (nchunks + s - 1) / s;
        const int se = (nchunks + cps - 1) / cps;
        const double cost = std::ceil((double)tiles * se / sms) * (cps + fixed);
        if (cost < best_cost * 0.999) {
            best_cost = cost;
            best = cps;
        }
    }
    return best;
}

// out (N x kg) = scale * A Z for one group of <= 256 / ND columns
template <int ND>
static int dense_group(globe_ctx* ctx, const double* Z, int kg, double scale, double* out) {
    auto& g = ctx->gen;
    const int32_t N = ctx->coh.N;
    const int64_t np = g.adig_np;
    const int nch = (int)(np / BK);
    const int nmma = ((kg * ND + 15) / 16) * 16;
    const int rows = (int)g.adig_rows, tiles = rows / DROWS;
    const int cps = dense_cps(ctx, tiles, nch, nmma);
    const int splits = (nch + cps - 1) / cps;
    const int64_t ldp = rows;
    uint8_t* D;
    float* P;
    double* cst;
    unsigned* err;
    const int nbr = 304;
    GLOBE_RET(ws(ctx, WS_TC_D1, (size_t)nmma * np, &D));
    GLOBE_RET(ws(ctx, WS_TC_P1, (size_t)splits * nmma * ldp, &P));
    GLOBE_RET(ws(ctx, WS_TC_SCAL, (size_t)(2 * kg + 2 * nbr * kg + 8), &cst));
    GLOBE_RET(tc_err_word(ctx, &err));
    double* col = cst;
    double* pm = cst + 2 * kg;
    double* ps = pm + (size_t)nbr * kg;
    CUtensorMap mA, mB;
    GLOBE_RET(make_map(ctx, &mA, g.adig, (uint64_t)np, (uint64_t)rows, BK, BM, true));
    GLOBE_RET(make_map(ctx, &mB, D, (uint64_t)np, (uint64_t)nmma, BK, (uint32_t)nmma, true));
    const int nz = col_parts(N);
    unsigned* cnt;
    GLOBE_RET(tc_counters(ctx, kg, &cnt));
    k_col_maxsum<<<dim3(nz, kg), 256, 0, ctx->stream>>>(Z, N, N, pm, ps, cnt, col);
    GLOBE_LAUNCHED(ctx, "k_col_maxsum");
    if (nmma > kg * ND)   // digit rows past the kg columns stay zero
        GLOBE_CK(ctx, cudaMemsetAsync(D + (size_t)kg * ND * np, 0, (size_t)(nmma - kg * ND) * np, ctx->stream));
    k_digits<ND, false><<<dim3((unsigned)std::min<int64_t>(div_up(np / 4, 256), 1024), kg), 256, 0, ctx->stream>>>(
        Z, N, N, kg, col, D, np);
    GLOBE_LAUNCHED(ctx, "k_digits");
    {
        ProfScope p(ctx, GLOBE_PROF_GRM_PASS1);
        const int stall = ctx->stall_next_gemm;   // test hook (globe_debug_stall_next_gemm)
        ctx->stall_next_gemm = 0;
        GLOBE_RET(dense_dispatch(ctx, nmma, mA, mB, rows, nch, cps, P, ldp, err, stall));
    }
    k_dense_combine<ND><<<dim3(std::min(div_up(N, 256), 1024), kg), 256, 0, ctx->stream>>>(
        P, splits, nmma, ldp, N, np, g.adig_da, col, std::ldexp(scale, g.adig_e), out, N);
    GLOBE_LAUNCHED(ctx, "k_dense_combine");
    return GLOBE_OK;
}

static int dense_group_nd(globe_ctx* ctx, int nd, const double* Z, int kg, double scale, double* out) {
    switch (nd) {
        case 2: return dense_group<2>(ctx, Z, kg, scale, out);
        case 3: return dense_group<3>(ctx, Z, kg, scale, out);
        case 4: return dense_group<4>(ctx, Z, kg, scale, out);
        case 5: return dense_group<5>(ctx, Z, kg, scale, out);
        case 6: return dense_group<6>(ctx, Z, kg, scale, out);
        case 7: return dense_group<7>(ctx, Z, kg, scale, out);
        case 8: return dense_group<8>(ctx, Z, kg, scale, out);
        case 9: return dense_group<9>(ctx, Z, kg, scale, out);
    }
    return set_err(ctx, GLOBE_ERR_ARG, "unsupported digit count %d", nd);
}

int dense_apply_tc(globe_ctx* ctx, const double* Z, int k, double scale, double* out) {
    GLOBE_RET(dense_digit_planes(ctx));
    if (ctx->gen.adig_state != 1) return dense_apply_df(ctx, Z, k, scale, out);
    const int nd = ctx->digits;
    const int gmax = 256 / nd;   // MMA width <= 256; near-equal groups
    const int ng = (k + gmax - 1) / gmax;
    for (int gi = 0, c0 = 0; gi < ng; ++gi) {
        const int kg = k / ng + (gi < k % ng ? 1 : 0);
        GLOBE_RET(dense_group_nd(ctx, nd, Z + (size_t)c0 * ctx->coh.N, kg, scale, out + (size_t)c0 * ctx->coh.N));
        c0 += kg;
    }
    return GLOBE_OK;
}

}  // namespace globe
