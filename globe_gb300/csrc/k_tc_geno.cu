// k_tc_geno.cu -- genotype GRM product on the 5th-generation tensor cores.
//
//   out (N x k) = scale * Zs' (Zs Z),  zs(s,i) = (g - 2 f_s) inv_s      (PCGsolver.cpp:1130-1201)
//
// Written as two integer-genotype products plus FP64 rank-1 terms:
//   pass 1:  P1[s,c] = sum_i g(s,i) Z[i,c]        (rows = SNPs, K = individuals)
//            u[s,c]  = inv_s^2 (P1[s,c] - 2 f_s sum_i Z[i,c])
//   pass 2:  P2[i,c] = sum_s g(s,i) u[s,c]        (rows = individuals, K = SNPs)
//            out[i,c] = scale (P2[i,c] - sum_s 2 f_s u[s,c])
// g in {0,1,2} is exact in FP8 e4m3.  Each right-hand-side column is split
// into base-16 digits: x = 2^e sum_j d_j 16^-j with integer d_j in [-8,8],
// also exact in e4m3.  |g d| <= 16, so an FP32 sum of up to 2^20 such
// products is an exact integer: the tensor-core accumulation carries no
// rounding, and the digits are recombined in FP64.  With 12 digits the
// product matches an FP64 evaluation to ~1e-14 relative.
//
// Kernel (one CTA = 128 rows x one K range, M=128 x N=NMMA MMAs):
//   warp 0    TMA producer: packed 2-bit tile [128 rows x 32 B] and the digit
//             tile [NMMA rows x 128 B, 128B-swizzled] per stage (4 stages)
//   warp 1    TMEM allocation and the single-thread tcgen05.mma issue
//             (kind::f8f6f4, E4M3 x E4M3 -> F32, 4 MMAs of K=32 per stage)
//   warps 2-9 decode 2-bit codes to e4m3 bytes in shared memory (128B-swizzled
//             K-major layout), then the epilogue (tcgen05.ld -> FP32 partials)
// The decode of 16 genotypes (one 32-bit word) is 3 logic ops, 2 shifts and
// 4 byte permutes; it permutes K within each group of 16, which the digit
// tiles repeat (kpos()).
// Every mbarrier wait is bounded (globaltimer); on timeout the CTA records
// an error bit, waits (bounded) for its issued copies / MMAs and frees TMEM.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "internal.cuh"

namespace globe {
namespace tc {

constexpr int BM = 128;           // tile rows (TMEM lanes)
constexpr int BK = 128;           // K elements per stage (one 128-byte swizzle panel of e4m3)
constexpr int PKB = BK / 4;       // packed bytes per row per stage
constexpr int STAGES = 4;
constexpr int DSTAGES = 2;
constexpr int DEC_WARPS = 8;
constexpr int NTHREADS = (2 + DEC_WARPS) * 32;
constexpr int NDIG = 12;          // digits per right-hand-side column
constexpr int MAX_RHS_GROUP = 21; // 21 * 12 = 252 <= 256 MMA columns
constexpr uint64_t WAIT_LIMIT_NS = 2000000000ull;  // 2 s per wait
constexpr uint32_t LUT_G = 0x00380040u;  // code 00 -> 2.0 (0x40), 01 -> 0, 10 -> 1.0 (0x38), 11 -> 0

__host__ __device__ constexpr int ncols_alloc(int n) { return n <= 32 ? 32 : n <= 64 ? 64 : n <= 128 ? 128 : 256; }

template <int NMMA>
struct __align__(1024) Smem {
    uint8_t adec[DSTAGES][BM * BK];      // decoded A, SW128 K-major (16 KB each)
    uint8_t bt[STAGES][NMMA * BK];       // digit tiles (TMA, SW128)
    uint8_t pk[STAGES][BM * PKB];        // packed tiles (TMA, no swizzle)
    uint64_t full[STAGES], empty[STAGES], adfull[DSTAGES], adempty[DSTAGES], accfull;
    uint32_t tmem_base;
    int abort;
};

// ---- PTX wrappers ---------------------------------------------------------

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint64_t gtime() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t n) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(n) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(b)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(saddr(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait; false on timeout or when another role aborted
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, int* abort, unsigned* err, unsigned bit) {
    if (mbar_try(b, parity)) return true;
    const uint64_t t0 = gtime();
    while (true) {
        if (mbar_try(b, parity)) return true;
        if (*(volatile int*)abort) return false;
        if (gtime() - t0 > WAIT_LIMIT_NS) {
            *(volatile int*)abort = 1;
            atomicOr(err, bit);
            return false;
        }
    }
}
// bounded wait used on the way out (ignores the abort flag)
__device__ __forceinline__ void mbar_drain(uint64_t* b, uint32_t parity) {
    const uint64_t t0 = gtime();
    while (!mbar_try(b, parity) && gtime() - t0 < WAIT_LIMIT_NS) {
    }
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            saddr(dst)),
        "l"((uint64_t)tm), "r"(x), "r"(y), "r"(saddr(bar))
        : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void mma_f8(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
                 : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
// K-major operand, 128-byte swizzle: 8-row atoms of 1024 B (SBO), start advanced by 32 B per K=32 step
__device__ __forceinline__ uint64_t desc_sw128(uint32_t addr) {
    uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;             // LBO (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;   // SBO
    d |= (uint64_t)1 << 46;             // descriptor version
    d |= (uint64_t)2 << 61;             // SWIZZLE_128B
    return d;
}

__device__ __forceinline__ void decode_word(uint32_t w, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
    const uint32_t e = w & 0x33333333u;
    const uint32_t o = (w >> 2) & 0x33333333u;
    r0 = __byte_perm(LUT_G, 0u, e);
    r1 = __byte_perm(LUT_G, 0u, e >> 16);
    r2 = __byte_perm(LUT_G, 0u, o);
    r3 = __byte_perm(LUT_G, 0u, o >> 16);
}

template <int NMMA>
__global__ void __launch_bounds__(NTHREADS, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int rows, int nchunks,
              int cps, float* __restrict__ part, int64_t ldp, unsigned* __restrict__ err) {
    static_assert(NMMA % 32 == 0 && NMMA >= 32 && NMMA <= 256, "NMMA");
    constexpr uint32_t NCOLS = ncols_alloc(NMMA);
    extern __shared__ uint8_t smraw[];
    Smem<NMMA>& S = *reinterpret_cast<Smem<NMMA>*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = blockIdx.x, split = blockIdx.y;
    const int c0 = split * cps;
    const int nloc = min(nchunks, c0 + cps) - c0;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&S.full[s], 1);
            mbar_init(&S.empty[s], DEC_WARPS * 32 + 1);
        }
        for (int d = 0; d < DSTAGES; ++d) {
            mbar_init(&S.adfull[d], DEC_WARPS * 32);
            mbar_init(&S.adempty[d], 1);
        }
        mbar_init(&S.accfull, 1);
        S.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) tmem_alloc(&S.tmem_base, NCOLS);
    tc_before();
    __syncthreads();
    tc_after();
    const uint32_t tmem = S.tmem_base;
    int* abort = &S.abort;

    if (warp == 0) {
        if (lane == 0 && nloc > 0) {
            int issued = 0;
            for (int it = 0; it < nloc; ++it) {
                const int s = it % STAGES, n = it / STAGES;
                if (n > 0 && !mbar_wait(&S.empty[s], (n - 1) & 1, abort, err, 1u)) break;
                mbar_expect_tx(&S.full[s], BM * PKB + NMMA * BK);
                const int kc = c0 + it;
                tma_load_2d(S.pk[s], &tmA, kc * PKB, tile * BM, &S.full[s]);
                tma_load_2d(S.bt[s], &tmB, kc * BK, 0, &S.full[s]);
                issued = it + 1;
            }
            // copies still in flight complete into full[]; wait for the last ones before leaving
            for (int it = issued - 1; it >= 0 && it >= issued - STAGES; --it)
                mbar_drain(&S.full[it % STAGES], (it / STAGES) & 1);
        }
    } else if (warp == 1) {
        if (lane == 0 && nloc > 0) {
            const uint32_t idesc = (1u << 4) | ((uint32_t)(NMMA >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
            for (int it = 0; it < nloc; ++it) {
                const int s = it % STAGES, ds = it % DSTAGES;
                if (!mbar_wait(&S.full[s], (it / STAGES) & 1, abort, err, 2u)) break;
                if (!mbar_wait(&S.adfull[ds], (it / DSTAGES) & 1, abort, err, 4u)) break;
                tc_after();
                const uint32_t a0 = saddr(S.adec[ds]), b0 = saddr(S.bt[s]);
#pragma unroll
                for (int kk = 0; kk < BK / 32; ++kk)
                    mma_f8(tmem, desc_sw128(a0 + kk * 32), desc_sw128(b0 + kk * 32), idesc, (it | kk) != 0);
                mma_commit(&S.empty[s]);
                mma_commit(&S.adempty[ds]);
            }
            mma_commit(&S.accfull);  // tracks every MMA issued above
        }
    } else {
        const int dt = threadIdx.x - 64;      // 0..255
        const int row = dt >> 1, half = dt & 1;
        const uint32_t r7 = (uint32_t)(row & 7);
        bool ok = true;
        for (int it = 0; it < nloc && ok; ++it) {
            const int s = it % STAGES, ds = it % DSTAGES;
            if (!mbar_wait(&S.full[s], (it / STAGES) & 1, abort, err, 8u)) { ok = false; break; }
            if (it >= DSTAGES && !mbar_wait(&S.adempty[ds], ((it / DSTAGES) - 1) & 1, abort, err, 16u)) {
                ok = false;
                break;
            }
            const uint4 v = *reinterpret_cast<const uint4*>(S.pk[s] + row * PKB + half * 16);
            mbar_arrive(&S.empty[s]);
            uint8_t* dst = S.adec[ds] + (row >> 3) * 1024 + r7 * 128;
            const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                uint4 o;
                decode_word(w4[q], o.x, o.y, o.z, o.w);
                const uint32_t chunk = (uint32_t)(half * 4 + q);
                *reinterpret_cast<uint4*>(dst + ((chunk ^ r7) << 4)) = o;
            }
            fence_proxy_async();
            mbar_arrive(&S.adfull[ds]);
        }
        // epilogue: warp -> TMEM lane quadrant, two warps per quadrant split the columns
        bool go = ok && nloc > 0;
        if (go) go = mbar_wait(&S.accfull, 0, abort, err, 32u);
        go = __all_sync(0xffffffffu, go);   // tcgen05.ld is warp-collective
        if (go) {
            tc_after();
            const int quad = warp & 3;
            const int hc = (warp - 2) >> 2;
            const int r = tile * BM + quad * 32 + lane;
#pragma unroll 1
            for (int cb = hc * (NMMA / 2); cb < (hc + 1) * (NMMA / 2); cb += 16) {
                uint32_t v[16];
                tmem_ld16(tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)cb, v);
                if (r < rows) {
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        part[((int64_t)split * NMMA + cb + j) * ldp + r] = __uint_as_float(v[j]);
                }
            }
        }
    }
    // leave: MMAs that were issued must finish before TMEM is released
    if (warp == 1 && nloc > 0) mbar_drain(&S.accfull, 0);
    tc_before();
    __syncthreads();
    if (warp == 1) {
        tc_after();
        tmem_dealloc(tmem, NCOLS);
    }
}

// ---- digit and combine kernels ---------------------------------------------

__device__ __forceinline__ int kpos(int64_t i) {
    // K position of element i after the decode permutation within groups of 16
    const int q = (int)(i & 15);
    return (int)(i & ~15ll) + ((q & 1) ? 8 + (q >> 1) : (q >> 1));
}

__constant__ uint8_t E4M3_INT[17] = {0xD0, 0xCE, 0xCC, 0xCA, 0xC8, 0xC4, 0xC0, 0xB8, 0x00,
                                     0x38, 0x40, 0x44, 0x48, 0x4A, 0x4C, 0x4E, 0x50};

// per-column max |x| and sum over n rows (partials per CTA)
__global__ void k_col_maxsum(const double* __restrict__ X, int64_t n, int64_t ld, double* __restrict__ pmax,
                             double* __restrict__ psum) {
    __shared__ double smx[32], ssm[32];
    const int c = blockIdx.y;
    double mx = 0, sm = 0;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const double v = X[r + c * ld];
        mx = fmax(mx, fabs(v));
        sm += v;
    }
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        sm += __shfl_xor_sync(0xffffffffu, sm, o);
    }
    if ((threadIdx.x & 31) == 0) {
        smx[threadIdx.x >> 5] = mx;
        ssm[threadIdx.x >> 5] = sm;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            a = fmax(a, smx[w]);
            b += ssm[w];
        }
        pmax[blockIdx.x + (size_t)c * gridDim.x] = a;
        psum[blockIdx.x + (size_t)c * gridDim.x] = b;
    }
}

// colinfo[c] = {scale exponent e_c (as double), column sum} from partials
__global__ void k_col_finish(const double* __restrict__ pmax, const double* __restrict__ psum, int nparts, int k,
                             double* __restrict__ colinfo) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k) return;
    double mx = 0, sm = 0;
    for (int j = 0; j < nparts; ++j) {
        mx = fmax(mx, pmax[j + (size_t)c * nparts]);
        sm += psum[j + (size_t)c * nparts];
    }
    int E = 0;
    if (mx > 0) frexp(mx, &E);
    colinfo[2 * c] = (double)(E - 3);  // |x 2^-e| < 8
    colinfo[2 * c + 1] = sm;
}

// digits of X (n x k, FP64) into D[(c*NDIG + j) * kpad + kpos(r)]  (e4m3)
__global__ void k_digits(const double* __restrict__ X, int64_t n, int64_t ld, int k, const double* __restrict__ colinfo,
                         uint8_t* __restrict__ D, int64_t kpad) {
    const int c = blockIdx.y;
    const int e = (int)colinfo[2 * c];
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        double x = ldexp(X[r + c * ld], -e);
        const int64_t p = kpos(r);
#pragma unroll
        for (int j = 0; j < NDIG; ++j) {
            const double d = rint(x);
            x = (x - d) * 16.0;
            D[((int64_t)c * NDIG + j) * kpad + p] = E4M3_INT[(int)d + 8];
        }
    }
}

// pass-1 epilogue in FP64: u[s,c] = inv_s^2 (2^e_c sum_j 16^-j P1 - 2 f_s S_c); partial max|u|, sum 2 f u
__global__ void k_combine1(const float* __restrict__ part, int nsplit, int nmma, int64_t ldp, int64_t rows, int k,
                           const double* __restrict__ colinfo, const double* __restrict__ f,
                           const double* __restrict__ inv, double* __restrict__ U, double* __restrict__ pmax,
                           double* __restrict__ psum) {
    __shared__ double smx[32], ssm[32];
    const int c = blockIdx.y;
    const int e = (int)colinfo[2 * c];
    const double Sc = colinfo[2 * c + 1];
    double mx = 0, sm = 0;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < rows; s += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0, w = 1.0;
        for (int j = 0; j < NDIG; ++j, w *= 0.0625) {
            double pj = 0.0;
            for (int y = 0; y < nsplit; ++y) pj += (double)part[((int64_t)y * nmma + c * NDIG + j) * ldp + s];
            acc += w * pj;
        }
        const double gv = ldexp(acc, e);
        const double iv = inv[s], fs = f[s];
        const double u = iv * iv * (gv - 2.0 * fs * Sc);
        U[s + c * rows] = u;
        mx = fmax(mx, fabs(u));
        sm += 2.0 * fs * u;
    }
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        sm += __shfl_xor_sync(0xffffffffu, sm, o);
    }
    if ((threadIdx.x & 31) == 0) {
        smx[threadIdx.x >> 5] = mx;
        ssm[threadIdx.x >> 5] = sm;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            a = fmax(a, smx[w]);
            b += ssm[w];
        }
        pmax[blockIdx.x + (size_t)c * gridDim.x] = a;
        psum[blockIdx.x + (size_t)c * gridDim.x] = b;
    }
}

// pass-2 epilogue: out[i,c] = scale (2^e_c sum_j 16^-j P2 - C2_c)
__global__ void k_combine2(const float* __restrict__ part, int nsplit, int nmma, int64_t ldp, int64_t rows, int k,
                           const double* __restrict__ colinfo, double scale, double* __restrict__ out, int64_t ldo) {
    const int c = blockIdx.y;
    const int e = (int)colinfo[2 * c];
    const double C2 = colinfo[2 * c + 1];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0, w = 1.0;
        for (int j = 0; j < NDIG; ++j, w *= 0.0625) {
            double pj = 0.0;
            for (int y = 0; y < nsplit; ++y) pj += (double)part[((int64_t)y * nmma + c * NDIG + j) * ldp + i];
            acc += w * pj;
        }
        out[i + c * ldo] = scale * (ldexp(acc, e) - C2);
    }
}

// individual-major copy: Gt[i][b] holds SNPs 4b..4b+3 of individual i; 64 SNPs x 256 individuals per tile
__global__ void k_transpose_codes(const uint8_t* __restrict__ G, int64_t Mk, int64_t stride, int32_t N,
                                  uint8_t* __restrict__ Gt, int64_t strideT) {
    __shared__ uint8_t t[64][64 + 4];
    const int64_t s0 = (int64_t)blockIdx.x * 64;
    for (int64_t i0 = (int64_t)blockIdx.y * 256; i0 < N; i0 += (int64_t)gridDim.y * 256) {
        // load 64 rows x 64 bytes (256 individuals); beyond Mk -> 0xFF (genotype 0)
        for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) {
            const int rs = e >> 6, b = e & 63;
            const int64_t s = s0 + rs, byte = i0 / 4 + b;
            t[rs][b] = (s < Mk && byte < stride) ? G[s * stride + byte] : (uint8_t)0xFF;
        }
        __syncthreads();
        // write 256 rows x 16 bytes (64 SNPs)
        for (int e = threadIdx.x; e < 256 * 16; e += blockDim.x) {
            const int il = e >> 4, ob = e & 15;
            const int64_t i = i0 + il;
            if (i < N) {
                unsigned v = 0;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int rs = ob * 4 + q;
                    const unsigned code = (t[rs][il >> 2] >> (2 * (il & 3))) & 3u;
                    v |= code << (2 * q);
                }
                Gt[i * strideT + s0 / 4 + ob] = (uint8_t)v;
            }
        }
        __syncthreads();
    }
}

// pad bytes of Gt beyond the last SNP byte: 0xFF
__global__ void k_fill_pad(uint8_t* __restrict__ Gt, int32_t N, int64_t strideT, int64_t from) {
    const int64_t w = strideT - from;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < (int64_t)N * w;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e / w, b = from + e % w;
        Gt[i * strideT + b] = 0xFF;
    }
}

}  // namespace tc

// ---- host side ---------------------------------------------------------------

using namespace tc;

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

static int make_map(globe_ctx* ctx, CUtensorMap* m, const void* base, uint64_t inner, uint64_t outer, uint32_t box_in,
                    uint32_t box_out, bool sw128) {
    auto fn = encode_fn();
    if (!fn) return set_err(ctx, GLOBE_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {inner};
    cuuint32_t box[2] = {box_in, box_out};
    cuuint32_t es[2] = {1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(base), dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, sw128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_err(ctx, GLOBE_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return GLOBE_OK;
}

int ensure_gt(globe_ctx* ctx) {
    auto& g = ctx->gen;
    if (g.gt) return GLOBE_OK;
    const int32_t N = ctx->coh.N;
    g.strideT = ((g.Mk + 3) / 4 + PKB - 1) / PKB * PKB;
    if (g.strideT < PKB) g.strideT = PKB;
    GLOBE_RET(dalloc(ctx, &g.gt, (size_t)N * g.strideT));
    const int64_t snp_bytes = (g.Mk + 3) / 4;
    if (g.Mk > 0) {
        dim3 grid((unsigned)((g.Mk + 63) / 64), (unsigned)std::min<int64_t>((N + 255) / 256, 64));
        k_transpose_codes<<<grid, 256, 0, ctx->stream>>>(g.geno, g.Mk, g.stride, N, g.gt, g.strideT);
        GLOBE_LAUNCHED(ctx, "k_transpose_codes");
    }
    // bytes past the last 64-SNP tile written above
    const int64_t written = (g.Mk + 63) / 64 * 16;
    const int64_t from = std::min<int64_t>(std::max<int64_t>(snp_bytes, written), g.strideT);
    if (from < g.strideT) {
        k_fill_pad<<<1024, 256, 0, ctx->stream>>>(g.gt, N, g.strideT, from);
        GLOBE_LAUNCHED(ctx, "k_fill_pad");
    }
    return GLOBE_OK;
}

template <int NMMA>
static int launch_gemm(globe_ctx* ctx, const CUtensorMap& mA, const CUtensorMap& mB, int rows, int nchunks, int splits,
                       float* part, int64_t ldp, unsigned* err) {
    const int cps = (nchunks + splits - 1) / splits;
    splits = (nchunks + cps - 1) / cps;
    const size_t smem = sizeof(Smem<NMMA>) + 1024;
    static bool attr = false;
    if (!attr) {
        GLOBE_CK(ctx, cudaFuncSetAttribute(k_tc_gemm<NMMA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr = true;
    }
    dim3 grid((unsigned)((rows + BM - 1) / BM), (unsigned)splits);
    k_tc_gemm<NMMA><<<grid, NTHREADS, smem, ctx->stream>>>(mA, mB, rows, nchunks, cps, part, ldp, err);
    GLOBE_LAUNCHED(ctx, "k_tc_gemm");
    return GLOBE_OK;
}

static int gemm_dispatch(globe_ctx* ctx, int nmma, const CUtensorMap& mA, const CUtensorMap& mB, int rows,
                         int nchunks, int splits, float* part, int64_t ldp, unsigned* err) {
    switch (nmma) {
        case 32: return launch_gemm<32>(ctx, mA, mB, rows, nchunks, splits, part, ldp, err);
        case 64: return launch_gemm<64>(ctx, mA, mB, rows, nchunks, splits, part, ldp, err);
        case 96: return launch_gemm<96>(ctx, mA, mB, rows, nchunks, splits, part, ldp, err);
        case 128: return launch_gemm<128>(ctx, mA, mB, rows, nchunks, splits, part, ldp, err);
        case 160: return launch_gemm<160>(ctx, mA, mB, rows, nchunks, splits, part, ldp, err);
        case 192: return launch_gemm<192>(ctx, mA, mB, rows, nchunks, splits, part, ldp, err);
        case 224: return launch_gemm<224>(ctx, mA, mB, rows, nchunks, splits, part, ldp, err);
        case 256: return launch_gemm<256>(ctx, mA, mB, rows, nchunks, splits, part, ldp, err);
    }
    return set_err(ctx, GLOBE_ERR_ARG, "unsupported MMA width %d", nmma);
}

static int eff_splits(int nchunks, int splits) {
    const int cps = (nchunks + splits - 1) / splits;
    return (nchunks + cps - 1) / cps;
}

static int pick_splits(int tiles, int nchunks) {
    int want = (8 * 152 + tiles - 1) / tiles;        // >= ~8 CTA waves
    int maxs = std::max(1, nchunks / 8);              // >= 8 stages per CTA
    want = std::min(want, maxs);
    want = std::max(want, (nchunks + 8191) / 8192);   // K per CTA <= 2^20 (exact FP32 sums)
    return std::max(1, want);
}

// out (N x k) = scale * Zs'(Zs Z) for one group of <= MAX_RHS_GROUP columns
static int tc_group(globe_ctx* ctx, const double* Z, int kg, double scale, double* out) {
    auto& g = ctx->gen;
    const int32_t N = ctx->coh.N;
    const int nmma = ((kg * NDIG + 31) / 32) * 32;
    // ---- pass 1 operands
    const int nch1 = (int)((g.stride + PKB - 1) / PKB);
    const int64_t kpad1 = (int64_t)nch1 * BK;
    const int nch2 = (int)(g.strideT / PKB);
    const int64_t kpad2 = (int64_t)nch2 * BK;
    const int tiles1 = (int)((g.Mk + BM - 1) / BM), tiles2 = (N + BM - 1) / BM;
    const int sp1 = pick_splits(tiles1, nch1), sp2 = pick_splits(tiles2, nch2);
    const int64_t ldp1 = (int64_t)tiles1 * BM, ldp2 = (int64_t)tiles2 * BM;
    uint8_t *D1, *D2;
    float *P1, *P2;
    double *U, *cst, *pm, *ps;
    unsigned* err;
    GLOBE_RET(ws(ctx, WS_TC_D1, (size_t)nmma * kpad1, &D1));
    GLOBE_RET(ws(ctx, WS_TC_D2, (size_t)nmma * kpad2, &D2));
    GLOBE_RET(ws(ctx, WS_TC_P1, (size_t)(sp1 + 1) * nmma * ldp1, &P1));
    GLOBE_RET(ws(ctx, WS_TC_P2, (size_t)(sp2 + 1) * nmma * ldp2, &P2));
    GLOBE_RET(ws(ctx, WS_TC_U, (size_t)g.Mk * kg + 1, &U));
    const int nbr = 304;
    GLOBE_RET(ws(ctx, WS_TC_SCAL, (size_t)(4 * kg + 2 * nbr * kg + 8), &cst));
    double* col1 = cst;           // 2*kg
    double* col2 = cst + 2 * kg;  // 2*kg
    pm = cst + 4 * kg;
    ps = pm + (size_t)nbr * kg;
    GLOBE_RET(ws(ctx, WS_TC_ERR, 4, &err));
    GLOBE_CK(ctx, cudaMemsetAsync(err, 0, sizeof(unsigned), ctx->stream));
    CUtensorMap mA1, mB1, mA2, mB2;
    GLOBE_RET(make_map(ctx, &mA1, g.geno, (uint64_t)g.stride, (uint64_t)g.Mk, PKB, BM, false));
    GLOBE_RET(make_map(ctx, &mB1, D1, (uint64_t)kpad1, (uint64_t)nmma, BK, (uint32_t)nmma, true));
    GLOBE_RET(make_map(ctx, &mA2, g.gt, (uint64_t)g.strideT, (uint64_t)N, PKB, BM, false));
    GLOBE_RET(make_map(ctx, &mB2, D2, (uint64_t)kpad2, (uint64_t)nmma, BK, (uint32_t)nmma, true));
    // ---- digits of Z
    k_col_maxsum<<<dim3(nbr, kg), 256, 0, ctx->stream>>>(Z, N, N, pm, ps);
    GLOBE_LAUNCHED(ctx, "k_col_maxsum");
    k_col_finish<<<1, 64, 0, ctx->stream>>>(pm, ps, nbr, kg, col1);
    GLOBE_LAUNCHED(ctx, "k_col_finish");
    GLOBE_CK(ctx, cudaMemsetAsync(D1, 0, (size_t)nmma * kpad1, ctx->stream));
    k_digits<<<dim3(div_up(N, 256) < 1024 ? div_up(N, 256) : 1024, kg), 256, 0, ctx->stream>>>(Z, N, N, kg, col1, D1,
                                                                                                 kpad1);
    GLOBE_LAUNCHED(ctx, "k_digits");
    // ---- pass 1
    {
        ProfScope p(ctx, GLOBE_PROF_GRM_PASS1);
        GLOBE_RET(gemm_dispatch(ctx, nmma, mA1, mB1, (int)g.Mk, nch1, sp1, P1, ldp1, err));
    }
    const int sp1e = eff_splits(nch1, sp1);
    k_combine1<<<dim3(nbr, kg), 256, 0, ctx->stream>>>(P1, sp1e, nmma, ldp1, g.Mk, kg, col1, g.f, g.inv, U, pm, ps);
    GLOBE_LAUNCHED(ctx, "k_combine1");
    k_col_finish<<<1, 64, 0, ctx->stream>>>(pm, ps, nbr, kg, col2);
    GLOBE_LAUNCHED(ctx, "k_col_finish");
    // ---- digits of u, pass 2
    GLOBE_CK(ctx, cudaMemsetAsync(D2, 0, (size_t)nmma * kpad2, ctx->stream));
    k_digits<<<dim3(div_up(g.Mk, 256) < 2048 ? div_up(g.Mk, 256) : 2048, kg), 256, 0, ctx->stream>>>(U, g.Mk, g.Mk, kg,
                                                                                                       col2, D2, kpad2);
    GLOBE_LAUNCHED(ctx, "k_digits");
    {
        ProfScope p(ctx, GLOBE_PROF_GRM_PASS2);
        GLOBE_RET(gemm_dispatch(ctx, nmma, mA2, mB2, N, nch2, sp2, P2, ldp2, err));
    }
    const int sp2e = eff_splits(nch2, sp2);
    k_combine2<<<dim3(div_up(N, 256) < 1024 ? div_up(N, 256) : 1024, kg), 256, 0, ctx->stream>>>(
        P2, sp2e, nmma, ldp2, N, kg, col2, scale, out, N);
    GLOBE_LAUNCHED(ctx, "k_combine2");
    return GLOBE_OK;
}

int geno_apply_tc(globe_ctx* ctx, const double* Z, int k, double scale, double* out) {
    auto& g = ctx->gen;
    const int32_t N = ctx->coh.N;
    if (g.Mk == 0) {
        GLOBE_CK(ctx, cudaMemsetAsync(out, 0, sizeof(double) * (size_t)N * k, ctx->stream));
        return GLOBE_OK;
    }
    GLOBE_RET(ensure_gt(ctx));
    for (int c0 = 0; c0 < k; c0 += MAX_RHS_GROUP) {
        const int kg = std::min(MAX_RHS_GROUP, k - c0);
        GLOBE_RET(tc_group(ctx, Z + (size_t)c0 * N, kg, scale, out + (size_t)c0 * N));
    }
    return GLOBE_OK;
}

int tc_check_error(globe_ctx* ctx) {
    unsigned h = 0;
    void* p = ctx->ws[WS_TC_ERR].p;
    if (!p) return GLOBE_OK;
    GLOBE_CK(ctx, cudaMemcpyAsync(&h, p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    GLOBE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (h) return set_err(ctx, GLOBE_ERR_CUDA, "tensor-core GRM kernel timed out waiting (code 0x%x)", h);
    return GLOBE_OK;
}

}  // namespace globe
