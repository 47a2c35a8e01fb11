// k_grm_geno.cu -- on-the-fly genotype GRM product in FP64 (the plain path).
//
//   out (N x k) = scale * Zs' (Zs Z),  zs(s,i) = (g - 2 f_s) inv_std_s,
//   missing -> g = 0, scale = sig2g / M            (PCGsolver.cpp:1130-1201)
//
// The genotypes are read from the SNP-major tile-blocked copy of the
// tensor-core path (blk1, tile codes; the only SNP-major copy kept).
// Pass 1 (w = Zs Z): one warp per SNP row; lanes stream 16-byte pieces of
// the row (64 samples each).  Pass 2 (Zs' w): a CTA owns 128 consecutive
// samples (one 32-byte chunk of every SNP row), stages SNP tiles in shared
// memory and splits the SNP range across CTAs (partials reduced in a fixed
// order).  zs per SNP is a table indexed by the 2-bit code, so the decode is a
// select, not arithmetic.  FP64 throughput bounds both passes.
#include "tc_common.cuh"

namespace globe {

__device__ __forceinline__ double zsel(unsigned code, double t0, double t1, double t2) {
    // tile code 00 -> t1 (g=0 or missing), 01 -> t2 (g=1), 10 -> t0 (g=2)
    return code == 1u ? t2 : (code == 2u ? t0 : t1);
}

template <int KC>
__global__ void __launch_bounds__(256) k_geno_p1(const uint8_t* __restrict__ blk, int nch, int64_t Mk,
                                                 int32_t N, const double* __restrict__ zs,
                                                 const double* __restrict__ Z, int64_t ldz, int kc,
                                                 double* __restrict__ W, int64_t ldw) {
    const int lane = threadIdx.x & 31;
    const int64_t s = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (s >= Mk) return;
    const double t0 = zs[4 * s], t1 = zs[4 * s + 1], t2 = zs[4 * s + 2];
    const int nchunks = (N + 63) >> 6;
    double acc[KC];
#pragma unroll
    for (int c = 0; c < KC; ++c) acc[c] = 0.0;
    for (int q = lane; q < nchunks; q += 32) {
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(blk + tc::blk_offset(s, (int64_t)q << 4, nch)));
        const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
        const int i0 = q << 6;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t w = w4[j];
#pragma unroll 4
            for (int e = 0; e < 16; ++e) {
                const int i = i0 + j * 16 + e;
                if (i < N) {
                    const double z = zsel((w >> (2 * e)) & 3u, t0, t1, t2);
#pragma unroll
                    for (int c = 0; c < KC; ++c)
                        if (c < kc) acc[c] += z * __ldg(Z + i + (size_t)c * ldz);
                }
            }
        }
    }
#pragma unroll
    for (int c = 0; c < KC; ++c) {
        double a = acc[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0 && c < kc) W[s + (size_t)c * ldw] = a;
    }
}

constexpr int P2_THREADS = 128;  // samples per CTA (32 bytes per SNP row)
constexpr int P2_TS = 64;        // SNPs per shared-memory tile

// SQUARE: accumulate zs^2 (genetic diagonal) instead of zs * W, as double-float sums of the
// FP64 squares split into float pairs (GB300's FP64 pipe would bound the 5e10 additions of
// the full workload at ~0.1 s; on the FP32 pipe they take a few ms).
template <int KC, bool SQUARE>
__global__ void __launch_bounds__(P2_THREADS) k_geno_p2(const uint8_t* __restrict__ blk, int nch,
                                                        int64_t Mk, int32_t N, const double* __restrict__ zs,
                                                        const float2* __restrict__ zsq,
                                                        const double* __restrict__ W, int64_t ldw, int kc,
                                                        int64_t s_per, double* __restrict__ part) {
    __shared__ __align__(16) uint8_t gb[P2_TS][32];
    __shared__ double zt[P2_TS][4];
    __shared__ double wt[P2_TS][KC > 0 ? KC : 1];
    __shared__ float2 zq[P2_TS][4];   // SQUARE: zs^2 by tile code as (hi, lo) floats
    const int tid = threadIdx.x;
    const int64_t i = (int64_t)blockIdx.x * P2_THREADS + tid;
    const int64_t byte0 = (int64_t)blockIdx.x * 32;   // this CTA's 32-byte chunk of every row
    const int64_t s_beg = (int64_t)blockIdx.y * s_per;
    int64_t s_end = s_beg + s_per;
    if (s_end > Mk) s_end = Mk;
    double acc[KC];
#pragma unroll
    for (int c = 0; c < KC; ++c) acc[c] = 0.0;
    float qh = 0.0f, ql = 0.0f;   // SQUARE: double-float sum
    const int sh = 2 * (tid & 3);
    const int bi = tid >> 2;
    for (int64_t s0 = s_beg; s0 < s_end; s0 += P2_TS) {
        const int ns = (int)((s_end - s0) < P2_TS ? (s_end - s0) : P2_TS);
        {   // 64 rows x 32 bytes, 16 bytes per thread
            const int rs = tid >> 1, half = tid & 1;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (rs < ns)
                v = __ldg(reinterpret_cast<const uint4*>(blk + tc::blk_offset(s0 + rs, byte0 + half * 16, nch)));
            *reinterpret_cast<uint4*>(&gb[rs][half * 16]) = v;
        }
        for (int e = tid; e < P2_TS * 4; e += P2_THREADS) {
            const int rs = e >> 2;
            if (SQUARE) zq[rs][e & 3] = rs < ns ? zsq[(s0 + rs) * 4 + (e & 3)] : make_float2(0.0f, 0.0f);
            else zt[rs][e & 3] = rs < ns ? zs[(s0 + rs) * 4 + (e & 3)] : 0.0;
        }
        if (!SQUARE) {
            for (int e = tid; e < P2_TS * KC; e += P2_THREADS) {
                const int rs = e / KC, c = e % KC;
                wt[rs][c] = (rs < ns && c < kc) ? W[(s0 + rs) + (size_t)c * ldw] : 0.0;
            }
        }
        __syncthreads();
        for (int rs = 0; rs < ns; ++rs) {
            const unsigned code = (gb[rs][bi] >> sh) & 3u;
            if (SQUARE) {
                const float2 q = zq[rs][code];
                tc::df_add(qh, ql, q.x, q.y);
            } else {
                const double z = zsel(code, zt[rs][0], zt[rs][1], zt[rs][2]);
#pragma unroll
                for (int c = 0; c < KC; ++c) acc[c] += z * wt[rs][c];
            }
        }
        __syncthreads();
    }
    if (SQUARE) acc[0] = (double)qh + (double)ql;
    if (i < N) {
        const size_t base = (size_t)blockIdx.y * (size_t)N * (SQUARE ? 1 : kc);
#pragma unroll
        for (int c = 0; c < KC; ++c)
            if (c < (SQUARE ? 1 : kc)) part[base + i + (size_t)c * N] = acc[c];
    }
}

// zsq[4 s + t] = zs^2 of tile code t as a (hi, lo) float pair (t: 0/3 -> g=0, 1 -> g=1, 2 -> g=2)
__global__ void k_zs_square(const double* __restrict__ zs, int64_t Mk, float2* __restrict__ zsq) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 4 * Mk) return;
    const double z = zs[(e & ~3ll) + tc::tile_to_plink((int)(e & 3))];
    const double q = z * z;
    const float hi = __double2float_rn(q);
    zsq[e] = make_float2(hi, __double2float_rn(q - (double)hi));
}

// out[e] = scale * sum_y part[y * n + e]  (fixed order)
__global__ void k_sum_splits(const double* __restrict__ part, int nsplit, int64_t n, double scale,
                             double* __restrict__ out, int64_t ldo, int64_t rows) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        double a = 0;
        for (int y = 0; y < nsplit; ++y) a += part[(size_t)y * n + e];
        const int64_t r = e % rows, c = e / rows;
        out[r + c * ldo] = scale * a;
    }
}

static int pick_splits(int64_t ctas_x, int64_t Mk) {
    int64_t want = (2 * 152 + ctas_x - 1) / ctas_x;
    int64_t maxs = (Mk + P2_TS - 1) / P2_TS;
    if (want > maxs) want = maxs;
    if (want < 1) want = 1;
    if (want > 256) want = 256;
    return (int)want;
}

template <int KC>
static int geno_chunk(globe_ctx* ctx, const double* Z, int kc, double scale, double* out, double* W,
                      double* part, int nsplit, int64_t s_per) {
    auto& g = ctx->gen;
    const int32_t N = ctx->coh.N;
    {
        ProfScope ps(ctx, GLOBE_PROF_GRM_PASS1);
        k_geno_p1<KC><<<div_up(g.Mk, 8), 256, 0, ctx->stream>>>(g.blk1, g.nch1, g.Mk, N, g.zs, Z, N, kc, W, g.Mk);
        GLOBE_LAUNCHED(ctx, "k_geno_p1");
    }
    dim3 grid(div_up(N, P2_THREADS), nsplit);
    {
        ProfScope ps(ctx, GLOBE_PROF_GRM_PASS2);
        k_geno_p2<KC, false><<<grid, P2_THREADS, 0, ctx->stream>>>(g.blk1, g.nch1, g.Mk, N, g.zs, nullptr, W, g.Mk, kc,
                                                                    s_per, part);
        GLOBE_LAUNCHED(ctx, "k_geno_p2");
    }
    int64_t n = (int64_t)N * kc;
    int nb = div_up(n, 256);
    if (nb > 4096) nb = 4096;
    k_sum_splits<<<nb, 256, 0, ctx->stream>>>(part, nsplit, n, scale, out, N, N);
    GLOBE_LAUNCHED(ctx, "k_sum_splits");
    return GLOBE_OK;
}

int geno_apply_f64(globe_ctx* ctx, const double* Z, int k, double scale, double* out) {
    auto& g = ctx->gen;
    const int32_t N = ctx->coh.N;
    if (g.Mk == 0) {
        GLOBE_CK(ctx, cudaMemsetAsync(out, 0, sizeof(double) * (size_t)N * k, ctx->stream));
        return GLOBE_OK;
    }
    GLOBE_RET(ensure_blk1(ctx));
    const int kcmax = 8;
    int kc0 = k < kcmax ? k : kcmax;
    double* W;
    GLOBE_RET(ws(ctx, WS_W, (size_t)g.Mk * kc0, &W));
    int64_t ctas_x = div_up(N, P2_THREADS);
    int nsplit = pick_splits(ctas_x, g.Mk);
    int64_t s_per = ((g.Mk + nsplit - 1) / nsplit + P2_TS - 1) / P2_TS * P2_TS;
    nsplit = (int)((g.Mk + s_per - 1) / s_per);
    double* part;
    GLOBE_RET(ws(ctx, WS_GPART, (size_t)nsplit * N * kc0, &part));
    for (int c0 = 0; c0 < k; c0 += kcmax) {
        int kc = (k - c0) < kcmax ? (k - c0) : kcmax;
        const double* Zc = Z + (size_t)c0 * N;
        double* oc = out + (size_t)c0 * N;
        int rc;
        if (kc == 1) rc = geno_chunk<1>(ctx, Zc, kc, scale, oc, W, part, nsplit, s_per);
        else if (kc == 2) rc = geno_chunk<2>(ctx, Zc, kc, scale, oc, W, part, nsplit, s_per);
        else if (kc <= 4) rc = geno_chunk<4>(ctx, Zc, kc, scale, oc, W, part, nsplit, s_per);
        else rc = geno_chunk<8>(ctx, Zc, kc, scale, oc, W, part, nsplit, s_per);
        GLOBE_RET(rc);
    }
    return GLOBE_OK;
}

int geno_diag(globe_ctx* ctx, double* d) {
    auto& g = ctx->gen;
    const int32_t N = ctx->coh.N;
    if (g.Mk == 0) {
        GLOBE_CK(ctx, cudaMemsetAsync(d, 0, sizeof(double) * N, ctx->stream));
        return GLOBE_OK;
    }
    GLOBE_RET(ensure_blk1(ctx));
    int64_t ctas_x = div_up(N, P2_THREADS);
    int nsplit = pick_splits(ctas_x, g.Mk);
    int64_t s_per = ((g.Mk + nsplit - 1) / nsplit + P2_TS - 1) / P2_TS * P2_TS;
    nsplit = (int)((g.Mk + s_per - 1) / s_per);
    double* part;
    GLOBE_RET(ws(ctx, WS_GPART, (size_t)nsplit * N, &part));
    float2* zsq;
    GLOBE_RET(ws(ctx, WS_W, (size_t)g.Mk * 4, &zsq));
    k_zs_square<<<div_up(4 * g.Mk, 256), 256, 0, ctx->stream>>>(g.zs, g.Mk, zsq);
    GLOBE_LAUNCHED(ctx, "k_zs_square");
    dim3 grid((unsigned)ctas_x, nsplit);
    k_geno_p2<1, true><<<grid, P2_THREADS, 0, ctx->stream>>>(g.blk1, g.nch1, g.Mk, N, g.zs, zsq, nullptr, 0, 1,
                                                              s_per, part);
    GLOBE_LAUNCHED(ctx, "k_geno_diag");
    // A_ii = (1/M) sum_s zs^2   (PCGsolver.cpp:986-988)
    k_sum_splits<<<div_up(N, 256), 256, 0, ctx->stream>>>(part, nsplit, N, 1.0 / (double)g.Mk, d, N, N);
    GLOBE_LAUNCHED(ctx, "k_sum_splits");
    return GLOBE_OK;
}

}  // namespace globe
