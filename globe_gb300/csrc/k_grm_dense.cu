// k_grm_dense.cu -- dense GRM product from the packed lower triangle: FP64
// (GLOBE_PREC_FP64), and double-float FP32 arithmetic for GLOBE_PREC_MIXED when the
// tensor-core digit planes of k_tc_dense.cu cannot be held (device memory, non-finite A).
//
//   out (N x k) = scale * A Z,  A(i,j) = lt[max(i,j)(max(i,j)+1)/2 + min(i,j)]
//   (PCGsolver.cpp:1202-1213, varCompEst.cpp:531-558)
//
// A CTA owns 64 output rows and walks all 64-column tiles of its row block.
// Tiles left of the diagonal are rows of the triangle (contiguous in j);
// tiles right of it are read as columns of the triangle (contiguous in i);
// both loads are coalesced.  Each element is read once per row block that
// needs it, i.e. twice overall, like the reference's full-square loop; in
// FP64 the kernel is bound by the FP64 pipe, not by these bytes.
#include <algorithm>

#include "internal.cuh"

namespace globe {

constexpr int DT = 64;

template <int KC>
__global__ void __launch_bounds__(256) k_dense_f64(const float* __restrict__ lt, int32_t N,
                                                   const double* __restrict__ Z, int kc, double scale,
                                                   double* __restrict__ out) {
    __shared__ float At[DT][DT + 1];
    __shared__ double Zt[DT][KC];
    const int tid = threadIdx.x;
    const int64_t I0 = (int64_t)blockIdx.x * DT;
    const int row = tid & (DT - 1);
    const int cg = tid >> 6;  // 0..3
    double acc[(KC + 3) / 4];
#pragma unroll
    for (int q = 0; q < (KC + 3) / 4; ++q) acc[q] = 0.0;
    for (int64_t J0 = 0; J0 < N; J0 += DT) {
        if (J0 + DT <= I0) {
            // strictly left of the diagonal block: A(i, j) = lt[i(i+1)/2 + j]
            const int jj = tid & (DT - 1);
            for (int m = tid >> 6; m < DT; m += 4) {
                const int64_t i = I0 + m, j = J0 + jj;
                At[m][jj] = (i < N) ? __ldg(lt + i * (i + 1) / 2 + j) : 0.0f;
            }
        } else if (J0 >= I0 + DT) {
            // strictly right: A(i, j) = lt[j(j+1)/2 + i], contiguous in i
            const int ii = tid & (DT - 1);
            for (int m = tid >> 6; m < DT; m += 4) {
                const int64_t i = I0 + ii, j = J0 + m;
                At[ii][m] = (i < N && j < N) ? __ldg(lt + j * (j + 1) / 2 + i) : 0.0f;
            }
        } else {
            const int jj = tid & (DT - 1);
            for (int m = tid >> 6; m < DT; m += 4) {
                const int64_t i = I0 + m, j = J0 + jj;
                float v = 0.0f;
                if (i < N && j < N) v = (i >= j) ? __ldg(lt + i * (i + 1) / 2 + j) : __ldg(lt + j * (j + 1) / 2 + i);
                At[m][jj] = v;
            }
        }
        for (int e = tid; e < DT * KC; e += 256) {
            const int j = e % DT, c = e / DT;
            Zt[j][c] = (J0 + j < N && c < kc) ? Z[J0 + j + (size_t)c * N] : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int j = 0; j < DT; ++j) {
            const double a = (double)At[row][j];
#pragma unroll
            for (int q = 0; q < (KC + 3) / 4; ++q) {
                const int c = cg + 4 * q;
                if (c < KC) acc[q] += a * Zt[j][c];
            }
        }
        __syncthreads();
    }
    const int64_t i = I0 + row;
    if (i < N) {
#pragma unroll
        for (int q = 0; q < (KC + 3) / 4; ++q) {
            const int c = cg + 4 * q;
            if (c < kc) out[i + (size_t)c * N] = scale * acc[q];
        }
    }
}

int dense_apply_f64(globe_ctx* ctx, const double* Z, int k, double scale, double* out) {
    const int32_t N = ctx->coh.N;
    const int kcmax = 8;
    for (int c0 = 0; c0 < k; c0 += kcmax) {
        int kc = (k - c0) < kcmax ? (k - c0) : kcmax;
        const double* Zc = Z + (size_t)c0 * N;
        double* oc = out + (size_t)c0 * N;
        int nb = div_up(N, DT);
        ProfScope ps(ctx, GLOBE_PROF_GRM_PASS1);
        if (kc <= 4) k_dense_f64<4><<<nb, 256, 0, ctx->stream>>>(ctx->gen.grm, N, Zc, kc, scale, oc);
        else k_dense_f64<8><<<nb, 256, 0, ctx->stream>>>(ctx->gen.grm, N, Zc, kc, scale, oc);
        GLOBE_LAUNCHED(ctx, "k_dense_f64");
    }
    return GLOBE_OK;
}

// ---- mixed precision: double-float arithmetic on the FP32 pipes ----------------
//
// GB300 runs FP64 at a small fraction of its FP32 rate, so the GLOBE_PREC_MIXED
// product keeps ~48-bit accuracy in FP32 arithmetic.  A(i,j) is exactly an FP32
// value.  Each right-hand side is split as z = zh + zl, two FP32 values.  The term
// a*z = p + e is formed exactly: p = a*zh rounded, e = fma(a, zh, -p) its error,
// and a*zl (relative size 2^-24) is folded into e.  The accumulator is a pair
// (s, c); s += p uses a two-sum whose exact error, with e, goes to c.  The error is
// ~2^-48 per term, relative to |a z|.  Column chunks of KC right-hand sides; the
// J range is split over gridDim.y CTAs, whose partials a second kernel adds in FP64.

// The _rn intrinsics keep every step rounded as written: the compiler never contracts
// them into FMAs, which would break the error-free product and two-sum.
__device__ __forceinline__ void df_acc(float& s, float& c, float a, float zh, float zl) {
    const float p = __fmul_rn(a, zh);
    float e = __fmaf_rn(a, zh, -p);                 // a*zh - p exactly
    e = __fmaf_rn(a, zl, e);
    const float t = __fadd_rn(s, p);
    const float bp = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));   // s + p - t exactly
    s = t;
    c = __fadd_rn(c, __fadd_rn(err, e));
}

template <int KC>
__global__ void __launch_bounds__(256) k_dense_df(const float* __restrict__ lt, int32_t N,
                                                  const double* __restrict__ Z, int kc, int tiles_per_split,
                                                  double scale, double* __restrict__ part, double* __restrict__ out) {
    __shared__ float At[DT][DT + 1];
    __shared__ float2 Zt[DT][KC];
    const int tid = threadIdx.x;
    const int64_t I0 = (int64_t)blockIdx.x * DT;
    const int row = tid & (DT - 1);
    const int cg = tid >> 6;  // 0..3
    constexpr int NQ = (KC + 3) / 4;
    float s[NQ], c[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) s[q] = c[q] = 0.0f;
    const int64_t Jb = (int64_t)blockIdx.y * tiles_per_split * DT;
    const int64_t Je = min((int64_t)N, Jb + (int64_t)tiles_per_split * DT);
    for (int64_t J0 = Jb; J0 < Je; J0 += DT) {
        if (J0 + DT <= I0) {
            const int jj = tid & (DT - 1);
            for (int m = tid >> 6; m < DT; m += 4) {
                const int64_t i = I0 + m, j = J0 + jj;
                At[m][jj] = (i < N) ? __ldg(lt + i * (i + 1) / 2 + j) : 0.0f;
            }
        } else if (J0 >= I0 + DT) {
            const int ii = tid & (DT - 1);
            for (int m = tid >> 6; m < DT; m += 4) {
                const int64_t i = I0 + ii, j = J0 + m;
                At[ii][m] = (i < N && j < N) ? __ldg(lt + j * (j + 1) / 2 + i) : 0.0f;
            }
        } else {
            const int jj = tid & (DT - 1);
            for (int m = tid >> 6; m < DT; m += 4) {
                const int64_t i = I0 + m, j = J0 + jj;
                float v = 0.0f;
                if (i < N && j < N) v = (i >= j) ? __ldg(lt + i * (i + 1) / 2 + j) : __ldg(lt + j * (j + 1) / 2 + i);
                At[m][jj] = v;
            }
        }
        for (int e = tid; e < DT * KC; e += 256) {
            const int j = e % DT, cc = e / DT;
            const double z = (J0 + j < N && cc < kc) ? Z[J0 + j + (size_t)cc * N] : 0.0;
            const float zh = __double2float_rn(z);
            Zt[j][cc] = make_float2(zh, __double2float_rn(z - (double)zh));
        }
        __syncthreads();
#pragma unroll 4
        for (int j = 0; j < DT; ++j) {
            const float a = At[row][j];
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                const int cc = cg + 4 * q;
                if (cc < KC) {
                    const float2 z = Zt[j][cc];
                    df_acc(s[q], c[q], a, z.x, z.y);
                }
            }
        }
        __syncthreads();
    }
    const int64_t i = I0 + row;
    if (i < N) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            const int cc = cg + 4 * q;
            if (cc < kc) {
                const double v = (double)s[q] + (double)c[q];
                if (gridDim.y == 1) out[i + (size_t)cc * N] = scale * v;
                else part[((size_t)blockIdx.y * kc + cc) * N + i] = v;
            }
        }
    }
}

// out[i, c] = scale * sum_y part[y, c, i]
__global__ void k_dense_sum(const double* __restrict__ part, int nsplit, int kc, int32_t N, double scale,
                            double* __restrict__ out) {
    const int c = blockIdx.y;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        double v = 0.0;
        for (int y = 0; y < nsplit; ++y) v += part[((size_t)y * kc + c) * N + i];
        out[i + (size_t)c * N] = scale * v;
    }
}

int dense_apply_df(globe_ctx* ctx, const double* Z, int k, double scale, double* out) {
    const int32_t N = ctx->coh.N;
    constexpr int KCM = 16;
    const int nb = div_up(N, DT), ntiles = div_up(N, DT);
    // about 4 CTAs per SM in flight: split the J range when the row blocks alone are few
    int nsplit = std::max(1, std::min(ntiles / 4, (4 * 152 + nb - 1) / nb));
    const int tps = div_up(ntiles, nsplit);
    nsplit = div_up(ntiles, tps);
    double* part = nullptr;
    if (nsplit > 1) GLOBE_RET(ws(ctx, WS_PART, (size_t)nsplit * KCM * N, &part));
    for (int c0 = 0; c0 < k; c0 += KCM) {
        const int kc = std::min(KCM, k - c0);
        const double* Zc = Z + (size_t)c0 * N;
        double* oc = out + (size_t)c0 * N;
        ProfScope ps(ctx, GLOBE_PROF_GRM_PASS1);
        const dim3 grid(nb, nsplit);
        if (kc <= 4) k_dense_df<4><<<grid, 256, 0, ctx->stream>>>(ctx->gen.grm, N, Zc, kc, tps, scale, part, oc);
        else if (kc <= 8) k_dense_df<8><<<grid, 256, 0, ctx->stream>>>(ctx->gen.grm, N, Zc, kc, tps, scale, part, oc);
        else k_dense_df<16><<<grid, 256, 0, ctx->stream>>>(ctx->gen.grm, N, Zc, kc, tps, scale, part, oc);
        GLOBE_LAUNCHED(ctx, "k_dense_df");
        if (nsplit > 1) {
            k_dense_sum<<<dim3(std::min(div_up(N, 256), 1024), kc), 256, 0, ctx->stream>>>(part, nsplit, kc, N, scale,
                                                                                          oc);
            GLOBE_LAUNCHED(ctx, "k_dense_sum");
        }
    }
    return GLOBE_OK;
}

__global__ void k_dense_diag(const float* __restrict__ lt, int32_t N, double* __restrict__ d) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) d[i] = (double)lt[i * (i + 1) / 2 + i];
}

int dense_diag(globe_ctx* ctx, double* d) {
    const int32_t N = ctx->coh.N;
    k_dense_diag<<<div_up(N, 256), 256, 0, ctx->stream>>>(ctx->gen.grm, N, d);
    GLOBE_LAUNCHED(ctx, "k_dense_diag");
    return GLOBE_OK;
}

}  // namespace globe
