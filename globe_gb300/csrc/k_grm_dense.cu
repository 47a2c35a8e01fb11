// k_grm_dense.cu -- dense GRM product from the packed lower triangle (FP64).
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
