// records.cuh -- launch shape shared by the record kernels (k_records.cu, k_records_df.cu).
#pragma once

#include "internal.cuh"

namespace globe {

constexpr int RB_THREADS = 256;  // 8 warps, one block of records per warp
constexpr int RB_WARPS = RB_THREADS / 32;
constexpr int TB_THREADS = 256;  // thread-per-block layout

// Launch shape of the record kernels: one thread per (block of <= SHORT_BLOCK records,
// column) over all blocks -- nbt CTAs per column, longer blocks skipped -- and one
// warp per longer block over the list coh.lblk (nbl CTAs).  Per-CTA partial sums of
// both go to part[slot + q * S], thread-layout CTAs first.
struct RecShape {
    int nbt, nbl, S;
};
inline RecShape rec_shape(const globe_ctx* ctx) {
    RecShape r;
    r.nbt = div_up(ctx->coh.N, TB_THREADS);
    r.nbl = ctx->coh.nlong > 0 ? div_up(ctx->coh.nlong, RB_WARPS) : 0;
    r.S = r.nbt + r.nbl;
    return r;
}

// Sum of one column's nparts partials by a CTA of 256 threads: four strided accumulators per
// thread, then a tree in sm (256 doubles); every thread returns the sum.  k_reduce_cols and the
// reductions that the record kernels' last CTAs finish both use it, so the order is one.
__device__ __forceinline__ double cta_reduce_256(const double* __restrict__ pc, int nparts, double* sm) {
    double a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    int j = threadIdx.x;
    for (; j + 3 * 256 < nparts; j += 4 * 256) {
        a0 += __ldcg(pc + j);
        a1 += __ldcg(pc + j + 256);
        a2 += __ldcg(pc + j + 2 * 256);
        a3 += __ldcg(pc + j + 3 * 256);
    }
    for (; j < nparts; j += 256) a0 += __ldcg(pc + j);
    sm[threadIdx.x] = (a0 + a1) + (a2 + a3);
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
        __syncthreads();
    }
    const double v = sm[0];
    __syncthreads();   // sm may be reused
    return v;
}

// The warp-per-block kernels stage per-warp partial sums of RCH columns at a time in static
// shared memory, sm[(j * RCH + cc) * RB_WARPS + warp] for quantity j < nq and column c0 + cc,
// so any number of columns fits.  flush_chunk sums them over the CTA's warps, in warp order,
// into part[slot + (j * kact + c0 + cc) * stride]; every thread of the CTA calls it.
constexpr int RCH = 32;
__device__ __forceinline__ void flush_chunk(const double* sm, int nq, int nc, int c0, int kact, double* part, int slot,
                                            int stride) {
    __syncthreads();
    for (int e = threadIdx.x; e < nq * nc; e += blockDim.x) {
        const int j = e / nc, cc = e - j * nc;
        double a = 0.0;
#pragma unroll
        for (int w = 0; w < RB_WARPS; ++w) a += sm[(j * RCH + cc) * RB_WARPS + w];
        part[slot + (size_t)(j * kact + c0 + cc) * stride] = a;
    }
    __syncthreads();
}

}  // namespace globe
