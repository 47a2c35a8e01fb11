// k_bed.cu -- PLINK 2-bit genotype statistics, filtering and layout.
//
// Per-SNP counts follow prepGenotypeInput (PCGsolver.cpp:700-743): A1 count
// = 2 #00 + #10 and missing = #01 over the N real samples (the phantom pairs
// of the last byte are excluded, which is what subtractPhantomGenotypes,
// PCGsolver.cpp:589-613, achieves by subtraction).  The float32 frequency,
// missing rate and filter use the same float operations as the reference, so
// the results are bit-exact.  The FP64 standardisation coefficients are the
// float->double restatement of getStdGenotype (PCGsolver.cpp:826-842).
#include "internal.cuh"

namespace globe {

// One warp per SNP row; byte-granular so any row alignment works.
__global__ void k_bed_stats(const uint8_t* __restrict__ bed, int64_t M, int64_t stride, int32_t N,
                            float min_maf, float max_miss, int64_t* __restrict__ alt_out,
                            int64_t* __restrict__ miss_out, float* __restrict__ maf_out,
                            float* __restrict__ mr_out, uint8_t* __restrict__ keep_out) {
    const int lane = threadIdx.x & 31;
    const int64_t s = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (s >= M) return;
    const int64_t bps = ((int64_t)N + 3) >> 2;
    const uint8_t* row = bed + s * stride;
    const int last_pairs = N - (int)((bps - 1) * 4);  // 1..4 real pairs in the last byte
    const unsigned last_mask = 0x55u & ((1u << (2 * last_pairs)) - 1u);
    long long a = 0, ms = 0;
    for (int64_t b = lane; b < bps; b += 32) {
        unsigned x = row[b];
        unsigned m = (b == bps - 1) ? last_mask : 0x55u;
        unsigned L = x & 0x55u, H = (x >> 1) & 0x55u;
        a += 2 * __popc(~(H | L) & m) + __popc(H & ~L & m);
        ms += __popc(L & ~H & m);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        ms += __shfl_xor_sync(0xffffffffu, ms, o);
    }
    if (lane == 0) {
        int n_obs = N - (int)ms;
        float f = (n_obs > 0) ? (float)a / (2.0f * (float)n_obs) : 0.0f;
        float mr = (float)ms / (float)N;
        bool k = (f >= min_maf && f <= (1.0f - min_maf) && mr <= max_miss);
        if (alt_out) alt_out[s] = a;
        if (miss_out) miss_out[s] = ms;
        if (maf_out) maf_out[s] = f;
        if (mr_out) mr_out[s] = mr;
        keep_out[s] = k ? 1 : 0;
    }
}

int bed_stats(globe_ctx* ctx, const uint8_t* d_bed, int64_t M, int64_t stride, int32_t N,
              float min_maf, float max_miss, int64_t* d_alt, int64_t* d_miss, float* d_maf,
              float* d_mr, uint8_t* d_keep) {
    if (M == 0) return GLOBE_OK;
    k_bed_stats<<<div_up(M, 8), 256, 0, ctx->stream>>>(d_bed, M, stride, N, min_maf, max_miss, d_alt,
                                                        d_miss, d_maf, d_mr, d_keep);
    GLOBE_LAUNCHED(ctx, "k_bed_stats");
    return GLOBE_OK;
}

// Copy kept rows into a padded layout.  Phantom pairs of the last byte and
// the padding bytes become code 11 (genotype 0), so a consumer that runs past
// N sees zeros.
__global__ void k_bed_compact(const uint8_t* __restrict__ in, int64_t stride_in,
                              const int64_t* __restrict__ idx, int64_t Mk, int64_t bps, int32_t N,
                              uint8_t* __restrict__ out, int64_t stride_out) {
    const int lane = threadIdx.x & 31;
    const int64_t k = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (k >= Mk) return;
    const uint8_t* src = in + idx[k] * stride_in;
    uint8_t* dst = out + k * stride_out;
    const int last_pairs = N - (int)((bps - 1) * 4);
    const unsigned keep_bits = (1u << (2 * last_pairs)) - 1u;
    for (int64_t b = lane; b < stride_out; b += 32) {
        unsigned v;
        if (b < bps - 1) v = src[b];
        else if (b == bps - 1) v = (src[b] & keep_bits) | (0xFFu & ~keep_bits);
        else v = 0xFFu;
        dst[b] = (uint8_t)v;
    }
}

int bed_compact(globe_ctx* ctx, const uint8_t* d_bed, int64_t stride_in, const int64_t* d_idx,
                int64_t Mk, int64_t bps, uint8_t* d_out, int64_t stride_out) {
    if (Mk == 0) return GLOBE_OK;
    k_bed_compact<<<div_up(Mk, 8), 256, 0, ctx->stream>>>(d_bed, stride_in, d_idx, Mk, bps,
                                                          ctx->coh.N, d_out, stride_out);
    GLOBE_LAUNCHED(ctx, "k_bed_compact");
    return GLOBE_OK;
}

// zs(code) = (g - 2f) * inv_std with g(00)=2, g(01 missing)=0, g(10)=1, g(11)=0.
__global__ void k_snp_coefs(const int64_t* __restrict__ alt, const int64_t* __restrict__ miss,
                            const int64_t* __restrict__ idx, int64_t Mk, int32_t N,
                            double* __restrict__ f_out, double* __restrict__ inv_out,
                            double* __restrict__ zs) {
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= Mk) return;
    int64_t s = idx[k];
    int n_obs = N - (int)miss[s];
    double f = (n_obs > 0) ? (double)alt[s] / (double)(2.0f * (float)n_obs) : 0.0;
    double den = 2.0 * f * (1.0 - f);
    double inv = (den > (double)1e-12f) ? 1.0 / sqrt(den) : 1.0;
    f_out[k] = f;
    inv_out[k] = inv;
    zs[k * 4 + 0] = (2.0 - 2.0 * f) * inv;
    zs[k * 4 + 1] = (0.0 - 2.0 * f) * inv;
    zs[k * 4 + 2] = (1.0 - 2.0 * f) * inv;
    zs[k * 4 + 3] = (0.0 - 2.0 * f) * inv;
}

int snp_coefs(globe_ctx* ctx, const int64_t* d_alt, const int64_t* d_miss, const int64_t* d_idx,
              int64_t Mk, int32_t N, double* d_f, double* d_inv, double* d_zs) {
    if (Mk == 0) return GLOBE_OK;
    k_snp_coefs<<<div_up(Mk, 256), 256, 0, ctx->stream>>>(d_alt, d_miss, d_idx, Mk, N, d_f, d_inv, d_zs);
    GLOBE_LAUNCHED(ctx, "k_snp_coefs");
    return GLOBE_OK;
}

// ---- synthetic genotypes (counter-based) --------------------------------

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ float u21(uint64_t h, int part) {
    return ((float)((h >> (21 * part)) & 0x1FFFFFull) + 0.5f) * (1.0f / 2097152.0f);
}

// One thread per output byte (4 samples).
__global__ void k_synth_bed(uint8_t* __restrict__ bed, int64_t M, int32_t N, int64_t stride,
                            uint64_t seed, float maf_lo, float maf_hi, float miss_rate) {
    const int64_t bps = ((int64_t)N + 3) >> 2;
    const int64_t s = blockIdx.y + (int64_t)blockIdx.z * gridDim.y;
    if (s >= M) return;
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < stride;
         b += (int64_t)gridDim.x * blockDim.x) {
        uint8_t v = 0;
        if (b < bps) {
            uint64_t hs = mix64(seed ^ mix64((uint64_t)s * 0x632BE59BD9B4E019ull));
            float p = maf_lo + (maf_hi - maf_lo) * u21(hs, 0);
            float pa1 = (u21(hs, 1) < 0.5f) ? 1.0f - p : p;
            unsigned byte = 0;
            for (int j = 0; j < 4; ++j) {
                int64_t i = b * 4 + j;
                unsigned code = 0;
                if (i < N) {
                    uint64_t h = mix64(hs ^ (uint64_t)(i + 1) * 0xD1342543DE82EF95ull);
                    int g = (u21(h, 0) < pa1) + (u21(h, 1) < pa1);
                    if (u21(h, 2) < miss_rate) code = 1;
                    else code = (g == 2) ? 0u : (g == 1 ? 2u : 3u);
                }
                byte |= code << (2 * j);
            }
            v = (uint8_t)byte;
        }
        bed[s * stride + b] = v;
    }
}

int synth_bed(globe_ctx* ctx, uint8_t* d_bed, int64_t M, int32_t N, int64_t stride, uint64_t seed,
              float maf_lo, float maf_hi, float miss_rate) {
    if (M == 0) return GLOBE_OK;
    int bx = div_up(stride, 256);
    if (bx > 64) bx = 64;
    int64_t gy = M < 65535 ? M : 65535;
    int64_t gz = (M + gy - 1) / gy;
    dim3 grid(bx, (unsigned)gy, (unsigned)gz);
    k_synth_bed<<<grid, 256, 0, ctx->stream>>>(d_bed, M, N, stride, seed, maf_lo, maf_hi, miss_rate);
    GLOBE_LAUNCHED(ctx, "k_synth_bed");
    return GLOBE_OK;
}

}  // namespace globe
