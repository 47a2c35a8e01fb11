// k_grm_build.cu -- the genetic relationship matrix of the kept SNPs,
//
//   A = Zs'Zs / M,   zs(s,i) = (g(s,i) - 2 f_s) inv_s,  missing g -> 0
//
// (getStdGenotype, PCGsolver.cpp:826-842, the standardisation the on-the-fly
// product uses), written as the float32 packed lower triangle, row major with
// the diagonal: the .grm.bin payload readFullGRM reads (PCGsolver.cpp:778-809)
// and readGRM reads (varCompEst.cpp:270-295).  The reference has no builder;
// a .grm.bin built here gives the dense path the same matrix as --geno.
//
// GLOBE_PREC_MIXED (tensor cores, exact up to the final float32 rounding).
// Column j of A is a pass-2 product of the genotype kernel (k_tc_gemm):
//   A_ij = 1/M sum_s (g(s,i) - 2 f_s) u(s,j),   u(s,j) = inv_s zs(s,j)
// u(s,j) is one of four values per SNP, one per 2-bit code.  Each is rounded
// once to a multiple of 2^(e-40) with one exponent e for the whole matrix
// (|u 2^-e| < 16) and split into 9 balanced base-32 digits, so the digit
// operand of column j is a table lookup on individual j's codes.  The MMAs
// sum g * digit exactly in FP32, the digits are recombined in int64, and the
// centring term sum_s 2 f_s u(s,j) is summed from the same rounded u (double-float per
// thread, FP64 across threads).
// Groups of 21 columns (189 digit rows, MMA N = 192) are the z dimension of
// one k_tc_gemm launch; row tiles wholly above a group's first column are
// skipped, so only the lower triangle is computed.
//
// GLOBE_PREC_FP64: k_grm_f64, 64 x 64 FP64 tiles over the lower triangle.
#include "tc_common.cuh"

namespace globe {
namespace tc {

constexpr int GRM_KG = 21;                                  // columns per group
constexpr int GRM_NMMA = (GRM_KG * NDIG + 15) / 16 * 16;    // 192
static_assert(GRM_KG <= 28 && GRM_NMMA <= 256, "group width");

// U4[4s + t] = inv_s zs_s: the value of u(s, .) for tile code t (the codes of blk2)
__global__ void k_grm_u4(const double* __restrict__ zs, const double* __restrict__ inv, int64_t Mk,
                         double* __restrict__ U4) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < 4 * Mk; e += (int64_t)gridDim.x * blockDim.x)
        U4[e] = inv[e >> 2] * zs[(e & ~3ll) + tile_to_plink((int)(e & 3))];
}

// Per SNP s < kpad and tile code c: the 9 e4m3 digits of I = round(u 2^(40-e)) (bytes 0..8 of
// dig[4s+c], most significant first; times geno_digit_mult(s)) and 2 f_s u~ with u~ = I 2^(e-40)
// the rounded value, as a float pair hi + lo (hi = the float nearest, lo = the float nearest
// the rest: ~48 bits).
// SNPs >= Mk (padding of the K range) get zero digits and zero.
__global__ void k_grm_table(const double* __restrict__ U4, const double* __restrict__ f, int64_t Mk, int64_t kpad,
                            const double* __restrict__ info, uint4* __restrict__ dig, float2* __restrict__ c2v) {
    const int e = (int)info[0];
    const double sc = ldexp(1.0, DBITS * (NDIG - 1) - e), back = ldexp(1.0, e - DBITS * (NDIG - 1));
    for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < 4 * kpad;
         x += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = x >> 2;
        uint4 out = make_uint4(0u, 0u, 0u, 0u);
        double cv = 0.0;
        if (s < Mk) {
            long long I = __double2ll_rn(U4[x] * sc);
            cv = 2.0 * f[s] * ll_times_pow2(I, back);
            uint32_t b[NDIG];
            const int mult = geno_digit_mult(s);   // even SNPs: 4 d (their genotypes decode to 2^-9 g)
#pragma unroll
            for (int j = NDIG - 1; j > 0; --j) {
                const int d = (int)((I + DHALF) & (2 * DHALF - 1)) - DHALF;
                I = (I - d) >> DBITS;
                b[j] = e4m3_int(mult * d);
            }
            b[0] = e4m3_int(mult * (int)I);
            out.x = b[0] | (b[1] << 8) | (b[2] << 16) | (b[3] << 24);
            out.y = b[4] | (b[5] << 8) | (b[6] << 16) | (b[7] << 24);
            out.z = b[8];
        }
        dig[x] = out;
        const float hi = __double2float_rn(cv);
        c2v[x] = make_float2(hi, __double2float_rn(cv - (double)hi));
    }
}

__device__ __forceinline__ uint32_t dig_byte(const uint4& v, int j) {
    const uint32_t w = j < 4 ? v.x : (j < 8 ? v.y : v.z);
    return (w >> (8 * (j & 3))) & 0xFFu;
}

constexpr int GD_Q = 32;      // 16-SNP groups per CTA (one per lane): 512 SNPs
constexpr int GD_COLS = 32;   // columns per CTA (four per warp)
constexpr int GD_PAD = 65;    // table slots per 16-SNP group: 64 entries + 1 (spreads shared-memory banks)
constexpr size_t GD_SMEM = (size_t)GD_Q * GD_PAD * (sizeof(uint4) + sizeof(float2));

// bytes [a0.k, a1.k, a2.k, a3.k] (byte k of each word)
__device__ __forceinline__ uint32_t gather_byte(uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t k) {
    const uint32_t sel = k | ((k + 4) << 4);
    uint32_t lo, hi, r;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(lo) : "r"(a0), "r"(a1), "r"(sel));
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(hi) : "r"(a2), "r"(a3), "r"(sel));
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(lo), "r"(hi), "r"(0x5410u));
    return r;
}

// Digit operand of the batch's columns jb .. jb + ncols - 1.  Column jj = z * GRM_KG + c
// goes to digit rows z * GRM_NMMA + c * NDIG + j, K positions in the decode order of the A
// operand (kpos_g: position P of a group of 16 holds SNP 4 (P % 4) + P / 4).
// A CTA covers 512 SNPs (32 groups of 16, one per lane) for 32 columns (four per warp): the
// table entries of its SNPs are staged once in shared memory, each lane reads the 16 codes
// of its group for one column (one 32-bit word of blk2, tile codes), gathers the 16 table
// entries and assembles the 9 digit rows 4 bytes at a time (3 prmt per word).  The centring
// sums come out per (CTA SNP range, column) in part[blockIdx.y * ncols + jj].
__global__ void __launch_bounds__(256) k_grm_digits(const uint8_t* __restrict__ blk2, int nch2, int32_t N, int jb,
                                                    int ncols, const uint4* __restrict__ dig,
                                                    const float2* __restrict__ c2v, int64_t kpad,
                                                    uint8_t* __restrict__ D, double* __restrict__ part) {
    extern __shared__ __align__(16) uint8_t gd_sm[];
    uint4* tdig = reinterpret_cast<uint4*>(gd_sm);
    float2* tc2 = reinterpret_cast<float2*>(gd_sm + (size_t)GD_Q * GD_PAD * sizeof(uint4));
    const int64_t nq = kpad >> 4;
    const int64_t q0 = (int64_t)blockIdx.y * GD_Q;
    for (int e = threadIdx.x; e < GD_Q * 64; e += blockDim.x) {
        const int ql = e >> 6, w = e & 63;          // w = 4 m + tile code
        const int64_t x = (q0 + ql) * 64 + w;        // entry of SNP 16 (q0 + ql) + m
        const bool in = q0 + ql < nq;
        tdig[ql * GD_PAD + w] = in ? __ldg(dig + x) : make_uint4(0u, 0u, 0u, 0u);
        tc2[ql * GD_PAD + w] = in ? __ldg(c2v + x) : make_float2(0.0f, 0.0f);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t q = q0 + lane;
    const bool qin = q < nq;
    const uint4* te = tdig + lane * GD_PAD;
    const float2* tc = tc2 + lane * GD_PAD;
    for (int cc = warp; cc < GD_COLS; cc += 8) {
        const int jj = blockIdx.x * GD_COLS + cc;
        if (jj >= ncols) break;                      // uniform across the warp
        const int64_t j = (int64_t)jb + jj;
        const int z = jj / GRM_KG, c = jj % GRM_KG;
        uint8_t* Dc = D + ((int64_t)z * GRM_NMMA + c * NDIG) * kpad;
        float ah = 0.0f, al = 0.0f;
        if (qin) {
            uint32_t o[NDIG][4];
#pragma unroll
            for (int d = 0; d < NDIG; ++d) o[d][0] = o[d][1] = o[d][2] = o[d][3] = 0u;
            if (j < N) {
                const int r = (int)(j & (BM - 1));
                const int64_t t = j / BM;
                const int swz = (r >> 2) & 1;
                const int64_t ch = q >> 3;
                const int qb = (int)(q & 7), h = qb >> 2;
                const uint32_t w = *reinterpret_cast<const uint32_t*>(
                    blk2 + (((t * nch2 + ch) * BM + r) * 2 + (h ^ swz)) * 16 + (qb & 3) * 4);
#pragma unroll
                for (int wq = 0; wq < 4; ++wq) {   // output word wq: positions 4 wq .. 4 wq + 3
                    uint4 e[4];
#pragma unroll
                    for (int b = 0; b < 4; ++b) {
                        const int P = 4 * wq + b;
                        const int m = 4 * (P & 3) + (P >> 2);
                        const int code = (int)((w >> (2 * m)) & 3u);
                        e[b] = te[m * 4 + code];
                        const float2 cv = tc[m * 4 + code];
                        df_add(ah, al, cv.x, cv.y);
                    }
#pragma unroll
                    for (int d = 0; d < 4; ++d) o[d][wq] = gather_byte(e[0].x, e[1].x, e[2].x, e[3].x, d);
#pragma unroll
                    for (int d = 4; d < 8; ++d) o[d][wq] = gather_byte(e[0].y, e[1].y, e[2].y, e[3].y, d - 4);
                    o[8][wq] = gather_byte(e[0].z, e[1].z, e[2].z, e[3].z, 0);
                }
            }
#pragma unroll
            for (int d = 0; d < NDIG; ++d)
                *reinterpret_cast<uint4*>(Dc + d * kpad + (q << 4)) = make_uint4(o[d][0], o[d][1], o[d][2], o[d][3]);
        }
        double acc = (double)ah + (double)al;
        for (int o2 = 16; o2 > 0; o2 >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o2);
        if (lane == 0) part[(int64_t)blockIdx.y * ncols + jj] = acc;
    }
}

// C2[jj] = sum over the SNP ranges of the centring partials, in range order
__global__ void k_grm_c2(const double* __restrict__ part, int nqb, int ncols, double* __restrict__ C2) {
    const int jj = blockIdx.x * blockDim.x + threadIdx.x;
    if (jj >= ncols) return;
    double a = 0.0;
    for (int y = 0; y < nqb; ++y) a += part[(int64_t)y * ncols + jj];
    C2[jj] = a;
}

// A_ij = (2^e sum_d 32^-d P_d(i, j) - C2_j) (1/M) rounded to float32, for the rows
// i = j0 + 32 blockIdx.x .. + 31 of group z = blockIdx.y (j0 = jb + z GRM_KG) and its
// columns j <= i; written to lt[i(i+1)/2 + j].  Values pass through shared memory so the
// row-contiguous writes of the packed triangle are coalesced.
__global__ void __launch_bounds__(256) k_grm_combine(const float* __restrict__ part, int nsplit, int64_t ldp,
                                                     int64_t pz, int32_t N, int jb, const double* __restrict__ C2,
                                                     const double* __restrict__ info, double inv_m,
                                                     float* __restrict__ lt) {
    __shared__ float sv[32][GRM_KG + 1];
    const int z = blockIdx.y;
    const int64_t j0 = (int64_t)jb + (int64_t)z * GRM_KG;
    const int64_t i0 = j0 + (int64_t)blockIdx.x * 32;
    if (j0 >= N || i0 >= N) return;
    double s_hi, s_lo;
    recombine_scales<NDIG>((int)info[0], s_hi, s_lo);
    const float* pzp = part + z * pz;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t i = i0 + lane;
    for (int c = warp; c < GRM_KG; c += 8) {
        float v = 0.0f;
        if (i < N && j0 + c < N)
            v = __double2float_rn((recombine<NDIG>(pzp, nsplit, GRM_NMMA, ldp, c, i, s_hi, s_lo) - C2[z * GRM_KG + c]) * inv_m);
        sv[lane][c] = v;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < 32 * GRM_KG; t += blockDim.x) {
        const int rr = t / GRM_KG, c = t % GRM_KG;
        const int64_t ii = i0 + rr, jj = j0 + c;
        if (ii < N && jj <= ii) lt[ii * (ii + 1) / 2 + jj] = sv[rr][c];
    }
}

// FP64: one CTA per 64 x 64 tile (ti, tj), tj <= ti, of the lower triangle; 256 threads,
// thread (ty, tx) holds rows ti*64 + ty + 16a and columns tj*64 + tx + 16b.  K runs over
// the SNP-major tile-blocked rows (blk1, tile codes) in chunks of 32 SNPs staged as zs
// values in shared memory.
__global__ void __launch_bounds__(256) k_grm_f64(const uint8_t* __restrict__ blk, int64_t Mk, int nch,
                                                 const double* __restrict__ zs, int32_t N, double M,
                                                 float* __restrict__ lt) {
    __shared__ double As[32][64], Bs[32][64];
    const int64_t b = blockIdx.x;
    int64_t ti = (int64_t)((sqrt(8.0 * (double)b + 1.0) - 1.0) * 0.5);
    while (ti * (ti + 1) / 2 > b) --ti;
    while ((ti + 1) * (ti + 2) / 2 <= b) ++ti;
    const int64_t tj = b - ti * (ti + 1) / 2;
    const int64_t ib = ti * 64, jbase = tj * 64;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[a][c] = 0.0;
    // loader: SNP ls = threadIdx.x / 8 of the chunk, individuals 8 * (threadIdx.x % 8) .. + 7
    const int ls = threadIdx.x >> 3, l8 = (threadIdx.x & 7) * 8;
    for (int64_t s0 = 0; s0 < Mk; s0 += 32) {
        const int64_t s = s0 + ls;
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const int64_t base = side ? jbase : ib;
            double(*dst)[64] = side ? Bs : As;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int64_t ind = base + l8 + q;
                double v = 0.0;
                if (s < Mk && ind < N) {
                    const unsigned code = (blk[blk_offset(s, ind >> 2, nch)] >> (2 * (ind & 3))) & 3u;
                    v = zs[s * 4 + tile_to_plink((int)code)];
                }
                dst[ls][l8 + q] = v;
            }
        }
        __syncthreads();
#pragma unroll 4
        for (int k = 0; k < 32; ++k) {
            double av[4], bv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) av[a] = As[k][ty + 16 * a];
#pragma unroll
            for (int c = 0; c < 4; ++c) bv[c] = Bs[k][tx + 16 * c];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[a][c] = fma(av[a], bv[c], acc[a][c]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int64_t i = ib + ty + 16 * a;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int64_t j = jbase + tx + 16 * c;
            if (i < N && j <= i) lt[i * (i + 1) / 2 + j] = __double2float_rn(acc[a][c] / M);
        }
    }
}

}  // namespace tc

using namespace tc;

// Temporary device buffers of one build, released on every exit path.
struct BuildBufs {
    globe_ctx* ctx;
    std::vector<void*> ps;
    explicit BuildBufs(globe_ctx* c) : ctx(c) {}
    template <class T>
    int get(T** p, size_t n) {
        int rc = dalloc(ctx, p, n);
        if (rc == GLOBE_OK) ps.push_back((void*)*p);
        return rc;
    }
    ~BuildBufs() {
        cudaStreamSynchronize(ctx->stream);
        for (void* p : ps) dfree(ctx, p);
    }
};

static int grm_build_tc(globe_ctx* ctx, float* lt) {
    auto& g = ctx->gen;
    const int32_t N = ctx->coh.N;
    GLOBE_RET(ensure_blk2(ctx));
    const int nch = g.nch2;
    const int64_t kpad = (int64_t)nch * BK;
    const int rpc = rows_per_cta(GRM_NMMA);
    const int tiles = (N + rpc - 1) / rpc;
    const int64_t ldp = (int64_t)tiles * rpc;
    const int splits = std::max(1, (nch + 4095) / 4096);   // K per CTA <= 2^19 (exact FP32 sums)
    const int spe = eff_splits(nch, splits);
    const int ngroups = (N + GRM_KG - 1) / GRM_KG;
    // groups per launch: digit operand + partials within ~2 GB
    const size_t per_group = (size_t)GRM_NMMA * kpad + (size_t)spe * GRM_NMMA * ldp * sizeof(float);
    size_t gfit = std::min<size_t>((size_t)ngroups, (size_t)65535);
    gfit = std::min<size_t>(gfit, ((size_t)2 << 30) / per_group);
    const int G = (int)std::max<size_t>(1, gfit);
    const int nbr = 304;
    BuildBufs B(ctx);
    double *U4, *C2, *info, *pm, *ps, *c2part;
    float2* c2v;
    uint4* dig;
    uint8_t* D;
    float* P;
    unsigned* err;
    GLOBE_RET(B.get(&U4, (size_t)4 * g.Mk));
    GLOBE_RET(B.get(&dig, (size_t)4 * kpad));
    GLOBE_RET(B.get(&c2v, (size_t)4 * kpad));
    GLOBE_RET(B.get(&C2, (size_t)G * GRM_KG));
    const int nqb = (int)((kpad / 16 + GD_Q - 1) / GD_Q);   // SNP ranges of k_grm_digits
    GLOBE_RET(B.get(&c2part, (size_t)nqb * G * GRM_KG));
    GLOBE_RET(B.get(&info, (size_t)2));
    GLOBE_RET(B.get(&pm, (size_t)nbr));
    GLOBE_RET(B.get(&ps, (size_t)nbr));
    GLOBE_RET(B.get(&D, (size_t)G * GRM_NMMA * kpad));
    GLOBE_RET(B.get(&P, (size_t)G * spe * GRM_NMMA * ldp));
    GLOBE_RET(tc_err_word(ctx, &err));
    // digit rows GRM_KG * NDIG .. GRM_NMMA - 1 of every group stay zero
    GLOBE_CK(ctx, cudaMemsetAsync(D, 0, (size_t)G * GRM_NMMA * kpad, ctx->stream));
    CUtensorMap mB;
    GLOBE_RET(make_map(ctx, &mB, D, (uint64_t)kpad, (uint64_t)G * GRM_NMMA, BK, (uint32_t)GRM_NMMA, true));
    {   // the digit kernel's staged table is above the default 48 KB (a per-device opt-in)
        static std::atomic<uint64_t> attr_set{0};
        const uint64_t bit = 1ull << (ctx->device & 63);
        if (!(attr_set.load() & bit)) {
            GLOBE_CK(ctx, cudaFuncSetAttribute(k_grm_digits, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)GD_SMEM));
            attr_set.fetch_or(bit);
        }
    }
    // digit table with one exponent for the whole matrix
    k_grm_u4<<<(unsigned)std::min<int64_t>(div_up(4 * g.Mk, 256), 4096), 256, 0, ctx->stream>>>(g.zs, g.inv, g.Mk,
                                                                                                 U4);
    GLOBE_LAUNCHED(ctx, "k_grm_u4");
    k_col_maxsum<<<dim3(nbr, 1), 256, 0, ctx->stream>>>(U4, 4 * g.Mk, 4 * g.Mk, pm, ps, nullptr, nullptr);
    GLOBE_LAUNCHED(ctx, "k_col_maxsum");
    k_col_finish<<<1, 128, 0, ctx->stream>>>(pm, ps, nbr, 1, info);
    GLOBE_LAUNCHED(ctx, "k_col_finish");
    k_grm_table<<<(unsigned)std::min<int64_t>(div_up(4 * kpad, 256), 4096), 256, 0, ctx->stream>>>(
        U4, g.f, g.Mk, kpad, info, dig, c2v);
    GLOBE_LAUNCHED(ctx, "k_grm_table");
    const int64_t pz = (int64_t)spe * GRM_NMMA * ldp;
    for (int jb = 0; jb < N; jb += G * GRM_KG) {
        const int gb = std::min(G, (N - jb + GRM_KG - 1) / GRM_KG);
        const int ncols = gb * GRM_KG;
        k_grm_digits<<<dim3((unsigned)div_up(ncols, GD_COLS), (unsigned)nqb), 256, GD_SMEM, ctx->stream>>>(
            g.blk2, nch, N, jb, ncols, dig, c2v, kpad, D, c2part);
        GLOBE_LAUNCHED(ctx, "k_grm_digits");
        k_grm_c2<<<div_up(ncols, 128), 128, 0, ctx->stream>>>(c2part, nqb, ncols, C2);
        GLOBE_LAUNCHED(ctx, "k_grm_c2");
        ZGrid zg;
        zg.nz = gb;
        zg.pz = pz;
        zg.skip0 = jb;
        zg.skipz = GRM_KG;
        {
            ProfScope p(ctx, GLOBE_PROF_GRM_BUILD_GEMM);
            GLOBE_RET(gemm_dispatch(ctx, GRM_NMMA, g.blk2, g.ntiles2, mB, N, nch, splits, P, ldp, err, zg));
        }
        k_grm_combine<<<dim3((unsigned)div_up(N - jb, 32), (unsigned)gb), 256, 0, ctx->stream>>>(
            P, spe, ldp, pz, N, jb, C2, info, 1.0 / (double)g.Mk, lt);
        GLOBE_LAUNCHED(ctx, "k_grm_combine");
    }
    return GLOBE_OK;
}

static int grm_build_f64(globe_ctx* ctx, float* lt) {
    auto& g = ctx->gen;
    const int32_t N = ctx->coh.N;
    const int64_t nt = (N + 63) / 64;
    const int64_t ntiles = nt * (nt + 1) / 2;
    if (ntiles > 0x7FFFFFFFll) return set_err(ctx, GLOBE_ERR_ARG, "N too large for the FP64 GRM build");
    GLOBE_RET(ensure_blk1(ctx));
    ProfScope p(ctx, GLOBE_PROF_GRM_BUILD_GEMM);
    k_grm_f64<<<(unsigned)ntiles, 256, 0, ctx->stream>>>(g.blk1, g.Mk, g.nch1, g.zs, N, (double)g.Mk, lt);
    GLOBE_LAUNCHED(ctx, "k_grm_f64");
    return GLOBE_OK;
}

}  // namespace globe

using namespace globe;

static int grm_ready(globe_ctx* ctx) {
    if (ctx->coh.N < 1 || ctx->gen.src != GSRC_GENO)
        return set_err(ctx, GLOBE_ERR_STATE, "load genotypes first (globe_load_bed / globe_load_bed_file)");
    if (ctx->gen.Mk < 1)
        return set_err(ctx, GLOBE_ERR_STATE, "no SNP passed the MAF / missingness filter: A = Zs'Zs / M is undefined");
    return GLOBE_OK;
}

extern "C" int globe_grm_build_dev(globe_ctx* ctx, float* d_lt) {
    if (!ctx) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    GLOBE_RET(grm_ready(ctx));
    if (!d_lt) return set_err(ctx, GLOBE_ERR_ARG, "globe_grm_build_dev: null output");
    ProfScope p(ctx, GLOBE_PROF_GRM_BUILD);
    if (ctx->prec == GLOBE_PREC_MIXED) return with_tc_check(ctx, GLOBE_PREC_MIXED, grm_build_tc(ctx, d_lt));
    return grm_build_f64(ctx, d_lt);
}

extern "C" int globe_grm_build(globe_ctx* ctx, float* lt) {
    if (!ctx) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    GLOBE_RET(grm_ready(ctx));
    if (!lt) return set_err(ctx, GLOBE_ERR_ARG, "globe_grm_build: null output");
    const int64_t N = ctx->coh.N;
    float* d = nullptr;
    GLOBE_RET(dalloc(ctx, &d, (size_t)(N * (N + 1) / 2)));
    int rc = globe_grm_build_dev(ctx, d);
    if (rc == GLOBE_OK) {
        cudaError_t e = cudaMemcpyAsync(lt, d, sizeof(float) * (size_t)(N * (N + 1) / 2), cudaMemcpyDeviceToHost,
                                        ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = cuda_err(ctx, e, "copy the GRM to the host");
    }
    cudaStreamSynchronize(ctx->stream);
    dfree(ctx, d);
    return rc;
}
