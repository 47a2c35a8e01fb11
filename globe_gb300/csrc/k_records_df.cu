// k_records_df.cu -- the record kernels of one block-PCG iteration in double-float.
//
// Under GLOBE_PREC_MIXED the record-level vectors of a solve (x, r, z, p, Vp) are held as
// double-float pairs (df.cuh), float2 in the 8 bytes of each double, from the end of the
// FP64 set-up to the end of the solve.  The three record kernels of an iteration then run
// on the FP32 pipe:
//   seg sums       p = z + beta p;  s0 = sum p, s1 = sum t p per individual  (J' p)
//   assemble       Vp = a0 + t a1 + sig2e p,  a0 = GZ + b0 s0 + b01 s1, a1 = b01 s0 + b1 s1
//   update         x += alpha p;  r -= alpha Vp;  z = Q^-1 r;  |r|^2, r'z
// the same operations as their FP64 forms in k_records.cu (PCGsolver.cpp:1095-1266 for V,
// :1014-1049 for Q), with the same two launch layouts (a thread per block of at most
// SHORT_BLOCK records, a warp per longer block).  What stays FP64: the GRM product's input
// (s0 is also written as double) and output (GZ), the preconditioner's 2x2 blocks (from
// which H is converted once per set of variance components), the per-column scalars, and
// every dot product past the CTA: p'Vp, |r|^2 and r'z are summed in double-float within a
// CTA and in FP64 across CTAs.
//
// Column c of the solve runs on s_c b_c (col_unscale): powers of two scale every value
// exactly, and keep the FP32 exponents near those of a unit right-hand side.
#include "df.cuh"
#include "records.cuh"

namespace globe {

using df::D;

// records per step of the thread-per-block loops: their loads issue together, ahead of the
// arithmetic, so that each thread keeps several loads in flight (the kernels wait on memory)
#ifndef REC_DF_RU
#define REC_DF_RU 4
#endif
constexpr int RU = REC_DF_RU;

struct VCdf {
    D e, b0, b01, b1;
};

// CTA sums of NQ double-float values per thread (thread-per-block layout), in double-float,
// then to FP64: sum over the CTA of v[j] -> part[blockIdx.x + q[j] * stride]
template <int NQ>
__device__ __forceinline__ void cta_sums_df(const D (&v)[NQ], const int (&q)[NQ], double* part, int stride) {
    __shared__ float2 sm[NQ][TB_THREADS / 32];
#pragma unroll
    for (int j = 0; j < NQ; ++j) {
        const D a = df::warp_sum(v[j]);
        if ((threadIdx.x & 31) == 0) df::store(&sm[j][threadIdx.x >> 5], a);
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < NQ; ++j) {
        if (threadIdx.x == j) {
            D a = df::zero();
#pragma unroll
            for (int w = 0; w < TB_THREADS / 32; ++w) a = df::add(a, df::load(&sm[j][w]));
            part[blockIdx.x + (size_t)q[j] * stride] = df::to_double(a);
        }
    }
}

// A column reduction finished inside a thread-per-block kernel when no warp-per-block launch
// contributes partials (no individual has more than SHORT_BLOCK records): the last of column
// c's CTAs (a per-column arrival count, zero between launches, reset by that CTA) sums the
// partials of quantity y < nq, part[y * S * kact + c * S + j], j < S, as k_reduce_cols would,
// into out[y][cols[c]]; with quot, quot[col] = num[col] / out[0][col] (0 where it is 0) and
// its double-float copy.
struct Fin {
    unsigned* cnt = nullptr;   // null: the host launches k_reduce_cols instead
    const int32_t* cols = nullptr;
    double* out[2] = {nullptr, nullptr};
    const double* num = nullptr;
    double* quot = nullptr;
    float2* quot_df = nullptr;
};

// every thread of the CTA calls it, after the CTA's partials are written
__device__ __forceinline__ void fin_last(const Fin& f, const double* part, int nq, int kact, int S) {
    __shared__ bool last;
    __shared__ double sm[256];
    const int c = blockIdx.y;
    if (threadIdx.x < nq) __threadfence();   // this CTA's partials (written by threads 0 .. nq-1), then its arrival
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&f.cnt[c], 1u) == gridDim.x - 1u;
    __syncthreads();
    if (!last) return;
    __threadfence();
    const int col = f.cols ? f.cols[c] : c;
    for (int y = 0; y < nq; ++y) {
        const double v = cta_reduce_256(part + (size_t)y * S * kact + (size_t)c * S, S, sm);
        if (threadIdx.x == 0) {
            f.out[y][col] = v;
            if (y == 0 && f.quot) {
                const double q = (v != 0.0) ? f.num[col] / v : 0.0;
                f.quot[col] = q;
                if (f.quot_df) df::store(f.quot_df + col, df::from_double(q));
            }
        }
    }
    if (threadIdx.x == 0) f.cnt[c] = 0u;
}

// ---------------------------------------------------------------------------
// Conversions

__global__ void k_to_df(const double* __restrict__ in, int64_t n, float2* __restrict__ out) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        df::store(out + e, df::from_double_scaled(in[e], 0));
}

// unsc[c] = col_unscale(bb[c]), once per solve
__global__ void k_col_unscale(const double* __restrict__ bb, int k, double* __restrict__ unsc) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < k) unsc[c] = col_unscale(bb[c]);
}

// 2^-e for the power of two u = 2^e, from its exponent bits
__device__ __forceinline__ int neg_exp2(double u) {
    return 1023 - (int)((__double_as_longlong(u) >> 52) & 0x7ff);
}

// column c (n rows, grid.y) of each pair with a destination: dst <- df(src / unsc[c]), src ==
// dst allowed (each element is read and written by one thread); rz[c] /= unsc[c]^2
__global__ void k_cols_to_df(DfCols v, int64_t n, const double* __restrict__ unsc, double* __restrict__ rz) {
    const int c = blockIdx.y;
    const int sh = neg_exp2(unsc[c]);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (!v.dst[j]) continue;
        const double* sc = v.src[j] + (size_t)c * n;
        float2* dc = reinterpret_cast<float2*>(v.dst[j] + (size_t)c * n);
        for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
            df::store(dc + e, df::from_double_scaled(sc[e], sh));
    }
    if (rz && blockIdx.x == 0 && threadIdx.x == 0) rz[c] = ldexp(rz[c], 2 * sh);
}

// in place, column c: v <- double(v) unsc[c]
__global__ void k_cols_from_df(double* v, int64_t n, const double* __restrict__ unsc) {
    const int c = blockIdx.y;
    const double u = unsc[c];
    double* vc = v + (size_t)c * n;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        vc[e] = df::to_double(df::load(reinterpret_cast<const float2*>(vc + e))) * u;
}

// CTAs per column of the conversions: ~4 elements per thread
static unsigned grid_for(int64_t n) {
    const int64_t b = (n + 1023) / 1024;
    return (unsigned)(b < 1 ? 1 : (b > 1024 ? 1024 : b));
}

int to_df(globe_ctx* ctx, const double* in, int64_t n, float2* out) {
    if (n < 1) return GLOBE_OK;
    k_to_df<<<grid_for(n), 256, 0, ctx->stream>>>(in, n, out);
    GLOBE_LAUNCHED(ctx, "k_to_df");
    return GLOBE_OK;
}

int col_unscales(globe_ctx* ctx, const double* bb, int k, double* unsc) {
    k_col_unscale<<<div_up(k, 128), 128, 0, ctx->stream>>>(bb, k, unsc);
    GLOBE_LAUNCHED(ctx, "k_col_unscale");
    return GLOBE_OK;
}

int cols_to_df(globe_ctx* ctx, const DfCols& v, int64_t n, int k, const double* unsc, double* rz) {
    k_cols_to_df<<<dim3(grid_for(n), k), 256, 0, ctx->stream>>>(v, n, unsc, rz);
    GLOBE_LAUNCHED(ctx, "k_cols_to_df");
    return GLOBE_OK;
}

int cols_from_df(globe_ctx* ctx, double* v, int64_t n, int k, const double* unsc) {
    k_cols_from_df<<<dim3(grid_for(n), k), 256, 0, ctx->stream>>>(v, n, unsc);
    GLOBE_LAUNCHED(ctx, "k_cols_from_df");
    return GLOBE_OK;
}

// ---------------------------------------------------------------------------
// Segment sums, optionally fused with p = z + beta p.  Zi (the GRM product's input) in
// FP64; S0, S1 (the assembly's) in double-float.  Column c of the outputs at i + c N.

__global__ void k_seg_sums_df_t(int32_t nblk, int64_t ld, int32_t N, const int32_t* __restrict__ bstart,
                                const int32_t* __restrict__ bind, const float2* __restrict__ t, float2* x,
                                const float2* __restrict__ z, const float2* __restrict__ beta,
                                const int32_t* __restrict__ cols, double* __restrict__ Zi, float2* __restrict__ S0,
                                float2* __restrict__ S1) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nblk) return;
    const int c = blockIdx.y;
    const int col = cols ? cols[c] : c;
    const int st = bstart[b], en = bstart[b + 1];
    if (!GLOBE_BOUNDS(st >= 0 && st <= en && en <= ld && bind[b] >= 0 && bind[b] < N, 0x0B01u)) return;
    if (en - st > SHORT_BLOCK) return;   // a warp per long block handles it
    float2* xc = x + (size_t)col * ld;
    D s0 = df::zero(), s1 = df::zero();
    if (beta) {
        const D bb = df::load(beta + col);
        const float2* zc = z + (size_t)col * ld;
        for (int r0 = st; r0 < en; r0 += RU) {   // the loads of RU records first, then the arithmetic
            D xv[RU], zv[RU], tv[RU];
#pragma unroll
            for (int u = 0; u < RU; ++u)
                if (r0 + u < en) {
                    xv[u] = df::load(xc + r0 + u);
                    zv[u] = df::load(zc + r0 + u);
                    tv[u] = df::load(t + r0 + u);
                }
#pragma unroll
            for (int u = 0; u < RU; ++u)
                if (r0 + u < en) {
                    const D v = df::madd(bb, xv[u], zv[u]);
                    df::store(xc + r0 + u, v);
                    s0 = df::add(s0, v);
                    s1 = df::madd(tv[u], v, s1);
                }
        }
    } else {
        for (int r0 = st; r0 < en; r0 += RU) {
            D xv[RU], tv[RU];
#pragma unroll
            for (int u = 0; u < RU; ++u)
                if (r0 + u < en) {
                    xv[u] = df::load(xc + r0 + u);
                    tv[u] = df::load(t + r0 + u);
                }
#pragma unroll
            for (int u = 0; u < RU; ++u)
                if (r0 + u < en) {
                    s0 = df::add(s0, xv[u]);
                    s1 = df::madd(tv[u], xv[u], s1);
                }
        }
    }
    const size_t o = (size_t)bind[b] + (size_t)c * N;
    Zi[o] = df::to_double(s0);
    df::store(S0 + o, s0);
    df::store(S1 + o, s1);
}

__global__ void k_seg_sums_df(int32_t nblk, int64_t ld, int32_t N, const int32_t* __restrict__ bstart,
                              const int32_t* __restrict__ bind, const float2* __restrict__ t, float2* x,
                              const float2* __restrict__ z, const float2* __restrict__ beta,
                              const int32_t* __restrict__ cols, int kact, double* __restrict__ Zi,
                              float2* __restrict__ S0, float2* __restrict__ S1, const int32_t* __restrict__ bl) {
    const int lane = threadIdx.x & 31;
    const int idx = blockIdx.x * RB_WARPS + (threadIdx.x >> 5);
    if (idx >= nblk) return;
    const int b = bl ? bl[idx] : idx;
    const int st = bstart[b], en = bstart[b + 1];
    const int i = bind[b];
    if (!GLOBE_BOUNDS(st >= 0 && st <= en && en <= ld && i >= 0 && i < N, 0x0C01u)) return;
    for (int c = 0; c < kact; ++c) {
        const int col = cols ? cols[c] : c;
        float2* xc = x + (size_t)col * ld;
        D s0 = df::zero(), s1 = df::zero();
        if (beta) {
            const D bb = df::load(beta + col);
            const float2* zc = z + (size_t)col * ld;
            for (int r = st + lane; r < en; r += 32) {
                const D v = df::madd(bb, df::load(xc + r), df::load(zc + r));
                df::store(xc + r, v);
                s0 = df::add(s0, v);
                s1 = df::madd(df::load(t + r), v, s1);
            }
        } else {
            for (int r = st + lane; r < en; r += 32) {
                const D v = df::load(xc + r);
                s0 = df::add(s0, v);
                s1 = df::madd(df::load(t + r), v, s1);
            }
        }
        s0 = df::warp_sum(s0);
        s1 = df::warp_sum(s1);
        if (lane == 0) {
            const size_t o = (size_t)i + (size_t)c * N;
            Zi[o] = df::to_double(s0);
            df::store(S0 + o, s0);
            df::store(S1 + o, s1);
        }
    }
}

int seg_sums_df(globe_ctx* ctx, float2* x, const float2* z, const float2* beta, const int32_t* cols, int kact,
                double* Zi, float2* S0, float2* S1) {
    auto& c = ctx->coh;
    const RecShape rs = rec_shape(ctx);
    k_seg_sums_df_t<<<dim3(rs.nbt, kact), TB_THREADS, 0, ctx->stream>>>(c.N, c.Nrec, c.N, c.bstart, c.bind, c.tdf, x,
                                                                          z, beta, cols, Zi, S0, S1);
    GLOBE_LAUNCHED(ctx, "k_seg_sums_df_t");
    if (rs.nbl) {
        k_seg_sums_df<<<rs.nbl, RB_THREADS, 0, ctx->stream>>>(c.nlong, c.Nrec, c.N, c.bstart, c.bind, c.tdf, x, z,
                                                               beta, cols, kact, Zi, S0, S1, c.lblk);
        GLOBE_LAUNCHED(ctx, "k_seg_sums_df");
    }
    return GLOBE_OK;
}

// ---------------------------------------------------------------------------
// out = J GZ + U D U' x + sig2e x, and the partial dots x'out

__global__ void k_vx_assemble_df_t(int32_t nblk, int64_t ld, int32_t N, const int32_t* __restrict__ bstart,
                                   const int32_t* __restrict__ bind, const float2* __restrict__ t, VCdf v,
                                   const float2* __restrict__ x, const double* __restrict__ GZ,
                                   const float2* __restrict__ S0, const float2* __restrict__ S1,
                                   const int32_t* __restrict__ cols, float2* __restrict__ out,
                                   double* __restrict__ part, int pstride, Fin fin) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    const int col = cols ? cols[c] : c;
    D dot[1] = {df::zero()};
    if (b < nblk && bstart[b + 1] - bstart[b] <= SHORT_BLOCK &&   // long blocks: a warp each
        GLOBE_BOUNDS(bstart[b] >= 0 && bstart[b + 1] <= ld && bind[b] >= 0 && bind[b] < N, 0x0D01u)) {
        const int st = bstart[b], en = bstart[b + 1];
        const size_t o = (size_t)bind[b] + (size_t)c * N;
        const D s0 = df::load(S0 + o), s1 = df::load(S1 + o);
        const D g = GZ ? df::from_double_scaled(GZ[o], 0) : df::zero();
        const D a0 = df::madd(v.b0, s0, df::madd(v.b01, s1, g));
        const D a1 = df::madd(v.b01, s0, df::mul(v.b1, s1));
        const float2* xc = x + (size_t)col * ld;
        float2* oc = out + (size_t)col * ld;
        for (int r0 = st; r0 < en; r0 += RU) {
            D xv[RU], tv[RU];
#pragma unroll
            for (int u = 0; u < RU; ++u)
                if (r0 + u < en) {
                    xv[u] = df::load(xc + r0 + u);
                    tv[u] = df::load(t + r0 + u);
                }
#pragma unroll
            for (int u = 0; u < RU; ++u)
                if (r0 + u < en) {
                    const D ov = df::madd(v.e, xv[u], df::madd(tv[u], a1, a0));
                    df::store(oc + r0 + u, ov);
                    dot[0] = df::madd(xv[u], ov, dot[0]);
                }
        }
    }
    if (part) {
        const int q[1] = {c};
        cta_sums_df<1>(dot, q, part, pstride);
        if (fin.cnt) fin_last(fin, part, 1, 0, pstride);
    }
}

__global__ void k_vx_assemble_df(int32_t nblk, int64_t ld, int32_t N, const int32_t* __restrict__ bstart,
                                 const int32_t* __restrict__ bind, const float2* __restrict__ t, VCdf v,
                                 const float2* __restrict__ x, const double* __restrict__ GZ,
                                 const float2* __restrict__ S0, const float2* __restrict__ S1,
                                 const int32_t* __restrict__ cols, int kact, float2* __restrict__ out,
                                 double* __restrict__ part, const int32_t* __restrict__ bl, int slot0, int pstride) {
    __shared__ double sm[RCH * RB_WARPS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int idx = blockIdx.x * RB_WARPS + warp;
    const bool live = idx < nblk;
    const int b = live ? (bl ? bl[idx] : idx) : 0;
    int st = 0, en = 0, i = 0;
    if (live) { st = bstart[b]; en = bstart[b + 1]; i = bind[b]; }
    if (live && !GLOBE_BOUNDS(st >= 0 && st <= en && en <= ld && i >= 0 && i < N, 0x0E01u)) st = en = i = 0;
    for (int c0 = 0; c0 < kact; c0 += RCH) {
        const int nc = min(RCH, kact - c0);
        for (int cc = 0; cc < nc; ++cc) {
            const int c = c0 + cc;
            const int col = cols ? cols[c] : c;
            D dot = df::zero();
            if (live) {
                const size_t o = (size_t)i + (size_t)c * N;
                const D s0 = df::load(S0 + o), s1 = df::load(S1 + o);
                const D g = GZ ? df::from_double_scaled(GZ[o], 0) : df::zero();
                const D a0 = df::madd(v.b0, s0, df::madd(v.b01, s1, g));
                const D a1 = df::madd(v.b01, s0, df::mul(v.b1, s1));
                const float2* xc = x + (size_t)col * ld;
                float2* oc = out + (size_t)col * ld;
                for (int r = st + lane; r < en; r += 32) {
                    const D xv = df::load(xc + r);
                    const D ov = df::madd(v.e, xv, df::madd(df::load(t + r), a1, a0));
                    df::store(oc + r, ov);
                    dot = df::madd(xv, ov, dot);
                }
            }
            if (part) {
                dot = df::warp_sum(dot);
                if (lane == 0) sm[cc * RB_WARPS + warp] = df::to_double(dot);
            }
        }
        if (part) flush_chunk(sm, 1, nc, c0, kact, part, slot0 + blockIdx.x, pstride);
    }
}

static VCdf vc_df(const globe_ctx* ctx) {
    VCdf v;
    v.e = df::from_double_host(ctx->vc[0]);
    v.b0 = df::from_double_host(ctx->vc[2]);
    v.b01 = df::from_double_host(ctx->vc[3]);
    v.b1 = df::from_double_host(ctx->vc[4]);
    return v;
}

int vx_assemble_df(globe_ctx* ctx, const float2* x, const double* GZ, const float2* S0, const float2* S1,
                   const int32_t* cols, int kact, float2* out, double* dot_out, const double* num, double* quot,
                   float2* quot_df) {
    auto& c = ctx->coh;
    const VCdf v = vc_df(ctx);
    const RecShape rs = rec_shape(ctx);
    double* part = nullptr;
    if (dot_out) GLOBE_RET(ws(ctx, WS_PART, (size_t)rs.S * kact * 2, &part));
    Fin fin;   // no long blocks: the p'Vp reduction (and alpha) finish in the kernel
    if (dot_out && rs.nbl == 0) {
        GLOBE_RET(tc_counters(ctx, (size_t)kact, &fin.cnt));
        fin.cols = cols;
        fin.out[0] = dot_out;
        fin.num = num;
        fin.quot = quot;
        fin.quot_df = quot_df;
    }
    k_vx_assemble_df_t<<<dim3(rs.nbt, kact), TB_THREADS, 0, ctx->stream>>>(c.N, c.Nrec, c.N, c.bstart, c.bind, c.tdf,
                                                                             v, x, GZ, S0, S1, cols, out, part, rs.S,
                                                                             fin);
    GLOBE_LAUNCHED(ctx, "k_vx_assemble_df_t");
    if (rs.nbl) {
        k_vx_assemble_df<<<rs.nbl, RB_THREADS, 0, ctx->stream>>>(c.nlong, c.Nrec, c.N, c.bstart, c.bind, c.tdf, v, x,
                                                                   GZ, S0, S1, cols, kact, out, part, c.lblk, rs.nbt,
                                                                   rs.S);
        GLOBE_LAUNCHED(ctx, "k_vx_assemble_df");
    }
    if (dot_out && !fin.cnt) GLOBE_RET(reduce_cols_div(ctx, part, rs.S, kact, cols, dot_out, num, quot, quot_df));
    return GLOBE_OK;
}

// ---------------------------------------------------------------------------
// x += a p; r -= a Vp; z = Q^-1 r = r/sig2e - (g0 + g1 t)/sig2e; partial |r|^2 and r'z.

__global__ void k_pcg_update_df_t(int32_t nblk, int64_t ld, const int32_t* __restrict__ bstart,
                                  const float2* __restrict__ t, D inv_e, const float2* __restrict__ H,
                                  const float2* __restrict__ alpha, float2* __restrict__ x, float2* __restrict__ r,
                                  const float2* __restrict__ p, const float2* __restrict__ Vp,
                                  float2* __restrict__ z, const int32_t* __restrict__ cols, int kact,
                                  double* __restrict__ part, int pstride, Fin fin) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    const int col = cols ? cols[c] : c;
    D acc[2] = {df::zero(), df::zero()};   // |r|^2, r'z
    if (b < nblk && bstart[b + 1] - bstart[b] <= SHORT_BLOCK &&
        GLOBE_BOUNDS(bstart[b] >= 0 && bstart[b + 1] <= ld, 0x0F01u)) {
        const int st = bstart[b], en = bstart[b + 1];
        const D a = df::load(alpha + col), na = df::neg(a);
        float2* xc = x + (size_t)col * ld;
        float2* rc = r + (size_t)col * ld;
        const float2* pc = p + (size_t)col * ld;
        const float2* vc = Vp + (size_t)col * ld;
        D s0 = df::zero(), s1 = df::zero();
        for (int q0 = st; q0 < en; q0 += RU) {   // the loads of RU records first, then the arithmetic
            D pv[RU], xv[RU], vv[RU], rv[RU], tv[RU];
#pragma unroll
            for (int u = 0; u < RU; ++u)
                if (q0 + u < en) {
                    pv[u] = df::load(pc + q0 + u);
                    xv[u] = df::load(xc + q0 + u);
                    vv[u] = df::load(vc + q0 + u);
                    rv[u] = df::load(rc + q0 + u);
                    tv[u] = df::load(t + q0 + u);
                }
#pragma unroll
            for (int u = 0; u < RU; ++u)
                if (q0 + u < en) {
                    df::store(xc + q0 + u, df::madd(a, pv[u], xv[u]));
                    const D rn = df::madd(na, vv[u], rv[u]);
                    df::store(rc + q0 + u, rn);
                    acc[0] = df::madd(rn, rn, acc[0]);
                    s0 = df::add(s0, rn);
                    s1 = df::madd(tv[u], rn, s1);
                }
        }
        const float2* hb = H + 4 * (size_t)b;
        const D g0 = df::madd(df::load(hb), s0, df::mul(df::load(hb + 1), s1));
        const D g1 = df::madd(df::load(hb + 2), s0, df::mul(df::load(hb + 3), s1));
        const D g0e = df::mul(g0, inv_e), g1e = df::mul(g1, inv_e);
        float2* zc = z + (size_t)col * ld;
        for (int q0 = st; q0 < en; q0 += RU) {
            D rv[RU], tv[RU];
#pragma unroll
            for (int u = 0; u < RU; ++u)
                if (q0 + u < en) {
                    rv[u] = df::load(rc + q0 + u);
                    tv[u] = df::load(t + q0 + u);
                }
#pragma unroll
            for (int u = 0; u < RU; ++u)
                if (q0 + u < en) {
                    const D zv = df::sub(df::mul(rv[u], inv_e), df::madd(g1e, tv[u], g0e));
                    df::store(zc + q0 + u, zv);
                    acc[1] = df::madd(rv[u], zv, acc[1]);
                }
        }
    }
    const int qi[2] = {c, kact + c};
    cta_sums_df<2>(acc, qi, part, pstride);
    if (fin.cnt) fin_last(fin, part, 2, kact, pstride);
}

__global__ void k_pcg_update_df(int32_t nblk, int64_t ld, const int32_t* __restrict__ bstart,
                                const float2* __restrict__ t, D inv_e, const float2* __restrict__ H,
                                const float2* __restrict__ alpha, float2* __restrict__ x, float2* __restrict__ r,
                                const float2* __restrict__ p, const float2* __restrict__ Vp, float2* __restrict__ z,
                                const int32_t* __restrict__ cols, int kact, double* __restrict__ part,
                                const int32_t* __restrict__ bl, int slot0, int pstride) {
    __shared__ double sm[2 * RCH * RB_WARPS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int idx = blockIdx.x * RB_WARPS + warp;
    const bool live = idx < nblk;
    const int b = live ? (bl ? bl[idx] : idx) : 0;
    int st = 0, en = 0;
    D h00 = df::zero(), h01 = df::zero(), h10 = df::zero(), h11 = df::zero();
    if (live) {
        st = bstart[b];
        en = bstart[b + 1];
        h00 = df::load(H + 4 * (size_t)b);
        h01 = df::load(H + 4 * (size_t)b + 1);
        h10 = df::load(H + 4 * (size_t)b + 2);
        h11 = df::load(H + 4 * (size_t)b + 3);
        if (!GLOBE_BOUNDS(st >= 0 && st <= en && en <= ld, 0x1001u)) st = en = 0;
    }
    for (int c0 = 0; c0 < kact; c0 += RCH) {
        const int nc = min(RCH, kact - c0);
        for (int cc = 0; cc < nc; ++cc) {
            const int c = c0 + cc;
            const int col = cols ? cols[c] : c;
            D rr = df::zero(), rz = df::zero();
            if (live) {
                const D a = df::load(alpha + col), na = df::neg(a);
                float2* xc = x + (size_t)col * ld;
                float2* rc = r + (size_t)col * ld;
                const float2* pc = p + (size_t)col * ld;
                const float2* vc = Vp + (size_t)col * ld;
                D s0 = df::zero(), s1 = df::zero();
                for (int q = st + lane; q < en; q += 32) {
                    df::store(xc + q, df::madd(a, df::load(pc + q), df::load(xc + q)));
                    const D rn = df::madd(na, df::load(vc + q), df::load(rc + q));
                    df::store(rc + q, rn);
                    rr = df::madd(rn, rn, rr);
                    s0 = df::add(s0, rn);
                    s1 = df::madd(df::load(t + q), rn, s1);
                }
                s0 = df::warp_sum(s0);
                s1 = df::warp_sum(s1);
                const D g0 = df::madd(h00, s0, df::mul(h01, s1)), g1 = df::madd(h10, s0, df::mul(h11, s1));
                const D g0e = df::mul(g0, inv_e), g1e = df::mul(g1, inv_e);
                float2* zc = z + (size_t)col * ld;
                for (int q = st + lane; q < en; q += 32) {
                    const D rn = df::load(rc + q);
                    const D zv = df::sub(df::mul(rn, inv_e), df::madd(g1e, df::load(t + q), g0e));
                    df::store(zc + q, zv);
                    rz = df::madd(rn, zv, rz);
                }
            }
            rr = df::warp_sum(rr);
            rz = df::warp_sum(rz);
            if (lane == 0) {
                sm[cc * RB_WARPS + warp] = df::to_double(rr);
                sm[(RCH + cc) * RB_WARPS + warp] = df::to_double(rz);
            }
        }
        flush_chunk(sm, 2, nc, c0, kact, part, slot0 + blockIdx.x, pstride);
    }
}

int pcg_update_df(globe_ctx* ctx, const float2* H, const float2* alpha, float2* x, float2* r, const float2* p,
                  const float2* Vp, float2* z, const int32_t* cols, int kact, double* rr, double* rz) {
    auto& c = ctx->coh;
    const RecShape rs = rec_shape(ctx);
    const D inv_e = df::from_double_host(1.0 / ctx->vc[0]);
    double* part;
    GLOBE_RET(ws(ctx, WS_PART, (size_t)rs.S * kact * 2, &part));
    Fin fin;   // no long blocks: the r'r and r'z reductions finish in the kernel
    if (rs.nbl == 0) {
        GLOBE_RET(tc_counters(ctx, (size_t)kact, &fin.cnt));
        fin.cols = cols;
        fin.out[0] = rr;
        fin.out[1] = rz;
    }
    k_pcg_update_df_t<<<dim3(rs.nbt, kact), TB_THREADS, 0, ctx->stream>>>(c.N, c.Nrec, c.bstart, c.tdf, inv_e, H,
                                                                            alpha, x, r, p, Vp, z, cols, kact, part,
                                                                            rs.S, fin);
    GLOBE_LAUNCHED(ctx, "k_pcg_update_df_t");
    if (rs.nbl) {
        k_pcg_update_df<<<rs.nbl, RB_THREADS, 0, ctx->stream>>>(c.nlong, c.Nrec, c.bstart, c.tdf, inv_e, H, alpha, x,
                                                                  r, p, Vp, z, cols, kact, part, c.lblk, rs.nbt, rs.S);
        GLOBE_LAUNCHED(ctx, "k_pcg_update_df");
    }
    if (fin.cnt) return GLOBE_OK;
    return reduce_cols2(ctx, part, rs.S, kact, cols, rr, rz);
}

// ---------------------------------------------------------------------------
// z = Q^-1 r and the partial r'z, every column (the solve's set-up from x0 = 0)

__global__ void k_precond_apply_df_t(int32_t nblk, int64_t ld, const int32_t* __restrict__ bstart,
                                     const float2* __restrict__ t, D inv_e, const float2* __restrict__ H,
                                     const float2* __restrict__ r, float2* __restrict__ z, double* __restrict__ part,
                                     int pstride) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    D rz[1] = {df::zero()};
    if (b < nblk && bstart[b + 1] - bstart[b] <= SHORT_BLOCK &&
        GLOBE_BOUNDS(bstart[b] >= 0 && bstart[b + 1] <= ld, 0x1101u)) {
        const int st = bstart[b], en = bstart[b + 1];
        const float2* rc = r + (size_t)c * ld;
        D s0 = df::zero(), s1 = df::zero();
        for (int q0 = st; q0 < en; q0 += RU) {
            D rv[RU], tv[RU];
#pragma unroll
            for (int u = 0; u < RU; ++u)
                if (q0 + u < en) {
                    rv[u] = df::load(rc + q0 + u);
                    tv[u] = df::load(t + q0 + u);
                }
#pragma unroll
            for (int u = 0; u < RU; ++u)
                if (q0 + u < en) {
                    s0 = df::add(s0, rv[u]);
                    s1 = df::madd(tv[u], rv[u], s1);
                }
        }
        const float2* hb = H + 4 * (size_t)b;
        const D g0 = df::madd(df::load(hb), s0, df::mul(df::load(hb + 1), s1));
        const D g1 = df::madd(df::load(hb + 2), s0, df::mul(df::load(hb + 3), s1));
        const D g0e = df::mul(g0, inv_e), g1e = df::mul(g1, inv_e);
        float2* zc = z + (size_t)c * ld;
        for (int q0 = st; q0 < en; q0 += RU) {
            D rv[RU], tv[RU];
#pragma unroll
            for (int u = 0; u < RU; ++u)
                if (q0 + u < en) {
                    rv[u] = df::load(rc + q0 + u);
                    tv[u] = df::load(t + q0 + u);
                }
#pragma unroll
            for (int u = 0; u < RU; ++u)
                if (q0 + u < en) {
                    const D zv = df::sub(df::mul(rv[u], inv_e), df::madd(g1e, tv[u], g0e));
                    df::store(zc + q0 + u, zv);
                    rz[0] = df::madd(rv[u], zv, rz[0]);
                }
        }
    }
    const int qi[1] = {c};
    cta_sums_df<1>(rz, qi, part, pstride);
}

__global__ void k_precond_apply_df(int32_t nblk, int64_t ld, const int32_t* __restrict__ bstart,
                                   const float2* __restrict__ t, D inv_e, const float2* __restrict__ H,
                                   const float2* __restrict__ r, float2* __restrict__ z, int k,
                                   double* __restrict__ part, const int32_t* __restrict__ bl, int slot0, int pstride) {
    __shared__ double sm[RCH * RB_WARPS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int idx = blockIdx.x * RB_WARPS + warp;
    const bool live = idx < nblk;
    const int b = live ? (bl ? bl[idx] : idx) : 0;
    int st = 0, en = 0;
    D h00 = df::zero(), h01 = df::zero(), h10 = df::zero(), h11 = df::zero();
    if (live) {
        st = bstart[b];
        en = bstart[b + 1];
        h00 = df::load(H + 4 * (size_t)b);
        h01 = df::load(H + 4 * (size_t)b + 1);
        h10 = df::load(H + 4 * (size_t)b + 2);
        h11 = df::load(H + 4 * (size_t)b + 3);
        if (!GLOBE_BOUNDS(st >= 0 && st <= en && en <= ld, 0x1201u)) st = en = 0;
    }
    for (int c0 = 0; c0 < k; c0 += RCH) {
        const int nc = min(RCH, k - c0);
        for (int cc = 0; cc < nc; ++cc) {
            const int c = c0 + cc;
            D rz = df::zero();
            if (live) {
                const float2* rc = r + (size_t)c * ld;
                D s0 = df::zero(), s1 = df::zero();
                for (int q = st + lane; q < en; q += 32) {
                    const D rv = df::load(rc + q);
                    s0 = df::add(s0, rv);
                    s1 = df::madd(df::load(t + q), rv, s1);
                }
                s0 = df::warp_sum(s0);
                s1 = df::warp_sum(s1);
                const D g0 = df::madd(h00, s0, df::mul(h01, s1)), g1 = df::madd(h10, s0, df::mul(h11, s1));
                const D g0e = df::mul(g0, inv_e), g1e = df::mul(g1, inv_e);
                float2* zc = z + (size_t)c * ld;
                for (int q = st + lane; q < en; q += 32) {
                    const D rv = df::load(rc + q);
                    const D zv = df::sub(df::mul(rv, inv_e), df::madd(g1e, df::load(t + q), g0e));
                    df::store(zc + q, zv);
                    rz = df::madd(rv, zv, rz);
                }
            }
            rz = df::warp_sum(rz);
            if (lane == 0) sm[cc * RB_WARPS + warp] = df::to_double(rz);
        }
        flush_chunk(sm, 1, nc, c0, k, part, slot0 + blockIdx.x, pstride);
    }
}

int precond_apply_df(globe_ctx* ctx, const float2* H, const float2* r, float2* z, int k, double* rz) {
    auto& c = ctx->coh;
    const RecShape rs = rec_shape(ctx);
    const D inv_e = df::from_double_host(1.0 / ctx->vc[0]);
    double* part;
    GLOBE_RET(ws(ctx, WS_PART, (size_t)rs.S * k * 2, &part));
    k_precond_apply_df_t<<<dim3(rs.nbt, k), TB_THREADS, 0, ctx->stream>>>(c.N, c.Nrec, c.bstart, c.tdf, inv_e, H, r,
                                                                            z, part, rs.S);
    GLOBE_LAUNCHED(ctx, "k_precond_apply_df_t");
    if (rs.nbl) {
        k_precond_apply_df<<<rs.nbl, RB_THREADS, 0, ctx->stream>>>(c.nlong, c.Nrec, c.bstart, c.tdf, inv_e, H, r, z,
                                                                    k, part, c.lblk, rs.nbt, rs.S);
        GLOBE_LAUNCHED(ctx, "k_precond_apply_df");
    }
    return reduce_cols(ctx, part, rs.S, k, nullptr, rz);
}

}  // namespace globe
