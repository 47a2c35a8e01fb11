// k_records.cu -- record-level kernels of the LGMM operator and block PCG.
//
// Records of one individual form one contiguous block.  All record-level
// work is per block, so segment sums, the 2x2 random intercept/slope term and
// the block preconditioner fuse without atomics.  Two layouts of the same
// kernels run side by side: one thread owns a (block, column) pair for blocks of
// at most SHORT_BLOCK records (grid.y = column); each longer block gets one warp
// that loops over the columns.
//
//   V x   = J (sig2g A J' x) + U D U' x + sig2e x          (PCGsolver.cpp:1095-1266)
//   U D U' x on block b = (D00 s0 + D01 s1) + t (D01 s0 + D11 s1),
//         s0 = sum x, s1 = sum t x  -- the O(n) form of the O(n^2) loop at
//         PCGsolver.cpp:1237-1254 (same matrix, different rounding).
//   Q_b = sig2e I + W C W', W = [1 t], C = D + diag(sig2g A_ii, 0): the block
//         of computePreconditioner_Block (PCGsolver.cpp:1014-1049).  Its
//         inverse by Woodbury: Q_b^-1 r = (r - W H W' r) / sig2e with
//         H = (sig2e I + C W'W)^-1 C, a 2x2 per individual.
//
// Reductions are deterministic: per-CTA partials, then a fixed-order reduce.
#include "df.cuh"
#include "records.cuh"

namespace globe {

// limits of precond_apply_scratch, which may set no kernel attribute: columns are
// grid rows (gridDim.y <= 65535), and dynamic shared memory stays at the default 48 KB
constexpr int NOALLOC_MAX_COLS = 65535;
constexpr size_t NOALLOC_SMEM_BYTES = 48 * 1024;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

struct VC {
    double e, g, b0, b01, b1;
};
__device__ __forceinline__ VC load_vc(const double* vc) { return VC{vc[0], vc[1], vc[2], vc[3], vc[4]}; }

// CTA-level reduction of per-warp values: vals[warp][q] -> part[slot + q*stride]
// smem layout: sm[q * RB_WARPS + warp]
__device__ __forceinline__ void cta_partials(double* sm, int nq, double* part, int slot, int stride) {
    __syncthreads();
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
        double a = 0.0;
#pragma unroll
        for (int w = 0; w < RB_WARPS; ++w) a += sm[q * RB_WARPS + w];
        part[slot + (size_t)q * stride] = a;
    }
}

// CTA sums of NQ values per thread (thread-per-block layout):
// sum over the CTA of v[j] -> part[blockIdx.x + q[j] * stride]
template <int NQ>
__device__ __forceinline__ void cta_sums(const double (&v)[NQ], const int (&q)[NQ], double* part, int stride) {
    __shared__ double sm[NQ][TB_THREADS / 32];
#pragma unroll
    for (int j = 0; j < NQ; ++j) {
        const double a = warp_sum(v[j]);
        if ((threadIdx.x & 31) == 0) sm[j][threadIdx.x >> 5] = a;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < NQ; ++j) {
        if (threadIdx.x == j) {
            double a = 0.0;
#pragma unroll
            for (int w = 0; w < TB_THREADS / 32; ++w) a += sm[j][w];
            part[blockIdx.x + (size_t)q[j] * stride] = a;
        }
    }
}

// ---------------------------------------------------------------------------

__global__ void k_block_moments(const int32_t* __restrict__ bstart, const double* __restrict__ t,
                                int32_t nblk, double* bn, double* bt, double* btt) {
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * RB_WARPS + (threadIdx.x >> 5);
    if (b >= nblk) return;
    const int st = bstart[b], en = bstart[b + 1];
    if (!GLOBE_BOUNDS(st >= 0 && st <= en, 0x0901u)) return;
    double s1 = 0, s2 = 0;
    for (int r = st + lane; r < en; r += 32) {
        double tr = t[r];
        s1 += tr;
        s2 += tr * tr;
    }
    s1 = warp_sum(s1);
    s2 = warp_sum(s2);
    if (lane == 0) {
        bn[b] = (double)(en - st);
        bt[b] = s1;
        btt[b] = s2;
    }
}

int block_moments(globe_ctx* ctx) {
    auto& c = ctx->coh;
    k_block_moments<<<div_up(c.N, RB_WARPS), RB_THREADS, 0, ctx->stream>>>(c.bstart, c.times(), c.N,
                                                                           c.bn, c.bt, c.btt);
    GLOBE_LAUNCHED(ctx, "k_block_moments");
    return GLOBE_OK;
}

// H_b = (sig2e I + C G)^-1 C,  C = [[b0 + g, b01], [b01, b1]],  G = [[n, St], [St, Stt]]
__global__ void k_build_H(int32_t nblk, const double* __restrict__ bn, const double* __restrict__ bt,
                          const double* __restrict__ btt, const int32_t* __restrict__ bind,
                          const double* __restrict__ gdiag, double gconst, VC v, double* __restrict__ H,
                          float2* __restrict__ Hdf) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nblk) return;
    if (gdiag && !GLOBE_BOUNDS(bind[b] >= 0 && bind[b] < nblk, 0x0A01u)) return;
    double g = gdiag ? v.g * gdiag[bind[b]] : gconst;
    double c00 = v.b0 + g, c01 = v.b01, c11 = v.b1;
    double g00 = bn[b], g01 = bt[b], g11 = btt[b];
    double m00 = v.e + c00 * g00 + c01 * g01;
    double m01 = c00 * g01 + c01 * g11;
    double m10 = c01 * g00 + c11 * g01;
    double m11 = v.e + c01 * g01 + c11 * g11;
    double det = m00 * m11 - m01 * m10;
    double i00 = m11 / det, i01 = -m01 / det, i10 = -m10 / det, i11 = m00 / det;
    const double h[4] = {i00 * c00 + i01 * c01, i00 * c01 + i01 * c11, i10 * c00 + i11 * c01,
                         i10 * c01 + i11 * c11};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        H[4 * b + j] = h[j];
        if (Hdf) df::store(Hdf + 4 * b + j, df::from_double(h[j]));   // the double-float record kernels' copy
    }
}

int build_H(globe_ctx* ctx, const double* gdiag, double gconst, double* H, float2* Hdf) {
    VC v{ctx->vc[0], ctx->vc[1], ctx->vc[2], ctx->vc[3], ctx->vc[4]};
    auto& c = ctx->coh;
    k_build_H<<<div_up(c.N, 128), 128, 0, ctx->stream>>>(c.N, c.bn, c.bt, c.btt, c.bind, gdiag, gconst, v, H, Hdf);
    GLOBE_LAUNCHED(ctx, "k_build_H");
    return GLOBE_OK;
}

// ---------------------------------------------------------------------------
// Segment sums (J' x and t-weighted), optionally fused with p = z + beta p.

__global__ void k_seg_sums(int32_t nblk, int64_t ld, int32_t N, const int32_t* __restrict__ bstart,
                           const int32_t* __restrict__ bind, const double* __restrict__ t,
                           double* x, const double* __restrict__ z, const double* __restrict__ beta,
                           const int32_t* __restrict__ cols, int kact, double* __restrict__ Zi,
                           double* __restrict__ S1, const int32_t* __restrict__ bl) {
    const int lane = threadIdx.x & 31;
    const int idx = blockIdx.x * RB_WARPS + (threadIdx.x >> 5);
    if (idx >= nblk) return;
    const int b = bl ? bl[idx] : idx;
    const int st = bstart[b], en = bstart[b + 1];
    const int i = bind[b];
    if (!GLOBE_BOUNDS(st >= 0 && st <= en && en <= ld && i >= 0 && i < N, 0x0101u)) return;
    for (int c = 0; c < kact; ++c) {
        const int col = cols ? cols[c] : c;
        double* xc = x + (size_t)col * ld;
        double s0 = 0, s1 = 0;
        if (beta) {
            const double bb = beta[col];
            const double* zc = z + (size_t)col * ld;
            for (int r = st + lane; r < en; r += 32) {
                double v = zc[r] + bb * xc[r];
                xc[r] = v;
                s0 += v;
                s1 += t[r] * v;
            }
        } else {
            for (int r = st + lane; r < en; r += 32) {
                double v = xc[r];
                s0 += v;
                s1 += t[r] * v;
            }
        }
        s0 = warp_sum(s0);
        s1 = warp_sum(s1);
        if (lane == 0) {
            Zi[i + (size_t)c * N] = s0;
            if (S1) S1[i + (size_t)c * N] = s1;
        }
    }
}

// thread-per-block layout: one thread per (block, column)
__global__ void k_seg_sums_t(int32_t nblk, int64_t ld, int32_t N, const int32_t* __restrict__ bstart,
                             const int32_t* __restrict__ bind, const double* __restrict__ t, double* x,
                             const double* __restrict__ z, const double* __restrict__ beta,
                             const int32_t* __restrict__ cols, double* __restrict__ Zi, double* __restrict__ S1) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nblk) return;
    const int c = blockIdx.y;
    const int col = cols ? cols[c] : c;
    const int st = bstart[b], en = bstart[b + 1];
    if (!GLOBE_BOUNDS(st >= 0 && st <= en && en <= ld && bind[b] >= 0 && bind[b] < N, 0x0201u)) return;
    if (en - st > SHORT_BLOCK) return;   // a warp per long block handles it
    double* xc = x + (size_t)col * ld;
    double s0 = 0, s1 = 0;
    if (beta) {
        const double bb = beta[col];
        const double* zc = z + (size_t)col * ld;
#pragma unroll 4
        for (int r = st; r < en; ++r) {
            const double v = zc[r] + bb * xc[r];
            xc[r] = v;
            s0 += v;
            s1 += t[r] * v;
        }
    } else {
#pragma unroll 4
        for (int r = st; r < en; ++r) {
            const double v = xc[r];
            s0 += v;
            s1 += t[r] * v;
        }
    }
    const int i = bind[b];
    Zi[i + (size_t)c * N] = s0;
    if (S1) S1[i + (size_t)c * N] = s1;
}

int seg_sums(globe_ctx* ctx, const double* x, const double* z, const double* beta, double* xout,
             const int32_t* cols, int kact, double* Zi, double* S1) {
    auto& c = ctx->coh;
    // in-place p update: xout must alias x when beta is given
    double* xx = beta ? xout : const_cast<double*>(x);
    const RecShape rs = rec_shape(ctx);
    k_seg_sums_t<<<dim3(rs.nbt, kact), TB_THREADS, 0, ctx->stream>>>(c.N, c.Nrec, c.N, c.bstart, c.bind, c.times(),
                                                                       xx, z, beta, cols, Zi, S1);
    GLOBE_LAUNCHED(ctx, "k_seg_sums_t");
    if (rs.nbl) {
        k_seg_sums<<<rs.nbl, RB_THREADS, 0, ctx->stream>>>(c.nlong, c.Nrec, c.N, c.bstart, c.bind, c.times(), xx, z,
                                                            beta, cols, kact, Zi, S1, c.lblk);
        GLOBE_LAUNCHED(ctx, "k_seg_sums");
    }
    return GLOBE_OK;
}

// ---------------------------------------------------------------------------
// out = J GZ + U D U' x + sig2e x  (+ per-column partial dot x'out)

__global__ void k_vx_assemble(int32_t nblk, int64_t ld, int32_t N, const int32_t* __restrict__ bstart,
                              const int32_t* __restrict__ bind, const double* __restrict__ t, VC v,
                              const double* __restrict__ x, const double* __restrict__ GZ,
                              const double* __restrict__ Zi, const double* __restrict__ S1,
                              const int32_t* __restrict__ cols, int kact, double* __restrict__ out,
                              double* __restrict__ part, const int32_t* __restrict__ bl, int slot0, int pstride) {
    __shared__ double sm[RCH * RB_WARPS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int idx = blockIdx.x * RB_WARPS + warp;
    const bool live = idx < nblk;
    const int b = live ? (bl ? bl[idx] : idx) : 0;
    int st = 0, en = 0, i = 0;
    if (live) { st = bstart[b]; en = bstart[b + 1]; i = bind[b]; }
    if (live && !GLOBE_BOUNDS(st >= 0 && st <= en && en <= ld && i >= 0 && i < N, 0x0301u)) st = en = i = 0;
    for (int c0 = 0; c0 < kact; c0 += RCH) {
        const int nc = min(RCH, kact - c0);
        for (int cc = 0; cc < nc; ++cc) {
            const int c = c0 + cc;
            const int col = cols ? cols[c] : c;
            double dot = 0;
            if (live) {
                const double s0 = Zi[i + (size_t)c * N], s1 = S1[i + (size_t)c * N];
                const double g = GZ ? GZ[i + (size_t)c * N] : 0.0;
                const double a0 = g + v.b0 * s0 + v.b01 * s1;
                const double a1 = v.b01 * s0 + v.b1 * s1;
                const double* xc = x + (size_t)col * ld;
                double* oc = out + (size_t)col * ld;
                for (int r = st + lane; r < en; r += 32) {
                    double xv = xc[r];
                    double o = a0 + t[r] * a1 + v.e * xv;
                    oc[r] = o;
                    dot += xv * o;
                }
            }
            if (part) {
                dot = warp_sum(dot);
                if (lane == 0) sm[cc * RB_WARPS + warp] = dot;
            }
        }
        if (part) flush_chunk(sm, 1, nc, c0, kact, part, slot0 + blockIdx.x, pstride);
    }
}

__global__ void k_vx_assemble_t(int32_t nblk, int64_t ld, int32_t N, const int32_t* __restrict__ bstart,
                                const int32_t* __restrict__ bind, const double* __restrict__ t, VC v,
                                const double* __restrict__ x, const double* __restrict__ GZ,
                                const double* __restrict__ Zi, const double* __restrict__ S1,
                                const int32_t* __restrict__ cols, double* __restrict__ out,
                                double* __restrict__ part, int pstride) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    const int col = cols ? cols[c] : c;
    double dot[1] = {0.0};
    if (b < nblk && bstart[b + 1] - bstart[b] <= SHORT_BLOCK &&   // long blocks: a warp each
        GLOBE_BOUNDS(bstart[b] >= 0 && bstart[b + 1] <= ld && bind[b] >= 0 && bind[b] < N, 0x0401u)) {
        const int st = bstart[b], en = bstart[b + 1], i = bind[b];
        const double s0 = Zi[i + (size_t)c * N], s1 = S1[i + (size_t)c * N];
        const double g = GZ ? GZ[i + (size_t)c * N] : 0.0;
        const double a0 = g + v.b0 * s0 + v.b01 * s1;
        const double a1 = v.b01 * s0 + v.b1 * s1;
        const double* xc = x + (size_t)col * ld;
        double* oc = out + (size_t)col * ld;
#pragma unroll 4
        for (int r = st; r < en; ++r) {
            const double xv = xc[r];
            const double o = a0 + t[r] * a1 + v.e * xv;
            oc[r] = o;
            dot[0] += xv * o;
        }
    }
    if (part) {
        const int q[1] = {c};
        cta_sums<1>(dot, q, part, pstride);
    }
}

int vx_assemble(globe_ctx* ctx, const double* x, const double* GZ, const double* Zi, const double* S1,
                const int32_t* cols, int kact, double* out, double* dot_out, const double* num, double* quot) {
    auto& c = ctx->coh;
    VC v{ctx->vc[0], ctx->vc[1], ctx->vc[2], ctx->vc[3], ctx->vc[4]};
    const RecShape rs = rec_shape(ctx);
    double* part = nullptr;
    if (dot_out) GLOBE_RET(ws(ctx, WS_PART, (size_t)rs.S * kact * 2, &part));
    k_vx_assemble_t<<<dim3(rs.nbt, kact), TB_THREADS, 0, ctx->stream>>>(c.N, c.Nrec, c.N, c.bstart, c.bind, c.times(),
                                                                          v, x, GZ, Zi, S1, cols, out, part, rs.S);
    GLOBE_LAUNCHED(ctx, "k_vx_assemble_t");
    if (rs.nbl) {
        k_vx_assemble<<<rs.nbl, RB_THREADS, 0, ctx->stream>>>(c.nlong, c.Nrec, c.N, c.bstart, c.bind, c.times(), v,
                                                                x, GZ, Zi, S1, cols, kact, out, part, c.lblk, rs.nbt,
                                                                rs.S);
        GLOBE_LAUNCHED(ctx, "k_vx_assemble");
    }
    if (dot_out) GLOBE_RET(reduce_cols_div(ctx, part, rs.S, kact, cols, dot_out, num, quot, nullptr));
    return GLOBE_OK;
}

// ---------------------------------------------------------------------------
// x += a p; r -= a Vp; z = Q^-1 r; partial |r|^2 and r'z.

__global__ void k_pcg_update(int32_t nblk, int64_t ld, const int32_t* __restrict__ bstart,
                             const double* __restrict__ t, double inv_e, const double* __restrict__ H,
                             const double* __restrict__ alpha, double* __restrict__ x, double* __restrict__ r,
                             const double* __restrict__ p, const double* __restrict__ Vp,
                             double* __restrict__ z, const int32_t* __restrict__ cols, int kact,
                             double* __restrict__ part, const int32_t* __restrict__ bl, int slot0, int pstride) {
    __shared__ double sm[2 * RCH * RB_WARPS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int idx = blockIdx.x * RB_WARPS + warp;
    const bool live = idx < nblk;
    const int b = live ? (bl ? bl[idx] : idx) : 0;
    int st = 0, en = 0;
    double h00 = 0, h01 = 0, h10 = 0, h11 = 0;
    if (live) {
        st = bstart[b];
        en = bstart[b + 1];
        h00 = H[4 * b];
        h01 = H[4 * b + 1];
        h10 = H[4 * b + 2];
        h11 = H[4 * b + 3];
        if (!GLOBE_BOUNDS(st >= 0 && st <= en && en <= ld, 0x0501u)) st = en = 0;
    }
    for (int c0 = 0; c0 < kact; c0 += RCH) {
        const int nc = min(RCH, kact - c0);
        for (int cc = 0; cc < nc; ++cc) {
            const int c = c0 + cc;
            const int col = cols ? cols[c] : c;
            double rr = 0, rz = 0;
            if (live) {
                const double a = alpha[col];
                double* xc = x + (size_t)col * ld;
                double* rc = r + (size_t)col * ld;
                const double* pc = p + (size_t)col * ld;
                const double* vc = Vp + (size_t)col * ld;
                double s0 = 0, s1 = 0;
                for (int q = st + lane; q < en; q += 32) {
                    xc[q] += a * pc[q];
                    double rn = rc[q] - a * vc[q];
                    rc[q] = rn;
                    rr += rn * rn;
                    s0 += rn;
                    s1 += t[q] * rn;
                }
                s0 = warp_sum(s0);
                s1 = warp_sum(s1);
                const double g0 = h00 * s0 + h01 * s1, g1 = h10 * s0 + h11 * s1;
                const double g0e = g0 * inv_e, g1e = g1 * inv_e;   // z = r/sig2e - (g0 + g1 t)/sig2e
                double* zc = z + (size_t)col * ld;
                for (int q = st + lane; q < en; q += 32) {
                    double rn = rc[q];
                    double zv = fma(rn, inv_e, -fma(g1e, t[q], g0e));
                    zc[q] = zv;
                    rz += rn * zv;
                }
            }
            rr = warp_sum(rr);
            rz = warp_sum(rz);
            if (lane == 0) {
                sm[cc * RB_WARPS + warp] = rr;
                sm[(RCH + cc) * RB_WARPS + warp] = rz;
            }
        }
        flush_chunk(sm, 2, nc, c0, kact, part, slot0 + blockIdx.x, pstride);
    }
}

__global__ void k_pcg_update_t(int32_t nblk, int64_t ld, const int32_t* __restrict__ bstart,
                               const double* __restrict__ t, double inv_e, const double* __restrict__ H,
                               const double* __restrict__ alpha, double* __restrict__ x, double* __restrict__ r,
                               const double* __restrict__ p, const double* __restrict__ Vp, double* __restrict__ z,
                               const int32_t* __restrict__ cols, int kact, double* __restrict__ part,
                               int pstride) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    const int col = cols ? cols[c] : c;
    double acc[2] = {0.0, 0.0};   // |r|^2, r'z
    if (b < nblk && bstart[b + 1] - bstart[b] <= SHORT_BLOCK &&
        GLOBE_BOUNDS(bstart[b] >= 0 && bstart[b + 1] <= ld, 0x0601u)) {
        const int st = bstart[b], en = bstart[b + 1];
        const double a = alpha[col];
        double* xc = x + (size_t)col * ld;
        double* rc = r + (size_t)col * ld;
        const double* pc = p + (size_t)col * ld;
        const double* vc = Vp + (size_t)col * ld;
        double s0 = 0, s1 = 0;
#pragma unroll 4
        for (int q = st; q < en; ++q) {
            xc[q] += a * pc[q];
            const double rn = rc[q] - a * vc[q];
            rc[q] = rn;
            acc[0] += rn * rn;
            s0 += rn;
            s1 += t[q] * rn;
        }
        const double g0 = H[4 * b] * s0 + H[4 * b + 1] * s1, g1 = H[4 * b + 2] * s0 + H[4 * b + 3] * s1;
        const double g0e = g0 * inv_e, g1e = g1 * inv_e;   // z = r/sig2e - (g0 + g1 t)/sig2e
        double* zc = z + (size_t)col * ld;
#pragma unroll 4
        for (int q = st; q < en; ++q) {
            const double rn = rc[q];
            const double zv = fma(rn, inv_e, -fma(g1e, t[q], g0e));
            zc[q] = zv;
            acc[1] += rn * zv;
        }
    }
    const int qi[2] = {c, kact + c};
    cta_sums<2>(acc, qi, part, pstride);
}

int pcg_update(globe_ctx* ctx, const double* H, const double* alpha, double* x, double* r, const double* p,
               const double* Vp, double* z, const int32_t* cols, int kact, double* rr, double* rz) {
    auto& c = ctx->coh;
    const RecShape rs = rec_shape(ctx);
    double* part;
    GLOBE_RET(ws(ctx, WS_PART, (size_t)rs.S * kact * 2, &part));
    k_pcg_update_t<<<dim3(rs.nbt, kact), TB_THREADS, 0, ctx->stream>>>(c.N, c.Nrec, c.bstart, c.times(),
                                                                         1.0 / ctx->vc[0], H, alpha, x, r, p, Vp, z,
                                                                         cols, kact, part, rs.S);
    GLOBE_LAUNCHED(ctx, "k_pcg_update_t");
    if (rs.nbl) {
        k_pcg_update<<<rs.nbl, RB_THREADS, 0, ctx->stream>>>(c.nlong, c.Nrec, c.bstart, c.times(), 1.0 / ctx->vc[0],
                                                               H, alpha, x, r, p, Vp, z, cols, kact, part, c.lblk,
                                                               rs.nbt, rs.S);
        GLOBE_LAUNCHED(ctx, "k_pcg_update");
    }
    return reduce_cols2(ctx, part, rs.S, kact, cols, rr, rz);
}

// z = Q^-1 r (+ partial r'z)
__global__ void k_precond_apply(int32_t nblk, int64_t ld, const int32_t* __restrict__ bstart,
                                const double* __restrict__ t, double inv_e, const double* __restrict__ H,
                                const double* __restrict__ r, double* __restrict__ z,
                                const int32_t* __restrict__ cols, int kact, double* __restrict__ part,
                                const int32_t* __restrict__ bl, int slot0, int pstride) {
    extern __shared__ double sm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int idx = blockIdx.x * RB_WARPS + warp;
    const bool live = idx < nblk;
    const int b = live ? (bl ? bl[idx] : idx) : 0;
    int st = 0, en = 0;
    double h00 = 0, h01 = 0, h10 = 0, h11 = 0;
    if (live) {
        st = bstart[b];
        en = bstart[b + 1];
        h00 = H[4 * b];
        h01 = H[4 * b + 1];
        h10 = H[4 * b + 2];
        h11 = H[4 * b + 3];
        if (!GLOBE_BOUNDS(st >= 0 && st <= en && en <= ld, 0x0701u)) st = en = 0;
    }
    for (int c = 0; c < kact; ++c) {
        const int col = cols ? cols[c] : c;
        double rz = 0;
        if (live) {
            const double* rc = r + (size_t)col * ld;
            double s0 = 0, s1 = 0;
            for (int q = st + lane; q < en; q += 32) {
                s0 += rc[q];
                s1 += t[q] * rc[q];
            }
            s0 = warp_sum(s0);
            s1 = warp_sum(s1);
            const double g0 = h00 * s0 + h01 * s1, g1 = h10 * s0 + h11 * s1;
            const double g0e = g0 * inv_e, g1e = g1 * inv_e;   // z = r/sig2e - (g0 + g1 t)/sig2e
            double* zc = z + (size_t)col * ld;
            for (int q = st + lane; q < en; q += 32) {
                double zv = fma(rc[q], inv_e, -fma(g1e, t[q], g0e));
                zc[q] = zv;
                rz += rc[q] * zv;
            }
        }
        if (part) {
            rz = warp_sum(rz);
            if (lane == 0) sm[c * RB_WARPS + warp] = rz;
        }
    }
    if (part) cta_partials(sm, kact, part, slot0 + blockIdx.x, pstride);
}

__global__ void k_precond_apply_t(int32_t nblk, int64_t ld, const int32_t* __restrict__ bstart,
                                  const double* __restrict__ t, double inv_e, const double* __restrict__ H,
                                  const double* __restrict__ r, double* __restrict__ z,
                                  const int32_t* __restrict__ cols, double* __restrict__ part, int pstride) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    const int col = cols ? cols[c] : c;
    double rz[1] = {0.0};
    if (b < nblk && bstart[b + 1] - bstart[b] <= SHORT_BLOCK &&
        GLOBE_BOUNDS(bstart[b] >= 0 && bstart[b + 1] <= ld, 0x0801u)) {
        const int st = bstart[b], en = bstart[b + 1];
        const double* rc = r + (size_t)col * ld;
        double s0 = 0, s1 = 0;
#pragma unroll 4
        for (int q = st; q < en; ++q) {
            s0 += rc[q];
            s1 += t[q] * rc[q];
        }
        const double g0 = H[4 * b] * s0 + H[4 * b + 1] * s1, g1 = H[4 * b + 2] * s0 + H[4 * b + 3] * s1;
        const double g0e = g0 * inv_e, g1e = g1 * inv_e;   // z = r/sig2e - (g0 + g1 t)/sig2e
        double* zc = z + (size_t)col * ld;
#pragma unroll 4
        for (int q = st; q < en; ++q) {
            const double zv = fma(rc[q], inv_e, -fma(g1e, t[q], g0e));
            zc[q] = zv;
            rz[0] += rc[q] * zv;
        }
    }
    if (part) {
        const int qi[1] = {c};
        cta_sums<1>(rz, qi, part, pstride);
    }
}

// z = Q^-1 r (+ r'z partials into part[slot + c * rs.S]): one thread per short block,
// one warp per long block
static int precond_launch(globe_ctx* ctx, const double* H, const double* r, double* z, const int32_t* cols, int kact,
                          double* part, const RecShape& rs) {
    auto& c = ctx->coh;
    k_precond_apply_t<<<dim3(rs.nbt, kact), TB_THREADS, 0, ctx->stream>>>(c.N, c.Nrec, c.bstart, c.times(),
                                                                            1.0 / ctx->vc[0], H, r, z, cols, part,
                                                                            rs.S);
    GLOBE_LAUNCHED(ctx, "k_precond_apply_t");
    if (rs.nbl) {
        const size_t sm = part ? sizeof(double) * RB_WARPS * kact : 0;
        k_precond_apply<<<rs.nbl, RB_THREADS, sm, ctx->stream>>>(c.nlong, c.Nrec, c.bstart, c.times(),
                                                                  1.0 / ctx->vc[0], H, r, z, cols, kact, part, c.lblk,
                                                                  rs.nbt, rs.S);
        GLOBE_LAUNCHED(ctx, "k_precond_apply");
    }
    return GLOBE_OK;
}

int precond_apply(globe_ctx* ctx, const double* H, const double* r, double* z, const int32_t* cols, int kact,
                  double* rz) {
    const RecShape rs = rec_shape(ctx);
    double* part = nullptr;
    if (rz) GLOBE_RET(ws(ctx, WS_PART, (size_t)rs.S * kact * 2, &part));
    GLOBE_RET(precond_launch(ctx, H, r, z, cols, kact, part, rs));
    if (rz) GLOBE_RET(reduce_cols(ctx, part, rs.S, kact, cols, rz));
    return GLOBE_OK;
}

// Same operator with the r'z partials in caller-provided scratch (part, part_cap
// doubles): launches kernels only, allocates nothing.  Each CTA writes its own
// partial slot, so the scratch needs no clearing.
int precond_apply_scratch(globe_ctx* ctx, const double* H, const double* r, double* z, int kact, double* part,
                          size_t part_cap, double* rz) {
    const RecShape rs = rec_shape(ctx);
    if (kact > NOALLOC_MAX_COLS)
        return set_err(ctx, GLOBE_ERR_ARG, "%d columns: at most %d per call (one grid row per column)", kact,
                       NOALLOC_MAX_COLS);
    if (rz && (size_t)rs.S * kact > part_cap)
        return set_err(ctx, GLOBE_ERR_ARG,
                       "r'z partials need %zu doubles of scratch (%d CTAs x %d columns); the static buffer holds %zu",
                       (size_t)rs.S * kact, rs.S, kact, part_cap);
    // the warp-per-block kernel stages its r'z partials in dynamic shared memory
    // (RB_WARPS doubles per column) and runs at the default 48 KB limit
    if (rz && rs.nbl && sizeof(double) * RB_WARPS * (size_t)kact > NOALLOC_SMEM_BYTES)
        return set_err(ctx, GLOBE_ERR_ARG,
                       "%d columns with r'z and individuals of more than %d records: at most %d columns (%zu bytes "
                       "of shared memory per column, %d available)",
                       kact, SHORT_BLOCK, (int)(NOALLOC_SMEM_BYTES / (sizeof(double) * RB_WARPS)),
                       sizeof(double) * RB_WARPS, NOALLOC_SMEM_BYTES);
    GLOBE_RET(precond_launch(ctx, H, r, z, nullptr, kact, rz ? part : nullptr, rs));
    if (rz) GLOBE_RET(reduce_cols(ctx, part, rs.S, kact, nullptr, rz));
    return GLOBE_OK;
}

// ---------------------------------------------------------------------------
// Column reductions

// Quantity y (grid.y) of column c (grid.x): part[y * qstride + j + c*nparts], j < nparts,
// summed into o.out[y][cols ? cols[c] : c]; with o.quot, also o.quot[col] = o.num[col] / sum
// (0 where the sum is 0) and its double-float copy o.quot_df -- the step length
// alpha = r'z / p'Vp fused into the p'Vp reduction.
struct ReduceOut {
    double* out[2] = {nullptr, nullptr};
    const double* num = nullptr;
    double* quot = nullptr;
    float2* quot_df = nullptr;
};

__global__ void k_reduce_cols(const double* __restrict__ part, int nparts, size_t qstride,
                              const int32_t* __restrict__ cols, ReduceOut o) {
    __shared__ double sm[256];
    const int c = blockIdx.x;
    const double v = cta_reduce_256(part + blockIdx.y * qstride + (size_t)c * nparts, nparts, sm);   // 256 threads
    if (threadIdx.x == 0) {
        const int col = cols ? cols[c] : c;
        o.out[blockIdx.y][col] = v;
        if (o.quot) {
            const double q = (v != 0.0) ? o.num[col] / v : 0.0;
            o.quot[col] = q;
            if (o.quot_df) df::store(o.quot_df + col, df::from_double(q));
        }
    }
}

// out[cols ? cols[c] : c] = sum_j part[j + c*nparts]
int reduce_cols(globe_ctx* ctx, const double* part, int nparts, int kact, const int32_t* cols, double* out) {
    ReduceOut o;
    o.out[0] = out;
    k_reduce_cols<<<kact, 256, 0, ctx->stream>>>(part, nparts, 0, cols, o);
    GLOBE_LAUNCHED(ctx, "k_reduce_cols");
    return GLOBE_OK;
}

// two quantities of kact columns each (the second's partials follow the first's), one launch
int reduce_cols2(globe_ctx* ctx, const double* part, int nparts, int kact, const int32_t* cols, double* out0,
                 double* out1) {
    ReduceOut o;
    o.out[0] = out0;
    o.out[1] = out1;
    k_reduce_cols<<<dim3(kact, 2), 256, 0, ctx->stream>>>(part, nparts, (size_t)nparts * kact, cols, o);
    GLOBE_LAUNCHED(ctx, "k_reduce_cols");
    return GLOBE_OK;
}

// out as reduce_cols, and quot[col] = num[col] / out[col] (0 where out is 0), quot_df its copy
int reduce_cols_div(globe_ctx* ctx, const double* part, int nparts, int kact, const int32_t* cols, double* out,
                    const double* num, double* quot, float2* quot_df) {
    ReduceOut o;
    o.out[0] = out;
    o.num = num;
    o.quot = quot;
    o.quot_df = quot_df;
    k_reduce_cols<<<kact, 256, 0, ctx->stream>>>(part, nparts, 0, cols, o);
    GLOBE_LAUNCHED(ctx, "k_reduce_cols");
    return GLOBE_OK;
}

// per-column partial dots a_c . b_c over n rows
__global__ void k_col_dots(const double* __restrict__ a, const double* __restrict__ b, int64_t n, int64_t lda,
                           int64_t ldb, const int32_t* __restrict__ cols, double* __restrict__ part) {
    __shared__ double sm[32];
    const int c = blockIdx.y;
    const int col = cols ? cols[c] : c;
    const double* ac = a + (size_t)col * lda;
    const double* bc = b + (size_t)col * ldb;
    double acc = 0;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        acc += ac[r] * bc[r];
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sm[w];
        part[blockIdx.x + (size_t)c * gridDim.x] = s;
    }
}

int col_dots(globe_ctx* ctx, const double* a, const double* b, int64_t n, int64_t lda, int64_t ldb,
             const int32_t* cols, int kact, double* out) {
    int nb = div_up(n, 256 * 4);
    if (nb > 304) nb = 304;
    if (nb < 1) nb = 1;
    double* part;
    GLOBE_RET(ws(ctx, WS_PART, (size_t)nb * kact * 2, &part));
    k_col_dots<<<dim3(nb, kact), 256, 0, ctx->stream>>>(a, b, n, lda, ldb, cols, part);
    GLOBE_LAUNCHED(ctx, "k_col_dots");
    return reduce_cols(ctx, part, nb, kact, cols, out);
}

// out = num / den (0 where den = 0), and its double-float copy when out_df is given
__global__ void k_scal_div(const double* __restrict__ num, const double* __restrict__ den, double* out, int k,
                           float2* __restrict__ out_df) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < k) {
        const double q = (den[c] != 0.0) ? num[c] / den[c] : 0.0;
        out[c] = q;
        if (out_df) df::store(out_df + c, df::from_double(q));
    }
}

int scal_alpha(globe_ctx* ctx, const double* num, const double* den, double* out, int k, float2* out_df) {
    k_scal_div<<<div_up(k, 128), 128, 0, ctx->stream>>>(num, den, out, k, out_df);
    GLOBE_LAUNCHED(ctx, "k_scal_div");
    return GLOBE_OK;
}

// out (m1 x m2) = X' S over Nrec rows; X Nrec x m1, S Nrec x m2.
__global__ void k_xt_mat(const double* __restrict__ X, int m1, const double* __restrict__ S, int64_t n,
                         double* __restrict__ part) {
    __shared__ double sm[32];
    const int pair = blockIdx.y;
    const int a = pair % m1, b = pair / m1;
    const double* xa = X + (size_t)a * n;
    const double* sb = S + (size_t)b * n;
    double acc = 0;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        acc += xa[r] * sb[r];
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sm[w];
        part[blockIdx.x + (size_t)pair * gridDim.x] = s;
    }
}

int xt_mat(globe_ctx* ctx, const double* X, int m1, const double* S, int m2, double* out) {
    int64_t n = ctx->coh.Nrec;
    int nb = div_up(n, 256 * 8);
    if (nb > 152) nb = 152;
    if (nb < 1) nb = 1;
    double* part;
    GLOBE_RET(ws(ctx, WS_GPART, (size_t)nb * m1 * m2, &part));
    k_xt_mat<<<dim3(nb, m1 * m2), 256, 0, ctx->stream>>>(X, m1, S, n, part);
    GLOBE_LAUNCHED(ctx, "k_xt_mat");
    return reduce_cols(ctx, part, nb, m1 * m2, nullptr, out);
}

// out[:, j] = A[:, j] - Bm c[:, j],  Bm Nrec x m, c m x kout (column-major)
__global__ void k_sub_mat(const double* __restrict__ A, const double* __restrict__ Bm, int m,
                          const double* __restrict__ c, double* __restrict__ out, int kout, int64_t n) {
    const int j = blockIdx.y;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        double acc = A[r + (size_t)j * n];
        for (int a = 0; a < m; ++a) acc -= Bm[r + (size_t)a * n] * c[a + (size_t)j * m];
        out[r + (size_t)j * n] = acc;
    }
}

int sub_mat(globe_ctx* ctx, const double* A, const double* Bm, int m, const double* c, double* out, int kout) {
    int64_t n = ctx->coh.Nrec;
    int nb = div_up(n, 256);
    if (nb > 1216) nb = 1216;
    k_sub_mat<<<dim3(nb, kout), 256, 0, ctx->stream>>>(A, Bm, m, c, out, kout, n);
    GLOBE_LAUNCHED(ctx, "k_sub_mat");
    return GLOBE_OK;
}

// bhat_i = (b0 s0 + b01 s1, b01 s0 + b1 s1)   (compute_bhat, PCGsolver.cpp:1475-1513)
__global__ void k_bhat(int32_t nblk, const int32_t* __restrict__ bstart, const int32_t* __restrict__ bind,
                       const double* __restrict__ t, VC v, const double* __restrict__ vr, double* __restrict__ bhat) {
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * RB_WARPS + (threadIdx.x >> 5);
    if (b >= nblk) return;
    double s0 = 0, s1 = 0;
    for (int r = bstart[b] + lane; r < bstart[b + 1]; r += 32) {
        s0 += vr[r];
        s1 += t[r] * vr[r];
    }
    s0 = warp_sum(s0);
    s1 = warp_sum(s1);
    if (lane == 0) {
        int i = bind[b];
        bhat[2 * i] = v.b0 * s0 + v.b01 * s1;
        bhat[2 * i + 1] = v.b01 * s0 + v.b1 * s1;
    }
}

int bhat_kernel(globe_ctx* ctx, const double* vr, double* bhat) {
    auto& c = ctx->coh;
    VC v{ctx->vc[0], ctx->vc[1], ctx->vc[2], ctx->vc[3], ctx->vc[4]};
    k_bhat<<<div_up(c.N, RB_WARPS), RB_THREADS, 0, ctx->stream>>>(c.N, c.bstart, c.bind, c.times(), v, vr, bhat);
    GLOBE_LAUNCHED(ctx, "k_bhat");
    return GLOBE_OK;
}

// f_theta (compute_f_theta_i, varCompEst.cpp:693-760):
//  f0 = vr, f1 = uhat_i / sig2g, f2 = w_i, f3 = t w_i + tw_i, f4 = tw_i t
__global__ void k_ftheta(int32_t nblk, int64_t n, const int32_t* __restrict__ bstart,
                         const int32_t* __restrict__ bind, const double* __restrict__ t, double inv_g,
                         const double* __restrict__ vr, const double* __restrict__ uh, double* __restrict__ f) {
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * RB_WARPS + (threadIdx.x >> 5);
    if (b >= nblk) return;
    const int st = bstart[b], en = bstart[b + 1];
    double w = 0, tw = 0;
    for (int r = st + lane; r < en; r += 32) {
        w += vr[r];
        tw += t[r] * vr[r];
    }
    w = warp_sum(w);
    tw = warp_sum(tw);
    const double u = uh[bind[b]] * inv_g;
    for (int r = st + lane; r < en; r += 32) {
        f[r] = vr[r];
        f[n + r] = u;
        f[2 * n + r] = w;
        f[3 * n + r] = t[r] * w + tw;
        f[4 * n + r] = tw * t[r];
    }
}

int ftheta_kernel(globe_ctx* ctx, const double* vr, const double* uh, double* fth) {
    auto& c = ctx->coh;
    k_ftheta<<<div_up(c.N, RB_WARPS), RB_THREADS, 0, ctx->stream>>>(c.N, c.Nrec, c.bstart, c.bind, c.times(),
                                                                    1.0 / ctx->vc[1], vr, uh, fth);
    GLOBE_LAUNCHED(ctx, "k_ftheta");
    return GLOBE_OK;
}

// ---- Monte-Carlo probes (sample_Yvs, varCompEst.cpp:775-797) ----------

__device__ __forceinline__ uint64_t pmix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// standard normal numbers 2 pair and 2 pair + 1 of stream `seed` (Box-Muller on two 53-bit
// uniforms): the cosine and sine halves of one draw
__device__ void stream_normal_pair(uint64_t seed, uint64_t pair, double& even, double& odd) {
    uint64_t h1 = pmix(seed ^ pmix(2 * pair + 1));
    uint64_t h2 = pmix(seed ^ pmix(2 * pair + 2));
    double u1 = ((double)(h1 >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    double u2 = ((double)(h2 >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    double rad = sqrt(-2.0 * log(u1));
    double s, c;
    sincospi(2.0 * u2, &s, &c);
    even = rad * c;
    odd = rad * s;
}

// standard normal number `idx` of stream `seed`
__device__ double stream_normal(uint64_t seed, uint64_t idx) {
    double e, o;
    stream_normal_pair(seed, idx >> 1, e, o);
    return (idx & 1) ? o : e;
}

// the per-individual normals of probe j (grid.y) in generated mode, once per individual rather
// than once per record: stream indices base .. base + L - 1 (base = j per, L = N or 3 N), i.e.
// z1 of individual i at base + i and, with time effects, z2a / z2b at base + N + 2 i (+ 1),
// into zi[3 j N + i], zi[(3 j + 1) N + i], zi[(3 j + 2) N + i]; one Box-Muller pair per step
__global__ void k_probe_ind(int32_t N, uint64_t seed, int no_time, size_t per, double* __restrict__ zi) {
    const int j = blockIdx.y;
    const uint64_t b = (uint64_t)j * per, L = (no_time ? 1u : 3u) * (uint64_t)N;
    const uint64_t p0 = b >> 1, p1 = (b + L - 1) >> 1;
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (uint64_t)gridDim.x * blockDim.x;
    double* z = zi + 3 * (size_t)j * N;
    for (uint64_t p = p0 + tid; p <= p1; p += nth) {
        double ze, zo;
        stream_normal_pair(seed, p, ze, zo);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int64_t m = (int64_t)(2 * p + h) - (int64_t)b;
            if (m < 0 || m >= (int64_t)L) continue;
            const double v = h ? zo : ze;
            if (m < N) {
                z[m] = v;
            } else {
                const int64_t m2 = m - N;
                z[(1 + (m2 & 1)) * (size_t)N + (m2 >> 1)] = v;
            }
        }
    }
}

// probe Y_j = sqrt(sig2g) Z1 + sqrt(sig2e) Z3 + the random-regression term (varCompEst.cpp:816-837;
// without time effects varCompEst_reducedModel_noTime.cpp:563-577), record r of probe j
__device__ __forceinline__ double probe_value(int no_time, double sg, double se, double L00, double L10, double L11,
                                              double z1, double z2a, double z2b, double z3, double tr) {
    if (no_time) return sg * z1 + se * z3;
    return sg * z1 + se * z3 + z2a * (L00 + L10 * tr) + z2b * L11 * tr;
}

// draws given: the normals of probe j at draws[j * per ...]; generated: the per-individual ones
// from k_probe_ind and the per-record one z3 (index base + N0 + r, N0 = N or 3 N) by Box-Muller
// pairs, one pair per thread step (both halves are records of the probe, except at its ends)
__global__ void k_probes(int64_t n, int32_t N, const int32_t* __restrict__ rind, const double* __restrict__ t,
                         double sg, double se, double L00, double L10, double L11,
                         const double* __restrict__ draws, const double* __restrict__ zi, uint64_t seed, int numMC,
                         int no_time, double* __restrict__ Y) {
    const int j = blockIdx.y;
    const size_t per = (no_time ? 1 : 3) * (size_t)N + n;
    const size_t N0 = (no_time ? 1 : 3) * (size_t)N;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (int64_t)gridDim.x * blockDim.x;
    if (draws) {
        const double* d = draws + (size_t)j * per;
        for (int64_t r = tid; r < n; r += nth) {
            const int i = rind[r];
            const double z2a = no_time ? 0.0 : d[N + 2 * (size_t)i], z2b = no_time ? 0.0 : d[N + 2 * (size_t)i + 1];
            Y[r + (size_t)j * n] = probe_value(no_time, sg, se, L00, L10, L11, d[i], z2a, z2b, d[N0 + r], t[r]);
        }
        return;
    }
    const uint64_t b3 = (uint64_t)j * per + N0;   // stream index of record 0's z3
    const uint64_t p0 = b3 >> 1, p1 = (b3 + (uint64_t)n - 1) >> 1;
    const double* z1s = zi + (3 * (size_t)j) * N;
    for (uint64_t p = p0 + (uint64_t)tid; p <= p1; p += (uint64_t)nth) {
        double ze, zo;
        stream_normal_pair(seed, p, ze, zo);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int64_t r = (int64_t)(2 * p + h) - (int64_t)b3;
            if (r < 0 || r >= n) continue;
            const int i = rind[r];
            const double z2a = no_time ? 0.0 : z1s[N + i], z2b = no_time ? 0.0 : z1s[2 * (size_t)N + i];
            Y[r + (size_t)j * n] = probe_value(no_time, sg, se, L00, L10, L11, z1s[i], z2a, z2b, h ? zo : ze, t[r]);
        }
    }
}

int probes_build(globe_ctx* ctx, const double* draws, int numMC, uint64_t seed, bool gen, double* Y, double* zi) {
    auto& c = ctx->coh;
    const double* v = ctx->vc;
    // compute_chol_2x2 (varCompEst.cpp:800-813); unused without time effects
    const int no_time = ctx->model == GLOBE_MODEL_NO_TIME ? 1 : 0;
    double L00 = 0, L10 = 0, L11 = 0;
    if (!no_time) {
        L00 = sqrt(v[2]);
        L10 = v[3] / L00;
        double d11 = v[4] - v[3] * v[3] / v[2];
        if (d11 < 0) d11 = 0;
        L11 = sqrt(d11);
    }
    if (gen) {
        const size_t per = (no_time ? 1 : 3) * (size_t)c.N + (size_t)c.Nrec;
        const int nbi = div_up(c.N, 256) < 1216 ? div_up(c.N, 256) : 1216;
        k_probe_ind<<<dim3(nbi, numMC), 256, 0, ctx->stream>>>(c.N, seed, no_time, per, zi);
        GLOBE_LAUNCHED(ctx, "k_probe_ind");
    }
    int nb = div_up(c.Nrec, 256);
    if (nb > 1216) nb = 1216;
    k_probes<<<dim3(nb, numMC), 256, 0, ctx->stream>>>(c.Nrec, c.N, c.rind, c.times(), sqrt(v[1]), sqrt(v[0]),
                                                       L00, L10, L11, gen ? nullptr : draws, zi, seed, numMC, no_time,
                                                       Y);
    GLOBE_LAUNCHED(ctx, "k_probes");
    return GLOBE_OK;
}

// trace terms: for probe j, f~_k from (VR_j, UH_j) and dot with TY_j
// (estimateTrace_PdV, varCompEst.cpp:955-968).  out[j*5 + k].  The launch shape of the record
// kernels: a thread per (individual of at most SHORT_BLOCK records, probe) -- grid.y = probe --
// and a warp per longer individual over every probe, partials part[slot + (5 j + k) * S].

// the five terms of probe j over one individual's records [st, en)
__device__ __forceinline__ void trace_block(const double* __restrict__ vr, const double* __restrict__ ty,
                                            const double* __restrict__ t, double u, int st, int en, int step,
                                            double (&acc)[5], bool warp) {
    double w = 0, tw = 0;
    for (int r = st; r < en; r += step) {
        w += vr[r];
        tw += t[r] * vr[r];
    }
    if (warp) {
        w = warp_sum(w);
        tw = warp_sum(tw);
    }
    for (int r = st; r < en; r += step) {
        const double y = ty[r], tr = t[r];
        acc[0] += vr[r] * y;
        acc[1] += u * y;
        acc[2] += w * y;
        acc[3] += (tr * w + tw) * y;
        acc[4] += tw * tr * y;
    }
}

__global__ void k_trace_terms_t(int32_t nblk, int64_t n, int32_t N, const int32_t* __restrict__ bstart,
                                const int32_t* __restrict__ bind, const double* __restrict__ t, double inv_g,
                                const double* __restrict__ VR, const double* __restrict__ UH,
                                const double* __restrict__ TY, double* __restrict__ part, int pstride) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    double acc[5] = {0, 0, 0, 0, 0};
    if (b < nblk && bstart[b + 1] - bstart[b] <= SHORT_BLOCK &&   // long blocks: a warp each
        GLOBE_BOUNDS(bstart[b] >= 0 && bstart[b + 1] <= n && bind[b] >= 0 && bind[b] < N, 0x1301u)) {
        const int i = bind[b];
        trace_block(VR + (size_t)j * n, TY + (size_t)j * n, t, UH[i + (size_t)j * N] * inv_g, bstart[b], bstart[b + 1],
                    1, acc, false);
    }
    const int q[5] = {5 * j, 5 * j + 1, 5 * j + 2, 5 * j + 3, 5 * j + 4};
    cta_sums<5>(acc, q, part, pstride);
}

__global__ void k_trace_terms(int32_t nblk, int64_t n, int32_t N, const int32_t* __restrict__ bstart,
                              const int32_t* __restrict__ bind, const double* __restrict__ t, double inv_g,
                              const double* __restrict__ VR, const double* __restrict__ UH,
                              const double* __restrict__ TY, int numMC, double* __restrict__ part,
                              const int32_t* __restrict__ bl, int slot0, int pstride) {
    extern __shared__ double sm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int idx = blockIdx.x * RB_WARPS + warp;
    const bool live = idx < nblk;
    const int b = live ? (bl ? bl[idx] : idx) : 0;
    int st = 0, en = 0, i = 0;
    if (live) { st = bstart[b]; en = bstart[b + 1]; i = bind[b]; }
    if (live && !GLOBE_BOUNDS(st >= 0 && st <= en && en <= n && i >= 0 && i < N, 0x1401u)) st = en = i = 0;
    for (int j = 0; j < numMC; ++j) {
        double acc[5] = {0, 0, 0, 0, 0};
        if (live)
            trace_block(VR + (size_t)j * n, TY + (size_t)j * n, t, UH[i + (size_t)j * N] * inv_g, st + lane, en, 32, acc,
                        true);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            double s = warp_sum(acc[k]);
            if (lane == 0) sm[(j * 5 + k) * RB_WARPS + warp] = s;
        }
    }
    cta_partials(sm, numMC * 5, part, slot0 + blockIdx.x, pstride);
}

int trace_terms(globe_ctx* ctx, const double* VR, const double* UH, const double* TY, int numMC, double* out) {
    auto& c = ctx->coh;
    const RecShape rs = rec_shape(ctx);
    double* part;
    GLOBE_RET(ws(ctx, WS_GPART, (size_t)rs.S * numMC * 5, &part));
    k_trace_terms_t<<<dim3(rs.nbt, numMC), TB_THREADS, 0, ctx->stream>>>(c.N, c.Nrec, c.N, c.bstart, c.bind,
                                                                           c.times(), 1.0 / ctx->vc[1], VR, UH, TY,
                                                                           part, rs.S);
    GLOBE_LAUNCHED(ctx, "k_trace_terms_t");
    if (rs.nbl) {
        const size_t sm = sizeof(double) * RB_WARPS * numMC * 5;
        if (sm > 48 * 1024)
            GLOBE_CK(ctx, cudaFuncSetAttribute(k_trace_terms, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        k_trace_terms<<<rs.nbl, RB_THREADS, sm, ctx->stream>>>(c.nlong, c.Nrec, c.N, c.bstart, c.bind, c.times(),
                                                                1.0 / ctx->vc[1], VR, UH, TY, numMC, part, c.lblk,
                                                                rs.nbt, rs.S);
        GLOBE_LAUNCHED(ctx, "k_trace_terms");
    }
    return reduce_cols(ctx, part, rs.S, numMC * 5, nullptr, out);
}

}  // namespace globe
