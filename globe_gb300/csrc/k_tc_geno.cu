// k_tc_geno.cu -- genotype GRM product on the 5th-generation tensor cores.
//
//   out (N x k) = scale * Zs' (Zs Z),  zs(s,i) = (g - 2 f_s) inv_s      (PCGsolver.cpp:1130-1201)
//
// Written as two integer-genotype products plus FP64 rank-1 terms:
//   pass 1:  P1[s,c] = sum_i g(s,i) Z[i,c]        (rows = SNPs, K = individuals)
//            u[s,c]  = inv_s^2 (P1[s,c] - 2 f_s sum_i Z[i,c])
//   pass 2:  P2[i,c] = sum_s g(s,i) u[s,c]        (rows = individuals, K = SNPs)
//            out[i,c] = scale (P2[i,c] - sum_s 2 f_s u[s,c])
// g in {0,1,2} is decoded to e4m3 as 2^-9 g or 2^-7 g (the tile code masked in
// place; even and odd genotypes of a word).  Each right-hand-side column is split
// into balanced base-32 digits: x = 2^e sum_j d_j 32^-j with integer d_j in
// [-16,16], exact in e4m3 (every integer up to 16 is, and 4x that), the digit
// operand holding 4 d where the genotype carries 2^-9.  Every product is
// g d 2^-7 with |g d| <= 32, so an FP32 sum of up to 2^19 of them is an exact
// multiple of 2^-7: the tensor-core accumulation carries no rounding, and the
// digits are recombined in int64 / FP64.  With 9 digits (45 bits) the product
// matches an FP64 evaluation to ~1e-13 relative.
//
// Kernel (one CTA = MT x 128 rows x one K range, M=128 x N=NMMA MMAs per tile):
//   warp 0     bulk copies of the packed 2-bit tiles (tile-blocked layout: each
//              128-row x 32-byte stage is one contiguous 4 KB block)
//   warp 1     TMA of the digit tiles [NMMA rows x 128 B, 128B-swizzled]
//   warp 2     TMEM allocation and the single-thread tcgen05.mma issue
//              (kind::f8f6f4, E4M3 x E4M3 -> F32, A from TMEM, B from smem)
//   warps 3-10 decode 2-bit codes to e4m3 bytes in registers and store them
//              straight into TMEM (tcgen05.st) as the A operand, then the
//              epilogue (tcgen05.ld -> FP32 partials)
// Keeping the decoded operand out of shared memory matters: staged through
// smem it costs ~4 bytes of smem traffic per genotype and caps the kernel
// near 40% of HBM bandwidth.
// The decode of 16 genotypes (one 32-bit word) is 4 masks and 1 shift; it
// permutes K within each group of 16, which the digit tiles repeat (kpos_g()).
// Every mbarrier wait is bounded (globaltimer); on timeout the CTA records
// an error bit, waits (bounded) for its issued copies / MMAs and frees TMEM.
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <cstdarg>
#include <cstdio>
#include <vector>

#include "tc_ptx.cuh"

namespace globe {
namespace tc {

#ifndef TC_ASTAGES
#define TC_ASTAGES 6
#endif
#ifndef TC_BSTAGES
#define TC_BSTAGES 4
#endif
#ifndef TC_DSTAGES
#define TC_DSTAGES 2
#endif
#ifndef TC_DEC_PRE
#define TC_DEC_PRE 8     // 16-byte units a decoder warp decodes before it waits for its TMEM slot
#endif
#ifndef TC_STW
#define TC_STW 16        // columns per tcgen05.st: 16 (a unit), 8 (a unit in two), 32 (a tile row's two
                         // units; 1% slower at k = 5)
#endif
#ifndef TC_SLEEP_DEC
#define TC_SLEEP_DEC 1   // decoders suspend in their waits too
#endif
constexpr int ASTAGES = TC_ASTAGES;  // packed-genotype ring (keeps DRAM reads in flight)
constexpr int BSTAGES = TC_BSTAGES;  // digit-tile ring (L2-resident operand)
constexpr int DSTAGES = TC_DSTAGES;  // decoded-A ring
// Row tiles per CTA (one MMA-issuing warp each): an M=128, K=32 MMA occupies
// its issuing context ~157 cycles whatever N is, so small-N products need
// several concurrent issue streams to use the tensor pipe; TMEM (512
// columns) bounds MT * NMMA + DSTAGES * MT * 32.  At k = 5 a stage takes ~1000
// cycles: copies without the TMEM stores or without the MMAs run 12% / 16%
// faster, but a deeper decoded-A ring (3 tiles, 3 slots; or 4 slots at width
// 128) does not help, and the stage time stays ~1000 cycles with 3 tiles per CTA
// as with 4 -- the stores and the MMAs' TMEM reads of A share what bounds it.
// Moving one or two tiles' decoded A to shared memory (MMA from two descriptors)
// is slower still (+10%, +30%): shared memory is the tighter of the two.
// Decoders: two sets of 8 warps take the stages in turn (set = stage parity, so
// each set owns one slot of the decoded-A ring) -- one set's load / TMEM-store
// latency overlaps the other set's decode.  Within a set, warp (quadrant q, j)
// covers TMEM lanes 32q..32q+31 of the 16-byte units u = j*MT .. j*MT+MT-1 of a
// row (unit u = tile u/2, half u%2).
template <int NMMA>
struct Geo {
    static constexpr int MT = NMMA <= 64 ? 4 : (NMMA <= 192 ? 2 : 1);
    static constexpr int NSET = 2;                         // decoder sets
    static constexpr int DECW = 16;                        // decoder warps (NSET x 4 quadrants x 2)
    static constexpr int DBASE = MT > 2 ? 8 : 4;           // first decoder warp (multiple of 4)
    static constexpr int NTHREADS = (DBASE + DECW) * 32;
    static constexpr int UPW = MT;                         // 16-byte units per warp and stage
    static constexpr int TPW = MT >= 2 ? MT / 2 : 1;       // tiles per warp
    static constexpr int DPT = MT >= 2 ? 4 : 8;            // warps of one set per tile (adfull count)
    static constexpr int ES = MT >= 2 ? 2 : 4;             // warps sharing a (tile, quadrant) epilogue
};

// MT row tiles of 128 share every digit tile.  TMEM columns: accumulators
// [0, MT*NMMA), then DSTAGES x MT decoded A tiles of 32 columns (K = 128 e4m3).
template <int NMMA, int MT>
struct __align__(1024) Smem {
    uint8_t bt[BSTAGES][NMMA * BK];         // digit tiles (TMA, SW128), 1024-aligned
    uint8_t pk[ASTAGES][MT * BM * PKB];     // packed tiles (bulk copies)
    uint64_t afull[ASTAGES], aempty[ASTAGES], bfull[BSTAGES], bempty[BSTAGES];
    uint64_t adfull[MT][DSTAGES], adempty[MT][DSTAGES], accfull[MT];
    uint32_t tmem_base;
    int abort;
};


// one decoded 16-byte unit (16 columns of one lane quadrant)
__device__ __forceinline__ void tmem_st_unit(uint32_t taddr, const uint32_t (&v)[16]) {
    if (TC_STW == 8) {
        tmem_st8(taddr, v);
        tmem_st8(taddr + 8, v + 8);
    } else {
        tmem_st16(taddr, v);
    }
}
// 16 tile codes (genotype j of the word at bits 2j) -> 16 e4m3 bytes, by masks in place:
//   r0 = w & 0x03030303         genotypes 0, 4, 8, 12   as 0x00 / 0x01 / 0x02 = 2^-9 g
//   r1 = w & 0x0C0C0C0C         genotypes 1, 5, 9, 13   as 0x00 / 0x04 / 0x08 = 2^-7 g
//   r2 = (w >> 4) & 0x03030303  genotypes 2, 6, 10, 14  (2^-9 g)
//   r3 = (w >> 4) & 0x0C0C0C0C  genotypes 3, 7, 11, 15  (2^-7 g)
// 5 integer instructions per 16 genotypes.  The K order is kpos_g; the digit operand carries
// 4 d at the even genotypes (r0, r2), so every product is g d 2^-7.
__device__ __forceinline__ void decode_word(uint32_t w, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
    const uint32_t h = w >> 4;
    r0 = w & 0x03030303u;
    r1 = w & 0x0C0C0C0Cu;
    r2 = h & 0x03030303u;
    r3 = h & 0x0C0C0C0Cu;
}

// A operand: tile-blocked packed genotypes, block (tile t, chunk c) = 128 rows x 32 B contiguous at
// blk + (t * nchunks + c) * 4096 (the two 16-byte halves of row r swapped when bit 2 of r is set,
// which makes the decoders' shared-memory reads conflict-free); one stage = MT bulk copies.
template <int NMMA>
__global__ void __launch_bounds__(Geo<NMMA>::NTHREADS, 1)
    k_tc_gemm(const uint8_t* __restrict__ blk, const __grid_constant__ CUtensorMap tmB, int rows, int nchunks,
              int cps, float* __restrict__ part, int64_t ldp, int64_t pz, int skip0, int skipz,
              unsigned* __restrict__ err, int stall) {
    using G = Geo<NMMA>;
    constexpr int MT = G::MT;
    static_assert(NMMA % 16 == 0 && NMMA >= 16 && NMMA <= 256, "NMMA");
    constexpr int ACOL0 = MT * NMMA;                     // first TMEM column of the decoded A stages
    static_assert(MT * NMMA + DSTAGES * MT * 32 <= 512, "TMEM columns");
    constexpr uint32_t NCOLS = ncols_alloc(MT * NMMA + DSTAGES * MT * 32);
    constexpr int ROWS = MT * BM;
    extern __shared__ uint8_t smraw[];
    Smem<NMMA, MT>& S = *reinterpret_cast<Smem<NMMA, MT>*>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row0 = blockIdx.x * ROWS, split = blockIdx.y, z = blockIdx.z;
    if (row0 + ROWS <= skip0 + z * skipz) return;   // whole CTA, before any barrier or TMEM use
    part += z * pz;
    const int c0 = split * cps;
    const int nloc = min(nchunks, c0 + cps) - c0;

    if (threadIdx.x == 0) {
        for (int s = 0; s < ASTAGES; ++s) {
            mbar_init(&S.afull[s], 1);
            mbar_init(&S.aempty[s], G::DECW / G::NSET);
        }
        for (int s = 0; s < BSTAGES; ++s) {
            mbar_init(&S.bfull[s], 1);
            mbar_init(&S.bempty[s], MT);
        }
        for (int m = 0; m < MT; ++m) {
            for (int d = 0; d < DSTAGES; ++d) {
                mbar_init(&S.adfull[m][d], G::DPT);
                mbar_init(&S.adempty[m][d], 1);
            }
            mbar_init(&S.accfull[m], 1);
        }
        S.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 2) tmem_alloc(&S.tmem_base, NCOLS);
    tc_before();
    __syncthreads();
    tc_after();
    const uint32_t tmem = S.tmem_base;
    int* abort = &S.abort;

    if (warp == 0) {
        // packed genotype tiles: up to ASTAGES chunks ahead of the decoders
        if (lane == 0 && nloc > 0) {
            int issued = 0;
            for (int it = 0; it < nloc; ++it) {
                const int s = it % ASTAGES, n = it / ASTAGES;
                if (n > 0 && !mbar_wait(&S.aempty[s], (n - 1) & 1, abort, err, 1u)) break;
                mbar_expect_tx(&S.afull[s], ROWS * PKB);
#pragma unroll
                for (int m = 0; m < MT; ++m) {
                    const int64_t t = (int64_t)blockIdx.x * MT + m;
                    bulk_load(S.pk[s] + m * (BM * PKB), blk + (t * nchunks + (c0 + it)) * (int64_t)(BM * PKB),
                              BM * PKB, &S.afull[s]);
                }
                issued = it + 1;
            }
            for (int it = issued - 1; it >= 0 && it >= issued - ASTAGES; --it)
                mbar_drain(&S.afull[it % ASTAGES], (it / ASTAGES) & 1);
        }
    } else if (warp == 1) {
        // digit tiles: up to BSTAGES chunks ahead of the MMAs
        if (lane == 0 && nloc > 0) {
            int issued = 0;
            for (int it = 0; it < nloc; ++it) {
                const int s = it % BSTAGES, n = it / BSTAGES;
                if (n > 0 && !mbar_wait(&S.bempty[s], (n - 1) & 1, abort, err, 2u)) break;
                if (stall && it == 0) {   // test hook: the stage is never loaded, so its waits run out
                    issued = 1;
                    continue;
                }
                mbar_expect_tx(&S.bfull[s], NMMA * BK);
                tma_load_2d(S.bt[s], &tmB, (c0 + it) * BK, z * NMMA, &S.bfull[s]);
                issued = it + 1;
            }
            for (int it = issued - 1; it >= 0 && it >= issued - BSTAGES; --it)
                mbar_drain(&S.bfull[it % BSTAGES], (it / BSTAGES) & 1);
        }
    } else if (warp >= 2 && warp < 2 + MT) {
        // one MMA issue stream per row tile
        const int m = warp - 2;
        if (lane == 0 && nloc > 0) {
            const uint32_t idesc = (1u << 4) | ((uint32_t)(NMMA >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
            const uint32_t dcol = tmem + (uint32_t)(m * NMMA);
            // B descriptors differ only in their start address (bits 0-13, address / 16): slot sb
            // and K step kk add sb * NMMA * BK / 16 + 2 kk, which stays inside the field
            const uint64_t dbase = desc_sw128(saddr(S.bt[0]));
            int sb = 0, ds = 0;
            uint32_t pb = 0, pd = 0;
            for (int it = 0; it < nloc; ++it) {
                if (!mbar_wait(&S.bfull[sb], pb, abort, err, 4u)) break;
                if (!mbar_wait(&S.adfull[m][ds], pd, abort, err, 8u)) break;
                tc_after();
                const uint32_t acol = tmem + (uint32_t)(ACOL0 + (ds * MT + m) * 32);
                const uint64_t bd = dbase + (uint64_t)(sb * ((NMMA * BK) >> 4));
#pragma unroll
                for (int kk = 0; kk < BK / 32; ++kk)
                    mma_f8_ta(dcol, acol + (uint32_t)(kk * 8), bd + (uint64_t)(2 * kk), idesc, (it | kk) != 0);
                mma_commit(&S.bempty[sb]);
                mma_commit(&S.adempty[m][ds]);
                if (++sb == BSTAGES) { sb = 0; pb ^= 1u; }
                if (++ds == DSTAGES) { ds = 0; pd ^= 1u; }
            }
            mma_commit(&S.accfull[m]);  // tracks every MMA this thread issued
        }
    } else if (warp >= G::DBASE) {
        static_assert(DSTAGES % G::NSET == 0 && ASTAGES % G::NSET == 0, "each ring slot belongs to one decoder set");
        const int dw = warp - G::DBASE;
        const int set = dw >> 3, j = (dw >> 2) & 1, quad = warp & 3;
        const int t0 = (j * MT) >> 1;                  // first tile of this warp
        const int r = quad * 32 + lane;                // row within a tile
        const uint32_t lane_addr = (uint32_t)(quad * 32) << 16;
        const int swz = (r >> 2) & 1;
        bool ok = true;
        for (int it = set; it < nloc && ok; it += G::NSET) {
            // (slots and phases from it: running counters here cost registers and ~15% of the pass)
            const int sa = it % ASTAGES, ds = it % DSTAGES;
            const uint32_t pa = (it / ASTAGES) & 1, pdd = (it / DSTAGES) & 1;
            if (!mbar_wait<TC_SLEEP_DEC != 0>(&S.afull[sa], pa, abort, err, 16u)) { ok = false; break; }
            uint4 v[G::UPW];
#pragma unroll
            for (int i = 0; i < G::UPW; ++i) {
                const int u = j * MT + i, m = u >> 1, h = u & 1;
                v[i] = *reinterpret_cast<const uint4*>(S.pk[sa] + m * (BM * PKB) + (r * 2 + (h ^ swz)) * 16);
            }
            constexpr int PRE = TC_DEC_PRE < G::UPW ? TC_DEC_PRE : G::UPW;
            uint32_t o[G::UPW][16];
#pragma unroll
            for (int i = 0; i < PRE; ++i) {
                decode_word(v[i].x, o[i][0], o[i][1], o[i][2], o[i][3]);
                decode_word(v[i].y, o[i][4], o[i][5], o[i][6], o[i][7]);
                decode_word(v[i].z, o[i][8], o[i][9], o[i][10], o[i][11]);
                decode_word(v[i].w, o[i][12], o[i][13], o[i][14], o[i][15]);
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&S.aempty[sa]);   // packed stage consumed
            // the decoded slot is free once the MMAs of the stage DSTAGES back completed; the decode
            // above already overlapped them
            if (it >= DSTAGES) {
#pragma unroll
                for (int q = 0; q < G::TPW; ++q)
                    if (ok && !mbar_wait<TC_SLEEP_DEC != 0>(&S.adempty[t0 + q][ds], pdd ^ 1u, abort,
                                                            err, 32u))
                        ok = false;
                if (!ok) break;
                tc_after();   // order the stores after the MMAs that read the slot
            }
#pragma unroll
            for (int i = 0; i < G::UPW; ++i) {
                const int u = j * MT + i, m = u >> 1, h = u & 1;
                if (i >= PRE) {   // the rest of the units, decoded after the wait
                    decode_word(v[i].x, o[i][0], o[i][1], o[i][2], o[i][3]);
                    decode_word(v[i].y, o[i][4], o[i][5], o[i][6], o[i][7]);
                    decode_word(v[i].z, o[i][8], o[i][9], o[i][10], o[i][11]);
                    decode_word(v[i].w, o[i][12], o[i][13], o[i][14], o[i][15]);
                }
                if (TC_STW == 32 && G::UPW % 2 == 0) {
                    // units i, i+1 are the two halves of one tile's row: one 32-column store
                    if (h == 1) tmem_st32(tmem + lane_addr + (uint32_t)(ACOL0 + (ds * MT + m) * 32), o[i - 1], o[i]);
                } else {
                    tmem_st_unit(tmem + lane_addr + (uint32_t)(ACOL0 + (ds * MT + m) * 32 + h * 16), o[i]);
                }
            }
            tmem_wait_st();
            tc_before();
            __syncwarp();
            if (lane == 0) {
#pragma unroll
                for (int q = 0; q < G::TPW; ++q) mbar_arrive(&S.adfull[t0 + q][ds]);
            }
        }
        // epilogue: the ES warps covering a (tile, quadrant) split its accumulator columns
        const int e0 = MT >= 2 ? set : set * 2 + j;
#pragma unroll 1
        for (int q = 0; q < G::TPW; ++q) {
            const int m = t0 + q;
            bool go = ok && nloc > 0;
            if (go) go = mbar_wait(&S.accfull[m], 0, abort, err, 64u);
            go = __all_sync(0xffffffffu, go);   // tcgen05.ld is warp-collective
            if (!go) {
                ok = false;
                continue;
            }
            tc_after();
            const int rr = row0 + m * BM + r;
#pragma unroll 1
            for (int cb = e0 * 16; cb < NMMA; cb += G::ES * 16) {
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
    if (warp >= 2 && warp < 2 + MT && nloc > 0) mbar_drain(&S.accfull[warp - 2], 0);
    tc_before();
    __syncthreads();
    if (warp == 2) {
        tc_after();
        tmem_dealloc(tmem, NCOLS);
    }
}

// ---- digit and combine kernels ---------------------------------------------



// colinfo = {scale exponent e (as double), column sum} of one column from its nparts partials;
// one warp (the lanes read the partials through L2, so a CTA that did not write them sees
// them once their writers' fences are past)
__device__ __forceinline__ void col_finish_warp(const double* __restrict__ pm, const double* __restrict__ ps,
                                                int nparts, double* __restrict__ colinfo) {
    const int lane = threadIdx.x & 31;
    double mx = 0, sm = 0;
    for (int j = lane; j < nparts; j += 32) {
        mx = fmax(mx, __ldcg(pm + j));
        sm += __ldcg(ps + j);
    }
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        sm += __shfl_xor_sync(0xffffffffu, sm, o);
    }
    if (lane == 0) {
        // A column holding NaN or +-Inf has a non-finite sum (fmax drops NaN, the sum keeps it).
        // It is marked by a NaN sum and a zero exponent: k_digits gives it zero digits, and every
        // epilogue writes NaN for it (through the centring term, or explicitly), as FP64 would.
        const bool bad = !isfinite(sm) || !isfinite(mx);
        int E = 0;
        if (!bad && mx > 0) frexp(mx, &E);
        colinfo[0] = bad ? 0.0 : (double)(E - (DBITS - 1));  // |x 2^-e| < 16
        colinfo[1] = bad ? __longlong_as_double(0x7ff8000000000000ll) : sm;
    }
}

// colinfo[c] = {scale exponent e_c (as double), column sum} from partials; one warp per column
__global__ void k_col_finish(const double* __restrict__ pmax, const double* __restrict__ psum, int nparts, int k,
                             double* __restrict__ colinfo) {
    const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (c >= k) return;
    col_finish_warp(pmax + (size_t)c * nparts, psum + (size_t)c * nparts, nparts, colinfo + 2 * c);
}

// The same inside the kernel that wrote the partials: the last of the column's gridDim.x CTAs
// to finish (a per-column arrival count, which that CTA resets for the next launch) forms
// colinfo[c], in the same order as k_col_finish.  Every thread of the CTA calls it, after
// thread 0 wrote the CTA's partials.
__device__ __forceinline__ void col_finish_last(const double* __restrict__ pmax, const double* __restrict__ psum,
                                                int c, unsigned* __restrict__ cnt, double* __restrict__ colinfo) {
    __shared__ bool last;
    const int nparts = (int)gridDim.x;
    if (threadIdx.x == 0) {
        __threadfence();   // this CTA's partials, then its arrival
        last = atomicAdd(&cnt[c], 1u) == (unsigned)nparts - 1u;
    }
    __syncthreads();
    if (last && threadIdx.x < 32) {
        __threadfence();
        col_finish_warp(pmax + (size_t)c * nparts, psum + (size_t)c * nparts, nparts, colinfo + 2 * c);
        if (threadIdx.x == 0) cnt[c] = 0u;
    }
}

// per-column max |x| and sum over n rows (partials per CTA); with colinfo, the last CTA of
// each column also forms colinfo[c] (col_finish_last)
__global__ void k_col_maxsum(const double* __restrict__ X, int64_t n, int64_t ld, double* __restrict__ pmax,
                             double* __restrict__ psum, unsigned* __restrict__ cnt, double* __restrict__ colinfo) {
    __shared__ double smx[32], ssm[32];
    const int c = blockIdx.y;
    double mx = 0, sm = 0;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const double v = X[r + c * ld];
        mx = absmax_bits(mx, v);
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
    if (colinfo) col_finish_last(pmax, psum, c, cnt, colinfo);
}

// pass-1 epilogue in FP64: u[s,c] = inv_s^2 (2^e_c sum_j 32^-j P1 - 2 f_s S_c); partial max|u|, sum 2 f u,
// and from the column's last CTA colinfo2[c]
template <int ND>
__global__ void k_combine1(const float* __restrict__ part, int nsplit, int nmma, int64_t ldp, int64_t rows, int k,
                           const double* __restrict__ colinfo, const double* __restrict__ f,
                           const double* __restrict__ inv, double* __restrict__ U, double* __restrict__ pmax,
                           double* __restrict__ psum, unsigned* __restrict__ cnt, double* __restrict__ colinfo2) {
    __shared__ double smx[32], ssm[32];
    const int c = blockIdx.y;
    double s_hi, s_lo;
    recombine_scales<ND>((int)colinfo[2 * c], s_hi, s_lo);
    const double Sc = colinfo[2 * c + 1];
    double mx = 0, sm = 0;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < rows; s += (int64_t)gridDim.x * blockDim.x) {
        const double gv = recombine<ND>(part, nsplit, nmma, ldp, c, s, s_hi, s_lo);
        const double iv = inv[s], fs = f[s];
        const double u = iv * iv * (gv - 2.0 * fs * Sc);
        U[s + c * rows] = u;
        mx = absmax_bits(mx, u);
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
    col_finish_last(pmax, psum, c, cnt, colinfo2);   // u's digit scale and centring sum
}

// pass-2 epilogue: out[i,c] = scale (2^e_c sum_j 32^-j P2 - C2_c)
template <int ND>
__global__ void k_combine2(const float* __restrict__ part, int nsplit, int nmma, int64_t ldp, int64_t rows, int k,
                           const double* __restrict__ colinfo, double scale, double* __restrict__ out, int64_t ldo) {
    const int c = blockIdx.y;
    double s_hi, s_lo;
    recombine_scales<ND>((int)colinfo[2 * c], s_hi, s_lo);
    const double C2 = colinfo[2 * c + 1];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += (int64_t)gridDim.x * blockDim.x) {
        out[i + c * ldo] = scale * (recombine<ND, 4>(part, nsplit, nmma, ldp, c, i, s_hi, s_lo) - C2);
    }
}

// blk2 from blk1 by 2-bit block transposes.  blk1 block (t1, c1) holds SNP rows 128 t1 .. + 127
// and individuals 128 c1 .. + 127 (32 bytes per row); blk2 block (t2, c2) holds individual rows
// 128 t2 .. and SNPs 128 c2 .. -- the transpose of blk1 block (c2, t2).  Blocks of blk2 past blk1's
// individual chunks are padding (tile code 10 everywhere, 0xAA).  One 4 KB block at a time per
// CTA: rows staged in shared memory, each thread assembles 16 bytes (64 SNPs) of one individual.
__global__ void __launch_bounds__(256) k_blk_transpose(const uint8_t* __restrict__ blk1, int nch1, int ntiles1,
                                                       uint8_t* __restrict__ blk2, int nch2, int ntiles2) {
    __shared__ uint8_t in[BM][PKB + 1];   // SNP rows x 32 bytes (+1: spreads banks)
    const int64_t nblk = (int64_t)ntiles2 * nch2;
    const int tid = threadIdx.x;
    for (int64_t b = blockIdx.x; b < nblk; b += gridDim.x) {
        const int64_t t2 = b / nch2;
        const int c2 = (int)(b % nch2);
        const int64_t t1 = c2, c1 = t2;
        const bool have = t1 < ntiles1 && c1 < nch1;
        {   // row r, logical half h (physical halves swapped when bit 2 of r is set)
            const int r = tid >> 1, h = tid & 1;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (have)
                v = *reinterpret_cast<const uint4*>(blk1 + (((t1 * nch1 + c1) * BM + r) * 2 + (h ^ ((r >> 2) & 1))) * 16);
            const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int q = 0; q < 16; ++q) in[r][h * 16 + q] = (uint8_t)(w[q >> 2] >> (8 * (q & 3)));
        }
        __syncthreads();
        {   // individual i, logical half hh: SNPs 64 hh .. + 63 of the block
            const int i = tid >> 1, hh = tid & 1;
            const int ib = i >> 2, sh = 2 * (i & 3);
            uint32_t w[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                uint32_t word = 0;
#pragma unroll
                for (int e = 0; e < 16; ++e)
                    word |= (uint32_t)((in[64 * hh + 16 * q + e][ib] >> sh) & 3u) << (2 * e);
                w[q] = word;
            }
            *reinterpret_cast<uint4*>(blk2 + (((t2 * nch2 + c2) * BM + i) * 2 + (hh ^ ((i >> 2) & 1))) * 16) =
                make_uint4(w[0], w[1], w[2], w[3]);
        }
        __syncthreads();
    }
}

// row-major packed rows (stride bytes) -> tile-blocked layout of tile codes, 16 bytes per
// thread; rows >= nrows and bytes >= stride become PLINK 0xFF (genotype 0)
__global__ void k_blockify(const uint8_t* __restrict__ src, int64_t nrows, int64_t stride, int64_t ntiles,
                           int64_t nch, uint8_t* __restrict__ dst) {
    const int64_t total = ntiles * nch * (BM * PKB / 16);
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t blkid = e / (BM * PKB / 16);
        const int within = (int)(e % (BM * PKB / 16));
        const int r = within >> 1, h = within & 1;
        const int64_t t = blkid / nch, c = blkid % nch;
        const int64_t row = t * BM + r, byte = c * PKB + h * 16;
        uint4 v = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu);
        if (row < nrows && byte < stride) {
            if (byte + 16 <= stride) {
                v = *reinterpret_cast<const uint4*>(src + row * stride + byte);
            } else {
                uint8_t tmp[16];
                for (int q = 0; q < 16; ++q) tmp[q] = byte + q < stride ? src[row * stride + byte + q] : (uint8_t)0xFF;
                v = *reinterpret_cast<const uint4*>(tmp);
            }
        }
        v = make_uint4(recode_tile(v.x), recode_tile(v.y), recode_tile(v.z), recode_tile(v.w));
        const int64_t phys = (blkid * BM + r) * 2 + (h ^ ((r >> 2) & 1));   // halves swapped when bit 2 of r is set
        *reinterpret_cast<uint4*>(dst + phys * 16) = v;
    }
}

}  // namespace tc

// ---- host side ---------------------------------------------------------------

using namespace tc;

static int encode_map(globe_ctx* ctx, CUtensorMap* m, const void* base, uint64_t inner, uint64_t outer,
                      uint32_t box_in, uint32_t box_out, bool sw128);

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

int make_map(globe_ctx* ctx, CUtensorMap* m, const void* base, uint64_t inner, uint64_t outer, uint32_t box_in,
                    uint32_t box_out, bool sw128) {
    // a map depends only on these values: reuse the encoding of an earlier call
    const std::vector<uint64_t> key = {(uint64_t)(uintptr_t)base, inner, outer, box_in, box_out, sw128 ? 1u : 0u};
    const auto hit = ctx->map_cache.find(key);
    if (hit != ctx->map_cache.end()) {
        std::memcpy(m, hit->second.data(), sizeof(CUtensorMap));
        return GLOBE_OK;
    }
    GLOBE_RET(encode_map(ctx, m, base, inner, outer, box_in, box_out, sw128));
    if (ctx->map_cache.size() > 256) ctx->map_cache.clear();
    ctx->map_cache[key].assign(reinterpret_cast<const uint8_t*>(m), reinterpret_cast<const uint8_t*>(m) + sizeof(CUtensorMap));
    return GLOBE_OK;
}

static int encode_map(globe_ctx* ctx, CUtensorMap* m, const void* base, uint64_t inner, uint64_t outer,
                      uint32_t box_in, uint32_t box_out, bool sw128) {
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

static int blockify(globe_ctx* ctx, const uint8_t* src, int64_t nrows, int64_t stride, uint8_t** dst, int* nch,
                    int* ntiles) {
    *nch = (int)((stride + PKB - 1) / PKB);
    *ntiles = (int)((nrows + BM - 1) / BM);
    // whole CTAs: round the tile count up to a multiple of TILE_PAD (a CTA owns 1 to 4 tiles)
    *ntiles = (*ntiles + TILE_PAD - 1) / TILE_PAD * TILE_PAD;
    GLOBE_RET(dalloc(ctx, dst, (size_t)(*ntiles) * (*nch) * BM * PKB));
    const int64_t total = (int64_t)(*ntiles) * (*nch) * (BM * PKB / 16);
    k_blockify<<<(unsigned)std::min<int64_t>((total + 255) / 256, 65535), 256, 0, ctx->stream>>>(
        src, nrows, stride, *ntiles, *nch, *dst);
    GLOBE_LAUNCHED(ctx, "k_blockify");
    return GLOBE_OK;
}

// The SNP-major tile-blocked copy (blk1) from the compacted rows, which are freed: every
// genotype kernel reads the tile-blocked copies.  Called when genotypes are loaded.
int ensure_blk1(globe_ctx* ctx) {
    auto& g = ctx->gen;
    if (g.blk1) return GLOBE_OK;
    if (!g.geno) return set_err(ctx, GLOBE_ERR_STATE, "no genotype rows to lay out");
    GLOBE_RET(blockify(ctx, g.geno, g.Mk, g.stride, &g.blk1, &g.nch1, &g.ntiles1));
    GLOBE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    dfree(ctx, g.geno);   // the compacted rows live on as blk1
    g.geno = nullptr;
    return GLOBE_OK;
}

// The individual-major tile-blocked copy (blk2, the tensor-core pass-2 operand) by block
// transposes of blk1; built on the first tensor-core use, so FP64-only work holds one copy.
int ensure_blk2(globe_ctx* ctx) {
    auto& g = ctx->gen;
    if (g.blk2) return GLOBE_OK;
    GLOBE_RET(ensure_blk1(ctx));
    const int32_t N = ctx->coh.N;
    g.strideT = ((g.Mk + 3) / 4 + PKB - 1) / PKB * PKB;   // individual-major row: SNP bytes, whole chunks
    if (g.strideT < PKB) g.strideT = PKB;
    g.nch2 = (int)(g.strideT / PKB);
    g.ntiles2 = (int)((N + BM - 1) / BM);
    g.ntiles2 = (g.ntiles2 + TILE_PAD - 1) / TILE_PAD * TILE_PAD;   // whole CTAs of 1 to 4 tiles
    GLOBE_RET(dalloc(ctx, &g.blk2, (size_t)g.ntiles2 * g.nch2 * BM * PKB));
    const int64_t nblk = (int64_t)g.ntiles2 * g.nch2;
    k_blk_transpose<<<(unsigned)std::min<int64_t>(nblk, 152 * 16), 256, 0, ctx->stream>>>(g.blk1, g.nch1, g.ntiles1,
                                                                                         g.blk2, g.nch2, g.ntiles2);
    GLOBE_LAUNCHED(ctx, "k_blk_transpose");
    GLOBE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return GLOBE_OK;
}

template <int NMMA>
static int launch_gemm(globe_ctx* ctx, const uint8_t* blk, int ntiles, const CUtensorMap& mB, int rows, int nchunks,
                       int splits, float* part, int64_t ldp, unsigned* err, const ZGrid& zg) {
    using G = Geo<NMMA>;
    // every CTA bulk-copies all G::MT of its row tiles: the last one must lie inside blk
    const int64_t ctas_x = (rows + G::MT * BM - 1) / (G::MT * BM);
    if (ctas_x * G::MT > ntiles)
        return set_err(ctx, GLOBE_ERR_ARG, "k_tc_gemm: %lld CTAs of %d row tiles need %lld tiles; the copy holds %d",
                       (long long)ctas_x, G::MT, (long long)(ctas_x * G::MT), ntiles);
    const int cps = (nchunks + splits - 1) / splits;
    splits = (nchunks + cps - 1) / cps;
    const size_t smem = sizeof(Smem<NMMA, G::MT>) + 1024;
    // the shared-memory opt-in is a per-device attribute of the kernel
    static std::atomic<uint64_t> attr_set{0};
    const uint64_t bit = 1ull << (ctx->device & 63);
    if (!(attr_set.load() & bit)) {
        GLOBE_CK(ctx, cudaFuncSetAttribute(k_tc_gemm<NMMA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set.fetch_or(bit);
    }
    dim3 grid((unsigned)((rows + G::MT * BM - 1) / (G::MT * BM)), (unsigned)splits, (unsigned)zg.nz);
    k_tc_gemm<NMMA><<<grid, G::NTHREADS, smem, ctx->stream>>>(blk, mB, rows, nchunks, cps, part, ldp, zg.pz,
                                                               zg.skip0, zg.skipz, err, zg.stall);
    GLOBE_LAUNCHED(ctx, "k_tc_gemm");
    return GLOBE_OK;
}

int rows_per_cta(int nmma) { return BM * (nmma <= 64 ? 4 : (nmma <= 192 ? 2 : 1)); }

int gemm_dispatch(globe_ctx* ctx, int nmma, const uint8_t* mA, int ntiles, const CUtensorMap& mB, int rows, int nchunks,
                  int splits, float* part, int64_t ldp, unsigned* err, const ZGrid& zg) {
    switch (nmma) {
        case 16: return launch_gemm<16>(ctx, mA, ntiles, mB, rows, nchunks, splits, part, ldp, err, zg);
        case 32: return launch_gemm<32>(ctx, mA, ntiles, mB, rows, nchunks, splits, part, ldp, err, zg);
        case 48: return launch_gemm<48>(ctx, mA, ntiles, mB, rows, nchunks, splits, part, ldp, err, zg);
        case 64: return launch_gemm<64>(ctx, mA, ntiles, mB, rows, nchunks, splits, part, ldp, err, zg);
        case 80: return launch_gemm<80>(ctx, mA, ntiles, mB, rows, nchunks, splits, part, ldp, err, zg);
        case 96: return launch_gemm<96>(ctx, mA, ntiles, mB, rows, nchunks, splits, part, ldp, err, zg);
        case 112: return launch_gemm<112>(ctx, mA, ntiles, mB, rows, nchunks, splits, part, ldp, err, zg);
        case 128: return launch_gemm<128>(ctx, mA, ntiles, mB, rows, nchunks, splits, part, ldp, err, zg);
        case 144: return launch_gemm<144>(ctx, mA, ntiles, mB, rows, nchunks, splits, part, ldp, err, zg);
        case 160: return launch_gemm<160>(ctx, mA, ntiles, mB, rows, nchunks, splits, part, ldp, err, zg);
        case 176: return launch_gemm<176>(ctx, mA, ntiles, mB, rows, nchunks, splits, part, ldp, err, zg);
        case 192: return launch_gemm<192>(ctx, mA, ntiles, mB, rows, nchunks, splits, part, ldp, err, zg);
        case 208: return launch_gemm<208>(ctx, mA, ntiles, mB, rows, nchunks, splits, part, ldp, err, zg);
        case 224: return launch_gemm<224>(ctx, mA, ntiles, mB, rows, nchunks, splits, part, ldp, err, zg);
        case 240: return launch_gemm<240>(ctx, mA, ntiles, mB, rows, nchunks, splits, part, ldp, err, zg);
        case 256: return launch_gemm<256>(ctx, mA, ntiles, mB, rows, nchunks, splits, part, ldp, err, zg);
    }
    return set_err(ctx, GLOBE_ERR_ARG, "unsupported MMA width %d", nmma);
}

int eff_splits(int nchunks, int splits) {
    const int cps = (nchunks + splits - 1) / splits;
    return (nchunks + cps - 1) / cps;
}

// Split-K candidates for `tiles` CTA row blocks of `nchunks` K stages.  One CTA runs per SM,
// so the pass takes about ceil(CTAs / SMs) waves of (stages per CTA + a fixed CTA cost: setup,
// pipeline fill and drain, epilogue).  The count minimising that estimate comes first, within
// K per CTA <= 2^19 (exact FP32 sums) and >= 8 stages per CTA; then up to 4 more effective
// counts whose estimate is within 25% of it, 3 in all (the autotuner times them).  Example: 196 row
// blocks x 3907 stages gives 10 splits (1960 CTAs, 12.9 waves on 152 SMs) where aiming at ~8
// waves gave 7 (1372 CTAs, 9.03 waves: a tenth wave of 4 CTAs).
static std::vector<int> split_candidates_model(globe_ctx* ctx, int tiles, int nchunks);
static const std::vector<int>& split_candidates(globe_ctx* ctx, int tiles, int nchunks) {
    auto& v = ctx->split_cache[{tiles, nchunks}];
    if (v.empty()) v = split_candidates_model(ctx, tiles, nchunks);
    return v;
}
static std::vector<int> split_candidates_model(globe_ctx* ctx, int tiles, int nchunks) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess || sms < 1) sms = 152;
    constexpr int CTA_COST = 8;                       // fixed cost of a CTA, in stages
    const int lo = std::max(1, (nchunks + 4095) / 4096);
    const int hi = std::max(lo, std::min(64, nchunks / 8));
    std::vector<std::pair<double, int>> est;          // (cost, split count) per effective count
    int prev_se = -1;
    for (int s = lo; s <= hi; ++s) {
        const int cps = (nchunks + s - 1) / s;
        const int se = (nchunks + cps - 1) / cps;
        if (se == prev_se) continue;
        prev_se = se;
        const double waves = std::ceil((double)tiles * se / sms);
        est.push_back({waves * (cps + CTA_COST), s});
    }
    std::stable_sort(est.begin(), est.end(),
                     [](const std::pair<double, int>& a, const std::pair<double, int>& b) { return a.first < b.first * 0.999; });
    std::vector<int> out;
    for (const auto& e : est)
        if (out.size() < 3 && e.first <= est[0].first * 1.25) out.push_back(e.second);
    return out;
}

// Tuned choices shared by every context of the process, per device and shape: a shape is
// timed once however many contexts use it.
static std::mutex g_tune_mu;
static std::map<std::vector<int64_t>, int> g_tuned;

static bool tuned_lookup(globe_ctx* ctx, std::vector<int64_t> key, int* out) {
    key.push_back(ctx->device);
    std::lock_guard<std::mutex> lock(g_tune_mu);
    const auto hit = g_tuned.find(key);
    if (hit == g_tuned.end()) return false;
    *out = hit->second;
    return true;
}

static void tuned_store(globe_ctx* ctx, std::vector<int64_t> key, int v) {
    key.push_back(ctx->device);
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tuned[key] = v;
}

static void tune_note(globe_ctx* ctx, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (!ctx->tune_log.empty()) ctx->tune_log += ",";
    ctx->tune_log += buf;
}

// Time each of `nc` variants (run(i) issues variant i on the stream) over `rounds` rounds with
// CUDA events on the context's stream; the last round's times go to ms[].  Within a round the
// variants run last to first, so a first-launch cost falls on an alternative, not on variant 0.
// Returns the index of the fastest: variant 0 unless another is more than 1% faster.
template <class F>
static int time_variants(globe_ctx* ctx, int nc, int rounds, F&& run, std::vector<float>& ms, int* best) {
    std::vector<cudaEvent_t> ev(2 * nc, nullptr);
    for (auto& e : ev) GLOBE_CK(ctx, cudaEventCreate(&e));
    int rc = GLOBE_OK;
    for (int r = 0; r < rounds && rc == GLOBE_OK; ++r)
        for (int i = nc - 1; i >= 0 && rc == GLOBE_OK; --i) {
            cudaEventRecord(ev[2 * i], ctx->stream);
            rc = run(i);
            cudaEventRecord(ev[2 * i + 1], ctx->stream);
        }
    if (rc == GLOBE_OK) rc = cudaStreamSynchronize(ctx->stream) == cudaSuccess ? GLOBE_OK : GLOBE_ERR_CUDA;
    ms.assign(nc, 0.0f);
    *best = 0;
    for (int i = 0; i < nc && rc == GLOBE_OK; ++i) {
        cudaEventElapsedTime(&ms[i], ev[2 * i], ev[2 * i + 1]);
        if (ms[i] < ms[*best] * 0.99f) *best = i;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    if (rc != GLOBE_OK) return set_err(ctx, rc, "autotuning: %s", cudaGetErrorString(cudaGetLastError()));
    return GLOBE_OK;
}

// The split count of one genotype pass: the test override, the tuned choice of this shape, or
// -- on its first use in the process, with autotuning on, outside graph capture and event
// profiling -- each candidate launched once and timed, the fastest kept.  Every count gives the
// same result bits (the split partials are exact and are summed in int64), so the candidates
// run on the real operands and the pass's own launch follows.
static int tune_splits(globe_ctx* ctx, int pass, int nmma, const uint8_t* blk, int ntiles, const CUtensorMap& mB,
                       int rows, int nchunks, const std::vector<int>& cand, float* part, int64_t ldp, unsigned* err,
                       int* out) {
    if (ctx->force_splits > 0) {   // at least the count that keeps K per CTA <= 2^19
        *out = std::max(ctx->force_splits, (nchunks + 4095) / 4096);
        return GLOBE_OK;
    }
    const std::vector<int64_t> key = {1, pass, nmma, rows, nchunks};
    *out = cand[0];
    if (!ctx->autotune || cand.size() < 2) return GLOBE_OK;
    if (tuned_lookup(ctx, key, out)) return GLOBE_OK;
    if (ctx->capturing || ctx->prof_on) return GLOBE_OK;
    std::vector<float> ms;
    int best = 0;
    GLOBE_RET(time_variants(ctx, (int)cand.size(), 1, [&](int i) {
        return gemm_dispatch(ctx, nmma, blk, ntiles, mB, rows, nchunks, cand[i], part, ldp, err, ZGrid());
    }, ms, &best));
    *out = cand[best];
    tuned_store(ctx, key, *out);
    std::string t;
    for (size_t i = 0; i < cand.size(); ++i) {
        char b[48];
        std::snprintf(b, sizeof b, "%s\"%d\": %.4f", i ? ", " : "", cand[i], ms[i]);
        t += b;
    }
    tune_note(ctx, "{\"kind\": \"splits\", \"pass\": %d, \"mma_width\": %d, \"rows\": %d, \"k_stages\": %d, "
              "\"model\": %d, \"choice\": %d, \"ms\": {%s}}", pass, nmma, rows, nchunks, cand[0], *out, t.c_str());
    return GLOBE_OK;
}

// out (N x k) = scale * Zs'(Zs Z) for one group of <= 256 / ND columns, ND digits per column
template <int ND>
static int tc_group(globe_ctx* ctx, const double* Z, int kg, double scale, double* out) {
    auto& g = ctx->gen;
    const int32_t N = ctx->coh.N;
    const int nmma = ((kg * ND + 15) / 16) * 16;
    // ---- pass 1 operands
    const int nch1 = g.nch1;
    const int64_t kpad1 = (int64_t)nch1 * BK;
    const int nch2 = g.nch2;
    const int64_t kpad2 = (int64_t)nch2 * BK;
    const int rpc = rows_per_cta(nmma);
    const int tiles1 = (int)((g.Mk + rpc - 1) / rpc), tiles2 = (N + rpc - 1) / rpc;
    const std::vector<int>& cand1 = split_candidates(ctx, tiles1, nch1);
    const std::vector<int>& cand2 = split_candidates(ctx, tiles2, nch2);
    auto most = [&](const std::vector<int>& c, int nch) {   // partial slots for any count used below
        int m = std::max(ctx->force_splits, (nch + 4095) / 4096);
        for (int v : c) m = std::max(m, v);
        return m;
    };
    const int spmax1 = most(cand1, nch1), spmax2 = most(cand2, nch2);
    const int64_t ldp1 = (int64_t)tiles1 * rpc, ldp2 = (int64_t)tiles2 * rpc;
    uint8_t *D1, *D2;
    float *P1, *P2;
    double *U, *cst, *pm, *ps;
    unsigned* err;
    GLOBE_RET(ws(ctx, WS_TC_D1, (size_t)nmma * kpad1, &D1));
    GLOBE_RET(ws(ctx, WS_TC_D2, (size_t)nmma * kpad2, &D2));
    GLOBE_RET(ws(ctx, WS_TC_P1, (size_t)(spmax1 + 1) * nmma * ldp1, &P1));
    GLOBE_RET(ws(ctx, WS_TC_P2, (size_t)(spmax2 + 1) * nmma * ldp2, &P2));
    GLOBE_RET(ws(ctx, WS_TC_U, (size_t)g.Mk * kg + 1, &U));
    const int nbr = 304;
    GLOBE_RET(ws(ctx, WS_TC_SCAL, (size_t)(4 * kg + 2 * nbr * kg + 8), &cst));
    double* col1 = cst;           // 2*kg
    double* col2 = cst + 2 * kg;  // 2*kg
    pm = cst + 4 * kg;
    ps = pm + (size_t)nbr * kg;
    GLOBE_RET(tc_err_word(ctx, &err));
    CUtensorMap mB1, mB2;
    GLOBE_RET(make_map(ctx, &mB1, D1, (uint64_t)kpad1, (uint64_t)nmma, BK, (uint32_t)nmma, true));
    GLOBE_RET(make_map(ctx, &mB2, D2, (uint64_t)kpad2, (uint64_t)nmma, BK, (uint32_t)nmma, true));
    // ---- digits of Z
    const int nz = col_parts(N);
    unsigned* cnt;
    GLOBE_RET(tc_counters(ctx, 2 * kg, &cnt));
    k_col_maxsum<<<dim3(nz, kg), 256, 0, ctx->stream>>>(Z, N, N, pm, ps, cnt, col1);
    GLOBE_LAUNCHED(ctx, "k_col_maxsum");
    // digit rows past the kg columns stay zero
    if (nmma > kg * ND)
        GLOBE_CK(ctx, cudaMemsetAsync(D1 + (size_t)kg * ND * kpad1, 0, (size_t)(nmma - kg * ND) * kpad1,
                                      ctx->stream));
    k_digits<ND, true><<<dim3((unsigned)std::min<int64_t>(div_up(kpad1 / 4, 256), 1024), kg), 256, 0, ctx->stream>>>(
        Z, N, N, kg, col1, D1, kpad1);
    GLOBE_LAUNCHED(ctx, "k_digits");
    // ---- pass 1
    int sp1 = 0;
    GLOBE_RET(tune_splits(ctx, 1, nmma, g.blk1, g.ntiles1, mB1, (int)g.Mk, nch1, cand1, P1, ldp1, err, &sp1));
    {
        ProfScope p(ctx, GLOBE_PROF_GRM_PASS1);
        ZGrid zg;
        zg.stall = ctx->stall_next_gemm;
        ctx->stall_next_gemm = 0;
        GLOBE_RET(gemm_dispatch(ctx, nmma, g.blk1, g.ntiles1, mB1, (int)g.Mk, nch1, sp1, P1, ldp1, err, zg));
    }
    const int sp1e = eff_splits(nch1, sp1);
    k_combine1<ND><<<dim3(nbr, kg), 256, 0, ctx->stream>>>(P1, sp1e, nmma, ldp1, g.Mk, kg, col1, g.f, g.inv, U, pm, ps,
                                                           cnt + kg, col2);
    GLOBE_LAUNCHED(ctx, "k_combine1");
    // ---- digits of u, pass 2
    if (nmma > kg * ND)
        GLOBE_CK(ctx, cudaMemsetAsync(D2 + (size_t)kg * ND * kpad2, 0, (size_t)(nmma - kg * ND) * kpad2,
                                      ctx->stream));
    k_digits<ND, true><<<dim3((unsigned)std::min<int64_t>(div_up(kpad2 / 4, 256), 2048), kg), 256, 0, ctx->stream>>>(
        U, g.Mk, g.Mk, kg, col2, D2, kpad2);
    GLOBE_LAUNCHED(ctx, "k_digits");
    int sp2 = 0;
    GLOBE_RET(tune_splits(ctx, 2, nmma, g.blk2, g.ntiles2, mB2, N, nch2, cand2, P2, ldp2, err, &sp2));
    {
        ProfScope p(ctx, GLOBE_PROF_GRM_PASS2);
        GLOBE_RET(gemm_dispatch(ctx, nmma, g.blk2, g.ntiles2, mB2, N, nch2, sp2, P2, ldp2, err, ZGrid()));
    }
    const int sp2e = eff_splits(nch2, sp2);
    k_combine2<ND><<<dim3(div_up(N, 256) < 1024 ? div_up(N, 256) : 1024, kg), 256, 0, ctx->stream>>>(
        P2, sp2e, nmma, ldp2, N, kg, col2, scale, out, N);
    GLOBE_LAUNCHED(ctx, "k_combine2");
    return GLOBE_OK;
}

static int tc_group_nd(globe_ctx* ctx, int nd, const double* Z, int kg, double scale, double* out) {
    switch (nd) {
        case 2: return tc_group<2>(ctx, Z, kg, scale, out);
        case 3: return tc_group<3>(ctx, Z, kg, scale, out);
        case 4: return tc_group<4>(ctx, Z, kg, scale, out);
        case 5: return tc_group<5>(ctx, Z, kg, scale, out);
        case 6: return tc_group<6>(ctx, Z, kg, scale, out);
        case 7: return tc_group<7>(ctx, Z, kg, scale, out);
        case 8: return tc_group<8>(ctx, Z, kg, scale, out);
        case 9: return tc_group<9>(ctx, Z, kg, scale, out);
    }
    return set_err(ctx, GLOBE_ERR_ARG, "unsupported digit count %d", nd);
}

int geno_apply_tc(globe_ctx* ctx, const double* Z, int k, double scale, double* out) {
    auto& g = ctx->gen;
    const int32_t N = ctx->coh.N;
    if (g.Mk == 0) {
        GLOBE_CK(ctx, cudaMemsetAsync(out, 0, sizeof(double) * (size_t)N * k, ctx->stream));
        return GLOBE_OK;
    }
    GLOBE_RET(ensure_blk2(ctx));
    const int nd = ctx->digits;
    // near-equal groups of <= 256 / nd columns (MMA width <= 256).  Groups wider than
    // 192 / nd (MMA width > 192) run one row tile per CTA, which costs more per column than
    // two groups of two tiles once k > 256 / nd: then groups of <= 192 / nd columns
    // (at 9 digits: 28 and 21; 65 -> 17 + 16 + 16 + 16).
    const int gmax = 256 / nd, gtwo = 192 / nd;
    int ng = (k + gmax - 1) / gmax;
    if (ng > 1) ng = (k + gtwo - 1) / gtwo;
    auto run = [&](int ngroups) -> int {
        for (int gi = 0, c0 = 0; gi < ngroups; ++gi) {
            const int kg = k / ngroups + (gi < k % ngroups ? 1 : 0);
            GLOBE_RET(tc_group_nd(ctx, nd, Z + (size_t)c0 * N, kg, scale, out + (size_t)c0 * N));
            c0 += kg;
        }
        return GLOBE_OK;
    };
    // Column grouping: the rule above, or -- for 9 or more columns, on first use of (k, digits,
    // N, SNPs), with autotuning on, outside capture and profiling -- the faster of it and one
    // group more, timed over two rounds (the first also tunes the groups' split counts).  Each column's digits and sums do not depend on its group, so every grouping
    // gives the same bits and the last run's output stands.
    const std::vector<int64_t> key = {2, k, nd, N, (int64_t)g.Mk};
    if (!ctx->autotune || ctx->force_splits > 0 || k < 9) return run(ng);
    int chosen = ng;
    if (tuned_lookup(ctx, key, &chosen)) return run(chosen);
    if (ctx->capturing || ctx->prof_on || ng + 1 > k) return run(ng);
    const std::vector<int> cand = {ng, ng + 1};
    std::vector<float> ms;
    int best = 0;
    GLOBE_RET(time_variants(ctx, (int)cand.size(), 2, [&](int i) { return run(cand[i]); }, ms, &best));
    tuned_store(ctx, key, cand[best]);
    std::string t;
    for (size_t i = 0; i < cand.size(); ++i) {
        char b[48];
        std::snprintf(b, sizeof b, "%s\"%d\": %.4f", i ? ", " : "", cand[i], ms[i]);
        t += b;
    }
    tune_note(ctx, "{\"kind\": \"groups\", \"columns\": %d, \"digits\": %d, \"model\": %d, \"choice\": %d, "
              "\"ms\": {%s}}", k, nd, ng, cand[best], t.c_str());
    return run(cand[best]);
}

// The tensor-core kernels' error word: word 0 of the WS_TC_ERR slot (words 1-2 serve
// k_dense_absmax).  Cleared once, when the slot is created; the kernels only set bits in it
// and tc_check_error reads and clears it, so a timeout in any product of a solve is still
// reported when the solve ends.
int tc_err_word(globe_ctx* ctx, unsigned** err) {
    const bool fresh = ctx->ws[WS_TC_ERR].p == nullptr;
    GLOBE_RET(ws(ctx, WS_TC_ERR, 4, err));
    if (fresh) GLOBE_CK(ctx, cudaMemsetAsync(*err, 0, 4 * sizeof(unsigned), ctx->stream));
    return GLOBE_OK;
}

// per-column arrival counts of col_finish_last, zero between launches: (re)created zeroed when
// more are needed (never inside a capture, where allocation is refused; every shape's first
// product runs outside one)
int tc_counters(globe_ctx* ctx, size_t n, unsigned** cnt) {
    const bool fresh = ctx->ws[WS_TC_CNT].bytes < n * sizeof(unsigned);
    GLOBE_RET(ws(ctx, WS_TC_CNT, n, cnt));
    if (fresh) GLOBE_CK(ctx, cudaMemsetAsync(*cnt, 0, ctx->ws[WS_TC_CNT].bytes, ctx->stream));
    return GLOBE_OK;
}

int tc_check_error(globe_ctx* ctx) {
    unsigned h = 0;
    void* p = ctx->ws[WS_TC_ERR].p;
    if (!p) return GLOBE_OK;
    GLOBE_CK(ctx, cudaMemcpyAsync(&h, p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    GLOBE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (!h) return GLOBE_OK;
    GLOBE_CK(ctx, cudaMemsetAsync(p, 0, sizeof(unsigned), ctx->stream));
    return set_err(ctx, GLOBE_ERR_CUDA, "tensor-core GRM kernel timed out waiting (code 0x%x)", h);
}

int with_tc_check(globe_ctx* ctx, int precision, int rc) {
    if (precision != GLOBE_PREC_MIXED) return rc;
    const int rt = tc_check_error(ctx);
    return rt != GLOBE_OK ? rt : rc;
}

}  // namespace globe
