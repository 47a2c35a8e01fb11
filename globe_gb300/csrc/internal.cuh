// internal.cuh -- context state and shared helpers of libglobe_gb300.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "globe.h"

namespace globe {

// Device layout of one cohort (all column-major, ld = rows):
//   X      Nrec x (p+1), time = last column            (double)
//   y      Nrec                                        (double)
//   blocks: one per individual, records contiguous;   bstart[N+1], bind[N]
//           (individual of block b), rind[Nrec] (individual of record r)
//   moments per block: n, sum t, sum t^2              (double, N each)
// Genetic source:
//   genotype: kept SNP rows, `stride` bytes each (multiple of 16), PLINK
//             2-bit codes; per-SNP zs table zs[s*4 + code] (double) with
//             zs = (g - 2f) * inv_std, missing -> g = 0
//   dense:    packed lower triangle float32, N(N+1)/2
constexpr int SHORT_BLOCK = 48;   // longest record block handled by one thread in the record kernels

struct Cohort {
    int64_t Nrec = 0;
    int32_t N = 0, p = 0;
    double* X = nullptr;
    double* y = nullptr;
    int32_t* bstart = nullptr;
    int32_t* bind = nullptr;
    int32_t* rind = nullptr;
    double* bn = nullptr;
    double* bt = nullptr;
    double* btt = nullptr;
    int32_t max_block = 0;
    int32_t* lblk = nullptr;   // blocks with more than SHORT_BLOCK records (device list)
    int32_t nlong = 0;
    float2* tdf = nullptr;     // times as double-float pairs (the double-float record kernels)
    double tmax = 0;           // max |t|
    const double* times() const { return X + (size_t)p * Nrec; }
};

enum GeneticSource { GSRC_NONE = 0, GSRC_GENO = 1, GSRC_DENSE = 2 };

struct Genetic {
    int src = GSRC_NONE;
    // genotype source
    int64_t Mk = 0;          // kept SNPs
    int64_t stride = 0;      // bytes per SNP row (multiple of 16)
    uint8_t* geno = nullptr; // Mk x stride compacted rows (PLINK codes), freed once blk1 exists
    double* zs = nullptr;    // Mk x 4
    double* f = nullptr;     // Mk
    double* inv = nullptr;   // Mk
    int64_t strideT = 0;     // bytes of an individual-major row of blk2 (whole 32-byte chunks)
    // tile-blocked copies (tile codes): block (tile, chunk) = 128 rows x 32 B
    uint8_t* blk1 = nullptr;   // SNP-major: every genotype kernel (built at load)
    uint8_t* blk2 = nullptr;   // individual-major: tensor-core pass 2, GRM build (first use)
    int nch1 = 0, ntiles1 = 0, nch2 = 0, ntiles2 = 0;
    // dense source
    float* grm = nullptr;    // N(N+1)/2
    // digit planes of the dense GRM for the tensor-core product (first GLOBE_PREC_MIXED use):
    // adig_da planes of adig_rows / adig_da rows x adig_np bytes, A ~ 2^adig_e sum_d a_d 32^-d
    uint8_t* adig = nullptr;
    int adig_state = 0;      // 0 not built, 1 ready, -1 unusable (memory, non-finite A): double-float kernel
    int adig_da = 0, adig_e = 0;
    int64_t adig_np = 0, adig_rows = 0;
    // both
    double* gdiag = nullptr; // A_ii
    bool gdiag_ok = false;
};

// Growable device workspace slots.
struct Slot {
    void* p = nullptr;
    size_t bytes = 0;
};

enum SlotId {
    WS_R, WS_Z, WS_P, WS_VP, WS_ZI, WS_GZ, WS_S1, WS_PART, WS_SCAL, WS_COLS, WS_W,
    WS_GPART, WS_B, WS_TMP1, WS_TMP2, WS_TMP3, WS_TMP4, WS_H, WS_HSTAR, WS_PROBE,
    WS_UH, WS_SMALL, WS_IO1, WS_IO2, WS_BHAT, WS_FB, WS_FX,
    WS_TC_D1, WS_TC_D2, WS_TC_P1, WS_TC_P2, WS_TC_U, WS_TC_SCAL, WS_TC_ERR, WS_LOOP, WS_S0DF, WS_HDF, WS_TC_CNT, WS_COUNT
};

// Scalars kept on the device during a solve (per column, k entries each).
struct PcgScalars {
    double* rz;     // r'z
    double* rz_new;
    double* pvp;    // p'Vp
    double* alpha;
    double* beta;
    double* rr;     // |r|^2
    double* bb;     // |b|^2
};

}  // namespace globe

struct globe_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    int64_t dev_bytes = 0;
    int64_t launches = 0;
    globe::Cohort coh;
    globe::Genetic gen;
    double vc[5] = {0, 0, 0, 0, 0};
    bool vc_set = false;
    int prec = GLOBE_PREC_FP64;   // precision of operator calls (globe_set_precision / PCG options)
    int model = GLOBE_MODEL_FULL; // GLOBE_MODEL_NO_TIME: components (sig2e, sig2g) only
    int digits = 9;               // base-32 digits per column of the tensor-core product (globe_set_digits)
    int stall_next_gemm = 0;      // test hook of the bounded waits (globe_debug_stall_next_gemm)
    // autotuning of the tensor-core genotype product (k_tc_geno.cu): split-K counts and column
    // groupings, timed on first use and shared by the process's contexts; 0 = the cost model
    // only (globe_set_autotune)
    int autotune = 1;
    int force_splits = 0;         // test hook: every tensor-core launch uses this split count
    // host-side results that repeat every product of a shape: split-K candidates per
    // (row blocks, K stages) and encoded tensor maps per (base, sizes, box, swizzle)
    std::map<std::pair<int, int>, std::vector<int>> split_cache;
    std::map<std::vector<uint64_t>, std::vector<uint8_t>> map_cache;
    std::string tune_log;         // this context's decisions, JSON objects, comma separated
    int nvc() const { return model == GLOBE_MODEL_NO_TIME ? 2 : 5; }
    bool precond_ok = false;      // H built for the current vc
    globe::Slot ws[globe::WS_COUNT];
    // MME state (V^-1 X, (X'V^-1X)^-1, V^-1 r, uhat) kept for AIREML terms
    double* vinv_X = nullptr;
    double* vinv_r = nullptr;
    double* uhat = nullptr;
    double* f_theta = nullptr;    // Nrec x 5, last globe_aireml_grad
    std::vector<double> xtvx_inv;
    bool mme_ok = false;
    bool fth_ok = false;
    std::vector<std::pair<void*, size_t>> allocs;  // persistent allocations (freed on destroy)
    double* hpin = nullptr;       // pinned host scratch for per-iteration scalars
    size_t hpin_n = 0;
    // CUDA graphs of the block-PCG iteration body (globe_set_graphs), one per parity of the
    // swapped r'z buffers; updated in place from each call's capture
    int graphs = 1;
    cudaGraphExec_t pcg_graph[2] = {nullptr, nullptr};
    // the device-side PCG loop of the last call (one WHILE conditional node), and whether to use it
    cudaGraphExec_t pcg_loop = nullptr;
    int device_loop = 1;
    int64_t device_loop_runs = 0;
    // record kernels of GLOBE_PREC_MIXED solves in double-float (k_records_df.cu), and how many
    // solves ran them (globe_set_record_df)
    int record_df = 1;
    int64_t record_df_runs = 0;
    bool capturing = false;       // a stream capture is open: allocation is refused
    // event profiling (globe_prof_*)
    bool prof_on = false;
    struct ProfEv {
        int kind;
        cudaEvent_t a, b;
    };
    std::vector<ProfEv> prof_pool;
    size_t prof_used = 0;
    int64_t prof_count[GLOBE_PROF_KINDS] = {0};
    double prof_ms[GLOBE_PROF_KINDS] = {0};
};

namespace globe {

int set_err(globe_ctx* ctx, int code, const char* fmt, ...);
int cuda_err(globe_ctx* ctx, cudaError_t e, const char* what);

// persistent device allocation tracked by the context
int dalloc_bytes(globe_ctx* ctx, void** p, size_t bytes);
template <class T>
int dalloc(globe_ctx* ctx, T** p, size_t n) {
    return dalloc_bytes(ctx, (void**)p, n * sizeof(T));
}
void dfree(globe_ctx* ctx, void* p);
// workspace slot of at least `bytes`
int wslot(globe_ctx* ctx, int id, size_t bytes, void** out);
template <class T>
int ws(globe_ctx* ctx, int id, size_t n, T** out) {
    return wslot(ctx, id, n * sizeof(T), (void**)out);
}

#define GLOBE_CK(ctx, call)                                          \
    do {                                                             \
        cudaError_t e__ = (call);                                    \
        if (e__ != cudaSuccess) return ::globe::cuda_err(ctx, e__, #call); \
    } while (0)

#define GLOBE_RET(call)                 \
    do {                                \
        int rc__ = (call);              \
        if (rc__ != GLOBE_OK) return rc__; \
    } while (0)

// launch bookkeeping: count + error check
int after_launch(globe_ctx* ctx, const char* name);
#define GLOBE_LAUNCHED(ctx, name) GLOBE_RET(::globe::after_launch(ctx, name))

inline int div_up(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// profiling scopes: prof_begin returns a handle (or -1 when off)
int prof_begin(globe_ctx* ctx, int kind);
void prof_end(globe_ctx* ctx, int h);
// An NVTX range for the lifetime of a scope: the solve's structure (solves, iterations,
// GRM products and their passes, AIREML steps) on an Nsight Systems or ncu --nvtx
// timeline.  Without a tool attached the calls return at once.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};
inline const char* prof_kind_name(int kind) {
    static const char* names[GLOBE_PROF_KINDS] = {"GRM product", "GRM pass 1", "GRM pass 2", "PCG iteration",
                                                  "GRM build", "GRM build GEMM", "profile kind 6", "profile kind 7"};
    return (kind >= 0 && kind < GLOBE_PROF_KINDS) ? names[kind] : "profile kind";
}
// CUDA-event timing of one kind of work (globe_prof_enable) and its NVTX range
struct ProfScope {
    globe_ctx* c;
    int h;
    NvtxRange r;
    ProfScope(globe_ctx* ctx, int kind) : c(ctx), h(prof_begin(ctx, kind)), r(prof_kind_name(kind)) {}
    ~ProfScope() { prof_end(c, h); }
};

// ---- bounds-checked debug build -------------------------------------------------
// Built with -DGLOBE_CHECK_BOUNDS (e.g. GLOBE_BUILD_TAG=bounds GLOBE_NVCC_FLAGS=
// -DGLOBE_CHECK_BOUNDS), the kernels check the indices they take from data (record
// ranges, individual indices) before using them.  A failed check records its code in a
// device word of its translation unit (the first one wins) and the access is skipped;
// nothing traps.  globe_debug_bounds reads and clears the words.  Without the macro
// GLOBE_BOUNDS(cond, code) is the constant true and the checks compile away.
int register_bounds_word(int (*query)(unsigned* code, bool clear));
int query_bounds_words(unsigned* first_code);   // 0: none failed, 1: a code, < 0: error
#if defined(GLOBE_CHECK_BOUNDS) && defined(__CUDACC__)
static __device__ unsigned g_bounds_code = 0u;   // one per translation unit
__device__ __forceinline__ bool bounds_ok(bool ok, unsigned code) {
    if (!ok) atomicCAS(&g_bounds_code, 0u, code);
    return ok;
}
static int query_bounds_word_tu(unsigned* code, bool clear) {
    if (cudaMemcpyFromSymbol(code, g_bounds_code, sizeof(unsigned)) != cudaSuccess) return -1;
    const unsigned zero = 0u;
    if (clear && cudaMemcpyToSymbol(g_bounds_code, &zero, sizeof(unsigned)) != cudaSuccess) return -1;
    return 0;
}
static const int g_bounds_registered = register_bounds_word(&query_bounds_word_tu);
#define GLOBE_BOUNDS(cond, code) ::globe::bounds_ok((cond), (code))
#else
#define GLOBE_BOUNDS(cond, code) true
#endif

// ---- kernels entry points (defined in the k_*.cu files) ----

// k_bed.cu
int bed_stats(globe_ctx* ctx, const uint8_t* d_bed, int64_t M, int64_t stride, int32_t N,
              float min_maf, float max_miss, int64_t* d_alt, int64_t* d_miss, float* d_maf,
              float* d_mr, uint8_t* d_keep);
int bed_compact(globe_ctx* ctx, const uint8_t* d_bed, int64_t stride_in, const int64_t* d_idx,
                int64_t Mk, int64_t bps, uint8_t* d_out, int64_t stride_out);
int snp_coefs(globe_ctx* ctx, const int64_t* d_alt, const int64_t* d_miss, const int64_t* d_idx,
              int64_t Mk, int32_t N, double* d_f, double* d_inv, double* d_zs);
int synth_bed(globe_ctx* ctx, uint8_t* d_bed, int64_t M, int32_t N, int64_t stride, uint64_t seed,
              float maf_lo, float maf_hi, float miss_rate);

// k_records.cu
int block_moments(globe_ctx* ctx);
int build_H(globe_ctx* ctx, const double* gdiag, double gconst, double* H, float2* Hdf = nullptr);
int seg_sums(globe_ctx* ctx, const double* x, const double* z, const double* beta, double* xout,
             const int32_t* cols, int kact, double* Zi, double* S1);
// with dot_out and quot: also quot[col] = num[col] / dot_out[col] (the step length, fused)
int vx_assemble(globe_ctx* ctx, const double* x, const double* GZ, const double* Zi,
                const double* S1, const int32_t* cols, int kact, double* out, double* dot_out,
                const double* num = nullptr, double* quot = nullptr);
int pcg_update(globe_ctx* ctx, const double* H, const double* alpha, double* x, double* r,
               const double* p, const double* Vp, double* z, const int32_t* cols, int kact,
               double* rr, double* rz);
int precond_apply(globe_ctx* ctx, const double* H, const double* r, double* z,
                  const int32_t* cols, int kact, double* rz);
int precond_apply_scratch(globe_ctx* ctx, const double* H, const double* r, double* z, int kact, double* part,
                          size_t part_cap, double* rz);
int col_dots(globe_ctx* ctx, const double* a, const double* b, int64_t n, int64_t lda, int64_t ldb,
             const int32_t* cols, int kact, double* out);
int scal_alpha(globe_ctx* ctx, const double* num, const double* den, double* out, int kact,
               float2* out_df = nullptr);
int xt_mat(globe_ctx* ctx, const double* X, int m1, const double* S, int m2, double* out);
int sub_mat(globe_ctx* ctx, const double* A, const double* Bm, int m, const double* c, double* out,
            int kout);
int bhat_kernel(globe_ctx* ctx, const double* vr, double* bhat);
int ftheta_kernel(globe_ctx* ctx, const double* vr, const double* uh, double* fth);
// gen: normals from the stream of seed (zi: 3 N numMC doubles of scratch); else from draws
int probes_build(globe_ctx* ctx, const double* draws, int numMC, uint64_t seed, bool gen, double* Y,
                 double* zi);
int trace_terms(globe_ctx* ctx, const double* VR, const double* UH, const double* TY, int numMC,
                double* out);

// k_records_df.cu: the iteration's record kernels on double-float vectors (float2 in the
// place of each double); Zi, GZ, the partial sums and the scalars stay FP64
int to_df(globe_ctx* ctx, const double* in, int64_t n, float2* out);
struct DfCols {   // up to 4 (source, destination) column blocks; unused destinations null
    const double* src[4] = {nullptr, nullptr, nullptr, nullptr};
    double* dst[4] = {nullptr, nullptr, nullptr, nullptr};
};
int col_unscales(globe_ctx* ctx, const double* bb, int k, double* unsc);   // unsc[c] = col_unscale(bb[c])
int cols_to_df(globe_ctx* ctx, const DfCols& v, int64_t n, int k, const double* unsc, double* rz);
int precond_apply_df(globe_ctx* ctx, const float2* H, const float2* r, float2* z, int k, double* rz);
int cols_from_df(globe_ctx* ctx, double* v, int64_t n, int k, const double* unsc);
int seg_sums_df(globe_ctx* ctx, float2* x, const float2* z, const float2* beta, const int32_t* cols, int kact,
                double* Zi, float2* S0, float2* S1);
int vx_assemble_df(globe_ctx* ctx, const float2* x, const double* GZ, const float2* S0, const float2* S1,
                   const int32_t* cols, int kact, float2* out, double* dot_out, const double* num = nullptr,
                   double* quot = nullptr, float2* quot_df = nullptr);
int pcg_update_df(globe_ctx* ctx, const float2* H, const float2* alpha, float2* x, float2* r, const float2* p,
                  const float2* Vp, float2* z, const int32_t* cols, int kact, double* rr, double* rz);

// k_grm_geno.cu
int geno_apply_f64(globe_ctx* ctx, const double* Z, int k, double scale, double* out);
int geno_diag(globe_ctx* ctx, double* d);

// k_grm_dense.cu
int dense_apply_f64(globe_ctx* ctx, const double* Z, int k, double scale, double* out);
int dense_apply_df(globe_ctx* ctx, const double* Z, int k, double scale, double* out);
int dense_diag(globe_ctx* ctx, double* d);

// k_tc_dense.cu
int dense_digit_planes(globe_ctx* ctx);   // (re)builds the digit planes for the context's digit count
int dense_apply_tc(globe_ctx* ctx, const double* Z, int k, double scale, double* out);

// k_tc_geno.cu
int ensure_blk1(globe_ctx* ctx);   // SNP-major tile-blocked copy; frees the compacted rows
int ensure_blk2(globe_ctx* ctx);   // individual-major tile-blocked copy (first tensor-core use)
int load_bed_rows(globe_ctx* ctx, const uint8_t* d_bed, int64_t M, int64_t stride, float min_maf, float max_miss,
                  int64_t* d_alt, int64_t* d_miss, float* d_maf, float* d_mr, uint8_t* d_keep, globe_bed_info* info);
int geno_apply_tc(globe_ctx* ctx, const double* Z, int k, double scale, double* out);
int tc_err_word(globe_ctx* ctx, unsigned** err);   // the kernels' timeout word (cleared when created)
int tc_check_error(globe_ctx* ctx);                 // reads and clears it: GLOBE_ERR_CUDA if set
int tc_counters(globe_ctx* ctx, size_t n, unsigned** cnt);   // >= n zeroed per-column arrival counts
// rc of a call at `precision`, or the tensor-core timeout behind it (the root cause) if one was set
int with_tc_check(globe_ctx* ctx, int precision, int rc);

// solver.cu
int grm_apply_dev(globe_ctx* ctx, const double* Z, int k, double* out);
int ensure_gdiag(globe_ctx* ctx);
int ensure_precond(globe_ctx* ctx);
int vx_dev(globe_ctx* ctx, const double* x, int k, double* out);
int pcg_dev(globe_ctx* ctx, const double* B, double* X, int k, const globe_pcg_opts* o,
            globe_pcg_info* info);
int reduce_cols(globe_ctx* ctx, const double* part, int nparts, int kact, const int32_t* cols, double* out);
int reduce_cols2(globe_ctx* ctx, const double* part, int nparts, int kact, const int32_t* cols, double* out0,
                 double* out1);
int reduce_cols_div(globe_ctx* ctx, const double* part, int nparts, int kact, const int32_t* cols, double* out,
                    const double* num, double* quot, float2* quot_df);

}  // namespace globe
