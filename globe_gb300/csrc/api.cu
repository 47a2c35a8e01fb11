// api.cu -- context, memory and input loading of the C ABI (include/globe.h).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.cuh"

namespace globe {

static thread_local std::string g_create_err;

int set_err(globe_ctx* ctx, int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (ctx) ctx->err = buf;
    else g_create_err = buf;
    return code;
}

int cuda_err(globe_ctx* ctx, cudaError_t e, const char* what) {
    return set_err(ctx, e == cudaErrorMemoryAllocation ? GLOBE_ERR_NOMEM : GLOBE_ERR_CUDA, "%s: %s (%s)", what,
                   cudaGetErrorString(e), cudaGetErrorName(e));
}

int dalloc_bytes(globe_ctx* ctx, void** p, size_t bytes) {
    *p = nullptr;
    if (ctx->capturing) return set_err(ctx, GLOBE_ERR_STATE, "device allocation during CUDA graph capture");
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(ctx, GLOBE_ERR_NOMEM, "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
    }
    ctx->dev_bytes += (int64_t)bytes;
    ctx->allocs.emplace_back(*p, bytes);
    return GLOBE_OK;
}

void dfree(globe_ctx* ctx, void* p) {
    if (!p) return;
    for (auto it = ctx->allocs.begin(); it != ctx->allocs.end(); ++it)
        if (it->first == p) {
            ctx->dev_bytes -= (int64_t)it->second;
            ctx->allocs.erase(it);
            break;
        }
    cudaFree(p);
}

int wslot(globe_ctx* ctx, int id, size_t bytes, void** out) {
    Slot& s = ctx->ws[id];
    if (s.bytes < bytes) {
        // growth synchronises the stream: not while a capture is open (the caller then runs
        // the same work directly)
        if (ctx->capturing) return set_err(ctx, GLOBE_ERR_STATE, "workspace growth during CUDA graph capture");
        if (s.p) {
            cudaStreamSynchronize(ctx->stream);
            cudaFree(s.p);
            ctx->dev_bytes -= (int64_t)s.bytes;
            s.p = nullptr;
            s.bytes = 0;
        }
        size_t want = bytes + bytes / 4 + 256;
        cudaError_t e = cudaMalloc(&s.p, want);
        if (e != cudaSuccess) {
            cudaGetLastError();
            s.p = nullptr;
            return set_err(ctx, GLOBE_ERR_NOMEM, "workspace cudaMalloc(%zu bytes) failed: %s", want,
                           cudaGetErrorString(e));
        }
        s.bytes = want;
        ctx->dev_bytes += (int64_t)want;
    }
    *out = s.p;
    return GLOBE_OK;
}

int after_launch(globe_ctx* ctx, const char* name) {
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(ctx, e, name);
    return GLOBE_OK;
}

static void prof_flush(globe_ctx* ctx) {
    cudaStreamSynchronize(ctx->stream);
    for (size_t i = 0; i < ctx->prof_used; ++i) {
        auto& e = ctx->prof_pool[i];
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, e.a, e.b) == cudaSuccess) {
            ctx->prof_count[e.kind] += 1;
            ctx->prof_ms[e.kind] += ms;
        } else {
            cudaGetLastError();
        }
    }
    ctx->prof_used = 0;
}

int prof_begin(globe_ctx* ctx, int kind) {
    if (!ctx->prof_on || kind < 0 || kind >= GLOBE_PROF_KINDS) return -1;
    if (ctx->prof_used >= 4096) prof_flush(ctx);
    if (ctx->prof_used == ctx->prof_pool.size()) {
        globe_ctx::ProfEv e{kind, nullptr, nullptr};
        if (cudaEventCreate(&e.a) != cudaSuccess || cudaEventCreate(&e.b) != cudaSuccess) {
            cudaGetLastError();
            return -1;
        }
        ctx->prof_pool.push_back(e);
    }
    int h = (int)ctx->prof_used++;
    ctx->prof_pool[h].kind = kind;
    cudaEventRecord(ctx->prof_pool[h].a, ctx->stream);
    return h;
}

void prof_end(globe_ctx* ctx, int h) {
    if (h < 0) return;
    cudaEventRecord(ctx->prof_pool[h].b, ctx->stream);
}

static void free_cohort(globe_ctx* ctx) {
    auto& c = ctx->coh;
    for (void* p : {(void*)c.X, (void*)c.y, (void*)c.bstart, (void*)c.bind, (void*)c.rind, (void*)c.bn,
                    (void*)c.bt, (void*)c.btt, (void*)c.lblk, (void*)c.tdf})
        dfree(ctx, p);
    c = Cohort();
    for (void* p : {(void*)ctx->vinv_X, (void*)ctx->vinv_r, (void*)ctx->uhat, (void*)ctx->f_theta}) dfree(ctx, p);
    ctx->vinv_X = ctx->vinv_r = ctx->uhat = ctx->f_theta = nullptr;
    ctx->mme_ok = ctx->fth_ok = false;
    ctx->precond_ok = false;
}

static void free_genetic(globe_ctx* ctx) {
    auto& g = ctx->gen;
    for (void* p : {(void*)g.geno, (void*)g.zs, (void*)g.f, (void*)g.inv, (void*)g.grm, (void*)g.gdiag,
                    (void*)g.blk1, (void*)g.blk2, (void*)g.adig})
        dfree(ctx, p);
    g = Genetic();
    ctx->precond_ok = false;
    ctx->mme_ok = ctx->fth_ok = false;
}

// registry of the bounds-check words (one per translation unit of a checked build)
static std::vector<int (*)(unsigned*, bool)>& bounds_queries() {
    static std::vector<int (*)(unsigned*, bool)> q;
    return q;
}
int register_bounds_word(int (*query)(unsigned* code, bool clear)) {
    bounds_queries().push_back(query);
    return (int)bounds_queries().size();
}
int query_bounds_words(unsigned* first_code) {
    int found = 0;
    for (auto q : bounds_queries()) {
        unsigned c = 0;
        if (q(&c, true) != 0) return -1;
        if (c != 0 && !found) {
            *first_code = c;
            found = 1;
        }
    }
    return found;
}

}  // namespace globe

using namespace globe;

extern "C" {

int globe_create(globe_ctx** out, int device) {
    if (!out) return set_err(nullptr, GLOBE_ERR_ARG, "globe_create: null output pointer");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return set_err(nullptr, GLOBE_ERR_CUDA, "no CUDA device available (%s)",
                       e != cudaSuccess ? cudaGetErrorString(e) : "0 devices");
    if (device < 0 || device >= n) return set_err(nullptr, GLOBE_ERR_ARG, "device %d out of range [0,%d)", device, n);
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return set_err(nullptr, GLOBE_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    globe_ctx* ctx = new globe_ctx();
    ctx->device = device;
    e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete ctx;
        return set_err(nullptr, GLOBE_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
    ctx->hpin_n = 1 << 14;
    e = cudaMallocHost(&ctx->hpin, sizeof(double) * ctx->hpin_n);
    if (e != cudaSuccess) {
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return set_err(nullptr, GLOBE_ERR_CUDA, "cudaMallocHost: %s", cudaGetErrorString(e));
    }
    *out = ctx;
    return GLOBE_OK;
}

void globe_destroy(globe_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto& a : ctx->allocs) cudaFree(a.first);
    for (auto& s : ctx->ws)
        if (s.p) cudaFree(s.p);
    if (ctx->hpin) cudaFreeHost(ctx->hpin);
    for (auto& g : ctx->pcg_graph)
        if (g) cudaGraphExecDestroy(g);
    if (ctx->pcg_loop) cudaGraphExecDestroy(ctx->pcg_loop);
    for (auto& e : ctx->prof_pool) {
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
    }
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* globe_last_error(const globe_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_err.c_str(); }

int globe_set_graphs(globe_ctx* ctx, int on) {
    if (!ctx) return GLOBE_ERR_ARG;
    if (on != 0 && on != 1) return set_err(ctx, GLOBE_ERR_ARG, "globe_set_graphs: on must be 0 or 1, got %d", on);
    ctx->graphs = on;
    return GLOBE_OK;
}

int globe_get_graphs(const globe_ctx* ctx) { return ctx ? ctx->graphs : -1; }

int globe_set_device_loop(globe_ctx* ctx, int on) {
    if (!ctx) return GLOBE_ERR_ARG;
    if (on != 0 && on != 1)
        return set_err(ctx, GLOBE_ERR_ARG, "globe_set_device_loop: on must be 0 or 1, got %d", on);
    ctx->device_loop = on;
    return GLOBE_OK;
}

int globe_get_device_loop(const globe_ctx* ctx) { return ctx ? ctx->device_loop : -1; }

int64_t globe_device_loop_runs(const globe_ctx* ctx) { return ctx ? ctx->device_loop_runs : -1; }

int globe_set_record_df(globe_ctx* ctx, int on) {
    if (!ctx) return GLOBE_ERR_ARG;
    if (on != 0 && on != 1) return set_err(ctx, GLOBE_ERR_ARG, "globe_set_record_df: on must be 0 or 1, got %d", on);
    ctx->record_df = on;
    return GLOBE_OK;
}

int globe_get_record_df(const globe_ctx* ctx) { return ctx ? ctx->record_df : -1; }

int64_t globe_record_df_solves(const globe_ctx* ctx) { return ctx ? ctx->record_df_runs : -1; }


int globe_set_autotune(globe_ctx* ctx, int on) {
    if (!ctx) return GLOBE_ERR_ARG;
    if (on != 0 && on != 1) return set_err(ctx, GLOBE_ERR_ARG, "globe_set_autotune: on must be 0 or 1, got %d", on);
    ctx->autotune = on;
    return GLOBE_OK;
}

int globe_get_autotune(const globe_ctx* ctx) { return ctx ? ctx->autotune : -1; }

int64_t globe_autotune_log(const globe_ctx* ctx, char* buf, int64_t cap) {
    if (!ctx) return -1;
    const std::string s = "[" + ctx->tune_log + "]";
    if (buf && cap > 0) {
        const int64_t n = std::min<int64_t>(cap - 1, (int64_t)s.size());
        std::memcpy(buf, s.data(), (size_t)n);
        buf[n] = 0;
    }
    return (int64_t)s.size();
}

int globe_debug_bounds(uint32_t* first_code) {
#ifdef GLOBE_CHECK_BOUNDS
    unsigned c = 0;
    const int r = globe::query_bounds_words(&c);
    if (r < 0) return GLOBE_ERR_CUDA;
    if (first_code) *first_code = r ? c : 0u;
    return r;
#else
    if (first_code) *first_code = 0u;
    return GLOBE_ERR_UNSUPPORTED;
#endif
}

int globe_debug_force_splits(globe_ctx* ctx, int splits) {
    if (!ctx) return GLOBE_ERR_ARG;
    if (splits < 0 || splits > 4096) return set_err(ctx, GLOBE_ERR_ARG, "force_splits: %d not in [0, 4096]", splits);
    ctx->force_splits = splits;
    return GLOBE_OK;
}

int globe_get_stream(globe_ctx* ctx, void** stream) {
    if (!ctx || !stream) return GLOBE_ERR_ARG;
    *stream = (void*)ctx->stream;
    return GLOBE_OK;
}

int globe_synchronize(globe_ctx* ctx) {
    if (!ctx) return GLOBE_ERR_ARG;
    GLOBE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return GLOBE_OK;
}

int64_t globe_device_bytes(const globe_ctx* ctx) { return ctx ? ctx->dev_bytes : 0; }
int64_t globe_kernel_launches(const globe_ctx* ctx) { return ctx ? ctx->launches : 0; }

int globe_prof_enable(globe_ctx* ctx, int on) {
    if (!ctx) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    prof_flush(ctx);
    for (int k = 0; k < GLOBE_PROF_KINDS; ++k) {
        ctx->prof_count[k] = 0;
        ctx->prof_ms[k] = 0.0;
    }
    ctx->prof_on = on != 0;
    return GLOBE_OK;
}

int globe_prof_query(globe_ctx* ctx, int kind, int64_t* count, double* ms) {
    if (!ctx || kind < 0 || kind >= GLOBE_PROF_KINDS) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    prof_flush(ctx);
    if (count) *count = ctx->prof_count[kind];
    if (ms) *ms = ctx->prof_ms[kind];
    return GLOBE_OK;
}

int globe_get_dims(const globe_ctx* ctx, int64_t* Nrec, int32_t* N, int32_t* p, int64_t* kept) {
    if (!ctx) return GLOBE_ERR_ARG;
    if (Nrec) *Nrec = ctx->coh.Nrec;
    if (N) *N = ctx->coh.N;
    if (p) *p = ctx->coh.p;
    if (kept) *kept = ctx->gen.src == GSRC_GENO ? ctx->gen.Mk : 0;
    return GLOBE_OK;
}

int globe_load_records(globe_ctx* ctx, int64_t Nrec, int32_t N, int32_t p, const int32_t* indiv,
                       const double* X, const double* y) {
    if (!ctx) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (Nrec < 1 || N < 1 || p < 0 || !indiv || !X || !y)
        return set_err(ctx, GLOBE_ERR_ARG, "globe_load_records: invalid sizes or null pointers");
    if (Nrec > INT32_MAX) return set_err(ctx, GLOBE_ERR_ARG, "globe_load_records: Nrec exceeds 2^31-1");
    // blocks = runs of one individual; each individual must form exactly one run
    std::vector<int32_t> bstart, bind, rind(Nrec);
    std::vector<uint8_t> seen(N, 0);
    int32_t maxb = 0;
    for (int64_t r = 0; r < Nrec; ++r) {
        int32_t i = indiv[r];
        if (i < 0 || i >= N)
            return set_err(ctx, GLOBE_ERR_FORMAT,
                           "record %lld: individual index %d outside [0,%d) (IDs must be 1..N, N = number of "
                           "distinct IDs)", (long long)r, i, N);
        if (r == 0 || indiv[r - 1] != i) {
            if (seen[i])
                return set_err(ctx, GLOBE_ERR_FORMAT,
                               "records of individual %d are not contiguous (records must be grouped by "
                               "individual)", i + 1);
            seen[i] = 1;
            if (!bstart.empty()) maxb = std::max<int32_t>(maxb, (int32_t)(r - bstart.back()));
            bstart.push_back((int32_t)r);
            bind.push_back(i);
        }
        rind[r] = i;
    }
    maxb = std::max<int32_t>(maxb, (int32_t)(Nrec - bstart.back()));
    if ((int32_t)bind.size() != N)
        return set_err(ctx, GLOBE_ERR_FORMAT, "%d individuals have records but N = %d", (int)bind.size(), N);
    bstart.push_back((int32_t)Nrec);
    for (int64_t e = 0; e < Nrec * (int64_t)(p + 1); ++e)
        if (!std::isfinite(X[e])) return set_err(ctx, GLOBE_ERR_FORMAT, "non-finite covariate/time value");
    for (int64_t e = 0; e < Nrec; ++e)
        if (!std::isfinite(y[e])) return set_err(ctx, GLOBE_ERR_FORMAT, "non-finite phenotype value");
    free_cohort(ctx);
    free_genetic(ctx);
    auto& c = ctx->coh;
    c.Nrec = Nrec;
    c.N = N;
    c.p = p;
    c.max_block = maxb;
    GLOBE_RET(dalloc(ctx, &c.X, (size_t)Nrec * (p + 1)));
    GLOBE_RET(dalloc(ctx, &c.y, (size_t)Nrec));
    GLOBE_RET(dalloc(ctx, &c.bstart, (size_t)N + 1));
    GLOBE_RET(dalloc(ctx, &c.bind, (size_t)N));
    GLOBE_RET(dalloc(ctx, &c.rind, (size_t)Nrec));
    GLOBE_RET(dalloc(ctx, &c.bn, (size_t)N));
    GLOBE_RET(dalloc(ctx, &c.bt, (size_t)N));
    GLOBE_RET(dalloc(ctx, &c.btt, (size_t)N));
    // blocks longer than SHORT_BLOCK records: the record kernels give each of them a warp
    std::vector<int32_t> lblk;
    for (int32_t b = 0; b < N; ++b)
        if (bstart[b + 1] - bstart[b] > SHORT_BLOCK) lblk.push_back(b);
    c.nlong = (int32_t)lblk.size();
    if (c.nlong > 0) {
        GLOBE_RET(dalloc(ctx, &c.lblk, (size_t)c.nlong));
        GLOBE_CK(ctx, cudaMemcpyAsync(c.lblk, lblk.data(), sizeof(int32_t) * c.nlong, cudaMemcpyHostToDevice,
                                      ctx->stream));
    }
    GLOBE_CK(ctx, cudaMemcpyAsync(c.X, X, sizeof(double) * Nrec * (p + 1), cudaMemcpyHostToDevice, ctx->stream));
    GLOBE_CK(ctx, cudaMemcpyAsync(c.y, y, sizeof(double) * Nrec, cudaMemcpyHostToDevice, ctx->stream));
    GLOBE_CK(ctx, cudaMemcpyAsync(c.bstart, bstart.data(), sizeof(int32_t) * (N + 1), cudaMemcpyHostToDevice,
                                  ctx->stream));
    GLOBE_CK(ctx, cudaMemcpyAsync(c.bind, bind.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice, ctx->stream));
    GLOBE_CK(ctx, cudaMemcpyAsync(c.rind, rind.data(), sizeof(int32_t) * Nrec, cudaMemcpyHostToDevice, ctx->stream));
    GLOBE_RET(block_moments(ctx));
    // the times as double-float pairs, for the double-float record kernels
    double tmax = 0.0;
    for (int64_t r = 0; r < Nrec; ++r) tmax = std::max(tmax, std::fabs(X[(int64_t)p * Nrec + r]));
    c.tmax = tmax;
    GLOBE_RET(dalloc(ctx, &c.tdf, (size_t)Nrec));
    GLOBE_RET(to_df(ctx, c.times(), Nrec, c.tdf));
    GLOBE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return GLOBE_OK;
}

int globe_set_individuals(globe_ctx* ctx, int32_t N) {
    if (!ctx) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (N < 1) return set_err(ctx, GLOBE_ERR_ARG, "globe_set_individuals: N must be >= 1");
    free_cohort(ctx);
    free_genetic(ctx);
    ctx->coh.N = N;
    return GLOBE_OK;
}

}  // extern "C"

namespace globe {

// statistics, filter and compaction of the kept SNP rows; the tile-blocked layout follows
// separately (ensure_blk1), after the callers have released their staging copies
int load_bed_rows(globe_ctx* ctx, const uint8_t* d_bed, int64_t M, int64_t stride, float min_maf, float max_miss,
                  int64_t* d_alt, int64_t* d_miss, float* d_maf, float* d_mr, uint8_t* d_keep, globe_bed_info* info) {
    if (!ctx) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    const int32_t N = ctx->coh.N;
    if (N < 1) return set_err(ctx, GLOBE_ERR_STATE, "load the record table first (N comes from it)");
    const int64_t bps = ((int64_t)N + 3) / 4;
    if (M < 0 || stride < bps || (M > 0 && !d_bed))
        return set_err(ctx, GLOBE_ERR_ARG, "globe_load_bed_dev: bad M/stride (stride %lld < %lld bytes per SNP)",
                       (long long)stride, (long long)bps);
    if (!(min_maf >= 0.0f && min_maf <= 0.5f && max_miss >= 0.0f && max_miss <= 1.0f))
        return set_err(ctx, GLOBE_ERR_ARG, "Invalid MAF or missing rate thresholds.");
    free_genetic(ctx);
    // per-SNP statistics (temporaries where the caller passed NULL)
    std::vector<void*> tmp;
    auto need = [&](auto** p, size_t n) -> int {
        if (*p) return GLOBE_OK;
        void* q;
        cudaError_t e = cudaMalloc(&q, n ? n : 16);
        if (e != cudaSuccess) return cuda_err(ctx, e, "cudaMalloc(stats)");
        tmp.push_back(q);
        *p = (std::remove_reference_t<decltype(*p)>)q;
        return GLOBE_OK;
    };
    int rc = GLOBE_OK;
    if ((rc = need(&d_alt, sizeof(int64_t) * M)) || (rc = need(&d_miss, sizeof(int64_t) * M)) ||
        (rc = need(&d_keep, (size_t)M))) {
        for (void* q : tmp) cudaFree(q);
        return rc;
    }
    auto cleanup = [&]() {
        cudaStreamSynchronize(ctx->stream);
        for (void* q : tmp) cudaFree(q);
    };
    rc = bed_stats(ctx, d_bed, M, stride, N, min_maf, max_miss, d_alt, d_miss, d_maf, d_mr, d_keep);
    std::vector<uint8_t> keep(M);
    if (rc == GLOBE_OK && M > 0) {
        cudaError_t e = cudaMemcpyAsync(keep.data(), d_keep, M, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = cuda_err(ctx, e, "copy keep mask");
    }
    if (rc != GLOBE_OK) { cleanup(); return rc; }
    std::vector<int64_t> idx;
    idx.reserve(M);
    for (int64_t s = 0; s < M; ++s)
        if (keep[s]) idx.push_back(s);
    auto& g = ctx->gen;
    g.Mk = (int64_t)idx.size();
    g.stride = (bps + 15) / 16 * 16;
    int64_t* d_idx = nullptr;
    if ((rc = dalloc(ctx, &d_idx, idx.size() + 1)) != GLOBE_OK) { cleanup(); return rc; }
    if (g.Mk > 0) {
        cudaError_t e = cudaMemcpyAsync(d_idx, idx.data(), sizeof(int64_t) * g.Mk, cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) { cleanup(); return cuda_err(ctx, e, "copy kept index"); }
    }
    if ((rc = dalloc(ctx, &g.geno, (size_t)g.Mk * g.stride)) || (rc = dalloc(ctx, &g.zs, (size_t)g.Mk * 4)) ||
        (rc = dalloc(ctx, &g.f, (size_t)g.Mk)) || (rc = dalloc(ctx, &g.inv, (size_t)g.Mk)) ||
        (rc = dalloc(ctx, &g.gdiag, (size_t)N))) {
        cleanup();
        return rc;
    }
    if ((rc = bed_compact(ctx, d_bed, stride, d_idx, g.Mk, bps, g.geno, g.stride)) ||
        (rc = snp_coefs(ctx, d_alt, d_miss, d_idx, g.Mk, N, g.f, g.inv, g.zs))) {
        cleanup();
        return rc;
    }
    cleanup();
    dfree(ctx, d_idx);
    g.src = GSRC_GENO;
    g.gdiag_ok = false;
    ctx->precond_ok = false;
    if (info) {
        info->M = M;
        info->kept = g.Mk;
    }
    GLOBE_CK(ctx, cudaGetLastError());
    return GLOBE_OK;
}

}  // namespace globe

extern "C" {

int globe_load_bed_dev(globe_ctx* ctx, const uint8_t* d_bed, int64_t M, int64_t stride, float min_maf,
                       float max_miss, int64_t* d_alt, int64_t* d_miss, float* d_maf, float* d_mr, uint8_t* d_keep,
                       globe_bed_info* info) {
    int rc = load_bed_rows(ctx, d_bed, M, stride, min_maf, max_miss, d_alt, d_miss, d_maf, d_mr, d_keep, info);
    // the tile-blocked copy the genotype kernels read; the compacted rows are freed
    if (rc == GLOBE_OK && ctx->gen.Mk > 0) rc = ensure_blk1(ctx);
    return rc;
}

int globe_load_bed(globe_ctx* ctx, const uint8_t* bed, int64_t M, float min_maf, float max_miss,
                   int64_t* alt_count, int64_t* miss_count, float* maf, float* miss_rate, uint8_t* keep,
                   globe_bed_info* info) {
    if (!ctx) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    const int32_t N = ctx->coh.N;
    if (N < 1) return set_err(ctx, GLOBE_ERR_STATE, "load the record table first (N comes from it)");
    if (M < 0 || (M > 0 && !bed)) return set_err(ctx, GLOBE_ERR_ARG, "globe_load_bed: bad arguments");
    const int64_t bps = ((int64_t)N + 3) / 4;
    uint8_t* d_bed = nullptr;
    int64_t* d_alt = nullptr;
    int64_t* d_miss = nullptr;
    float* d_maf = nullptr;
    float* d_mr = nullptr;
    uint8_t* d_keep = nullptr;
    int rc;
    if ((rc = dalloc(ctx, &d_bed, (size_t)M * bps)) || (rc = dalloc(ctx, &d_alt, (size_t)M)) ||
        (rc = dalloc(ctx, &d_miss, (size_t)M)) || (rc = dalloc(ctx, &d_maf, (size_t)M)) ||
        (rc = dalloc(ctx, &d_mr, (size_t)M)) || (rc = dalloc(ctx, &d_keep, (size_t)M)))
        goto done;
    if (M > 0) {
        cudaError_t e = cudaMemcpyAsync(d_bed, bed, (size_t)M * bps, cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) { rc = cuda_err(ctx, e, "copy .bed payload"); goto done; }
    }
    rc = load_bed_rows(ctx, d_bed, M, bps, min_maf, max_miss, d_alt, d_miss, d_maf, d_mr, d_keep, info);
    if (rc == GLOBE_OK && M > 0) {
        cudaError_t e = cudaSuccess;
        if (alt_count && e == cudaSuccess) e = cudaMemcpyAsync(alt_count, d_alt, 8 * M, cudaMemcpyDeviceToHost, ctx->stream);
        if (miss_count && e == cudaSuccess) e = cudaMemcpyAsync(miss_count, d_miss, 8 * M, cudaMemcpyDeviceToHost, ctx->stream);
        if (maf && e == cudaSuccess) e = cudaMemcpyAsync(maf, d_maf, 4 * M, cudaMemcpyDeviceToHost, ctx->stream);
        if (miss_rate && e == cudaSuccess) e = cudaMemcpyAsync(miss_rate, d_mr, 4 * M, cudaMemcpyDeviceToHost, ctx->stream);
        if (keep && e == cudaSuccess) e = cudaMemcpyAsync(keep, d_keep, M, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) rc = cuda_err(ctx, e, "copy SNP statistics");
    }
done:
    cudaStreamSynchronize(ctx->stream);
    for (void* p : {(void*)d_bed, (void*)d_alt, (void*)d_miss, (void*)d_maf, (void*)d_mr, (void*)d_keep}) dfree(ctx, p);
    // tile-blocked layout once the staging copy of the payload is gone
    if (rc == GLOBE_OK && ctx->gen.Mk > 0) rc = ensure_blk1(ctx);
    return rc;
}

int globe_load_grm(globe_ctx* ctx, const float* grm_lt, int32_t N) {
    if (!ctx) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->coh.N < 1) return set_err(ctx, GLOBE_ERR_STATE, "load the record table first (N comes from it)");
    if (N != ctx->coh.N)
        return set_err(ctx, GLOBE_ERR_ARG, "GRM has N = %d but the record table has %d individuals", N, ctx->coh.N);
    if (!grm_lt) return set_err(ctx, GLOBE_ERR_ARG, "globe_load_grm: null GRM");
    free_genetic(ctx);
    auto& g = ctx->gen;
    size_t nelt = (size_t)N * (N + 1) / 2;
    GLOBE_RET(dalloc(ctx, &g.grm, nelt));
    GLOBE_RET(dalloc(ctx, &g.gdiag, (size_t)N));
    GLOBE_CK(ctx, cudaMemcpyAsync(g.grm, grm_lt, nelt * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    GLOBE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    g.src = GSRC_DENSE;
    g.gdiag_ok = false;
    ctx->precond_ok = false;
    return GLOBE_OK;
}

int globe_set_vc(globe_ctx* ctx, const double vc[5]) {
    if (!ctx || !vc) return GLOBE_ERR_ARG;
    for (int k = 0; k < 5; ++k)
        if (!std::isfinite(vc[k])) return set_err(ctx, GLOBE_ERR_ARG, "variance component %d is not finite", k);
    if (!(vc[0] > 0.0)) return set_err(ctx, GLOBE_ERR_ARG, "sig2e must be > 0 (got %g)", vc[0]);
    double v[5];
    std::memcpy(v, vc, sizeof(v));
    if (ctx->model == GLOBE_MODEL_NO_TIME) v[2] = v[3] = v[4] = 0.0;   // no time effects
    bool same = ctx->vc_set;
    for (int k = 0; k < 5; ++k) same = same && ctx->vc[k] == v[k];
    if (same) return GLOBE_OK;
    std::memcpy(ctx->vc, v, sizeof(double) * 5);
    ctx->vc_set = true;
    ctx->precond_ok = false;
    ctx->mme_ok = ctx->fth_ok = false;
    return GLOBE_OK;
}

int globe_set_model(globe_ctx* ctx, int model) {
    if (!ctx) return GLOBE_ERR_ARG;
    if (model != GLOBE_MODEL_FULL && model != GLOBE_MODEL_NO_TIME)
        return set_err(ctx, GLOBE_ERR_ARG, "unknown model %d", model);
    if (ctx->model == model) return GLOBE_OK;
    ctx->model = model;
    if (ctx->vc_set && model == GLOBE_MODEL_NO_TIME) {
        ctx->vc[2] = ctx->vc[3] = ctx->vc[4] = 0.0;
        ctx->precond_ok = false;
    }
    ctx->mme_ok = ctx->fth_ok = false;
    return GLOBE_OK;
}

int globe_get_model(const globe_ctx* ctx) { return ctx ? ctx->model : GLOBE_MODEL_FULL; }

int globe_set_digits(globe_ctx* ctx, int nd) {
    if (!ctx) return GLOBE_ERR_ARG;
    if (nd < 2 || nd > 9) return set_err(ctx, GLOBE_ERR_ARG, "digits per column must be in [2, 9], got %d", nd);
    ctx->digits = nd;
    return GLOBE_OK;
}

int globe_get_digits(const globe_ctx* ctx) { return ctx ? ctx->digits : 9; }

int globe_debug_stall_next_gemm(globe_ctx* ctx) {
    if (!ctx) return GLOBE_ERR_ARG;
    ctx->stall_next_gemm = 1;
    return GLOBE_OK;
}

int globe_set_precision(globe_ctx* ctx, int precision) {
    if (!ctx) return GLOBE_ERR_ARG;
    if (precision != GLOBE_PREC_FP64 && precision != GLOBE_PREC_MIXED)
        return set_err(ctx, GLOBE_ERR_ARG, "unknown precision mode %d", precision);
    ctx->prec = precision;
    return GLOBE_OK;
}

int globe_synth_bed_dev(globe_ctx* ctx, uint8_t* d_bed, int64_t M, int32_t N, int64_t stride, uint64_t seed,
                        float maf_lo, float maf_hi, float miss_rate) {
    if (!ctx || !d_bed || M < 0 || N < 1 || stride < ((int64_t)N + 3) / 4)
        return set_err(ctx, GLOBE_ERR_ARG, "globe_synth_bed_dev: bad arguments");
    cudaSetDevice(ctx->device);
    return synth_bed(ctx, d_bed, M, N, stride, seed, maf_lo, maf_hi, miss_rate);
}

}  // extern "C"
