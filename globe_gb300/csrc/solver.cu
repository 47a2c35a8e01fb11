// solver.cu -- operator application, block PCG, MME and AIREML terms.
//
// Host-side orchestration of the kernels in k_*.cu.  The PCG recurrences,
// dot products and the small (p+1)-sized systems are FP64.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "df.cuh"
#include "internal.cuh"

namespace globe {

int check_ready(globe_ctx* ctx) {
    if (ctx->coh.Nrec < 1) return set_err(ctx, GLOBE_ERR_STATE, "no record table loaded");
    if (ctx->gen.src == GSRC_NONE) return set_err(ctx, GLOBE_ERR_STATE, "no genotypes or GRM loaded");
    if (!ctx->vc_set) return set_err(ctx, GLOBE_ERR_STATE, "variance components not set");
    return GLOBE_OK;
}

int grm_apply_dev(globe_ctx* ctx, const double* Z, int k, double* out) {
    ProfScope ps(ctx, GLOBE_PROF_GRM);
    if (ctx->gen.src == GSRC_GENO) {
        const double scale = ctx->vc[1] * (ctx->gen.Mk > 0 ? 1.0 / (double)ctx->gen.Mk : 0.0);
        if (ctx->prec == GLOBE_PREC_MIXED) return geno_apply_tc(ctx, Z, k, scale, out);
        return geno_apply_f64(ctx, Z, k, scale, out);
    }
    if (ctx->gen.src == GSRC_DENSE)
        return ctx->prec == GLOBE_PREC_MIXED ? dense_apply_tc(ctx, Z, k, ctx->vc[1], out)
                                             : dense_apply_f64(ctx, Z, k, ctx->vc[1], out);
    return set_err(ctx, GLOBE_ERR_STATE, "no genetic relationship source loaded");
}

int ensure_gdiag(globe_ctx* ctx) {
    auto& g = ctx->gen;
    if (g.gdiag_ok) return GLOBE_OK;
    if (g.src == GSRC_GENO) GLOBE_RET(geno_diag(ctx, g.gdiag));
    else if (g.src == GSRC_DENSE) GLOBE_RET(dense_diag(ctx, g.gdiag));
    else return set_err(ctx, GLOBE_ERR_STATE, "no genetic relationship source loaded");
    g.gdiag_ok = true;
    return GLOBE_OK;
}

int ensure_precond(globe_ctx* ctx) {
    if (ctx->precond_ok) return GLOBE_OK;
    GLOBE_RET(ensure_gdiag(ctx));
    double* H;
    float2* Hdf;
    GLOBE_RET(ws(ctx, WS_H, (size_t)ctx->coh.N * 4, &H));
    GLOBE_RET(ws(ctx, WS_HDF, (size_t)ctx->coh.N * 4, &Hdf));
    GLOBE_RET(build_H(ctx, ctx->gen.gdiag, 0.0, H, Hdf));
    ctx->precond_ok = true;
    return GLOBE_OK;
}

static double* Hptr(globe_ctx* ctx) { return (double*)ctx->ws[WS_H].p; }

int vx_dev(globe_ctx* ctx, const double* x, int k, double* out) {
    const int32_t N = ctx->coh.N;
    double *Zi, *S1, *GZ;
    GLOBE_RET(ws(ctx, WS_ZI, (size_t)N * k, &Zi));
    GLOBE_RET(ws(ctx, WS_S1, (size_t)N * k, &S1));
    GLOBE_RET(ws(ctx, WS_GZ, (size_t)N * k, &GZ));
    GLOBE_RET(seg_sums(ctx, x, nullptr, nullptr, nullptr, nullptr, k, Zi, S1));
    GLOBE_RET(grm_apply_dev(ctx, Zi, k, GZ));
    GLOBE_RET(vx_assemble(ctx, x, GZ, Zi, S1, nullptr, k, out, nullptr));
    return GLOBE_OK;
}

__global__ void k_sub(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out, int64_t n) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        out[e] = a[e] - b[e];
}

static int sub_vec(globe_ctx* ctx, const double* a, const double* b, double* out, int64_t n) {
    int nb = div_up(n, 256);
    if (nb > 4096) nb = 4096;
    k_sub<<<nb, 256, 0, ctx->stream>>>(a, b, out, n);
    GLOBE_LAUNCHED(ctx, "k_sub");
    return GLOBE_OK;
}

static int d2h(globe_ctx* ctx, double* h, const double* d, size_t n) {
    GLOBE_CK(ctx, cudaMemcpyAsync(h, d, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    GLOBE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return GLOBE_OK;
}

static int pcg_run(globe_ctx* ctx, const double* B, double* X, int k, const globe_pcg_opts* o, globe_pcg_info* info);

int pcg_dev(globe_ctx* ctx, const double* B, double* X, int k, const globe_pcg_opts* o, globe_pcg_info* info) {
    if (!o) return set_err(ctx, GLOBE_ERR_ARG, "null PCG options");
    if (o->precision != GLOBE_PREC_FP64 && o->precision != GLOBE_PREC_MIXED)
        return set_err(ctx, GLOBE_ERR_ARG, "unknown precision mode %d", o->precision);
    const int saved = ctx->prec;
    ctx->prec = o->precision;
    const int rc = pcg_run(ctx, B, X, k, o, info);
    ctx->prec = saved;
    return with_tc_check(ctx, o->precision, rc);
}

// Captures `body` (stream work only, nothing run) into a graph and makes ctx->pcg_graph[slot]
// run it: the cached executable is updated in place when the topology matches, else
// instantiated anew.  Allocation is refused while the capture is open.  Returns false, with
// nothing run and the error message restored, if any step fails.
template <class F>
static bool capture_body(globe_ctx* ctx, int slot, F&& body, int64_t* nlaunch) {
    const std::string err0 = ctx->err;
    const int64_t l0 = ctx->launches;
    if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    ctx->capturing = true;
    const int rc = body();
    ctx->capturing = false;
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    *nlaunch = ctx->launches - l0;
    ctx->launches = l0;
    bool ok = rc == GLOBE_OK && e == cudaSuccess && g != nullptr;
    if (ok) {
        cudaGraphExec_t& x = ctx->pcg_graph[slot];
        cudaGraphExecUpdateResultInfo upd;
        if (!(x && cudaGraphExecUpdate(x, g, &upd) == cudaSuccess)) {
            cudaGetLastError();
            if (x) cudaGraphExecDestroy(x);
            x = nullptr;
            if (cudaGraphInstantiate(&x, g, 0) != cudaSuccess) {
                x = nullptr;
                ok = false;
            }
        }
    }
    if (g) cudaGraphDestroy(g);
    if (!ok) {
        cudaGetLastError();
        ctx->err = err0;
    }
    return ok;
}

// ---- the PCG iterations after the first, as one device-side loop -------------------
//
// One graph: a kernel that arms a WHILE conditional node, then the node, whose body is
// one iteration (the same kernels, in the same order, as a host-driven iteration) followed
// by k_pcg_check_shift, which applies the stopping rule of the host loop below to the device
// copies of r'r and p'Vp, sets the node's condition, and shifts beta / r'z.
// So the iterations run without a host synchronisation each, with bit-identical
// results and iteration counts.  The condition's launch default is 0: only the arming
// kernel opens the loop, so a condition that could not be set leaves the loop unrun
// (the host then sees no iteration and carries on itself); inside it every path of the
// check sets it, and the iteration cap always closes it.

struct PcgLoopState {
    double last;          // last max ratio (PCGsolver rule, stagnation)
    long long rhs_iters;  // sum over iterations of active columns
    int it;               // iterations completed
    int stag;             // iterations in a row with < 0.5% improvement
    int status;           // 0 running, 1 converged, 2 stagnated, 3 iteration cap, 4 breakdown
    int err_col;          // column of a breakdown
};

__global__ void k_pcg_loop_arm(cudaGraphConditionalHandle h) { cudaGraphSetConditional(h, 1u); }

// the host loop's stopping rule (pcg_run) on the device: one thread, after iteration st->it + 1
__device__ void pcg_check(const double* __restrict__ rr, const double* __restrict__ pvp,
                          const double* __restrict__ bb, const int32_t* __restrict__ cols, int kact, int k,
                          double tol, int rule, int maxit, const double* __restrict__ unsc, PcgLoopState* st,
                          cudaGraphConditionalHandle h) {
    const int it = st->it + 1;
    st->it = it;
    st->rhs_iters += kact;
    for (int c = 0; c < kact; ++c) {
        const int j = cols[c];
        if (!(pvp[j] > 0.0) || !isfinite(rr[j])) {
            st->status = 4;
            st->err_col = j;
            cudaGraphSetConditional(h, 0u);
            return;
        }
    }
    bool stop = false;
    if (rule == GLOBE_RULE_PCGSOLVER) {
        const double small_b = (double)1e-12f;  // PCGsolver.cpp:1365, :1393
        double mx = 0.0;
        for (int j = 0; j < k; ++j) {
            const double nb = sqrt(bb[j]);
            const double u = unsc ? unsc[j] : 1.0;
            const double q = nb > small_b ? sqrt(rr[j]) * u / nb : 0.0;
            if (q > mx) mx = q;
        }
        if (mx < tol) {
            st->status = 1;
            stop = true;
        } else {
            const double last = st->last;
            if (last - mx < (double)5e-3f * last) ++st->stag;
            else st->stag = 0;
            st->last = mx;
            if (st->stag >= 10) {
                st->status = 2;
                stop = true;
            }
        }
    } else {
        bool all = true;
        for (int j = 0; j < k; ++j)
            if (bb[j] > 0.0 && !(sqrt(rr[j]) * (unsc ? unsc[j] : 1.0) < tol * sqrt(bb[j]))) {
                all = false;
                break;
            }
        if (all) {
            st->status = 1;
            stop = true;
        }
    }
    if (!stop && it >= maxit) {
        st->status = 3;
        stop = true;
    }
    cudaGraphSetConditional(h, stop ? 0u : 1u);
}

// The end of a device-loop iteration, one launch: thread 0 applies the stopping rule
// (pcg_check); every column c < k takes beta = r'z(new) / r'z(old) (0 where r'z(old) = 0, as
// k_scal_div) and its double-float copy when beta_df is given, then r'z(old) = r'z(new).
// The check reads r'r and p'Vp only, so the two parts are independent.
__global__ void k_pcg_check_shift(const double* __restrict__ rr, const double* __restrict__ pvp,
                                  const double* __restrict__ bb, const int32_t* __restrict__ cols, int kact, int k,
                                  double tol, int rule, int maxit, const double* __restrict__ unsc, PcgLoopState* st,
                                  cudaGraphConditionalHandle h, double* __restrict__ rz,
                                  const double* __restrict__ rz2, double* __restrict__ beta,
                                  float2* __restrict__ beta_df) {
    if (blockIdx.x == 0 && threadIdx.x == 0) pcg_check(rr, pvp, bb, cols, kact, k, tol, rule, maxit, unsc, st, h);
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < k) {
        const double o = rz[c], nw = rz2[c];
        const double bt = (o != 0.0) ? nw / o : 0.0;
        beta[c] = bt;
        if (beta_df) df::store(beta_df + c, df::from_double(bt));
        rz[c] = nw;
    }
}

// Build and run the loop graph; body(h) issues one iteration and its check on the stream.
// Returns GLOBE_OK with *ran = false (nothing run) when the graph cannot be built.
template <class F>
static int run_device_loop(globe_ctx* ctx, F&& body, int64_t* nlaunch, bool* ran) {
    *ran = false;
    const std::string err0 = ctx->err;
    const int64_t l0 = ctx->launches;
    cudaGraph_t g = nullptr;
    cudaGraphConditionalHandle h;
    bool ok = cudaGraphCreate(&g, 0) == cudaSuccess &&
              cudaGraphConditionalHandleCreate(&h, g, 0u, cudaGraphCondAssignDefault) == cudaSuccess;
    // the arming kernel, captured into g
    cudaGraphNode_t arm = nullptr;
    if (ok) {
        ok = cudaStreamBeginCaptureToGraph(ctx->stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) ==
             cudaSuccess;
        if (ok) {
            k_pcg_loop_arm<<<1, 1, 0, ctx->stream>>>(h);
            cudaGraph_t gg = nullptr;
            ok = cudaStreamEndCapture(ctx->stream, &gg) == cudaSuccess && gg == g;
            size_t nn = 1;
            ok = ok && cudaGraphGetNodes(g, &arm, &nn) == cudaSuccess && nn == 1;
        }
    }
    cudaGraph_t bodyg = nullptr;
    if (ok) {
        cudaGraphNodeParams np = {};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        ok = cudaGraphAddNode(&node, g, &arm, nullptr, 1, &np) == cudaSuccess;
        if (ok) bodyg = np.conditional.phGraph_out[0];
    }
    int rc = GLOBE_OK;
    if (ok) {
        ok = cudaStreamBeginCaptureToGraph(ctx->stream, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) ==
             cudaSuccess;
        if (ok) {
            ctx->capturing = true;
            rc = body(h);
            ctx->capturing = false;
            cudaGraph_t gb = nullptr;
            ok = cudaStreamEndCapture(ctx->stream, &gb) == cudaSuccess && rc == GLOBE_OK;
        }
    }
    *nlaunch = ctx->launches - l0;
    ctx->launches = l0;
    if (ok) {
        if (ctx->pcg_loop) cudaGraphExecDestroy(ctx->pcg_loop);
        ctx->pcg_loop = nullptr;
        ok = cudaGraphInstantiate(&ctx->pcg_loop, g, 0) == cudaSuccess;
        if (!ok) ctx->pcg_loop = nullptr;
    }
    if (g) cudaGraphDestroy(g);
    if (!ok) {
        cudaGetLastError();
        ctx->err = err0;
        return GLOBE_OK;
    }
    GLOBE_CK(ctx, cudaGraphLaunch(ctx->pcg_loop, ctx->stream));
    *ran = true;
    return GLOBE_OK;
}

// Whether a GLOBE_PREC_MIXED solve may run its record kernels in double-float: with each
// column scaled to a unit-size right-hand side, the variance components and times bound every
// value of the iteration well inside FP32's exponent range.  Otherwise the FP64 kernels run.
static bool df_records_ok(const globe_ctx* ctx) {
    const double lo = std::ldexp(1.0, -30), hi = std::ldexp(1.0, 30);
    if (!(ctx->vc[0] >= lo && ctx->vc[0] <= hi)) return false;
    for (int j = 1; j < 5; ++j)
        if (!(std::fabs(ctx->vc[j]) <= hi)) return false;
    return ctx->coh.tdf != nullptr && ctx->coh.tmax <= hi;
}

static int pcg_run(globe_ctx* ctx, const double* B, double* X, int k, const globe_pcg_opts* o, globe_pcg_info* info) {
    GLOBE_RET(check_ready(ctx));
    if (k < 1) return set_err(ctx, GLOBE_ERR_ARG, "number of right-hand sides must be >= 1");
    if (!(o->tol >= 0) || o->maxit < 0) return set_err(ctx, GLOBE_ERR_ARG, "bad tolerance / iteration cap");
    auto& c = ctx->coh;
    const int64_t n = c.Nrec;
    const int32_t N = c.N;
    GLOBE_RET(ensure_precond(ctx));
    double *r, *z, *p, *Vp, *Zi, *GZ, *S1, *scal, *part;
    int32_t* dcols;
    GLOBE_RET(ws(ctx, WS_R, (size_t)n * k, &r));
    GLOBE_RET(ws(ctx, WS_Z, (size_t)n * k, &z));
    GLOBE_RET(ws(ctx, WS_P, (size_t)n * k, &p));
    GLOBE_RET(ws(ctx, WS_VP, (size_t)n * k, &Vp));
    GLOBE_RET(ws(ctx, WS_ZI, (size_t)N * k, &Zi));
    GLOBE_RET(ws(ctx, WS_GZ, (size_t)N * k, &GZ));
    GLOBE_RET(ws(ctx, WS_S1, (size_t)N * k, &S1));
    GLOBE_RET(ws(ctx, WS_SCAL, (size_t)10 * k, &scal));
    GLOBE_RET(ws(ctx, WS_COLS, (size_t)k, &dcols));
    GLOBE_RET(ws(ctx, WS_PART, (size_t)std::max<int64_t>(div_up(N, 8), 304) * k * 2, &part));
    PcgLoopState* dstate;
    GLOBE_RET(ws(ctx, WS_LOOP, 1, &dstate));
    const double* H = Hptr(ctx);
    double* rz = scal;
    double* rz2 = scal + k;
    double* pvp = scal + 2 * k;
    double* alpha = scal + 3 * k;
    double* beta = scal + 4 * k;
    double* rr = scal + 5 * k;
    double* bb = scal + 6 * k;
    double* dunsc = scal + 7 * k;   // per-column unscale factors of a double-float solve
    float2* alpha_df = reinterpret_cast<float2*>(scal + 8 * k);   // double-float copies of alpha, beta
    float2* beta_df = reinterpret_cast<float2*>(scal + 9 * k);
    if ((size_t)4 * k > ctx->hpin_n) return set_err(ctx, GLOBE_ERR_ARG, "too many right-hand sides (%d)", k);
    double* h_rr = ctx->hpin;
    double* h_bb = ctx->hpin + k;
    double* h_pvp = ctx->hpin + 2 * k;

    // Under GLOBE_PREC_MIXED the iterations run on double-float vectors (df_records_ok): x, r,
    // z and p hold pairs, column c scaled by 1/unsc[c] (a power of two, col_unscale), and x is
    // converted back when the loop ends, however it ends.  From x0 = 0 the set-up itself runs
    // in double-float (r = b scaled, z = Q^-1 r); from another start point it runs in FP64 and
    // x, r, z, p are converted in place.  r'z follows the scaling; the host and the device
    // check unscale r'r exactly (sqrt(rr) unsc = sqrt(rr unsc^2)).
    const bool df = ctx->prec == GLOBE_PREC_MIXED && ctx->record_df && df_records_ok(ctx);
    const bool df_setup = df && o->x0mode == GLOBE_X0_ZERO;
    float2* Hdf = reinterpret_cast<float2*>(ctx->ws[WS_HDF].p);
    float2* S0df = nullptr;
    if (df) GLOBE_RET(ws(ctx, WS_S0DF, (size_t)N * k, &S0df));
    auto F = [](double* v) { return reinterpret_cast<float2*>(v); };

    GLOBE_RET(col_dots(ctx, B, B, n, n, n, nullptr, k, bb));
    if (df) GLOBE_RET(col_unscales(ctx, bb, k, dunsc));
    switch (o->x0mode) {
        case GLOBE_X0_ZERO:
            GLOBE_CK(ctx, cudaMemsetAsync(X, 0, sizeof(double) * n * k, ctx->stream));
            if (df_setup) {
                DfCols v;
                v.src[0] = B;
                v.dst[0] = r;
                GLOBE_RET(cols_to_df(ctx, v, n, k, dunsc, nullptr));
            } else {
                GLOBE_CK(ctx, cudaMemcpyAsync(r, B, sizeof(double) * n * k, cudaMemcpyDeviceToDevice, ctx->stream));
            }
            break;
        case GLOBE_X0_PRECOND:
            GLOBE_RET(precond_apply(ctx, H, B, X, nullptr, k, nullptr));
            GLOBE_RET(vx_dev(ctx, X, k, Vp));
            GLOBE_RET(sub_vec(ctx, B, Vp, r, n * k));
            break;
        case GLOBE_X0_GIVEN:
            GLOBE_RET(vx_dev(ctx, X, k, Vp));
            GLOBE_RET(sub_vec(ctx, B, Vp, r, n * k));
            break;
        default:
            return set_err(ctx, GLOBE_ERR_ARG, "unknown x0 mode %d", o->x0mode);
    }
    if (df_setup) GLOBE_RET(precond_apply_df(ctx, Hdf, F(r), F(z), k, rz));
    else GLOBE_RET(precond_apply(ctx, H, r, z, nullptr, k, rz));
    GLOBE_CK(ctx, cudaMemcpyAsync(p, z, sizeof(double) * n * k, cudaMemcpyDeviceToDevice, ctx->stream));
    // from x0 = 0, r = b: r'r is b'b (the same kernel on the same values)
    const bool r_is_b = o->x0mode == GLOBE_X0_ZERO;
    if (!r_is_b) GLOBE_RET(col_dots(ctx, r, r, n, n, n, nullptr, k, rr));
    GLOBE_CK(ctx, cudaMemcpyAsync(h_bb, bb, sizeof(double) * k, cudaMemcpyDeviceToHost, ctx->stream));
    if (!r_is_b) GLOBE_CK(ctx, cudaMemcpyAsync(h_rr, rr, sizeof(double) * k, cudaMemcpyDeviceToHost, ctx->stream));
    GLOBE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (r_is_b) std::copy(h_bb, h_bb + k, h_rr);

    std::vector<double> nb(k), nr(k);
    for (int j = 0; j < k; ++j) {
        nb[j] = std::sqrt(h_bb[j]);
        nr[j] = std::sqrt(h_rr[j]);
    }
    const double small_b = (double)1e-12f;  // PCGsolver.cpp:1365, :1393
    auto max_ratio = [&]() {
        double m = 0.0;
        for (int j = 0; j < k; ++j) {
            double q = nb[j] > small_b ? nr[j] / nb[j] : 0.0;
            if (q > m) m = q;
        }
        return m;
    };
    // Columns with b = 0 have the solution x = 0 and never enter the loop
    // (the reference divides 0 by 0 there).
    std::vector<int32_t> cols;
    for (int j = 0; j < k; ++j)
        if (h_bb[j] > 0.0) cols.push_back(j);
        else GLOBE_CK(ctx, cudaMemsetAsync(X + (size_t)j * n, 0, sizeof(double) * n, ctx->stream));

    std::vector<double> unsc(k, 1.0);
    if (df) {
        for (int j = 0; j < k; ++j) unsc[j] = col_unscale(h_bb[j]);
        if (!df_setup) {   // x, r, z, p to double-float in place; r'z scaled with them
            DfCols v;
            double* vv[4] = {X, r, z, p};
            for (int j = 0; j < 4; ++j) v.src[j] = v.dst[j] = vv[j];
            GLOBE_RET(cols_to_df(ctx, v, n, k, dunsc, rz));
        }
        ctx->record_df_runs += 1;
    }
    // one iteration on the stream: the operator on p, alpha, and the updates up to r'r and r'z
    auto iteration = [&](bool first, int kc) -> int {
        if (df) {
            GLOBE_RET(seg_sums_df(ctx, F(p), first ? nullptr : F(z), first ? nullptr : beta_df, dcols, kc, Zi, S0df,
                                  F(S1)));
            GLOBE_RET(grm_apply_dev(ctx, Zi, kc, GZ));
            GLOBE_RET(vx_assemble_df(ctx, F(p), GZ, S0df, F(S1), dcols, kc, F(Vp), pvp, rz, alpha, alpha_df));
            return pcg_update_df(ctx, Hdf, alpha_df, F(X), F(r), F(p), F(Vp), F(z), dcols, kc, rr, rz2);
        }
        if (!first) GLOBE_RET(seg_sums(ctx, p, z, beta, p, dcols, kc, Zi, S1));
        else GLOBE_RET(seg_sums(ctx, p, nullptr, nullptr, nullptr, dcols, kc, Zi, S1));
        GLOBE_RET(grm_apply_dev(ctx, Zi, kc, GZ));
        GLOBE_RET(vx_assemble(ctx, p, GZ, Zi, S1, dcols, kc, Vp, pvp, rz, alpha));   // alpha = r'z / p'Vp
        return pcg_update(ctx, H, alpha, X, r, p, Vp, z, dcols, kc, rr, rz2);
    };

    std::vector<int32_t> uploaded;
    double last = max_ratio();
    const double stag_frac = (double)5e-3f;
    int stag = 0, it = 0;
    bool converged = false, stagnated = false;
    int64_t rhs_iters = 0;
    if (cols.empty()) converged = true;
    bool use_graph = ctx->graphs && !ctx->prof_on;   // profiling times each pass with events
    std::vector<int32_t> gcols[2];                   // column set each graph was captured for
    int64_t glaunch[2] = {0, 0};                     // kernels per replay
    auto iterate = [&]() -> int {
        for (it = 0; it < o->maxit && !cols.empty(); ++it) {
            const int kact = (int)cols.size();
            ProfScope iter_scope(ctx, GLOBE_PROF_PCG_ITER);
            if (cols != uploaded) {
                GLOBE_CK(ctx, cudaMemcpyAsync(dcols, cols.data(), sizeof(int32_t) * kact, cudaMemcpyHostToDevice,
                                              ctx->stream));
                uploaded = cols;
            }
            // the iteration's stream work, up to the copies of the two k-vectors the host checks
            auto body = [&](bool first) -> int {
                GLOBE_RET(iteration(first, kact));
                GLOBE_CK(ctx, cudaMemcpyAsync(h_rr, rr, sizeof(double) * k, cudaMemcpyDeviceToHost, ctx->stream));
                GLOBE_CK(ctx, cudaMemcpyAsync(h_pvp, pvp, sizeof(double) * k, cudaMemcpyDeviceToHost, ctx->stream));
                return GLOBE_OK;
            };
            // The first iteration runs directly (it also builds what the products make on first
            // use).  Later ones replay a graph of the body, captured once per call, parity of the
            // swapped r'z buffers and column set; a failed capture falls back to direct launches.
            bool ran = false;
            if (it > 0 && use_graph) {
                const int slot = rz == scal ? 0 : 1;
                if (gcols[slot] != cols) {
                    gcols[slot].clear();
                    if (capture_body(ctx, slot, [&]() { return body(false); }, &glaunch[slot])) gcols[slot] = cols;
                    else use_graph = false;
                }
                if (use_graph) {
                    GLOBE_CK(ctx, cudaGraphLaunch(ctx->pcg_graph[slot], ctx->stream));
                    ctx->launches += glaunch[slot];
                    ran = true;
                }
            }
            if (!ran) GLOBE_RET(body(it == 0));
            GLOBE_CK(ctx, cudaStreamSynchronize(ctx->stream));
            rhs_iters += kact;
            for (int j : cols) {
                if (!(h_pvp[j] > 0.0) || !std::isfinite(h_rr[j]))
                    return set_err(ctx, GLOBE_ERR_NUMERIC, "PCG breakdown in column %d at iteration %d (p'Vp = %g)", j,
                                   it + 1, h_pvp[j] * unsc[j] * unsc[j]);
                nr[j] = std::sqrt(h_rr[j]) * unsc[j];
            }
            if (o->rule == GLOBE_RULE_PCGSOLVER) {
                double mx = max_ratio();
                if (mx < o->tol) { converged = true; ++it; break; }
                double impr = last - mx;
                if (impr < stag_frac * last) ++stag;
                else stag = 0;
                last = mx;
                if (stag >= 10) { stagnated = true; ++it; break; }
            } else {
                bool all = true;
                for (int j = 0; j < k; ++j)
                    if (h_bb[j] > 0.0 && !(nr[j] < o->tol * nb[j])) { all = false; break; }
                if (all) { converged = true; ++it; break; }
            }
            if (o->mask) {
                std::vector<int32_t> keep;
                for (int j : cols)
                    if (!(nr[j] < o->tol * nb[j])) keep.push_back(j);
                if (keep.empty()) { converged = true; ++it; break; }
                cols.swap(keep);
            }
            GLOBE_RET(scal_alpha(ctx, rz2, rz, beta, k, df ? beta_df : nullptr));
            std::swap(rz, rz2);
            // after the first iteration, the rest as one device-side loop (no per-iteration
            // synchronisation) when graphs are on and the column set cannot change
            if (it == 0 && use_graph && ctx->device_loop && !o->mask && o->maxit > 1) {
                const PcgLoopState st0{last, 0, 1, stag, 0, -1};
                GLOBE_CK(ctx, cudaMemcpyAsync(dstate, &st0, sizeof st0, cudaMemcpyHostToDevice, ctx->stream));
                const int kc = kact;
                auto loop_body = [&](cudaGraphConditionalHandle h) -> int {
                    GLOBE_RET(iteration(false, kc));
                    k_pcg_check_shift<<<div_up(k, 128), 128, 0, ctx->stream>>>(
                        rr, pvp, bb, dcols, kc, k, o->tol, o->rule, o->maxit, df ? dunsc : nullptr, dstate, h, rz, rz2,
                        beta, df ? beta_df : nullptr);
                    GLOBE_LAUNCHED(ctx, "k_pcg_check_shift");
                    return GLOBE_OK;
                };
                int64_t per_it = 0;
                bool ran = false;
                GLOBE_RET(run_device_loop(ctx, loop_body, &per_it, &ran));
                if (ran) {
                    PcgLoopState st;
                    double* h_scr = ctx->hpin + 3 * k;   // k doubles: the final r'r
                    GLOBE_CK(ctx, cudaMemcpyAsync(&st, dstate, sizeof st, cudaMemcpyDeviceToHost, ctx->stream));
                    GLOBE_CK(ctx, cudaMemcpyAsync(h_scr, rr, sizeof(double) * k, cudaMemcpyDeviceToHost, ctx->stream));
                    GLOBE_CK(ctx, cudaMemcpyAsync(h_pvp, pvp, sizeof(double) * k, cudaMemcpyDeviceToHost, ctx->stream));
                    GLOBE_CK(ctx, cudaStreamSynchronize(ctx->stream));
                    if (st.it > 1) {   // the loop ran (see run_device_loop)
                        ctx->launches += per_it * (st.it - 1) + 1;
                        ctx->device_loop_runs += 1;
                        rhs_iters += st.rhs_iters;
                        for (int j : cols) nr[j] = std::sqrt(h_scr[j]) * unsc[j];
                        if (st.status == 4)
                            return set_err(ctx, GLOBE_ERR_NUMERIC,
                                           "PCG breakdown in column %d at iteration %d (p'Vp = %g)", st.err_col, st.it,
                                           h_pvp[st.err_col] * unsc[st.err_col] * unsc[st.err_col]);
                        converged = st.status == 1;
                        stagnated = st.status == 2;
                        it = st.it;
                        break;
                    }
                }
                use_graph = use_graph && ran;
            }
        }
        return GLOBE_OK;
    };
    const int rc = iterate();
    if (df) {   // x back to FP64, whatever ended the loop (an earlier error's message is kept)
        const std::string e0 = ctx->err;
        const int rc2 = cols_from_df(ctx, X, n, k, dunsc);
        if (rc != GLOBE_OK) ctx->err = e0;
        else if (rc2 != GLOBE_OK) return rc2;
    }
    if (rc != GLOBE_OK) return rc;
    if (info) {
        info->iters = it;
        info->inner_iters = it;
        info->rhs_iters = rhs_iters;
        info->max_rel_res = max_ratio();
        info->converged = converged ? 1 : 0;
        info->stagnated = stagnated ? 1 : 0;
    }
    return GLOBE_OK;
}

// (m x m) inverse, Gauss-Jordan with partial pivoting, column-major
bool small_inverse(std::vector<double>& A, int m) {
    std::vector<double> I(m * m, 0.0);
    for (int i = 0; i < m; ++i) I[i * m + i] = 1.0;
    for (int col = 0; col < m; ++col) {
        int pr = col;
        for (int r = col + 1; r < m; ++r)
            if (std::fabs(A[col * m + r]) > std::fabs(A[col * m + pr])) pr = r;
        if (A[col * m + pr] == 0.0) return false;
        if (pr != col)
            for (int j = 0; j < m; ++j) {
                std::swap(A[j * m + col], A[j * m + pr]);
                std::swap(I[j * m + col], I[j * m + pr]);
            }
        double d = A[col * m + col];
        for (int j = 0; j < m; ++j) {
            A[j * m + col] /= d;
            I[j * m + col] /= d;
        }
        for (int r = 0; r < m; ++r) {
            if (r == col) continue;
            double f = A[col * m + r];
            if (f == 0.0) continue;
            for (int j = 0; j < m; ++j) {
                A[j * m + r] -= f * A[j * m + col];
                I[j * m + r] -= f * I[j * m + col];
            }
        }
    }
    A.swap(I);
    return true;
}

// out = P V = V - V^-1X (X'V^-1X)^-1 X' V  for V (Nrec x m)
static int project_dev(globe_ctx* ctx, const double* V, int m, double* out) {
    const int p1 = ctx->coh.p + 1;
    double* small;
    GLOBE_RET(ws(ctx, WS_SMALL, (size_t)2 * p1 * m + 64, &small));
    GLOBE_RET(xt_mat(ctx, ctx->coh.X, p1, V, m, small));
    std::vector<double> xv(p1 * m), cc(p1 * m);
    GLOBE_RET(d2h(ctx, xv.data(), small, (size_t)p1 * m));
    const auto& inv = ctx->xtvx_inv;
    for (int j = 0; j < m; ++j)
        for (int a = 0; a < p1; ++a) {
            double acc = 0.0;
            for (int b = 0; b < p1; ++b) acc += inv[b * p1 + a] * xv[j * p1 + b];
            cc[j * p1 + a] = acc;
        }
    double* dc = small + (size_t)p1 * m;
    GLOBE_CK(ctx, cudaMemcpyAsync(dc, cc.data(), sizeof(double) * p1 * m, cudaMemcpyHostToDevice, ctx->stream));
    GLOBE_RET(sub_mat(ctx, V, ctx->vinv_X, p1, dc, out, m));
    return GLOBE_OK;
}

}  // namespace globe

using namespace globe;

// ---------------------------------------------------------------------------
// C ABI

template <class F>
static int host_io(globe_ctx* ctx, const double* in, size_t nin, double* out, size_t nout, F&& body) {
    double *din, *dout;
    GLOBE_RET(ws(ctx, WS_IO1, nin, &din));
    GLOBE_RET(ws(ctx, WS_IO2, nout, &dout));
    if (in) GLOBE_CK(ctx, cudaMemcpyAsync(din, in, sizeof(double) * nin, cudaMemcpyHostToDevice, ctx->stream));
    GLOBE_RET(body(din, dout));
    GLOBE_CK(ctx, cudaMemcpyAsync(out, dout, sizeof(double) * nout, cudaMemcpyDeviceToHost, ctx->stream));
    GLOBE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return GLOBE_OK;
}

extern "C" {

int globe_grm_apply_dev(globe_ctx* ctx, const double* d_Z, double* d_out, int k) {
    if (!ctx || !d_Z || !d_out || k < 1) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    GLOBE_RET(check_ready(ctx));
    return grm_apply_dev(ctx, d_Z, k, d_out);
}

int globe_grm_apply(globe_ctx* ctx, const double* Z, double* out, int k) {
    if (!ctx || !Z || !out || k < 1) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    GLOBE_RET(check_ready(ctx));
    size_t n = (size_t)ctx->coh.N * k;
    const int rc = host_io(ctx, Z, n, out, n, [&](double* a, double* b) { return grm_apply_dev(ctx, a, k, b); });
    return with_tc_check(ctx, ctx->prec, rc);
}

int globe_vx_dev(globe_ctx* ctx, const double* d_x, double* d_out, int k) {
    if (!ctx || !d_x || !d_out || k < 1) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    GLOBE_RET(check_ready(ctx));
    return vx_dev(ctx, d_x, k, d_out);
}

int globe_vx(globe_ctx* ctx, const double* x, double* out, int k) {
    if (!ctx || !x || !out || k < 1) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    GLOBE_RET(check_ready(ctx));
    size_t n = (size_t)ctx->coh.Nrec * k;
    const int rc = host_io(ctx, x, n, out, n, [&](double* a, double* b) { return vx_dev(ctx, a, k, b); });
    return with_tc_check(ctx, ctx->prec, rc);
}

int globe_precond_apply(globe_ctx* ctx, const double* r, double* z, int k) {
    if (!ctx || !r || !z || k < 1) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    GLOBE_RET(check_ready(ctx));
    GLOBE_RET(ensure_precond(ctx));
    size_t n = (size_t)ctx->coh.Nrec * k;
    return host_io(ctx, r, n, z, n, [&](double* a, double* b) {
        return precond_apply(ctx, (const double*)ctx->ws[WS_H].p, a, b, nullptr, k, nullptr);
    });
}

int globe_genetic_diag(globe_ctx* ctx, double* diag) {
    if (!ctx || !diag) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->coh.N < 1 || ctx->gen.src == GSRC_NONE)
        return set_err(ctx, GLOBE_ERR_STATE, "records and a genetic source must be loaded");
    GLOBE_RET(ensure_gdiag(ctx));
    return d2h(ctx, diag, ctx->gen.gdiag, ctx->coh.N);
}

int globe_pcg_dev(globe_ctx* ctx, const double* d_B, double* d_X, int k, const globe_pcg_opts* opts,
                  globe_pcg_info* info) {
    NvtxRange nvtx("globe_pcg_dev");
    if (!ctx || !d_B || !d_X) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    return pcg_dev(ctx, d_B, d_X, k, opts, info);
}

int globe_pcg(globe_ctx* ctx, const double* B, double* X, int k, const globe_pcg_opts* opts, globe_pcg_info* info) {
    NvtxRange nvtx("globe_pcg");
    if (!ctx || !B || !X || k < 1) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    GLOBE_RET(check_ready(ctx));
    size_t n = (size_t)ctx->coh.Nrec * k;
    double *dB, *dX;
    GLOBE_RET(ws(ctx, WS_IO1, n, &dB));
    GLOBE_RET(ws(ctx, WS_IO2, n, &dX));
    GLOBE_CK(ctx, cudaMemcpyAsync(dB, B, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    if (opts && opts->x0mode == GLOBE_X0_GIVEN)
        GLOBE_CK(ctx, cudaMemcpyAsync(dX, X, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    GLOBE_RET(pcg_dev(ctx, dB, dX, k, opts, info));
    GLOBE_CK(ctx, cudaMemcpyAsync(X, dX, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    GLOBE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return GLOBE_OK;
}

// ---- MME and AIREML score: right-hand sides, solves, and what follows them ----

static int mme_prepare(globe_ctx* ctx) {
    auto& c = ctx->coh;
    const int64_t n = c.Nrec;
    const int k = c.p + 2;
    if (!ctx->vinv_X) GLOBE_RET(dalloc(ctx, &ctx->vinv_X, (size_t)n * k));
    if (!ctx->vinv_r) GLOBE_RET(dalloc(ctx, &ctx->vinv_r, (size_t)n));
    if (!ctx->uhat) GLOBE_RET(dalloc(ctx, &ctx->uhat, (size_t)c.N));
    ctx->mme_ok = ctx->fth_ok = false;
    return GLOBE_OK;
}

// B (Nrec x (p+2)) = [X y]
static int mme_rhs(globe_ctx* ctx, double* B) {
    auto& c = ctx->coh;
    const int64_t n = c.Nrec;
    const int p1 = c.p + 1;
    GLOBE_CK(ctx, cudaMemcpyAsync(B, c.X, sizeof(double) * n * p1, cudaMemcpyDeviceToDevice, ctx->stream));
    GLOBE_CK(ctx, cudaMemcpyAsync(B + (size_t)n * p1, c.y, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
    return GLOBE_OK;
}

// From ctx->vinv_X = V^-1 [X y]: beta, V^-1 r, u-hat, b-hat (fitMME, varCompEst.cpp:587-685).
// with_uhat = false leaves u-hat to the caller (the fused AIREML evaluation forms it in one
// GRM product with the probes' u-hat); the MME is then not marked complete.
static int mme_finish(globe_ctx* ctx, double* beta, double* uhat, double* bhat, double* vinv_r,
                      bool with_uhat = true) {
    auto& c = ctx->coh;
    const int64_t n = c.Nrec;
    const int32_t N = c.N;
    const int p1 = c.p + 1, k = c.p + 2;
    double* S = ctx->vinv_X;  // [V^-1 X | V^-1 y]
    double* small;
    GLOBE_RET(ws(ctx, WS_SMALL, (size_t)p1 * (p1 + 2) + 64, &small));
    GLOBE_RET(xt_mat(ctx, c.X, p1, S, k, small));  // [X'V^-1X | X'V^-1y]
    std::vector<double> xs((size_t)p1 * k);
    GLOBE_RET(d2h(ctx, xs.data(), small, xs.size()));
    std::vector<double> A(xs.begin(), xs.begin() + (size_t)p1 * p1);
    if (!small_inverse(A, p1)) return set_err(ctx, GLOBE_ERR_NUMERIC, "X'V^-1X is singular");
    std::vector<double> b(p1);
    for (int a = 0; a < p1; ++a) {
        double acc = 0;
        for (int q = 0; q < p1; ++q) acc += A[q * p1 + a] * xs[(size_t)p1 * p1 + q];
        b[a] = acc;
    }
    ctx->xtvx_inv = A;
    double* dbeta = small + (size_t)p1 * k;
    GLOBE_CK(ctx, cudaMemcpyAsync(dbeta, b.data(), sizeof(double) * p1, cudaMemcpyHostToDevice, ctx->stream));
    GLOBE_RET(sub_mat(ctx, S + (size_t)n * p1, S, p1, dbeta, ctx->vinv_r, 1));
    double *Zi, *S1, *dbhat;
    GLOBE_RET(ws(ctx, WS_ZI, (size_t)N, &Zi));
    GLOBE_RET(ws(ctx, WS_S1, (size_t)N, &S1));
    if (with_uhat) {
        GLOBE_RET(seg_sums(ctx, ctx->vinv_r, nullptr, nullptr, nullptr, nullptr, 1, Zi, S1));
        GLOBE_RET(grm_apply_dev(ctx, Zi, 1, ctx->uhat));
    }
    GLOBE_RET(ws(ctx, WS_BHAT, (size_t)2 * N, &dbhat));
    GLOBE_RET(bhat_kernel(ctx, ctx->vinv_r, dbhat));
    if (beta) std::memcpy(beta, b.data(), sizeof(double) * p1);
    if (uhat) GLOBE_CK(ctx, cudaMemcpyAsync(uhat, ctx->uhat, sizeof(double) * N, cudaMemcpyDeviceToHost, ctx->stream));
    if (bhat) GLOBE_CK(ctx, cudaMemcpyAsync(bhat, dbhat, sizeof(double) * 2 * N, cudaMemcpyDeviceToHost, ctx->stream));
    if (vinv_r) GLOBE_CK(ctx, cudaMemcpyAsync(vinv_r, ctx->vinv_r, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    GLOBE_CK(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->mme_ok = with_uhat;
    return GLOBE_OK;
}

static int mme_impl(globe_ctx* ctx, const globe_pcg_opts* opts, double* beta, double* uhat, double* bhat,
                    double* vinv_r, globe_pcg_info* info) {
    if (!ctx || !opts) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    GLOBE_RET(check_ready(ctx));
    GLOBE_RET(mme_prepare(ctx));
    const int64_t n = ctx->coh.Nrec;
    const int k = ctx->coh.p + 2;
    double* B;
    GLOBE_RET(ws(ctx, WS_B, (size_t)n * k, &B));
    GLOBE_RET(mme_rhs(ctx, B));
    GLOBE_RET(pcg_dev(ctx, B, ctx->vinv_X, k, opts, info));
    return mme_finish(ctx, beta, uhat, bhat, vinv_r);
}

static int grad_check(globe_ctx* ctx, int numMC) {
    if (numMC < 1) return set_err(ctx, GLOBE_ERR_ARG, "numMC must be >= 1");
    if (!(ctx->vc[1] > 0.0)) return set_err(ctx, GLOBE_ERR_ARG, "AIREML needs sig2g > 0");
    if (ctx->model == GLOBE_MODEL_FULL && !(ctx->vc[2] > 0.0))
        return set_err(ctx, GLOBE_ERR_ARG, "AIREML needs sig2b0 > 0 (the time effects' probe Cholesky factor)");
    return GLOBE_OK;
}

// Probes Y_v ~ N(0, V*) and TY = V*^-1 Y (the PCG start), sample_Yvs and
// estimateTrace_PdV (varCompEst.cpp:775-862)
// VR and UH have one leading column more than the probes (VR0 / UH0): the fused evaluation
// puts V^-1 r there and gets u-hat from the same GRM product as the probes' u-hat.
struct ProbeBufs {
    double *Y, *TY, *VR, *UH, *Hs, *VR0, *UH0;
};

static int grad_probes(globe_ctx* ctx, const double* probes, int numMC, uint64_t seed, ProbeBufs& pb) {
    const int64_t n = ctx->coh.Nrec;
    const int32_t N = ctx->coh.N;
    GLOBE_RET(ws(ctx, WS_TMP1, (size_t)n * numMC, &pb.Y));
    GLOBE_RET(ws(ctx, WS_TMP2, (size_t)n * numMC, &pb.TY));
    GLOBE_RET(ws(ctx, WS_TMP4, (size_t)n * (numMC + 1), &pb.VR0));
    GLOBE_RET(ws(ctx, WS_UH, (size_t)N * (numMC + 1), &pb.UH0));
    pb.VR = pb.VR0 + n;
    pb.UH = pb.UH0 + N;
    GLOBE_RET(ws(ctx, WS_HSTAR, (size_t)N * 4, &pb.Hs));
    if (probes) {
        double* dd;
        size_t cnt = (size_t)numMC * ((ctx->model == GLOBE_MODEL_NO_TIME ? 1 : 3) * (size_t)N + n);
        GLOBE_RET(ws(ctx, WS_PROBE, cnt, &dd));
        GLOBE_CK(ctx, cudaMemcpyAsync(dd, probes, sizeof(double) * cnt, cudaMemcpyHostToDevice, ctx->stream));
        GLOBE_RET(probes_build(ctx, dd, numMC, seed, false, pb.Y, nullptr));
    } else {
        double* zi;   // per-individual normals (the injected-draws buffer is free in this mode)
        GLOBE_RET(ws(ctx, WS_PROBE, (size_t)3 * N * numMC, &zi));
        GLOBE_RET(probes_build(ctx, nullptr, numMC, seed, true, pb.Y, zi));
    }
    // V*^-1 Y by the Woodbury block inverse with g = sig2g (varCompEst.cpp:839-862)
    GLOBE_RET(build_H(ctx, nullptr, ctx->vc[1], pb.Hs));
    GLOBE_RET(precond_apply(ctx, pb.Hs, pb.Y, pb.TY, nullptr, numMC, nullptr));
    return GLOBE_OK;
}

// From the MME (V^-1 r, u-hat) and VY = V^-1 Y: f_theta, the first-order terms, the
// Monte-Carlo trace and the score (computeDerivative_first, varCompEst.cpp:693-1012).
// with_uhat: u-hat is not formed yet; it comes out of the probes' GRM product (column 0 of
// VR0 / UH0).  Every column of a GRM product is computed on its own, so the values are the
// same as from two products.
static int grad_finish(globe_ctx* ctx, int numMC, const double* VY, const ProbeBufs& pb, double* f_theta,
                       double* first, double* trace, double* grad, bool with_uhat = false) {
    auto& c = ctx->coh;
    const int64_t n = c.Nrec;
    const int32_t N = c.N;
    if (!ctx->f_theta) GLOBE_RET(dalloc(ctx, &ctx->f_theta, (size_t)n * 5));
    double* fth = ctx->f_theta;
    GLOBE_RET(project_dev(ctx, VY, numMC, pb.VR));
    double *Zi, *S1;
    GLOBE_RET(ws(ctx, WS_ZI, (size_t)N * (numMC + 1), &Zi));
    GLOBE_RET(ws(ctx, WS_S1, (size_t)N * (numMC + 1), &S1));
    if (with_uhat) {
        GLOBE_CK(ctx, cudaMemcpyAsync(pb.VR0, ctx->vinv_r, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                      ctx->stream));
        GLOBE_RET(seg_sums(ctx, pb.VR0, nullptr, nullptr, nullptr, nullptr, numMC + 1, Zi, S1));
        GLOBE_RET(grm_apply_dev(ctx, Zi, numMC + 1, pb.UH0));
        GLOBE_CK(ctx, cudaMemcpyAsync(ctx->uhat, pb.UH0, sizeof(double) * N, cudaMemcpyDeviceToDevice,
                                      ctx->stream));
        ctx->mme_ok = true;
    } else {
        GLOBE_RET(seg_sums(ctx, pb.VR, nullptr, nullptr, nullptr, nullptr, numMC, Zi, S1));
        GLOBE_RET(grm_apply_dev(ctx, Zi, numMC, pb.UH));
    }
    GLOBE_RET(ftheta_kernel(ctx, ctx->vinv_r, ctx->uhat, fth));
    double* small;
    GLOBE_RET(ws(ctx, WS_SMALL, (size_t)numMC * 5 + 64, &small));
    GLOBE_RET(xt_mat(ctx, ctx->vinv_r, 1, fth, 5, small));
    double h_first[5];
    GLOBE_RET(d2h(ctx, h_first, small, 5));
    GLOBE_RET(ws(ctx, WS_SMALL, (size_t)numMC * 5 + 64, &small));
    GLOBE_RET(trace_terms(ctx, pb.VR, pb.UH, pb.TY, numMC, small));
    std::vector<double> tt((size_t)numMC * 5);
    GLOBE_RET(d2h(ctx, tt.data(), small, tt.size()));
    double h_trace[5], h_grad[5];
    const int nc = ctx->nvc();
    for (int q = 0; q < 5; ++q) {
        double a = 0;
        for (int j = 0; j < numMC; ++j) a += tt[(size_t)j * 5 + q];
        h_trace[q] = a / numMC;
        h_grad[q] = 0.5 * (h_first[q] - h_trace[q]);  // varCompEst.cpp:1006-1010
        if (q >= nc) h_first[q] = h_trace[q] = h_grad[q] = 0.0;   // no such component in this model
    }
    if (first) std::memcpy(first, h_first, sizeof(h_first));
    if (trace) std::memcpy(trace, h_trace, sizeof(h_trace));
    if (grad) std::memcpy(grad, h_grad, sizeof(h_grad));
    if (f_theta) GLOBE_RET(d2h(ctx, f_theta, fth, (size_t)n * 5));
    ctx->fth_ok = true;
    return GLOBE_OK;
}

static int aireml_grad_impl(globe_ctx* ctx, const double* probes, int numMC, uint64_t seed, const globe_pcg_opts* opts,
                            double* f_theta, double* first, double* trace, double* grad, globe_pcg_info* info) {
    if (!ctx || !opts || numMC < 1) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    GLOBE_RET(check_ready(ctx));
    if (!ctx->mme_ok) return set_err(ctx, GLOBE_ERR_STATE, "call globe_mme at the current components first");
    GLOBE_RET(grad_check(ctx, numMC));
    ProbeBufs pb;
    GLOBE_RET(grad_probes(ctx, probes, numMC, seed, pb));
    const int64_t n = ctx->coh.Nrec;
    double* VY;
    GLOBE_RET(ws(ctx, WS_TMP3, (size_t)n * numMC, &VY));
    GLOBE_CK(ctx, cudaMemcpyAsync(VY, pb.TY, sizeof(double) * n * numMC, cudaMemcpyDeviceToDevice, ctx->stream));
    globe_pcg_opts o = *opts;
    o.rule = GLOBE_RULE_AIREML;
    o.x0mode = GLOBE_X0_GIVEN;
    GLOBE_RET(pcg_dev(ctx, pb.Y, VY, numMC, &o, info));
    return grad_finish(ctx, numMC, VY, pb, f_theta, first, trace, grad);
}

// MME and score with one block solve of [X y | probes]: the MME columns start from
// Q^-1 b (fitMME's use_initial_guess), the probe columns from V*^-1 Y.
static int aireml_eval_impl(globe_ctx* ctx, const double* probes, int numMC, uint64_t seed,
                            const globe_pcg_opts* opts, double* first, double* trace, double* grad,
                            globe_pcg_info* info) {
    if (!ctx || !opts || numMC < 1) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    GLOBE_RET(check_ready(ctx));
    GLOBE_RET(grad_check(ctx, numMC));
    GLOBE_RET(mme_prepare(ctx));
    ProbeBufs pb;
    GLOBE_RET(grad_probes(ctx, probes, numMC, seed, pb));
    const int64_t n = ctx->coh.Nrec;
    const int k = ctx->coh.p + 2, kt = k + numMC;
    double *FB, *FX;
    GLOBE_RET(ws(ctx, WS_FB, (size_t)n * kt, &FB));
    GLOBE_RET(ws(ctx, WS_FX, (size_t)n * kt, &FX));
    GLOBE_RET(mme_rhs(ctx, FB));
    GLOBE_CK(ctx, cudaMemcpyAsync(FB + (size_t)n * k, pb.Y, sizeof(double) * n * numMC, cudaMemcpyDeviceToDevice,
                                  ctx->stream));
    GLOBE_RET(ensure_precond(ctx));
    GLOBE_RET(precond_apply(ctx, Hptr(ctx), FB, FX, nullptr, k, nullptr));
    GLOBE_CK(ctx, cudaMemcpyAsync(FX + (size_t)n * k, pb.TY, sizeof(double) * n * numMC, cudaMemcpyDeviceToDevice,
                                  ctx->stream));
    globe_pcg_opts o = *opts;
    o.rule = GLOBE_RULE_AIREML;
    o.x0mode = GLOBE_X0_GIVEN;
    GLOBE_RET(pcg_dev(ctx, FB, FX, kt, &o, info));
    GLOBE_CK(ctx, cudaMemcpyAsync(ctx->vinv_X, FX, sizeof(double) * n * k, cudaMemcpyDeviceToDevice, ctx->stream));
    GLOBE_RET(mme_finish(ctx, nullptr, nullptr, nullptr, nullptr, false));
    return grad_finish(ctx, numMC, FX + (size_t)n * k, pb, nullptr, first, trace, grad, true);
}

// The GRM products outside the PCG solves (u-hat, the probes' u-hat) run at the
// precision of the solve: opts->precision holds for the whole call.
struct PrecScope {
    globe_ctx* ctx;
    int saved;
    PrecScope(globe_ctx* c, int p) : ctx(c), saved(c->prec) { c->prec = p; }
    ~PrecScope() { ctx->prec = saved; }
};

static int check_prec(globe_ctx* ctx, const globe_pcg_opts* o) {
    if (o->precision != GLOBE_PREC_FP64 && o->precision != GLOBE_PREC_MIXED)
        return set_err(ctx, GLOBE_ERR_ARG, "unknown precision mode %d", o->precision);
    return GLOBE_OK;
}

int globe_mme(globe_ctx* ctx, const globe_pcg_opts* opts, double* beta, double* uhat, double* bhat, double* vinv_r,
              globe_pcg_info* info) {
    NvtxRange nvtx("globe_mme");
    if (!ctx || !opts) return GLOBE_ERR_ARG;
    GLOBE_RET(check_prec(ctx, opts));
    int rc;
    {
        PrecScope ps(ctx, opts->precision);
        rc = mme_impl(ctx, opts, beta, uhat, bhat, vinv_r, info);
    }
    return with_tc_check(ctx, opts->precision, rc);
}

int globe_aireml_grad(globe_ctx* ctx, const double* probes, int numMC, uint64_t seed, const globe_pcg_opts* opts,
                      double* f_theta, double* first, double* trace, double* grad, globe_pcg_info* info) {
    NvtxRange nvtx("globe_aireml_grad");
    if (!ctx || !opts) return GLOBE_ERR_ARG;
    GLOBE_RET(check_prec(ctx, opts));
    int rc;
    {
        PrecScope ps(ctx, opts->precision);
        rc = aireml_grad_impl(ctx, probes, numMC, seed, opts, f_theta, first, trace, grad, info);
    }
    return with_tc_check(ctx, opts->precision, rc);
}

int globe_aireml_eval(globe_ctx* ctx, const double* probes, int numMC, uint64_t seed, const globe_pcg_opts* opts,
                      double* first, double* trace, double* grad, globe_pcg_info* info) {
    NvtxRange nvtx("globe_aireml_eval");
    if (!ctx || !opts) return GLOBE_ERR_ARG;
    GLOBE_RET(check_prec(ctx, opts));
    int rc;
    {
        PrecScope ps(ctx, opts->precision);
        rc = aireml_eval_impl(ctx, probes, numMC, seed, opts, first, trace, grad, info);
    }
    return with_tc_check(ctx, opts->precision, rc);
}

int globe_aireml_ai(globe_ctx* ctx, const globe_pcg_opts* opts, double* ai, globe_pcg_info* info) {
    NvtxRange nvtx("globe_aireml_ai");
    if (!ctx || !opts || !ai) return GLOBE_ERR_ARG;
    cudaSetDevice(ctx->device);
    GLOBE_RET(check_ready(ctx));
    if (!ctx->fth_ok) return set_err(ctx, GLOBE_ERR_STATE, "call globe_aireml_grad first");
    const int64_t n = ctx->coh.Nrec;
    const int nc = ctx->nvc();   // f_theta columns of this model
    double *Vf, *Pf, *small;
    GLOBE_RET(ws(ctx, WS_TMP1, (size_t)n * nc, &Vf));
    GLOBE_RET(ws(ctx, WS_TMP2, (size_t)n * nc, &Pf));
    globe_pcg_opts o = *opts;
    o.rule = GLOBE_RULE_AIREML;
    o.x0mode = GLOBE_X0_PRECOND;
    GLOBE_RET(pcg_dev(ctx, ctx->f_theta, Vf, nc, &o, info));
    GLOBE_RET(project_dev(ctx, Vf, nc, Pf));
    GLOBE_RET(ws(ctx, WS_SMALL, 64, &small));
    GLOBE_RET(xt_mat(ctx, ctx->f_theta, nc, Pf, nc, small));
    double h[25];
    GLOBE_RET(d2h(ctx, h, small, (size_t)nc * nc));
    for (int e = 0; e < 25; ++e) ai[e] = 0.0;
    for (int c = 0; c < nc; ++c)
        for (int r = 0; r < nc; ++r) ai[c * 5 + r] = 0.5 * h[c * nc + r];  // varCompEst.cpp:1038
    return GLOBE_OK;
}

}  // extern "C"
