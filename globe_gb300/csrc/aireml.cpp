// aireml.cpp -- AIREML outer loop (host C++) and its trust-region steps.
//
// Two models: runAIREML's five components, and runAIREML_reducedModel's two
// (sig2e, sig2g; no time effects, varCompEst_reducedModel_noTime.cpp:782-1090),
// chosen by globe_set_model on the context.
//
// The loop mirrors runAIREML's main and oneIter_AIREML
// (varCompEst.cpp:1148-1344, :1415-1491): gradient from the Monte-Carlo score,
// AI matrix, a constrained quadratic model step, step halving, the rho test
// and the trust-radius update, with the same constants.  The model step is
// the one part the reference hands to NLopt's MMA (a closed binary); here it
// is solved by a primal-dual interior-point method written from the problem:
//
//   max  g'p - p'Ap/2  s.t.  |p_k| <= 10,  sum_k A_kk p_k <= Delta,
//        theta_k + p_k >= 1e-5 (k != 3),
//        (theta_3+p_3)^2 <= (theta_2+p_2)(theta_4+p_4) - 1e-3.
//
// The last constraint is written in the equivalent convex form
// sqrt(4 x3^2 + 4e-3 + (x2 - x4)^2) <= x2 + x4 (x = theta + p), so the
// problem is convex and its solution unique when A is positive definite.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "globe.h"

namespace globe {
int set_err(globe_ctx* ctx, int code, const char* fmt, ...);   // api.cu
}

namespace {

// NVTX range for a scope (AIREML iterations and gradient evaluations on a profiler timeline)
struct Nvtx {
    explicit Nvtx(const char* name) { nvtxRangePushA(name); }
    ~Nvtx() { nvtxRangePop(); }
};

struct Cons {
    // c(p) <= 0 ; gradient; Hessian (only the covariance constraint has one)
    int kind;  // 0 linear (a'p + b), 1 covariance
    double a[5];
    double b;
};

struct TRProblem {
    double th[5], g[5], A[25];
    std::vector<Cons> cons;
};

double cov_val(const TRProblem& P, const double* p, double* grad, double* hess) {
    const double x2 = P.th[2] + p[2], x3 = P.th[3] + p[3], x4 = P.th[4] + p[4];
    const double d = x2 - x4;
    const double q = 4.0 * x3 * x3 + 4e-3 + d * d;
    const double r = std::sqrt(q);
    if (grad) {
        for (int k = 0; k < 5; ++k) grad[k] = 0.0;
        grad[2] = d / r - 1.0;
        grad[3] = 4.0 * x3 / r;
        grad[4] = -d / r - 1.0;
    }
    if (hess) {
        // Hessian of sqrt(u'Mu + c) with u = (x2, x3, x4):  (M r - (Mu)(Mu)'/r) / r^2
        for (int e = 0; e < 25; ++e) hess[e] = 0.0;
        const double mu[3] = {d, 4.0 * x3, -d};  // M u, M = [[1,0,-1],[0,4,0],[-1,0,1]]
        const double M[3][3] = {{1, 0, -1}, {0, 4, 0}, {-1, 0, 1}};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) hess[(2 + j) * 5 + (2 + i)] = (M[i][j] - mu[i] * mu[j] / q) / r;
    }
    return r - (x2 + x4);
}

double cval(const TRProblem& P, const Cons& c, const double* p, double* grad, double* hess) {
    if (c.kind == 1) return cov_val(P, p, grad, hess);
    double v = c.b;
    for (int k = 0; k < 5; ++k) v += c.a[k] * p[k];
    if (grad)
        for (int k = 0; k < 5; ++k) grad[k] = c.a[k];
    if (hess)
        for (int e = 0; e < 25; ++e) hess[e] = 0.0;
    return v;
}

bool solve5(double* M, double* rhs) {
    // Gaussian elimination with partial pivoting, M column-major 5x5
    const int n = 5;
    for (int c = 0; c < n; ++c) {
        int pr = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(M[c * n + r]) > std::fabs(M[c * n + pr])) pr = r;
        if (M[c * n + pr] == 0.0) return false;
        if (pr != c) {
            for (int j = 0; j < n; ++j) std::swap(M[j * n + c], M[j * n + pr]);
            std::swap(rhs[c], rhs[pr]);
        }
        for (int r = c + 1; r < n; ++r) {
            double f = M[c * n + r] / M[c * n + c];
            for (int j = c; j < n; ++j) M[j * n + r] -= f * M[j * n + c];
            rhs[r] -= f * rhs[c];
        }
    }
    for (int r = n - 1; r >= 0; --r) {
        double s = rhs[r];
        for (int j = r + 1; j < n; ++j) s -= M[j * n + r] * rhs[j];
        rhs[r] = s / M[r * n + r];
    }
    return true;
}

// returns 0 solved, 1 infeasible, 2 not converged
int solve_tr(const double* theta, const double* g, const double* A, double delta, double* pout) {
    TRProblem P;
    std::memcpy(P.th, theta, sizeof(P.th));
    double amax = 1.0;
    for (int e = 0; e < 25; ++e) amax = std::fmax(amax, std::fabs(A[e]));
    for (int k = 0; k < 5; ++k) P.g[k] = g[k] / amax;
    for (int e = 0; e < 25; ++e) P.A[e] = 0.5 * (A[e] + A[(e % 5) * 5 + e / 5]) / amax;  // symmetric part
    for (int k = 0; k < 5; ++k) {
        Cons up{0, {0, 0, 0, 0, 0}, -10.0};
        up.a[k] = 1.0;
        Cons lo{0, {0, 0, 0, 0, 0}, -10.0};
        lo.a[k] = -1.0;
        P.cons.push_back(up);
        P.cons.push_back(lo);
    }
    double sdiag = 0.0;
    for (int k = 0; k < 5; ++k) sdiag += std::fabs(A[k * 5 + k]);
    if (delta < 10.0 * sdiag * 1.000001) {  // otherwise it can never bind inside the box
        Cons tr{0, {0, 0, 0, 0, 0}, -delta};
        for (int k = 0; k < 5; ++k) tr.a[k] = A[k * 5 + k];
        // scale the row to unit size for conditioning
        double nrm = 0;
        for (int k = 0; k < 5; ++k) nrm = std::fmax(nrm, std::fabs(tr.a[k]));
        if (nrm > 0) {
            for (int k = 0; k < 5; ++k) tr.a[k] /= nrm;
            tr.b /= nrm;
        }
        P.cons.push_back(tr);
    }
    for (int k = 0; k < 5; ++k) {
        if (k == 3) continue;
        Cons pos{0, {0, 0, 0, 0, 0}, 1e-5 - theta[k]};
        pos.a[k] = -1.0;
        P.cons.push_back(pos);
    }
    P.cons.push_back(Cons{1, {0, 0, 0, 0, 0}, 0.0});
    const int m = (int)P.cons.size();

    double p[5] = {0, 0, 0, 0, 0};
    std::vector<double> s(m), lam(m, 1.0), c(m), J(m * 5);
    for (int i = 0; i < m; ++i) {
        c[i] = cval(P, P.cons[i], p, nullptr, nullptr);
        s[i] = std::fmax(-c[i], 1e-2);
    }
    auto residual = [&](const double* pp, const std::vector<double>& ss, const std::vector<double>& ll,
                        double mu_t, double* rd, std::vector<double>& rp, std::vector<double>& rc) {
        double gr[5];
        for (int k = 0; k < 5; ++k) {
            double a = -P.g[k];
            for (int j = 0; j < 5; ++j) a += P.A[j * 5 + k] * pp[j];
            rd[k] = a;
        }
        for (int i = 0; i < m; ++i) {
            double ci = cval(P, P.cons[i], pp, gr, nullptr);
            for (int k = 0; k < 5; ++k) rd[k] += ll[i] * gr[k];
            rp[i] = ci + ss[i];
            rc[i] = ss[i] * ll[i] - mu_t;
        }
        double nrm = 0;
        for (int k = 0; k < 5; ++k) nrm = std::fmax(nrm, std::fabs(rd[k]));
        for (int i = 0; i < m; ++i) nrm = std::fmax(nrm, std::fmax(std::fabs(rp[i]), std::fabs(rc[i])));
        return nrm;
    };
    std::vector<double> rp(m), rc(m), dl(m), ds(m), ns(m), nl(m), rp2(m), rc2(m);
    double rd[5], rd2[5];
    for (int it = 0; it < 300; ++it) {
        double mu = 0;
        for (int i = 0; i < m; ++i) mu += s[i] * lam[i];
        mu /= m;
        double err = residual(p, s, lam, 0.0, rd, rp, rc);
        if (err < 1e-13 && mu < 1e-14) {
            for (int k = 0; k < 5; ++k) pout[k] = p[k];
            return 0;
        }
        const double target = 0.1 * mu;
        residual(p, s, lam, target, rd, rp, rc);
        // W = A + sum lam_i hess_i ; K = W + J' S^-1 Lam J
        double K[25], gr[5], hs[25];
        for (int e = 0; e < 25; ++e) K[e] = P.A[e];
        double rhs[5];
        for (int k = 0; k < 5; ++k) rhs[k] = -rd[k];
        for (int i = 0; i < m; ++i) {
            cval(P, P.cons[i], p, gr, hs);
            for (int k = 0; k < 5; ++k) J[i * 5 + k] = gr[k];
            const double w = lam[i] / s[i];
            for (int a = 0; a < 5; ++a)
                for (int b = 0; b < 5; ++b) K[b * 5 + a] += lam[i] * hs[b * 5 + a] + w * gr[a] * gr[b];
            // rhs -= J' (S^-1 Lam rp - S^-1 rc)
            const double q = w * rp[i] - rc[i] / s[i];
            for (int k = 0; k < 5; ++k) rhs[k] -= gr[k] * q;
        }
        double dp[5];
        std::memcpy(dp, rhs, sizeof(dp));
        if (!solve5(K, dp)) return 2;
        for (int i = 0; i < m; ++i) {
            double jd = 0;
            for (int k = 0; k < 5; ++k) jd += J[i * 5 + k] * dp[k];
            dl[i] = (lam[i] / s[i]) * (jd + rp[i] - rc[i] / lam[i]);
            ds[i] = -(rc[i] + s[i] * dl[i]) / lam[i];
        }
        double amax_ = 1.0;
        for (int i = 0; i < m; ++i) {
            if (ds[i] < 0) amax_ = std::fmin(amax_, -0.995 * s[i] / ds[i]);
            if (dl[i] < 0) amax_ = std::fmin(amax_, -0.995 * lam[i] / dl[i]);
        }
        double alpha = amax_;
        const double e0 = residual(p, s, lam, target, rd2, rp2, rc2);
        double pn[5];
        for (int bt = 0; bt < 40; ++bt) {
            for (int k = 0; k < 5; ++k) pn[k] = p[k] + alpha * dp[k];
            for (int i = 0; i < m; ++i) {
                ns[i] = s[i] + alpha * ds[i];
                nl[i] = lam[i] + alpha * dl[i];
            }
            double e1 = residual(pn, ns, nl, target, rd2, rp2, rc2);
            if (e1 <= (1.0 - 1e-4 * alpha) * e0 || bt == 39) break;
            alpha *= 0.5;
        }
        std::memcpy(p, pn, sizeof(p));
        s = ns;
        lam = nl;
    }
    // not converged to full tolerance: accept if primal feasible
    bool feas = true;
    for (int i = 0; i < m; ++i)
        if (cval(P, P.cons[i], p, nullptr, nullptr) > 1e-9) feas = false;
    for (int k = 0; k < 5; ++k) pout[k] = p[k];
    return feas ? 0 : 1;
}

}  // namespace

extern "C" int globe_trust_region_step(const double theta[5], const double grad[5], const double ai[25], double delta,
                                       double p[5], int* status) {
    if (!theta || !grad || !ai || !p) return GLOBE_ERR_ARG;
    for (int k = 0; k < 5; ++k)
        if (!std::isfinite(theta[k]) || !std::isfinite(grad[k])) return GLOBE_ERR_ARG;
    for (int e = 0; e < 25; ++e)
        if (!std::isfinite(ai[e])) return GLOBE_ERR_ARG;
    int st = solve_tr(theta, grad, ai, delta, p);
    if (status) *status = st;
    return GLOBE_OK;
}

// ---------------------------------------------------------------------------
// Step of the model without time effects: two components, linear constraints only
//
//   max  g'p - p'Ap/2  s.t.  |p_k| <= 10,  A_00 p_0 + A_11 p_1 <= Delta,
//        theta_k + p_k >= 1e-5                (varCompEst_reducedModel_noTime.cpp:782-830)
//
// In two variables the maximiser is a stationary point of the objective restricted
// to the intersection of at most two active constraints (interior, an edge, or a
// vertex); every such candidate is formed and the best feasible one is kept.

namespace {

int solve_tr2(const double* th, const double* g, const double* A, double delta, double* pout) {
    const double S00 = A[0], S11 = A[3], S01 = 0.5 * (A[1] + A[2]);   // symmetric part
    struct Row {
        double a0, a1, b;   // a . p <= b
    };
    std::vector<Row> rows = {{1, 0, 10}, {-1, 0, 10}, {0, 1, 10}, {0, -1, 10}, {A[0], A[3], delta},
                             {-1, 0, th[0] - 1e-5}, {0, -1, th[1] - 1e-5}};
    auto feasible = [&](double p0, double p1) {
        for (const Row& r : rows) {
            const double lhs = r.a0 * p0 + r.a1 * p1;
            const double tol = 1e-12 * std::fmax(1.0, std::fmax(std::fabs(r.b), std::fabs(r.a0 * p0) + std::fabs(r.a1 * p1)));
            if (lhs > r.b + tol) return false;
        }
        return true;
    };
    auto obj = [&](double p0, double p1) {
        return g[0] * p0 + g[1] * p1 - 0.5 * (S00 * p0 * p0 + 2.0 * S01 * p0 * p1 + S11 * p1 * p1);
    };
    bool found = false;
    double best = -INFINITY, b0 = 0, b1 = 0;
    auto consider = [&](double p0, double p1) {
        if (!std::isfinite(p0) || !std::isfinite(p1) || !feasible(p0, p1)) return;
        const double f = obj(p0, p1);
        if (!found || f > best) {
            found = true;
            best = f;
            b0 = p0;
            b1 = p1;
        }
    };
    // interior: S p = g
    const double det = S00 * S11 - S01 * S01;
    if (det != 0.0) consider((S11 * g[0] - S01 * g[1]) / det, (S00 * g[1] - S01 * g[0]) / det);
    const int m = (int)rows.size();
    for (int i = 0; i < m; ++i) {
        // one active row: stationary point of the objective on the line a.p = b
        // [S a; a' 0] [p; lam] = [g; b]
        const Row& r = rows[i];
        const double M[3][3] = {{S00, S01, r.a0}, {S01, S11, r.a1}, {r.a0, r.a1, 0.0}};
        const double rhs[3] = {g[0], g[1], r.b};
        const double d3 = M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) -
                          M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
                          M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
        if (d3 != 0.0) {
            double x[3];
            for (int c = 0; c < 3; ++c) {   // Cramer's rule
                double T[3][3];
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) T[a][b] = b == c ? rhs[a] : M[a][b];
                x[c] = (T[0][0] * (T[1][1] * T[2][2] - T[1][2] * T[2][1]) -
                        T[0][1] * (T[1][0] * T[2][2] - T[1][2] * T[2][0]) +
                        T[0][2] * (T[1][0] * T[2][1] - T[1][1] * T[2][0])) / d3;
            }
            consider(x[0], x[1]);
        }
        for (int j = i + 1; j < m; ++j) {   // two active rows: their intersection
            const Row& q = rows[j];
            const double d2 = r.a0 * q.a1 - r.a1 * q.a0;
            if (d2 == 0.0) continue;
            consider((r.b * q.a1 - r.a1 * q.b) / d2, (r.a0 * q.b - r.b * q.a0) / d2);
        }
    }
    if (!found) return 1;
    pout[0] = b0;
    pout[1] = b1;
    return 0;
}

}  // namespace

extern "C" int globe_trust_region_step_no_time(const double theta[2], const double grad[2], const double ai[4],
                                               double delta, double p[2], int* status) {
    if (!theta || !grad || !ai || !p) return GLOBE_ERR_ARG;
    for (int k = 0; k < 2; ++k)
        if (!std::isfinite(theta[k]) || !std::isfinite(grad[k])) return GLOBE_ERR_ARG;
    for (int e = 0; e < 4; ++e)
        if (!std::isfinite(ai[e])) return GLOBE_ERR_ARG;
    const int st = solve_tr2(theta, grad, ai, delta, p);
    if (st != 0) p[0] = p[1] = 0.0;
    if (status) *status = st;
    return GLOBE_OK;
}

// ---------------------------------------------------------------------------
// AIREML loop

namespace {

struct Log {
    FILE* f = nullptr;
    void printf(const char* fmt, ...) {
        if (!f) return;
        va_list ap;
        va_start(ap, fmt);
        vfprintf(f, fmt, ap);
        va_end(ap);
        fflush(f);
    }
    void vec(const char* label, const double* v, int n) {
        if (!f) return;
        fprintf(f, "%s", label);
        for (int k = 0; k < n; ++k) fprintf(f, " %.17g", v[k]);
        fprintf(f, "\n");
        fflush(f);
    }
};

double dot5(const double* a, const double* b) {
    double s = 0;
    for (int k = 0; k < 5; ++k) s += a[k] * b[k];
    return s;
}
double quad5(const double* A, const double* p) {
    double s = 0;
    for (int a = 0; a < 5; ++a)
        for (int b = 0; b < 5; ++b) s += p[a] * A[b * 5 + a] * p[b];
    return s;
}
double norm5(const double* a) { return std::sqrt(dot5(a, a)); }

bool inv5(const double* A, double* out) {
    double M[25];
    std::memcpy(M, A, sizeof(M));
    for (int c = 0; c < 5; ++c) {
        double col[5] = {0, 0, 0, 0, 0};
        col[c] = 1.0;
        double W[25];
        std::memcpy(W, M, sizeof(W));
        if (!solve5(W, col)) return false;
        for (int r = 0; r < 5; ++r) out[c * 5 + r] = col[r];
    }
    return true;
}

uint64_t smix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct Driver {
    globe_ctx* ctx;
    const globe_aireml_opts* o;
    Log log;
    globe_pcg_opts pcg;
    int64_t probe_pos = 0;
    int64_t evals = 0;
    int64_t rhs_iters = 0;
    std::string err;

    int eval_grad(const double* th, double* grad) {
        Nvtx nvtx("AIREML gradient evaluation");
        int rc = globe_set_vc(ctx, th);
        if (rc) return rc;
        globe_pcg_info info{};
        globe_pcg_opts m = pcg;
        m.rule = GLOBE_RULE_AIREML;
        m.x0mode = GLOBE_X0_PRECOND;  // fitMME: use_initial_guess (varCompEst.cpp:642)
        const double* pr = nullptr;
        if (o->probes) {
            int64_t per = probes_per_eval();
            if (probe_pos + per > o->probes_len) {
                err = "injected probe draws exhausted";
                return GLOBE_ERR_ARG;
            }
            pr = o->probes + probe_pos;
            probe_pos += per;
        }
        double first[5], trace[5];
        const uint64_t seed = o->seed + 0x1000003ull * (uint64_t)evals;
        log.printf("Solving MME... ");
        if (o->fuse) {
            // one block solve of [X y | probes]
            rc = globe_aireml_eval(ctx, pr, o->numMC, seed, &m, first, trace, grad, &info);
            if (rc) return rc;
            rhs_iters += info.rhs_iters;
            log.printf("Converged at iteration %d\nMME solved successfully.\nComputing derivatives.\n", info.iters);
        } else {
            rc = globe_mme(ctx, &m, nullptr, nullptr, nullptr, nullptr, &info);
            if (rc) return rc;
            rhs_iters += info.rhs_iters;
            log.printf("Converged at iteration %d\nMME solved successfully.\nComputing derivatives.\n", info.iters);
            rc = globe_aireml_grad(ctx, pr, o->numMC, seed, &m, nullptr, first, trace, grad, &info);
            if (rc) return rc;
            rhs_iters += info.rhs_iters;
        }
        ++evals;
        log.printf("Estimating trace terms... Converged at iteration %d\n", info.iters);
        log.vec("Gradient:", grad, 5);
        return GLOBE_OK;
    }
    int64_t n_rec = 0, n_ind = 0;
    int nc = 5;   // components of the model (2 without time effects)
    int64_t probes_per_eval() const { return (int64_t)o->numMC * ((nc == 5 ? 3 : 1) * n_ind + n_rec); }

    int eval_ai(double* ai) {
        globe_pcg_info info{};
        log.printf("Computing Vinv_f_theta (for Pf_theta -> AI matrix)... ");
        int rc = globe_aireml_ai(ctx, &pcg, ai, &info);
        if (rc) return rc;
        rhs_iters += info.rhs_iters;
        log.printf("Converged at iteration %d\nAI matrix: \n", info.iters);
        for (int r = 0; r < 5; ++r) {
            for (int c = 0; c < 5; ++c) log.printf(" %.17g", ai[c * 5 + r]);
            log.printf("\n");
        }
        return GLOBE_OK;
    }
};

}  // namespace

static int aireml_run_impl(globe_ctx* ctx, const globe_aireml_opts* o, const char* log_path,
                           globe_aireml_result* res) {
    if (o->numMC < 1 || o->maxiter < 0) return GLOBE_ERR_ARG;
    Driver d;
    d.ctx = ctx;
    d.o = o;
    int32_t Ni = 0;
    if (globe_get_dims(ctx, &d.n_rec, &Ni, nullptr, nullptr) != GLOBE_OK || Ni < 1) return GLOBE_ERR_STATE;
    d.n_ind = Ni;
    d.pcg.tol = o->pcg_tol > 0 ? o->pcg_tol : 1e-5;
    d.pcg.maxit = o->pcg_maxit > 0 ? o->pcg_maxit : 1000;
    d.pcg.rule = GLOBE_RULE_AIREML;
    d.pcg.x0mode = GLOBE_X0_PRECOND;
    d.pcg.mask = o->mask;
    d.pcg.precision = o->precision;
    if (log_path) {
        d.log.f = std::fopen(log_path, "w");
        if (!d.log.f) return GLOBE_ERR_IO;
    }
    std::memset(res, 0, sizeof(*res));
    // model: runAIREML (5 components) or runAIREML_reducedModel (sig2e, sig2g; no time effects)
    const int nc = globe_get_model(ctx) == GLOBE_MODEL_NO_TIME ? 2 : 5;
    d.nc = nc;
    double theta[5], grad[5], ai[25];
    std::memcpy(theta, o->theta0, sizeof(theta));
    for (int k = nc; k < 5; ++k) theta[k] = 0.0;
    if (nc == 5)
        d.log.printf("Running AI-REML...\nInitial variance components: \n  sig2e = %.17g, \n  sig2g = %.17g, \n"
                     "  sig2b0 = %.17g, \n  sigb01 = %.17g, \n  sig2b1 = %.17g\n",
                     theta[0], theta[1], theta[2], theta[3], theta[4]);
    else
        d.log.printf("Running AI-REML...\nInitial variance components: \n  sig2e = %.17g, \n  sig2g = %.17g\n",
                     theta[0], theta[1]);
    double Delta = 1e20;
    bool dangerous = false, converged = false;
    int num_rej = 0;
    const bool grad_check = true;
    double gnt = 0.0;
    uint64_t restart_state = o->seed ^ 0xA5A5A5A5ull;
    int rc = GLOBE_OK;
    int i;
#define TRY(x)                      \
    do {                            \
        rc = (x);                   \
        if (rc != GLOBE_OK) goto out; \
    } while (0)
    for (i = 0; i < o->maxiter; ++i) {
        Nvtx nvtx_iter("AIREML iteration");
        d.log.printf("\n=================================\n---------- Iteration %d ----------\n"
                     "=================================\n", i + 1);
        if (i == 0) {
            TRY(d.eval_grad(theta, grad));
            TRY(d.eval_ai(ai));
        }
        if (i == 1) {
            gnt = 0.1 * norm5(grad);
            d.log.printf("Gradient norm threshold: %.17g\n", gnt);
        }
        if (num_rej > 5) {
            // varCompEst.cpp:1431-1451 draws the restart with rand(); here a
            // seeded stream (same distribution, U[0.1, 0.9])
            d.log.printf("Too many rejections at current point. Re-initalizing optimization.\n");
            for (int k = 0; k < nc; ++k) {
                restart_state = smix(restart_state);
                theta[k] = 0.1 + 0.8 * ((double)(restart_state >> 11) * (1.0 / 9007199254740992.0));
            }
            if (nc == 5 && theta[3] > std::sqrt(theta[2] * theta[4]))
                theta[3] = std::sqrt(theta[2] * theta[4]) - 1e-3;
            d.log.vec("Re-initialized variance components:", theta, nc);
            TRY(d.eval_grad(theta, grad));
            TRY(d.eval_ai(ai));
            num_rej = 0;
        }
        double theta_old[5];
        std::memcpy(theta_old, theta, sizeof(theta));
        {
            // ---- oneIter_AIREML (varCompEst.cpp:1148-1344) ----
            double p[5] = {0, 0, 0, 0, 0};
            int st = 0;
            if (nc == 5) {
                rc = globe_trust_region_step(theta, grad, ai, Delta, p, &st);
            } else {
                const double ai2[4] = {ai[0], ai[1], ai[5], ai[6]};
                rc = globe_trust_region_step_no_time(theta, grad, ai2, Delta, p, &st);
            }
            if (rc != GLOBE_OK) {
                d.err = "trust-region step: the gradient or the AI matrix is not finite";
                goto out;
            }
            if (st != 0) {
                d.log.printf("Step solver failed (status %d). Reducing trust region radius.\n", st);
                Delta *= 0.75;
                dangerous = true;
                num_rej += 1;
            } else {
                const double pred = dot5(grad, p) - 0.5 * quad5(ai, p);
                d.log.printf("Predicted change in log-likelihood: %.17g\n", pred);
                d.log.vec("Predicted step:", p, nc);
                double scale = 1.0;
                bool accepted = false, conv_here = false;
                int red = 0;
                while (!accepted && red <= 10) {
                    double sp[5], tn[5];
                    for (int k = 0; k < 5; ++k) {
                        sp[k] = scale * p[k];
                        tn[k] = theta[k] + sp[k];
                    }
                    d.log.printf("Trying step with scale %.17g\n", scale);
                    d.log.vec("theta_new:", tn, nc);
                    bool violated = false;
                    for (int k = 0; k < nc; ++k) {
                        if (k != 3 && tn[k] < 1e-6) { tn[k] = 1e-6; violated = true; }
                        if (tn[k] > 10.0) { tn[k] = 10.0; violated = true; }
                    }
                    if (nc == 5 && tn[3] > std::sqrt(tn[2] * tn[4])) {
                        tn[3] = std::sqrt(tn[2] * tn[4]) - 1e-6;
                        violated = true;
                    }
                    if (violated) {
                        d.log.printf("Constraints violated at scale %.17g. Reducing step size.\n", scale);
                        scale *= 0.5;
                        red += 1;
                        continue;
                    }
                    d.log.printf("Computing gradient at theta_new...\n");
                    double gnew[5];
                    TRY(d.eval_grad(tn, gnew));
                    double gm[5];
                    for (int k = 0; k < 5; ++k) gm[k] = 0.5 * (grad[k] + gnew[k]);
                    const double dll = dot5(sp, gm);
                    const double preds = dot5(grad, sp) - 0.5 * quad5(ai, sp);
                    d.log.printf("Predicted change in log-likelihood (scaled): %.17g\n", preds);
                    d.log.printf("(Approximate) Actual change in log-likelihood: %.17g\n", dll);
                    if (scale == 1.0 && preds < 1e-2) {
                        d.log.printf("Converged: predicted log-likelihood improvement below threshold.\n");
                        dangerous = false;
                        conv_here = true;
                        break;
                    }
                    double rho;
                    if (grad_check && norm5(grad) > gnt && norm5(gnew) > 2.0 * norm5(grad)) {
                        d.log.printf("Dangerous model deviation detected at scale %.17g. Reducing step size.\n", scale);
                        scale *= 0.5;
                        red += 1;
                        continue;
                    }
                    rho = dll / preds;
                    d.log.printf("Rho: %.17g\n", rho);
                    double npd = 0;
                    for (int k = 0; k < 5; ++k) npd += std::fabs(ai[k * 5 + k] * sp[k]);
                    if (rho < 0.25) Delta = 0.25 * npd;
                    else if (rho > 0.99) Delta = std::fmax(Delta, 3.5 * npd);
                    if (rho > 0.25) {
                        std::memcpy(theta, tn, sizeof(theta));
                        std::memcpy(grad, gnew, sizeof(grad));
                        TRY(d.eval_ai(ai));
                        num_rej = 0;
                        accepted = true;
                    } else {
                        d.log.printf("Step rejected at scale %.17g, rho = %.17g. Reducing step size.\n", scale, rho);
                        scale *= 0.5;
                        red += 1;
                    }
                }
                if (!accepted && !conv_here) {
                    d.log.printf("Failed to accept a step after %d reductions.\n", red);
                    Delta *= 0.75;
                    dangerous = true;
                    num_rej += 1;
                }
            }
        }
        if (nc == 5)
            d.log.printf("Estimated variance components:  sig2e = %.17g, sig2g = %.17g, sig2b0 = %.17g, "
                         "sigb01 = %.17g, sig2b1 = %.17g\n", theta[0], theta[1], theta[2], theta[3], theta[4]);
        else
            d.log.printf("Estimated variance components:  sig2e = %.17g, sig2g = %.17g\n", theta[0], theta[1]);
        {
            double dif[5];
            for (int k = 0; k < 5; ++k) dif[k] = theta[k] - theta_old[k];
            const double delta = norm5(dif) / norm5(theta_old);
            if (delta < o->tol && !dangerous) {
                d.log.printf("Convergence reached after %d iterations.\n", i + 1);
                converged = true;
                ++i;
                break;
            }
            dangerous = false;
            d.log.printf("Convergence check: %.17g\nTrust region radius: %.17g\n", delta, Delta);
            if (Delta < 1e-4) {
                d.log.printf("Trust region radius too small. Terminating optimization.\n");
                ++i;
                break;
            }
        }
    }
    {
        double inv[25], aii[25];
        std::memcpy(aii, ai, sizeof(aii));
        for (int k = nc; k < 5; ++k) aii[k * 5 + k] = 1.0;   // block-diagonal: the model's block inverts alone
        bool ok = inv5(aii, inv);
        const char* nm[5] = {"   sig2e", "   sig2g", "  sig2b0", "  sigb01", "  sig2b1"};
        d.log.printf("Final variance components \xc2\xb1 SEs:\n");
        for (int k = 0; k < nc; ++k) {
            res->se[k] = ok ? std::sqrt(inv[k * 5 + k]) : NAN;
            d.log.printf("%s = %.17g \xc2\xb1 %.17g\n", nm[k], theta[k], res->se[k]);
        }
    }
    res->iterations = i;
    res->converged = converged ? 1 : 0;
    std::memcpy(res->theta, theta, sizeof(theta));
    std::memcpy(res->ai, ai, sizeof(ai));
    std::memcpy(res->grad, grad, sizeof(grad));
    res->grad_evals = d.evals;
    res->pcg_rhs_iters = d.rhs_iters;
out:
#undef TRY
    if (rc != GLOBE_OK && !d.err.empty()) globe::set_err(ctx, rc, "%s", d.err.c_str());
    if (rc != GLOBE_OK && d.log.f) d.log.printf("[error] %s\n", globe_last_error(ctx));
    if (d.log.f) std::fclose(d.log.f);
    // restore the context's components to the final estimate
    if (rc == GLOBE_OK) globe_set_vc(ctx, theta);
    return rc;
}

extern "C" int globe_aireml_run(globe_ctx* ctx, const globe_aireml_opts* o, const char* log_path,
                                globe_aireml_result* res) {
    if (!ctx || !o || !res) return GLOBE_ERR_ARG;
    if (o->digits == 0) return aireml_run_impl(ctx, o, log_path, res);
    // digits for this run only
    const int keep = globe_get_digits(ctx);
    int rc = globe_set_digits(ctx, o->digits);
    if (rc != GLOBE_OK) return rc;
    rc = aireml_run_impl(ctx, o, log_path, res);
    globe_set_digits(ctx, keep);
    return rc;
}
