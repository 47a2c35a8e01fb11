/*
 * globe_oracle.c -- CPU restatement of GLOBE's LGMM solve path.
 *
 * TEST INFRASTRUCTURE ONLY (see globe_oracle.h).  Written from the behaviour
 * of the reference (src/PCGsolver.cpp, src/varCompEst.cpp); every function
 * names the lines it restates.  Double precision unless stated.
 */
#include "globe_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* PLINK 2-bit decode and per-SNP statistics                            */
/* ------------------------------------------------------------------ */

/* PCGsolver.cpp:83-94 -- 00 -> 2, 10 -> 1, 11 -> 0, 01 -> missing (-1) */
static inline int decode_code(unsigned c) {
    switch (c & 3u) {
        case 0u: return 2;
        case 2u: return 1;
        case 3u: return 0;
        default: return -1;
    }
}

int64_t orc_bed_stats(const uint8_t* bed, int64_t M, int32_t N, float min_maf, float max_miss,
                      int64_t* alt, int64_t* miss, float* maf, float* miss_rate, uint8_t* keep) {
    const int64_t bps = ((int64_t)N + 3) / 4;
    const int rem = N % 4;
    const int phantom = rem == 0 ? 0 : 4 - rem;           /* PCGsolver.cpp:699-700 */
    int64_t kept = 0;
    for (int64_t s = 0; s < M; ++s) {
        const uint8_t* row = bed + s * bps;
        int64_t a = 0, ms = 0;
        for (int64_t b = 0; b < bps; ++b) {                  /* LUT counts :715-721 */
            unsigned x = row[b];
            for (int j = 0; j < 4; ++j) {
                unsigned c = (x >> (2 * j)) & 3u;
                if (c == 0u) a += 2;
                else if (c == 2u) a += 1;
                else if (c == 1u) ms += 1;
            }
        }
        if (phantom > 0) {                                   /* :589-613 */
            unsigned last = row[bps - 1];
            for (int q = 0; q < phantom; ++q) {
                int pair_idx = 3 - q;
                unsigned c = (last >> (2 * pair_idx)) & 3u;
                if (c == 0u) a -= 2;
                else if (c == 2u) a -= 1;
                else if (c == 1u) ms -= 1;
            }
        }
        int n_obs = N - (int)ms;                             /* :726-728, float arithmetic */
        float f = (n_obs > 0) ? (float)a / (2.0f * (float)n_obs) : 0.0f;
        float mr = (float)ms / (float)N;
        int k = (f >= min_maf && f <= (1.0f - min_maf) && mr <= max_miss);  /* :731-732 */
        if (alt) alt[s] = a;
        if (miss) miss[s] = ms;
        if (maf) maf[s] = f;
        if (miss_rate) miss_rate[s] = mr;
        if (keep) keep[s] = (uint8_t)k;
        kept += k;
    }
    return kept;
}

void orc_std_params(const int64_t* alt, const int64_t* miss, int64_t M, int32_t N, double* f,
                    double* inv_std) {
    for (int64_t s = 0; s < M; ++s) {
        int n_obs = N - (int)miss[s];
        double fs = (n_obs > 0) ? (double)alt[s] / (double)(2.0f * (float)n_obs) : 0.0;
        double den = 2.0 * fs * (1.0 - fs);                 /* :837-839 in double */
        f[s] = fs;
        inv_std[s] = (den > (double)1e-12f) ? 1.0 / sqrt(den) : 1.0;
    }
}

/* ------------------------------------------------------------------ */
/* Solver state                                                          */
/* ------------------------------------------------------------------ */

struct orc_solver {
    orc_model m;
    int32_t nblk;
    int64_t* bstart;   /* [nblk+1] contiguous runs of one individual */
    int32_t* bind;     /* [nblk] individual of each run */
    int64_t* qoff;     /* [nblk+1] offsets of the dense block inverses */
    double* qinv;
    double* gdiag;     /* [N] A_ii */
    int have_gdiag;
    /* MME state (varCompEst.cpp:33-45) */
    double* vinv_X;    /* [Nrec x (p+1)] */
    double* xtvx_inv;  /* [(p+1)^2] */
    double* vinv_r;    /* [Nrec] */
    double* uhat;      /* [N] */
};

static double zs_of(const orc_model* m, int64_t s, int32_t i) {
    /* getStdGenotype PCGsolver.cpp:826-842 (double build) */
    unsigned c = (m->geno[s * m->stride + i / 4] >> (2 * (i % 4))) & 3u;
    int g = decode_code(c);
    if (g < 0) g = 0;
    return ((double)g - 2.0 * m->f[s]) * m->inv_std[s];
}

void orc_grm_build(const uint8_t* geno, int64_t Mk, int64_t stride, int32_t N, const double* f,
                   const double* inv_std, float* lt) {
    /* individual-major zs, so that each A_ij is one contiguous dot product */
    double* Z = (double*)malloc(sizeof(double) * (size_t)N * (size_t)(Mk > 0 ? Mk : 1));
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < N; ++i)
        for (int64_t s = 0; s < Mk; ++s) {
            unsigned c = (geno[s * stride + i / 4] >> (2 * (i % 4))) & 3u;
            int g = decode_code(c);
            if (g < 0) g = 0;
            Z[(size_t)i * Mk + s] = ((double)g - 2.0 * f[s]) * inv_std[s];
        }
#pragma omp parallel for schedule(dynamic, 8)
    for (int32_t i = 0; i < N; ++i) {
        const double* zi = Z + (size_t)i * Mk;
        for (int32_t j = 0; j <= i; ++j) {
            const double* zj = Z + (size_t)j * Mk;
            double acc = 0.0;
            for (int64_t s = 0; s < Mk; ++s) acc += zi[s] * zj[s];
            lt[(size_t)i * (i + 1) / 2 + j] = (float)(acc / (double)Mk);
        }
    }
    free(Z);
}

orc_solver* orc_create(const orc_model* m) {
    orc_solver* s = (orc_solver*)calloc(1, sizeof(orc_solver));
    s->m = *m;
    /* block boundaries: PCGsolver.cpp:1002-1009 */
    int64_t nb = 1;
    for (int64_t r = 1; r < m->Nrec; ++r) nb += (m->indiv[r] != m->indiv[r - 1]);
    s->nblk = (int32_t)nb;
    s->bstart = (int64_t*)malloc(sizeof(int64_t) * (nb + 1));
    s->bind = (int32_t*)malloc(sizeof(int32_t) * nb);
    s->qoff = (int64_t*)malloc(sizeof(int64_t) * (nb + 1));
    int64_t b = 0;
    s->bstart[0] = 0;
    s->bind[0] = m->indiv[0];
    for (int64_t r = 1; r < m->Nrec; ++r)
        if (m->indiv[r] != m->indiv[r - 1]) {
            ++b;
            s->bstart[b] = r;
            s->bind[b] = m->indiv[r];
        }
    s->bstart[nb] = m->Nrec;
    s->qoff[0] = 0;
    for (b = 0; b < nb; ++b) {
        int64_t n = s->bstart[b + 1] - s->bstart[b];
        s->qoff[b + 1] = s->qoff[b] + n * n;
    }
    s->qinv = (double*)malloc(sizeof(double) * s->qoff[nb]);
    s->gdiag = (double*)malloc(sizeof(double) * m->N);
    int pp = m->p + 1;
    s->vinv_X = (double*)calloc((size_t)m->Nrec * pp, sizeof(double));
    s->xtvx_inv = (double*)calloc((size_t)pp * pp, sizeof(double));
    s->vinv_r = (double*)calloc((size_t)m->Nrec, sizeof(double));
    s->uhat = (double*)calloc((size_t)m->N, sizeof(double));
    return s;
}

void orc_destroy(orc_solver* s) {
    if (!s) return;
    free(s->bstart); free(s->bind); free(s->qoff); free(s->qinv); free(s->gdiag);
    free(s->vinv_X); free(s->xtvx_inv); free(s->vinv_r); free(s->uhat);
    free(s);
}

void orc_set_vc(orc_solver* s, const double vc[5]) { memcpy(s->m.vc, vc, sizeof(double) * 5); }

/* ------------------------------------------------------------------ */
/* GRM products                                                          */
/* ------------------------------------------------------------------ */

void orc_grm_apply(orc_solver* s, const double* Z, int k, double* out) {
    const orc_model* m = &s->m;
    const int32_t N = m->N;
    const double s2g = m->vc[1];
    memset(out, 0, sizeof(double) * (size_t)N * k);
    if (m->geno) {
        /* PCGsolver.cpp:1130-1201: w = Zs Z (pass 1), GZ = s2g/M Zs' w (pass 2) */
        const int64_t Mk = m->Mk;
        if (Mk == 0) return;
        double* W = (double*)calloc((size_t)Mk * k, sizeof(double));
        /* columns in groups of 256 (the accumulator); each column's sum runs in i order */
        for (int c0 = 0; c0 < k; c0 += 256) {
            const int kc = k - c0 < 256 ? k - c0 : 256;
#pragma omp parallel for schedule(dynamic, 64)
            for (int64_t sn = 0; sn < Mk; ++sn) {
                double acc[256];
                for (int c = 0; c < kc; ++c) acc[c] = 0.0;
                for (int32_t i = 0; i < N; ++i) {
                    double z = zs_of(m, sn, i);
                    for (int c = 0; c < kc; ++c) acc[c] += z * Z[(size_t)(c0 + c) * N + i];
                }
                for (int c = 0; c < kc; ++c) W[(size_t)(c0 + c) * Mk + sn] = acc[c];
            }
        }
        const double scale = s2g * (1.0 / (double)Mk);
#pragma omp parallel
        {
            double* loc = (double*)calloc((size_t)N * k, sizeof(double));
#pragma omp for schedule(static)
            for (int64_t sn = 0; sn < Mk; ++sn) {
                for (int32_t i = 0; i < N; ++i) {
                    double z = zs_of(m, sn, i);
                    for (int c = 0; c < k; ++c) loc[(size_t)c * N + i] += z * W[(size_t)c * Mk + sn];
                }
            }
#pragma omp critical
            for (size_t e = 0; e < (size_t)N * k; ++e) out[e] += scale * loc[e];
            free(loc);
        }
        free(W);
    } else {
        /* PCGsolver.cpp:1202-1213 (full square through the packed triangle) */
#pragma omp parallel for schedule(dynamic, 16)
        for (int32_t i = 0; i < N; ++i) {
            for (int32_t j = 0; j < N; ++j) {
                size_t ii = i > j ? (size_t)i : (size_t)j, jj = i > j ? (size_t)j : (size_t)i;
                double gij = (double)m->grm_lt[ii * (ii + 1) / 2 + jj];
                for (int c = 0; c < k; ++c) out[(size_t)c * N + i] += s2g * gij * Z[(size_t)c * N + j];
            }
        }
    }
}

void orc_genetic_diag(orc_solver* s, double* d) {
    const orc_model* m = &s->m;
    if (m->geno) {
        /* PCGsolver.cpp:951-988 */
        memset(d, 0, sizeof(double) * m->N);
        if (m->Mk == 0) return;
        for (int64_t sn = 0; sn < m->Mk; ++sn)
            for (int32_t i = 0; i < m->N; ++i) {
                double z = zs_of(m, sn, i);
                d[i] += z * z;
            }
        double inv = 1.0 / (double)m->Mk;
        for (int32_t i = 0; i < m->N; ++i) d[i] *= inv;
    } else {
        for (int32_t i = 0; i < m->N; ++i) d[i] = (double)m->grm_lt[(size_t)i * (i + 1) / 2 + i];
    }
}

/* ------------------------------------------------------------------ */
/* V x                                                                   */
/* ------------------------------------------------------------------ */

static double tval(const double* vc, double ti, double tj) {
    return vc[2] + vc[3] * (ti + tj) + vc[4] * (ti * tj);
}

void orc_vx(orc_solver* s, const double* x, int k, double* out) {
    const orc_model* m = &s->m;
    const int64_t Nrec = m->Nrec;
    const int32_t N = m->N;
    const double* t = m->X + (size_t)m->p * Nrec;
    double* Z = (double*)calloc((size_t)N * k, sizeof(double));
    double* GZ = (double*)malloc(sizeof(double) * (size_t)N * k);
    for (int64_t r = 0; r < Nrec; ++r)                     /* J' x  :1118-1125 */
        for (int c = 0; c < k; ++c) Z[(size_t)c * N + m->indiv[r]] += x[(size_t)c * Nrec + r];
    orc_grm_apply(s, Z, k, GZ);
    for (int64_t r = 0; r < Nrec; ++r)                     /* J GZ :1219-1225 */
        for (int c = 0; c < k; ++c) out[(size_t)c * Nrec + r] = GZ[(size_t)c * N + m->indiv[r]];
#pragma omp parallel for schedule(dynamic, 64)
    for (int32_t b = 0; b < s->nblk; ++b) {                /* time block :1237-1254 */
        int64_t st = s->bstart[b], n = s->bstart[b + 1] - st;
        for (int64_t i = 0; i < n; ++i)
            for (int64_t j = 0; j < n; ++j) {
                double v = tval(m->vc, t[st + i], t[st + j]);
                for (int c = 0; c < k; ++c) out[(size_t)c * Nrec + st + i] += v * x[(size_t)c * Nrec + st + j];
            }
    }
    for (int c = 0; c < k; ++c)                             /* residual :1259-1265 */
        for (int64_t r = 0; r < Nrec; ++r) out[(size_t)c * Nrec + r] += m->vc[0] * x[(size_t)c * Nrec + r];
    free(Z);
    free(GZ);
}

/* ------------------------------------------------------------------ */
/* Preconditioner                                                        */
/* ------------------------------------------------------------------ */

/* Gauss-Jordan inverse with partial pivoting, in place (n x n, col-major). */
static int gj_inverse(double* A, int n) {
    int* piv = (int*)malloc(sizeof(int) * n);
    double* I = (double*)calloc((size_t)n * n, sizeof(double));
    for (int i = 0; i < n; ++i) I[(size_t)i * n + i] = 1.0;
    int ok = 1;
    for (int c = 0; c < n; ++c) {
        int pr = c;
        double best = fabs(A[(size_t)c * n + c]);
        for (int r = c + 1; r < n; ++r)
            if (fabs(A[(size_t)c * n + r]) > best) { best = fabs(A[(size_t)c * n + r]); pr = r; }
        if (best == 0.0) { ok = 0; break; }
        if (pr != c)
            for (int j = 0; j < n; ++j) {
                double t1 = A[(size_t)j * n + c]; A[(size_t)j * n + c] = A[(size_t)j * n + pr]; A[(size_t)j * n + pr] = t1;
                double t2 = I[(size_t)j * n + c]; I[(size_t)j * n + c] = I[(size_t)j * n + pr]; I[(size_t)j * n + pr] = t2;
            }
        double d = A[(size_t)c * n + c];
        for (int j = 0; j < n; ++j) { A[(size_t)j * n + c] /= d; I[(size_t)j * n + c] /= d; }
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            double f = A[(size_t)c * n + r];
            if (f == 0.0) continue;
            for (int j = 0; j < n; ++j) {
                A[(size_t)j * n + r] -= f * A[(size_t)j * n + c];
                I[(size_t)j * n + r] -= f * I[(size_t)j * n + c];
            }
        }
    }
    memcpy(A, I, sizeof(double) * (size_t)n * n);
    free(I);
    free(piv);
    return ok;
}

void orc_precond_build(orc_solver* s) {
    const orc_model* m = &s->m;
    const double* t = m->X + (size_t)m->p * m->Nrec;
    if (!s->have_gdiag) { orc_genetic_diag(s, s->gdiag); s->have_gdiag = 1; }
    /* PCGsolver.cpp:1014-1049; varCompEst.cpp:384-410 (same block) */
#pragma omp parallel for schedule(dynamic, 64)
    for (int32_t b = 0; b < s->nblk; ++b) {
        int64_t st = s->bstart[b];
        int n = (int)(s->bstart[b + 1] - st);
        double* Q = s->qinv + s->qoff[b];
        double gval = m->vc[1] * s->gdiag[s->bind[b]];
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j)
                Q[(size_t)j * n + i] = gval + tval(m->vc, t[st + i], t[st + j]) + (i == j ? m->vc[0] : 0.0);
        gj_inverse(Q, n);
    }
}

void orc_precond_apply(orc_solver* s, const double* r, int k, double* z) {
    const int64_t Nrec = s->m.Nrec;
#pragma omp parallel for schedule(dynamic, 64)
    for (int32_t b = 0; b < s->nblk; ++b) {
        int64_t st = s->bstart[b];
        int n = (int)(s->bstart[b + 1] - st);
        const double* Q = s->qinv + s->qoff[b];
        for (int c = 0; c < k; ++c)
            for (int i = 0; i < n; ++i) {
                double acc = 0.0;
                for (int j = 0; j < n; ++j) acc += Q[(size_t)j * n + i] * r[(size_t)c * Nrec + st + j];
                z[(size_t)c * Nrec + st + i] = acc;
            }
    }
}

/* ------------------------------------------------------------------ */
/* Block PCG                                                             */
/* ------------------------------------------------------------------ */

static double col_dot(const double* a, const double* b, int64_t n) {
    double acc = 0.0;
    for (int64_t i = 0; i < n; ++i) acc += a[i] * b[i];
    return acc;
}

int orc_pcg(orc_solver* s, const double* B, double* X, int k, double tol, int maxit, int rule,
            int x0mode) {
    const int64_t n = s->m.Nrec;
    const size_t tot = (size_t)n * k;
    double* r = (double*)malloc(sizeof(double) * tot);
    double* z = (double*)malloc(sizeof(double) * tot);
    double* p = (double*)malloc(sizeof(double) * tot);
    double* Vp = (double*)malloc(sizeof(double) * tot);
    double* rs = (double*)malloc(sizeof(double) * k);
    double* nb = (double*)malloc(sizeof(double) * k);
    if (x0mode == 0) {
        memset(X, 0, sizeof(double) * tot);
        memcpy(r, B, sizeof(double) * tot);
    } else {
        if (x0mode == 1) orc_precond_apply(s, B, k, X);    /* varCompEst.cpp:466-473 */
        orc_vx(s, X, k, Vp);
        for (size_t e = 0; e < tot; ++e) r[e] = B[e] - Vp[e];
    }
    for (int c = 0; c < k; ++c) nb[c] = sqrt(col_dot(B + (size_t)c * n, B + (size_t)c * n, n));
    orc_precond_apply(s, r, k, z);
    memcpy(p, z, sizeof(double) * tot);
    for (int c = 0; c < k; ++c) rs[c] = col_dot(r + (size_t)c * n, z + (size_t)c * n, n);
    /* stagnation state, PCGsolver.cpp:1359-1375 */
    double last = 0.0;
    for (int c = 0; c < k; ++c)
        if (nb[c] > (double)1e-12f) {
            double ratio = sqrt(col_dot(r + (size_t)c * n, r + (size_t)c * n, n)) / nb[c];
            if (ratio > last) last = ratio;
        }
    const double stag_frac = (double)5e-3f;
    int stag = 0, it;
    for (it = 0; it < maxit; ++it) {
        orc_vx(s, p, k, Vp);
        for (int c = 0; c < k; ++c) {
            double* pc = p + (size_t)c * n;
            double* vc = Vp + (size_t)c * n;
            double alpha = rs[c] / col_dot(pc, vc, n);
            double* xc = X + (size_t)c * n;
            double* rc = r + (size_t)c * n;
            for (int64_t i = 0; i < n; ++i) { xc[i] += alpha * pc[i]; rc[i] -= alpha * vc[i]; }
        }
        if (rule == 0) {
            double mx = 0.0;
            for (int c = 0; c < k; ++c) {
                double nr = sqrt(col_dot(r + (size_t)c * n, r + (size_t)c * n, n));
                double ratio = nb[c] > (double)1e-12f ? nr / nb[c] : 0.0;
                if (ratio > mx) mx = ratio;
            }
            if (mx < tol) { ++it; break; }
            double impr = last - mx;
            if (impr < stag_frac * last) ++stag; else stag = 0;
            last = mx;
            if (stag >= 10) { ++it; break; }
        } else {
            int all = 1;
            for (int c = 0; c < k; ++c) {
                double nr = sqrt(col_dot(r + (size_t)c * n, r + (size_t)c * n, n));
                if (!(nr < tol * nb[c])) { all = 0; break; }
            }
            if (all) { ++it; break; }
        }
        orc_precond_apply(s, r, k, z);
        for (int c = 0; c < k; ++c) {
            double rn = col_dot(r + (size_t)c * n, z + (size_t)c * n, n);
            double beta = rn / rs[c];
            rs[c] = rn;
            double* pc = p + (size_t)c * n;
            const double* zc = z + (size_t)c * n;
            for (int64_t i = 0; i < n; ++i) pc[i] = zc[i] + beta * pc[i];
        }
    }
    free(r); free(z); free(p); free(Vp); free(rs); free(nb);
    return it;
}

/* ------------------------------------------------------------------ */
/* MME                                                                   */
/* ------------------------------------------------------------------ */

static void jt_vec(const orc_model* m, const double* v, double* w) {
    memset(w, 0, sizeof(double) * m->N);
    for (int64_t r = 0; r < m->Nrec; ++r) w[m->indiv[r]] += v[r];
}

int orc_mme(orc_solver* s, double tol, int maxit, int rule, int x0mode, double* beta, double* uhat,
            double* bhat, double* vinv_r) {
    const orc_model* m = &s->m;
    const int64_t n = m->Nrec;
    const int pp = m->p + 1, k = m->p + 2;
    const double* vc = m->vc;
    const double* t = m->X + (size_t)m->p * n;
    orc_precond_build(s);
    double* B = (double*)malloc(sizeof(double) * (size_t)n * k);
    double* S = (double*)malloc(sizeof(double) * (size_t)n * k);
    memcpy(B, m->X, sizeof(double) * (size_t)n * pp);
    memcpy(B + (size_t)n * pp, m->y, sizeof(double) * n);
    int it = orc_pcg(s, B, S, k, tol, maxit, rule, x0mode);
    memcpy(s->vinv_X, S, sizeof(double) * (size_t)n * pp);
    const double* vinv_y = S + (size_t)n * pp;
    double* A = s->xtvx_inv;
    for (int a = 0; a < pp; ++a)                            /* X' V^-1 X  PCGsolver.cpp:279 */
        for (int b = 0; b < pp; ++b) A[(size_t)b * pp + a] = col_dot(m->X + (size_t)a * n, S + (size_t)b * n, n);
    gj_inverse(A, pp);
    double* xty = (double*)malloc(sizeof(double) * pp);
    for (int a = 0; a < pp; ++a) xty[a] = col_dot(m->X + (size_t)a * n, vinv_y, n);
    for (int a = 0; a < pp; ++a) {
        double acc = 0.0;
        for (int b = 0; b < pp; ++b) acc += A[(size_t)b * pp + a] * xty[b];
        beta[a] = acc;
    }
    for (int64_t r = 0; r < n; ++r) {                       /* V^-1 r  :284 */
        double acc = vinv_y[r];
        for (int a = 0; a < pp; ++a) acc -= S[(size_t)a * n + r] * beta[a];
        s->vinv_r[r] = acc;
    }
    double* w = (double*)malloc(sizeof(double) * m->N);
    jt_vec(m, s->vinv_r, w);                                /* uhat  :1446-1473 */
    orc_grm_apply(s, w, 1, s->uhat);
    memset(bhat, 0, sizeof(double) * 2 * (size_t)m->N);    /* bhat  :1475-1513 */
    for (int64_t r = 0; r < n; ++r) {
        int i = m->indiv[r];
        bhat[2 * i] += s->vinv_r[r] * (vc[2] + vc[3] * t[r]);
        bhat[2 * i + 1] += s->vinv_r[r] * (vc[3] + vc[4] * t[r]);
    }
    if (uhat) memcpy(uhat, s->uhat, sizeof(double) * m->N);
    if (vinv_r) memcpy(vinv_r, s->vinv_r, sizeof(double) * n);
    free(B); free(S); free(xty); free(w);
    return it;
}

/* ------------------------------------------------------------------ */
/* AIREML terms                                                          */
/* ------------------------------------------------------------------ */

/* compute_f_theta_i varCompEst.cpp:693-760 */
static void f_theta(const orc_model* m, const double* vr, const double* uh, double* f) {
    const int64_t n = m->Nrec;
    const int32_t N = m->N;
    const double* t = m->X + (size_t)m->p * n;
    double* w = (double*)calloc(N, sizeof(double));
    double* tw = (double*)calloc(N, sizeof(double));
    for (int64_t r = 0; r < n; ++r) { w[m->indiv[r]] += vr[r]; tw[m->indiv[r]] += vr[r] * t[r]; }
    for (int64_t r = 0; r < n; ++r) {
        int i = m->indiv[r];
        f[r] = vr[r];
        f[n + r] = uh[i] / m->vc[1];
        f[2 * n + r] = w[i];
        f[3 * n + r] = t[r] * w[i] + tw[i];
        f[4 * n + r] = tw[i] * t[r];
    }
    free(w);
    free(tw);
}

/* P v = v - V^-1X (X'V^-1X)^-1 X' v  (varCompEst.cpp:957, :1030-1035) */
static void project(orc_solver* s, const double* v, double* out) {
    const orc_model* m = &s->m;
    const int64_t n = m->Nrec;
    const int pp = m->p + 1;
    double xv[64], c[64];
    for (int a = 0; a < pp; ++a) xv[a] = col_dot(m->X + (size_t)a * n, v, n);
    for (int a = 0; a < pp; ++a) {
        double acc = 0.0;
        for (int b = 0; b < pp; ++b) acc += s->xtvx_inv[(size_t)b * pp + a] * xv[b];
        c[a] = acc;
    }
    for (int64_t r = 0; r < n; ++r) {
        double acc = v[r];
        for (int a = 0; a < pp; ++a) acc -= s->vinv_X[(size_t)a * n + r] * c[a];
        out[r] = acc;
    }
}

int orc_aireml_grad(orc_solver* s, const double* probes, int numMC, double tol, int maxit,
                    double* fth, double* first, double* trace, double* grad) {
    const orc_model* m = &s->m;
    const int64_t n = m->Nrec;
    const int32_t N = m->N;
    const double* vc = m->vc;
    const double* t = m->X + (size_t)m->p * n;
    f_theta(m, s->vinv_r, s->uhat, fth);
    for (int k = 0; k < 5; ++k) first[k] = col_dot(s->vinv_r, fth + (size_t)k * n, n);
    /* compute_chol_2x2 :800-813 */
    double L00 = sqrt(vc[2]), L10 = vc[3] / L00;
    double d11 = vc[4] - vc[3] * vc[3] / vc[2];
    if (d11 < 0) d11 = 0;
    double L11 = sqrt(d11);
    /* sample_Yvs :775-797 */
    double* Y = (double*)malloc(sizeof(double) * (size_t)n * numMC);
    const double* pz = probes;
    for (int j = 0; j < numMC; ++j) {
        const double *Z1 = pz, *Z2 = pz + N, *Z3 = pz + 3 * (size_t)N;
        for (int64_t r = 0; r < n; ++r) {
            int i = m->indiv[r];
            Y[(size_t)j * n + r] = sqrt(vc[1]) * Z1[i] + sqrt(vc[0]) * Z3[r] +
                                   Z2[2 * i] * (L00 + L10 * t[r]) + Z2[2 * i + 1] * L11 * t[r];
        }
        pz += 3 * (size_t)N + n;
    }
    /* V*^-1 Y per block (:839-862): V* = s2g 11' + U D U' + s2e I */
    double* TY = (double*)malloc(sizeof(double) * (size_t)n * numMC);
    for (int32_t b = 0; b < s->nblk; ++b) {
        int64_t st = s->bstart[b];
        int nn = (int)(s->bstart[b + 1] - st);
        double* Q = (double*)malloc(sizeof(double) * (size_t)nn * nn);
        for (int i = 0; i < nn; ++i)
            for (int j = 0; j < nn; ++j)
                Q[(size_t)j * nn + i] = vc[1] + tval(vc, t[st + i], t[st + j]) + (i == j ? vc[0] : 0.0);
        gj_inverse(Q, nn);
        for (int c = 0; c < numMC; ++c)
            for (int i = 0; i < nn; ++i) {
                double acc = 0.0;
                for (int j = 0; j < nn; ++j) acc += Q[(size_t)j * nn + i] * Y[(size_t)c * n + st + j];
                TY[(size_t)c * n + st + i] = acc;
            }
        free(Q);
    }
    /* V^-1 Y by PCG from x0 = V*^-1 Y (:945-950) */
    double* VY = (double*)malloc(sizeof(double) * (size_t)n * numMC);
    memcpy(VY, TY, sizeof(double) * (size_t)n * numMC);
    int it = orc_pcg(s, Y, VY, numMC, tol, maxit, 1, 2);
    double* vr = (double*)malloc(sizeof(double) * n);
    double* w = (double*)malloc(sizeof(double) * N);
    double* uh = (double*)malloc(sizeof(double) * N);
    double* ft = (double*)malloc(sizeof(double) * (size_t)n * 5);
    for (int k = 0; k < 5; ++k) trace[k] = 0.0;
    for (int j = 0; j < numMC; ++j) {                       /* :955-968 */
        project(s, VY + (size_t)j * n, vr);
        jt_vec(m, vr, w);
        orc_grm_apply(s, w, 1, uh);
        f_theta(m, vr, uh, ft);
        for (int k = 0; k < 5; ++k) trace[k] += col_dot(ft + (size_t)k * n, TY + (size_t)j * n, n);
    }
    for (int k = 0; k < 5; ++k) {
        trace[k] /= numMC;
        grad[k] = 0.5 * (first[k] - trace[k]);               /* :1006-1010 */
    }
    free(Y); free(TY); free(VY); free(vr); free(w); free(uh); free(ft);
    return it;
}

int orc_aireml_ai(orc_solver* s, const double* fth, double tol, int maxit, double* ai) {
    const int64_t n = s->m.Nrec;
    double* Vf = (double*)malloc(sizeof(double) * (size_t)n * 5);
    double* Pf = (double*)malloc(sizeof(double) * (size_t)n * 5);
    int it = orc_pcg(s, fth, Vf, 5, tol, maxit, 1, 1);
    for (int k = 0; k < 5; ++k) project(s, Vf + (size_t)k * n, Pf + (size_t)k * n);
    for (int a = 0; a < 5; ++a)
        for (int b = 0; b < 5; ++b) ai[b * 5 + a] = 0.5 * col_dot(fth + (size_t)a * n, Pf + (size_t)b * n, n);
    free(Vf);
    free(Pf);
    return it;
}

/* ------------------------------------------------------------------ */
/* FP32 restatement with the reference's loop structure (timing only)    */
/* ------------------------------------------------------------------ */

struct ref_gdata {
    const uint8_t* const* chunks;
    int64_t per_chunk, bps;
};

static inline int ref_get_genotype(const struct ref_gdata* g, int64_t snp, int indiv) {
    /* getGenotype PCGsolver.cpp:812-824 (chunk lookup per element) */
    int chunk_idx = (int)(snp / g->per_chunk);
    int off = (int)(snp % g->per_chunk);
    size_t base = (size_t)off * g->bps;
    const uint8_t* p = g->chunks[chunk_idx];
    unsigned code = (p[base + indiv / 4] >> ((indiv % 4) * 2)) & 3u;
    return decode_code(code);
}

void orc_ref_vx_f32(int32_t N, int64_t Nrec, const int32_t* indiv, const float* times,
                    const uint8_t* geno, int64_t Mk, int64_t stride, const float* maf,
                    const float vc[5], const float* x, int k, float* out) {
    /* storage in 1 GB chunks as in prepGenotypeInput PCGsolver.cpp:666-697 */
    int64_t per_chunk = (int64_t)(1e9 / (double)stride);
    if (per_chunk == 0) per_chunk = 50000;
    int64_t nch = (Mk + per_chunk - 1) / per_chunk;
    const uint8_t** chunks = (const uint8_t**)malloc(sizeof(uint8_t*) * (nch > 0 ? nch : 1));
    for (int64_t c = 0; c < nch; ++c) chunks[c] = geno + (size_t)c * per_chunk * stride;
    struct ref_gdata g = {chunks, per_chunk, stride};
    float* Z = (float*)calloc((size_t)N * k, sizeof(float));
    float* GZ = (float*)calloc((size_t)N * k, sizeof(float));
    memset(out, 0, sizeof(float) * (size_t)Nrec * k);
    for (int64_t r = 0; r < Nrec; ++r)
        for (int c = 0; c < k; ++c) Z[(size_t)c * N + indiv[r]] += x[(size_t)c * Nrec + r];
    const float inv_num = Mk > 0 ? 1.0f / (float)Mk : 0.0f;
    const int64_t CH = 50000;
    for (int64_t s0 = 0; s0 < Mk; s0 += CH) {
        int64_t s1 = s0 + CH < Mk ? s0 + CH : Mk;
        float* part = (float*)calloc((size_t)(s1 - s0) * k, sizeof(float));
#pragma omp parallel for schedule(dynamic)
        for (int64_t sn = s0; sn < s1; ++sn) {
            float acc[256];
            for (int c = 0; c < k; ++c) acc[c] = 0.0f;
            for (int i = 0; i < N; ++i) {
                int gt = ref_get_genotype(&g, sn, i);
                if (gt < 0) gt = 0;
                float f = maf[sn];
                float den = 2.0f * f * (1.0f - f);
                float inv = (den > 1e-12f) ? (1.0f / sqrtf(den)) : 1.0f;
                float z = (gt - 2.0f * f) * inv;
                for (int c = 0; c < k; ++c) acc[c] += z * Z[(size_t)c * N + i];
            }
            for (int c = 0; c < k; ++c) part[(size_t)(sn - s0) * k + c] = acc[c];
        }
#pragma omp parallel for schedule(dynamic)
        for (int i = 0; i < N; ++i) {
            float res[256];
            for (int c = 0; c < k; ++c) res[c] = 0.0f;
            for (int64_t sn = s0; sn < s1; ++sn) {
                int gt = ref_get_genotype(&g, sn, i);
                if (gt < 0) gt = 0;
                float f = maf[sn];
                float den = 2.0f * f * (1.0f - f);
                float inv = (den > 1e-12f) ? (1.0f / sqrtf(den)) : 1.0f;
                float z = (gt - 2.0f * f) * inv;
                for (int c = 0; c < k; ++c) res[c] += z * part[(size_t)(sn - s0) * k + c];
            }
            for (int c = 0; c < k; ++c) GZ[(size_t)c * N + i] += vc[1] * inv_num * res[c];
        }
        free(part);
    }
    for (int64_t r = 0; r < Nrec; ++r)
        for (int c = 0; c < k; ++c) out[(size_t)c * Nrec + r] += GZ[(size_t)c * N + indiv[r]];
    /* time block and residual over contiguous runs */
    int64_t st = 0;
    while (st < Nrec) {
        int64_t en = st + 1;
        while (en < Nrec && indiv[en] == indiv[st]) ++en;
        for (int64_t i = st; i < en; ++i)
            for (int64_t j = st; j < en; ++j) {
                float v = vc[2] + vc[3] * (times[i] + times[j]) + vc[4] * (times[i] * times[j]);
                for (int c = 0; c < k; ++c) out[(size_t)c * Nrec + i] += v * x[(size_t)c * Nrec + j];
            }
        st = en;
    }
    for (int c = 0; c < k; ++c)
        for (int64_t r = 0; r < Nrec; ++r) out[(size_t)c * Nrec + r] += vc[0] * x[(size_t)c * Nrec + r];
    free(Z); free(GZ); free(chunks);
}
