/*
 * globe_oracle.h -- CPU restatement of GLOBE's LGMM solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the parity tests, smoke()
 * and bench.py's CPU-baseline leg compare against; the product never links,
 * loads or calls it.  Each function cites the reference code it restates
 * (paths inside the GLOBE source tree).  It is pinned against the upstream
 * programs themselves (built by oracle/build_ref.py) through the fixtures in
 * tests/golden/.
 *
 * Conventions: matrices are column-major (leading dimension = rows), record
 * arrays are in file order, individual indices are 0-based.
 */
#ifndef GLOBE_ORACLE_H
#define GLOBE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Per-SNP allele counts, float32 A1 frequency, missing rate and the MAF /
 * missingness filter, bit-exact with PCGsolver.cpp:96-123 (LUT),
 * :589-613 (phantom pairs of the last byte), :700-743 (counts, float maf,
 * filter).  bed = M rows of ceil(N/4) bytes, no magic.  Returns #kept. */
int64_t orc_bed_stats(const uint8_t* bed, int64_t M, int32_t N, float min_maf,
                      float max_miss, int64_t* alt, int64_t* miss, float* maf,
                      float* miss_rate, uint8_t* keep);

/* Double-precision A1 frequency and inverse std of the kept SNPs, with the
 * expressions of PCGsolver.cpp:728 and :837-840 evaluated in double (what the
 * float->double build of the reference computes). */
void orc_std_params(const int64_t* alt, const int64_t* miss, int64_t M, int32_t N,
                    double* f, double* inv_std);

/* A = Zs'Zs / Mk of the kept SNP rows (Mk rows of `stride` bytes), zs as
 * getStdGenotype (PCGsolver.cpp:826-842, missing -> 0), summed in double in
 * SNP order and rounded once to float32; written as the packed lower
 * triangle lt[i(i+1)/2 + j], j <= i (the .grm.bin layout readFullGRM reads,
 * PCGsolver.cpp:778-809). */
void orc_grm_build(const uint8_t* geno, int64_t Mk, int64_t stride, int32_t N, const double* f,
                   const double* inv_std, float* lt);

typedef struct {
    int32_t N;            /* individuals */
    int64_t Nrec;         /* records */
    int32_t p;            /* covariates; X has p+1 columns, time last */
    const int32_t* indiv; /* [Nrec], 0-based */
    const double* X;      /* [Nrec x (p+1)] */
    const double* y;      /* [Nrec] */
    /* genetic relationship source: genotypes (geno != 0) or dense GRM */
    const uint8_t* geno;  /* kept SNP rows, stride bytes each */
    int64_t Mk, stride;
    const double* f;      /* [Mk] */
    const double* inv_std;/* [Mk] */
    const float* grm_lt;  /* [N(N+1)/2] packed lower triangle */
    double vc[5];         /* sig2e sig2g sig2b0 sigb01 sig2b1 */
} orc_model;

typedef struct orc_solver orc_solver;

orc_solver* orc_create(const orc_model* m);
void orc_destroy(orc_solver* s);
void orc_set_vc(orc_solver* s, const double vc[5]);

/* out[N x k] = sig2g * A * Z.  Genotypes: sig2g/M * Zs'(Zs Z) with
 * zs = (g-2f)*inv_std, missing -> 0 (PCGsolver.cpp:1130-1201).  Dense:
 * sig2g * A_lt(i,j) * Z (PCGsolver.cpp:1202-1213). */
void orc_grm_apply(orc_solver* s, const double* Z, int k, double* out);
/* A_ii (PCGsolver.cpp:924-989). */
void orc_genetic_diag(orc_solver* s, double* d);
/* out[Nrec x k] = V x  (PCGsolver.cpp:1095-1266; time block within each
 * contiguous run of one individual). */
void orc_vx(orc_solver* s, const double* x, int k, double* out);
/* Rebuild the block preconditioner (PCGsolver.cpp:991-1058 /
 * varCompEst.cpp:355-411) for the current components. */
void orc_precond_build(orc_solver* s);
/* z = Q^-1 r per column (PCGsolver.cpp:1060-1093). */
void orc_precond_apply(orc_solver* s, const double* r, int k, double* z);

/* Block PCG.  rule 0: stop when max_j |r_j|/|b_j| < tol or after 10
 * iterations without 0.5% improvement (PCGsolver.cpp:1324-1444); rule 1:
 * stop when all |r_j| < tol |b_j| (varCompEst.cpp:453-528).  x0mode 0: x=0,
 * 1: x = Q^-1 b, 2: x given.  Returns iterations run. */
int orc_pcg(orc_solver* s, const double* B, double* X, int k, double tol, int maxit,
            int rule, int x0mode);

/* Fixed and random effects (PCGsolver.cpp:262-297, 1446-1513;
 * varCompEst.cpp:587-685).  Solves V [X y], forms beta, V^-1 r, uhat, bhat
 * and keeps V^-1 X and (X'V^-1X)^-1 for the AIREML terms. */
int orc_mme(orc_solver* s, double tol, int maxit, int rule, int x0mode, double* beta,
            double* uhat, double* bhat, double* vinv_r);

/* f_theta columns, score first terms, Monte-Carlo trace and gradient at the
 * current components, after orc_mme (varCompEst.cpp:693-1012).  probes holds
 * numMC x (N + 2N + Nrec) standard normal draws in the order the reference's
 * sample_Yvs consumes them (Z1, Z2, Z3 per sample). */
int orc_aireml_grad(orc_solver* s, const double* probes, int numMC, double tol, int maxit,
                    double* f_theta, double* first, double* trace, double* grad);
/* AI = 1/2 f' P f (varCompEst.cpp:1015-1041). */
int orc_aireml_ai(orc_solver* s, const double* f_theta, double tol, int maxit, double* ai);

/* ---- FP32 restatement with the reference's own loop structure, for the
 * timed CPU baseline only (PCGsolver.cpp:1095-1266 genotype branch and
 * :1324-1444).  Single precision throughout, genotype decoded per element as
 * in getGenotype/getStdGenotype (PCGsolver.cpp:811-842). */
void orc_ref_vx_f32(int32_t N, int64_t Nrec, const int32_t* indiv, const float* times,
                    const uint8_t* geno, int64_t Mk, int64_t stride, const float* maf,
                    const float vc[5], const float* x, int k, float* out);

#ifdef __cplusplus
}
#endif
#endif
