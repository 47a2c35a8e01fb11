/*
 * globe.h -- C ABI of the GB300-native GLOBE longitudinal genomic mixed-model
 * solve (libglobe_gb300.so).
 *
 * The reference (ahmadazim/GLOBE) has no library interface: its stable
 * boundary is the runPCGsolver / runAIREML command lines and their files.
 * Every entry point below replaces one internal function of those programs
 * and cites it (file:line in the GLOBE source tree).  The command-line
 * programs shipped here (runPCGsolver, runAIREML) are written on top of this
 * ABI only.
 *
 * Conventions
 *  - Every call returns an int status: GLOBE_OK (0) or a negative code;
 *    globe_last_error(ctx) then holds a message.  Nothing calls exit().
 *  - Matrices are column-major with the leading dimension equal to the row
 *    count (records, individuals or SNPs).
 *  - Host buffers are caller-owned and copied; "_dev" entry points take
 *    device pointers on the context's device and run on the context's stream.
 *  - Every wait inside the tensor-core kernels is bounded; one that runs out
 *    sets a device error word.  Calls that synchronise (the host-buffer
 *    operators, PCG, MME, AIREML, the GRM builder) read and clear it and return
 *    GLOBE_ERR_CUDA ("timed out"), ahead of any other error it caused; after an
 *    asynchronous _dev operator the next such call reports it.
 *  - One context = one GPU and one CUDA stream.  Calls on one context are not
 *    reentrant; distinct contexts are independent.
 *  - Variance components are ordered (sig2e, sig2g, sig2b0, sigb01, sig2b1)
 *    as in varCompEst.cpp:48-60.
 */
#ifndef GLOBE_H
#define GLOBE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GLOBE_OK 0
#define GLOBE_ERR_ARG (-1)         /* invalid argument / size mismatch */
#define GLOBE_ERR_CUDA (-2)        /* CUDA runtime error */
#define GLOBE_ERR_STATE (-3)       /* call order: data or components missing */
#define GLOBE_ERR_IO (-4)          /* file cannot be opened / read / written */
#define GLOBE_ERR_FORMAT (-5)      /* malformed input file */
#define GLOBE_ERR_NOMEM (-6)       /* device allocation failed */
#define GLOBE_ERR_NUMERIC (-7)     /* breakdown (non-finite or zero curvature) */
#define GLOBE_ERR_UNSUPPORTED (-8) /* option not available for this input */

/* precision of the GRM product and the solve's record arithmetic */
#define GLOBE_PREC_FP64 0   /* plain FP64 everywhere (the drop-in path) */
#define GLOBE_PREC_MIXED 1  /* genotype GRM product on the FP8 tensor cores with exact
                               base-32 digit slicing of the right-hand sides (9 digits =
                               45 bits by default, matches FP64 to ~1e-13; see
                               globe_set_digits); dense GRM on the same tensor
                               cores, A held as min(7, digits) e4m3 digit planes of
                               one fixed-point grid (7 N^2 bytes; A within 2^-34
                               max|A|), or in double-float FP32 arithmetic (~48 bits)
                               when the planes do not fit in free device memory or
                               A has a non-finite entry; inside PCG / MME / AIREML solves
                               the record-level vectors run in double-float FP32 pairs
                               and the scalars and dot products in FP64
                               (globe_set_record_df) */

/* models (globe_set_model) */
#define GLOBE_MODEL_FULL 0     /* random intercept and slope per individual (runAIREML) */
#define GLOBE_MODEL_NO_TIME 1  /* no time effects: V = sig2g J A J' + sig2e I, components
                                  (sig2e, sig2g) (runAIREML_reducedModel) */

/* PCG stopping rules */
#define GLOBE_RULE_PCGSOLVER 0 /* max_j |r_j|/|b_j| < tol, or 10 iterations with
                                  < 0.5% improvement (PCGsolver.cpp:1381-1415) */
#define GLOBE_RULE_AIREML 1    /* all_j |r_j| < tol |b_j| (varCompEst.cpp:505-508) */

/* PCG starting points (varCompEst.cpp:453-476) */
#define GLOBE_X0_ZERO 0      /* x0 = 0 (PCGsolver.cpp:1339-1344) */
#define GLOBE_X0_PRECOND 1   /* x0 = Q^-1 b ("use_initial_guess") */
#define GLOBE_X0_GIVEN 2     /* x0 = X on entry ("use_input_initial") */

typedef struct globe_ctx globe_ctx;

typedef struct {
    double tol;     /* relative residual tolerance (reference: 1e-5) */
    int maxit;      /* iteration cap (reference: 1000) */
    int rule;       /* GLOBE_RULE_* */
    int x0mode;     /* GLOBE_X0_* */
    int mask;       /* 1: freeze converged columns (per-column masking);
                       0: every column iterates until the rule stops all */
    int precision;  /* GLOBE_PREC_* */
} globe_pcg_opts;

typedef struct {
    int iters;          /* iterations of the (outer) solve */
    int inner_iters;    /* iterations run by the kernels (equals iters: the mixed
                           product is FP64-faithful, so there is no inner solve) */
    int64_t rhs_iters;  /* sum over iterations of active columns */
    double max_rel_res; /* max_j |b_j - V x_j| / |b_j| at exit (recurrence) */
    int converged;      /* 1 if the rule was met (not maxit / stagnation) */
    int stagnated;      /* 1 if PCGsolver's stagnation stop fired */
} globe_pcg_info;

typedef struct {
    int64_t M;       /* SNPs in the .bed */
    int64_t kept;    /* SNPs passing the MAF / missingness filter */
} globe_bed_info;

/* ---- context ---------------------------------------------------------- */

/* Create a context on `device` (one CUDA stream).  No reference
 * counterpart: the reference is a single process holding its state in the
 * structs of PCGsolver.cpp:32-75. */
int globe_create(globe_ctx** ctx, int device);
void globe_destroy(globe_ctx* ctx);
/* Last error message of ctx (or of the failing globe_create when ctx is
 * NULL).  Replaces the std::cerr + exit(EXIT_FAILURE) convention of
 * PCGsolver.cpp:338-444. */
const char* globe_last_error(const globe_ctx* ctx);
/* The context's cudaStream_t (for events / interop). */
int globe_get_stream(globe_ctx* ctx, void** stream);
int globe_synchronize(globe_ctx* ctx);
/* Device bytes currently held by the context. */
int64_t globe_device_bytes(const globe_ctx* ctx);
/* Number of kernels this context has launched (for accounting). */
int64_t globe_kernel_launches(const globe_ctx* ctx);
/* Sizes of the loaded inputs (any pointer may be NULL): records, individuals,
 * covariates, kept SNPs (0 for a dense GRM). */
int globe_get_dims(const globe_ctx* ctx, int64_t* Nrec, int32_t* N, int32_t* p, int64_t* kept_snps);

/* ---- inputs ----------------------------------------------------------- */

/* Record table: Nrec records of N individuals, p covariates plus time.
 * indiv: 0-based individual index of each record (the file's INDIV - 1,
 * PCGsolver.cpp:579); X: Nrec x (p+1) with time as the last column
 * (PCGsolver.cpp:581); y: phenotype.  Records of one individual must be
 * contiguous, and every index in 0..N-1 must occur (the reference assumes
 * both, PCGsolver.cpp:499-519, :1002-1009).  Replaces readInputData
 * (PCGsolver.cpp:529-587, varCompEst.cpp:199-262). */
int globe_load_records(globe_ctx* ctx, int64_t Nrec, int32_t N, int32_t p,
                       const int32_t* indiv, const double* X, const double* y);

/* Genotype-only context: N individuals (the lines of the .fam) and no record
 * table, for building a GRM (globe_grm_build).  Drops any loaded records and
 * genetic source.  The solver entry points still need globe_load_records.
 * No reference counterpart: the reference takes N from the record table
 * (PCGsolver.cpp:529-587) and has no GRM builder. */
int globe_set_individuals(globe_ctx* ctx, int32_t N);

/* PLINK .bed payload (the bytes after the 3-byte magic): M SNP rows of
 * ceil(N/4) bytes, N from globe_load_records.  Computes per-SNP A1 counts,
 * missing counts, the float32 A1 frequency and missing rate, applies the
 * filter maf in [min_maf, 1-min_maf], miss_rate <= max_miss -- bit-exact
 * with prepGenotypeInput (PCGsolver.cpp:615-763) -- and keeps the passing
 * SNPs in HBM as the genetic relationship source.  Any per-SNP output may
 * be NULL. */
int globe_load_bed(globe_ctx* ctx, const uint8_t* bed, int64_t M, float min_maf,
                   float max_miss, int64_t* alt_count, int64_t* miss_count, float* maf,
                   float* miss_rate, uint8_t* keep, globe_bed_info* info);
/* Same from a device buffer of M rows, `stride` bytes apart (stride >=
 * ceil(N/4)).  Per-SNP outputs are device pointers (may be NULL). */
int globe_load_bed_dev(globe_ctx* ctx, const uint8_t* d_bed, int64_t M, int64_t stride,
                       float min_maf, float max_miss, int64_t* d_alt, int64_t* d_miss,
                       float* d_maf, float* d_miss_rate, uint8_t* d_keep, globe_bed_info* info);
/* Same from <prefix>.bed on disk, streamed: whole SNP rows are read in chunks
 * of about chunk_bytes (0: 256 MB) into two pinned host buffers taken in turn,
 * each copied to the device while the next is read; host memory stays at two
 * chunks.  M is the number of lines of <prefix>.bim.  Replaces the serial
 * whole-file read of prepGenotypeInput (PCGsolver.cpp:706-749).  Per-SNP
 * outputs are host pointers (may be NULL), as in globe_load_bed. */
int globe_load_bed_file(globe_ctx* ctx, const char* prefix, float min_maf, float max_miss, int64_t chunk_bytes,
                        int64_t* alt_count, int64_t* miss_count, float* maf, float* miss_rate, uint8_t* keep,
                        globe_bed_info* info);

/* Dense GRM: float32 packed lower triangle, row major with the diagonal,
 * N(N+1)/2 values (.grm.bin payload).  Replaces readFullGRM
 * (PCGsolver.cpp:778-809) and readGRM (varCompEst.cpp:270-295). */
int globe_load_grm(globe_ctx* ctx, const float* grm_lt, int32_t N);

/* Genetic relationship matrix of the loaded genotypes, A = Zs'Zs / M_kept with
 * zs = (g - 2f) inv_std and missing g -> 0 (getStdGenotype,
 * PCGsolver.cpp:826-842: the matrix the --geno product applies), as the
 * float32 packed lower triangle, row major with the diagonal, N(N+1)/2 values:
 * the payload of <prefix>.grm.bin that readFullGRM (PCGsolver.cpp:778-809)
 * and readGRM (varCompEst.cpp:270-295) read.  The reference has no builder.
 * GLOBE_PREC_MIXED: tensor cores, each value the float32 rounding of an
 * evaluation exact to ~2^-41 max|inv_std zs| per term; GLOBE_PREC_FP64: FP64
 * arithmetic.  Needs at least one kept SNP (GLOBE_ERR_STATE otherwise). */
int globe_grm_build(globe_ctx* ctx, float* grm_lt);
/* Same into a device buffer of N(N+1)/2 floats. */
int globe_grm_build_dev(globe_ctx* ctx, float* d_grm_lt);

/* Variance components (sig2e, sig2g, sig2b0, sigb01, sig2b1).  sig2e must be
 * > 0 (the block preconditioner is singular otherwise). */
int globe_set_vc(globe_ctx* ctx, const double vc[5]);

/* Model of the variance components (GLOBE_MODEL_FULL by default).  Under
 * GLOBE_MODEL_NO_TIME -- varCompEst_reducedModel_noTime.cpp, the reference's
 * runAIREML_reducedModel -- the time effects are absent: globe_set_vc keeps
 * vc[0..1] and sets vc[2..4] = 0, the AIREML probes are Y = sqrt(sig2g) J Z1 +
 * sqrt(sig2e) Z3 (Z1 over individuals, Z3 over records, in that order per
 * probe; :563-577), and globe_aireml_grad / _eval / _ai fill components 0..1
 * only (the AI matrix in the top-left 2x2 of its 5x5 array). */
int globe_set_model(globe_ctx* ctx, int model);
int globe_get_model(const globe_ctx* ctx);

/* Precision of the operator calls below (globe_grm_apply, globe_vx):
 * GLOBE_PREC_FP64 (default) or GLOBE_PREC_MIXED (genotype GRM on the FP8
 * tensor cores with exact digit slicing; see globe_pcg_opts.precision).
 * PCG / MME / AIREML calls take the precision from their options. */
int globe_set_precision(globe_ctx* ctx, int precision);

/* GLOBE_PREC_MIXED rounds each right-hand-side column once to nd balanced
 * base-32 digits (2 <= nd <= 9, default 9) and multiplies every digit exactly:
 * a column x becomes x rounded to a multiple of 2^-(5(nd-1)+4) max|x| (both
 * passes round their input this way), so each product column is within a few
 * times that unit of the exact product (nd = 9: ~1e-13, nd = 6: ~5e-9,
 * nd = 5: ~1.5e-7, the reference's own FP32 level).  Fewer digits
 * mean fewer tensor-core columns: 20 columns take MMA width 192 at nd = 9 and
 * 128 at nd = 6.  A dense GRM is rounded the same way, to min(7, nd) digits
 * on one grid for the whole matrix (a multiple of 2^-(5(min(7,nd)-1)+3) max|A|;
 * nd >= 7: ~1e-10 relative product error, nd = 6: ~2e-8); its digit planes are
 * rebuilt on the first mixed product after the count changes.
 * No reference counterpart (the reference works in FP32). */
int globe_set_digits(globe_ctx* ctx, int nd);
int globe_get_digits(const globe_ctx* ctx);

/* CUDA graphs in the block PCG (on = 1, the default; 0 = direct launches).
 * Each globe_pcg call runs its first iteration directly. It then captures the
 * iteration's stream work (record kernels, GRM product, the copies of the
 * residual norms) once per parity of its swapped r'z buffers and column set,
 * and replays it, with the host checking the stopping rule after each
 * iteration (or, by default, once per solve: globe_set_device_loop).
 * Results are identical either way. Graphs are not used while event
 * profiling is on (globe_prof_enable), so that each pass is timed, nor when a
 * capture fails (e.g. a workspace would have to grow); the iteration then
 * launches the same kernels directly.  No reference counterpart. */
int globe_set_graphs(globe_ctx* ctx, int on);
int globe_get_graphs(const globe_ctx* ctx);

/* Device-side PCG loop (on = 1, the default; needs graphs on).  Without
 * per-column masking the column set of a solve cannot change, so after the
 * first iteration the rest run as one CUDA graph whose WHILE conditional node
 * repeats the iteration; a one-thread kernel at the end of each iteration
 * applies the stopping rule of the reference -- max_j |r_j|/|b_j| < tol and the
 * stagnation stop (PCGsolver.cpp:1373-1415), or all_j |r_j| < tol |b_j|
 * (varCompEst.cpp:505-508) -- to the device copies of the residual norms and
 * sets the node's condition.  No host synchronisation per iteration; the same
 * kernels in the same order, so the same results and iteration counts as the
 * host-checked loop (on = 0).  With masking, while profiling, or if the graph
 * cannot be built, the host checks every iteration.  globe_device_loop_runs
 * counts the solves that used it.  No reference counterpart. */
int globe_set_device_loop(globe_ctx* ctx, int on);
int globe_get_device_loop(const globe_ctx* ctx);
int64_t globe_device_loop_runs(const globe_ctx* ctx);

/* Double-float record kernels of GLOBE_PREC_MIXED solves (on = 1, the default;
 * 0 = FP64).  The block PCG's record-level vectors (x, r, z, p, Vp) are held
 * as pairs of FP32 numbers (about 48 significant bits) from the end of its
 * FP64 set-up to the end of the solve, and the iteration's segment sums,
 * operator assembly and update run on the FP32 pipe; the GRM product's input
 * and output, the per-column scalars and the dot products past each CTA stay
 * FP64.  Each column runs scaled by a power of two to a unit-size right-hand
 * side (exact), and x is returned in FP64.  A solve keeps the FP64 kernels
 * when sig2e lies outside [2^-30, 2^30], another component or a time exceeds
 * 2^30 in magnitude, or a right-hand side is not finite.
 * globe_record_df_solves counts the solves that used them.  FP64 solves
 * (GLOBE_PREC_FP64) never do.  No reference counterpart: the reference's
 * record loops run in its build's floating type (PCGsolver.cpp:1095-1266). */
int globe_set_record_df(globe_ctx* ctx, int on);
int globe_get_record_df(const globe_ctx* ctx);
int64_t globe_record_df_solves(const globe_ctx* ctx);

/* Autotuning of the tensor-core genotype product (on = 1, the default; 0 =
 * the analytic choices only).  On first use of a shape in the process --
 * outside graph capture and event profiling -- the product times its
 * candidates with CUDA events on the context's stream and keeps the fastest
 * for every context on that device:
 *  - the split-K count of each pass (per MMA width, rows and K stages): the
 *    wave-quantisation cost model's count and up to 2 more within 25% of its
 *    estimate, one launch each;
 *  - for 9 or more right-hand-side columns, the column grouping (per column
 *    count, digit count and genotype shape): the rule's group count and one
 *    more, two rounds each.
 * Every candidate gives the same result bits (exact sums in any split or
 * group), so the choice changes speed only.  globe_autotune_log writes this
 * context's timing decisions as a JSON array into buf (cap bytes,
 * NUL-terminated, truncated if short) and returns the full length.
 * globe_debug_force_splits(ctx, s), s > 0, makes every tensor-core genotype
 * pass use s splits (a test hook; 0 = off).  The reference hard-codes its SNP
 * chunk instead (SNP_CHUNK_SIZE, PCGsolver.cpp:1135). */
int globe_set_autotune(globe_ctx* ctx, int on);
int globe_get_autotune(const globe_ctx* ctx);
int64_t globe_autotune_log(const globe_ctx* ctx, char* buf, int64_t cap);
int globe_debug_force_splits(globe_ctx* ctx, int splits);

/* Bounds-checked debug build (the library compiled with -DGLOBE_CHECK_BOUNDS):
 * the kernels check the indices they take from data -- each block of records
 * inside [0, Nrec), each individual inside [0, N) -- and a failed check skips
 * its access and records a code (kernel << 8 | check).  Returns 0 if no check
 * failed since the last call, 1 if one did (first_code: its code), and clears;
 * GLOBE_ERR_UNSUPPORTED in a library built without the checks.  No reference
 * counterpart. */
int globe_debug_bounds(uint32_t* first_code);

/* Test hook for the tensor-core kernels' bounded waits: the next tensor-core
 * GRM product's first launch (genotype or dense) leaves its first stage
 * unloaded.  The MMA issuer's wait for it runs out after ~2 s, the CTA raises
 * its abort flag, drains its copies with bounded waits and frees TMEM, and the
 * call returns GLOBE_ERR_CUDA ("timed out ... code 0x4" from the genotype
 * kernel, "code 0x2" from the dense one); the context stays usable.  Nothing
 * faults and nothing waits without a limit.  Not for production use. */
int globe_debug_stall_next_gemm(globe_ctx* ctx);

/* ---- operators -------------------------------------------------------- */

/* out (N x k) = sig2g * A * Z for Z (N x k): the GRM product of
 * computeVx_multi with multGRM_uhat = true (PCGsolver.cpp:1127-1217,
 * :1446-1473), genotype branch sig2g/M Zs'(Zs Z) or dense branch. */
int globe_grm_apply(globe_ctx* ctx, const double* Z, double* out, int k);
int globe_grm_apply_dev(globe_ctx* ctx, const double* d_Z, double* d_out, int k);
/* out (Nrec x k) = V x (computeVx_multi, PCGsolver.cpp:1095-1266;
 * computeVx_multi_VC, varCompEst.cpp:322-352). */
int globe_vx(globe_ctx* ctx, const double* x, double* out, int k);
int globe_vx_dev(globe_ctx* ctx, const double* d_x, double* d_out, int k);
/* z = Q^-1 r with the per-individual block preconditioner
 * (computePreconditioner_Block + applyPreconditioner, PCGsolver.cpp:991-1093;
 * varCompEst.cpp:355-450).  Built from the current components. */
int globe_precond_apply(globe_ctx* ctx, const double* r, double* z, int k);
/* A_ii (computeGeneticDiagonal, PCGsolver.cpp:924-989). */
int globe_genetic_diag(globe_ctx* ctx, double* diag);

/* z = Q^-1 r on device buffers (Nrec x k, column-major), and d_rz[j] = r_j'z_j
 * (device, k doubles; may be NULL), without allocating device memory.  No
 * counterpart in the reference: it is the preconditioner of globe_precond_apply
 * for callers that may not allocate (e.g. work issued during CUDA stream
 * capture, or where the implicit device synchronisation of an allocation is
 * not allowed).
 *  - The r'z partials use one static 2 MiB device buffer (2^18 doubles).  A
 *    call needing more -- k x (ceil(N/256) + ceil(L/8)) doubles, L the number
 *    of individuals with more than 48 records -- returns GLOBE_ERR_ARG before
 *    launching anything.  Nothing in the buffer needs to start at zero.
 *  - Width limits, also checked before launching anything (GLOBE_ERR_ARG):
 *    k <= 65535; and with d_rz and any individual of more than 48 records,
 *    k <= 768 (64 bytes of shared memory per column, at the default 48 KB).
 *  - The buffer is shared by every context on a device: calls that overlap
 *    on the GPU (other streams or contexts on the same device) race on it.
 *  - The preconditioner must already be built at the current components
 *    (globe_precond_apply or globe_pcg once); otherwise GLOBE_ERR_STATE.
 *  - The first call on a device looks up the buffer's address; make that
 *    first call before any stream capture. */
int globe_precond_apply_dev_noalloc(globe_ctx* ctx, const double* d_r, double* d_z, int k, double* d_rz);

/* ---- solves ----------------------------------------------------------- */

/* Solve V X = B (Nrec x k) by block PCG (runPCG_multi,
 * PCGsolver.cpp:1324-1444; runPCG_multi_VC, varCompEst.cpp:453-528).  With
 * GLOBE_X0_GIVEN, X holds the starting point on entry. */
int globe_pcg(globe_ctx* ctx, const double* B, double* X, int k, const globe_pcg_opts* opts,
              globe_pcg_info* info);
int globe_pcg_dev(globe_ctx* ctx, const double* d_B, double* d_X, int k,
                  const globe_pcg_opts* opts, globe_pcg_info* info);

/* Mixed-model equations at the current components (main,
 * PCGsolver.cpp:262-297; fitMME, varCompEst.cpp:587-685): solves V [X y],
 * beta = (X'V^-1X)^-1 X'V^-1y, V^-1 r, uhat = sig2g A J' V^-1 r
 * (compute_uhat, :1446-1473), bhat_i = sum_r V^-1r (sig2b0 + sigb01 t,
 * sigb01 + sig2b1 t) (compute_bhat, :1475-1513).  Keeps V^-1X and
 * (X'V^-1X)^-1 for the AIREML terms.  Any output may be NULL. */
int globe_mme(globe_ctx* ctx, const globe_pcg_opts* opts, double* beta, double* uhat,
              double* bhat, double* vinv_r, globe_pcg_info* info);

/* AIREML score at the current components, after globe_mme
 * (computeDerivative_first + estimateTrace_PdV, varCompEst.cpp:693-1012).
 * probes: numMC x (N + 2N + Nrec) standard normal draws in the order
 * sample_Yvs consumes them (Z1, Z2, Z3 per probe, varCompEst.cpp:783-786),
 * or NULL to draw them on the GPU from `seed` (counter-based, reproducible).
 * f_theta (Nrec x 5, may be NULL) receives dV/dtheta_k V^-1 r; first, trace,
 * grad (5 each) receive the score terms. */
int globe_aireml_grad(globe_ctx* ctx, const double* probes, int numMC, uint64_t seed,
                      const globe_pcg_opts* opts, double* f_theta, double* first,
                      double* trace, double* grad, globe_pcg_info* info);

/* globe_mme followed by globe_aireml_grad's score, with the MME right-hand sides
 * [X y] and the numMC probes solved as one block PCG of p+2+numMC columns (MME
 * columns start from Q^-1 b, probe columns from V*^-1 Y).  The reference solves
 * them one after the other (fitMME, varCompEst.cpp:587-685, then
 * computeDerivative_first, :980-1012); the two solves are independent.  Leaves
 * the same state as globe_mme + globe_aireml_grad, so globe_aireml_ai may
 * follow. */
int globe_aireml_eval(globe_ctx* ctx, const double* probes, int numMC, uint64_t seed, const globe_pcg_opts* opts,
                      double* first, double* trace, double* grad, globe_pcg_info* info);
/* Average-information matrix AI = 1/2 f' P f (5 x 5) for the f_theta of the
 * last globe_aireml_grad (computeDerivative_AImat, varCompEst.cpp:1015-1041). */
int globe_aireml_ai(globe_ctx* ctx, const globe_pcg_opts* opts, double* ai,
                    globe_pcg_info* info);

/* Trust-region step of oneIter_AIREML (varCompEst.cpp:1148-1199): maximise
 * g'p - p'AI p/2 over p in [-10,10]^5 subject to sum_k AI_kk p_k <= delta,
 * theta_k + p_k >= 1e-5 (k != 3) and (theta_3+p_3)^2 <= (theta_2+p_2)(theta_4
 * +p_4) - 1e-3.  The reference solves this with NLopt's MMA (a closed
 * binary); this is a primal-dual interior-point method written from the
 * problem statement.  Host-only, FP64.  status: 0 solved, 1 infeasible,
 * 2 not converged. */
int globe_trust_region_step(const double theta[5], const double grad[5], const double ai[25],
                            double delta, double p[5], int* status);
/* Step of the reduced model (oneIter_AIREML, varCompEst_reducedModel_noTime.cpp:782-830):
 * maximise g'p - p'Ap/2 over 2 components s.t. |p_k| <= 10,
 * A_00 p_0 + A_11 p_1 <= delta, theta_k + p_k >= 1e-5; ai is 2x2 column-major.
 * Solved exactly by enumerating active sets.  status: 0 solved, 1 infeasible. */
int globe_trust_region_step_no_time(const double theta[2], const double grad[2], const double ai[4], double delta,
                                    double p[2], int* status);

typedef struct {
    int maxiter;       /* --maxiter (varCompEst.cpp:21, default 50) */
    double tol;        /* --tol (default 1e-3) */
    int numMC;         /* --numMC (default 15) */
    double theta0[5];  /* starting components (varCompEst.cpp:48-52 defaults) */
    double pcg_tol;    /* PCG tolerance (reference: 1e-5) */
    int pcg_maxit;     /* reference: 1000 */
    int precision;     /* GLOBE_PREC_* */
    int mask;          /* per-column convergence masking */
    uint64_t seed;     /* probe seed when probes == NULL */
    const double* probes;  /* optional injected draws, consumed in order */
    int64_t probes_len;
    int fuse;          /* 1: one block solve of MME + probes per gradient evaluation
                          (globe_aireml_eval); 0: two solves, as the reference */
    int digits;        /* GLOBE_PREC_MIXED: base-32 digits per column for this run
                          (globe_set_digits); 0 keeps the context's setting */
} globe_aireml_opts;

typedef struct {
    int iterations;     /* AIREML iterations run */
    int converged;
    double theta[5];    /* final components */
    double se[5];       /* sqrt(diag(AI^-1)) */
    double ai[25];
    double grad[5];
    int64_t grad_evals; /* gradient evaluations (each one fitMME + trace) */
    int64_t pcg_rhs_iters;
} globe_aireml_result;

/* The AIREML loop of runAIREML (main + oneIter_AIREML,
 * varCompEst.cpp:1148-1497) on the loaded records and dense GRM; progress
 * is written to `log_path` (NULL: no log) in the reference's .log layout. */
int globe_aireml_run(globe_ctx* ctx, const globe_aireml_opts* opts, const char* log_path,
                     globe_aireml_result* result);

/* ---- files ------------------------------------------------------------ */

/* Record table reader (checkInputs + readInputData, PCGsolver.cpp:465-587):
 * first call with X == NULL to get Nrec, N, p; second call fills indiv
 * (0-based), X (Nrec x (p+1), time last) and y. */
int globe_read_records(const char* path, int64_t* Nrec, int32_t* N, int32_t* p, int32_t* indiv,
                       double* X, double* y, char* err, int errlen);
/* Record table of the model without time effects (readInputData,
 * varCompEst_reducedModel_noTime.cpp:191-247): INDIV and PHENO by name, every
 * other column in file order a covariate; p = number of covariates and X is
 * Nrec x p.  To load it, pass p - 1 to globe_load_records (its last covariate
 * then takes the place of time, which the model does not use). */
int globe_read_records_no_time(const char* path, int64_t* Nrec, int32_t* N, int32_t* p, int32_t* indiv,
                               double* X, double* y, char* err, int errlen);
/* saveVector (utils.cpp:18-34): int32 length + float32 payload. */
int globe_save_vector_f32(const char* path, const double* v, int32_t n);
/* Same layout with a float64 payload (what the float->double build of the
 * reference writes; used for full-precision outputs). */
int globe_save_vector_f64(const char* path, const double* v, int32_t n);
/* PLINK trio: M = number of lines of <prefix>.bim (PCGsolver.cpp:631-639);
 * checks the .bed magic (6C 1B 01, SNP-major; :648-664) and that the file
 * holds M rows of ceil(N/4) bytes. */
int globe_bed_dims(const char* prefix, int32_t N, int64_t* M, char* err, int errlen);
/* Reads the M x ceil(N/4) payload after the magic into `payload`. */
int globe_read_bed(const char* prefix, int32_t N, int64_t M, uint8_t* payload, char* err, int errlen);
/* <prefix>.grm.bin: N(N+1)/2 float32 (readFullGRM, PCGsolver.cpp:778-809). */
int globe_read_grm(const char* prefix, int32_t N, float* grm_lt, char* err, int errlen);
/* Writes <prefix>.grm.bin: the N(N+1)/2 float32 values of grm_lt, no header
 * (the layout globe_read_grm and readFullGRM read). */
int globe_write_grm(const char* prefix, const float* grm_lt, int32_t N, char* err, int errlen);

/* ---- profiling ---------------------------------------------------------- */

/* CUDA-event timing of the context's own kernels, recorded on its stream.
 * No reference counterpart (the reference prints wall time per iteration,
 * varCompEst.cpp:1462-1464). */
#define GLOBE_PROF_GRM 0        /* one GRM product (all its launches) */
#define GLOBE_PROF_GRM_PASS1 1  /* genotype pass 1 (w = Zs v) / dense kernel */
#define GLOBE_PROF_GRM_PASS2 2  /* genotype pass 2 (Zs' w) */
#define GLOBE_PROF_PCG_ITER 3   /* one block-PCG iteration */
#define GLOBE_PROF_GRM_BUILD 4  /* one globe_grm_build[_dev] (all its launches) */
#define GLOBE_PROF_GRM_BUILD_GEMM 5  /* its GEMM launches (tensor-core or FP64) */
#define GLOBE_PROF_KINDS 8
/* on != 0 starts recording (and clears the counters); 0 stops. */
int globe_prof_enable(globe_ctx* ctx, int on);
/* Launch count and summed duration (ms) of `kind` since enabling;
 * synchronises the stream. */
int globe_prof_query(globe_ctx* ctx, int kind, int64_t* count, double* ms);

/* ---- benchmarking support --------------------------------------------- */

/* Fill d_bed (M rows, `stride` bytes apart) with PLINK-coded genotypes
 * drawn on the GPU: per SNP an A1 frequency U(maf_lo, maf_hi) (A1 flipped
 * for half the SNPs), g ~ Binomial(2, f), missing with probability
 * miss_rate, padding pairs 00.  Counter-based: the same (seed, SNP,
 * individual) always gives the same genotype.  No reference counterpart. */
int globe_synth_bed_dev(globe_ctx* ctx, uint8_t* d_bed, int64_t M, int32_t N, int64_t stride,
                        uint64_t seed, float maf_lo, float maf_hi, float miss_rate);

#ifdef __cplusplus
}
#endif
#endif /* GLOBE_H */
