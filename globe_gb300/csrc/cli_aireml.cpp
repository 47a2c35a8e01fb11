// runAIREML -- drop-in for the reference program of the same name.  Built a
// second time with GLOBE_NO_TIME defined, it is runAIREML_reducedModel
// (varCompEst_reducedModel_noTime.cpp:93-129, :967-1106): no time effects,
// components sig2e and sig2g (defaults 0.5, 0.5), record table of INDIV,
// PHENO and covariates.
// (varCompEst.cpp:103-133, :1347-1500): positional <input> <grm_prefix>
// <output_prefix>, optional --maxiter --tol --numMC --sig2e --sig2g --sig2b0
// --sigb01 --sig2b1 (unknown flags ignored, as in the reference), progress
// and the final "sigma +- SE" block written to <output_prefix>.log.
//
// Extra flags: --precision fp64|mixed, --pcgTol <v> (default 1e-5),
// --device <id>, --seed <n> (GPU probe stream), --probes <file> (float64
// standard normal draws consumed in the reference's sample_Yvs order).
// --geno <plink_prefix> [--minMAF v] [--maxMissingRate v] takes the genetic
// relationships from PLINK genotypes, as runPCGsolver --geno does
// (PCGsolver.cpp:615-763), instead of <grm_prefix>; the reference's
// runAIREML reads only a dense GRM.
// Each gradient evaluation solves the MME right-hand sides and the probes as
// one block PCG (globe_aireml_eval); --separateSolves solves them one after
// the other, as the reference does.  --digits <n> (with --precision mixed):
// base-32 digits per column of the tensor-core product (globe_set_digits).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "globe.h"

#ifdef GLOBE_NO_TIME
constexpr int NVC = 2;
#else
constexpr int NVC = 5;
#endif

static int fail(const char* msg) {
    std::fprintf(stderr, "Error: %s\n", msg);
    return EXIT_FAILURE;
}

int main(int argc, char** argv) {
    if (argc < 4) {
#ifdef GLOBE_NO_TIME
        std::fprintf(stderr,
                     "Usage: %s <input_filename> <grm_prefix> <output_prefix> [--maxiter <int>] [--tol <float>] "
                     "[--numMC <int>] [--sig2e <float>] [--sig2g <float>]\n",
                     argv[0]);
#else
        std::fprintf(stderr,
                     "Usage: %s <input_filename> <grm_prefix> <output_prefix> [--maxiter: optional] [--tol: optional] "
                     "[--numMC: optional] [--sig2e: optional] [--sig2g: optional] [--sig2b0: optional] [--sigb01: "
                     "optional] [--sig2b1: optional]\n",
                     argv[0]);
#endif
        return EXIT_FAILURE;
    }
    std::string input = argv[1], grm = argv[2], outp = argv[3], probes_file, geno;
    float min_maf = 0.01f, max_miss = 0.2f;   // runPCGsolver's defaults (PCGsolver.cpp:34-35)
    int fuse = 1, digits = 0;
    int maxiter = 50, numMC = 15, precision = GLOBE_PREC_FP64, device = 0;
    float tol = 1e-3f;
#ifdef GLOBE_NO_TIME
    // defaults of the reduced VarCompDataStruct (varCompEst_reducedModel_noTime.cpp:43-45)
    float th[5] = {0.5f, 0.5f, 0.0f, 0.0f, 0.0f};
#else
    // defaults of VarCompDataStruct (varCompEst.cpp:48-52), as float
    float th[5] = {0.5f, 0.3f, 0.2f, 0.1f, 0.1f};
#endif
    const char* vcflag[5] = {"--sig2e", "--sig2g", "--sig2b0", "--sigb01", "--sig2b1"};
    double pcg_tol = 1e-5;
    unsigned long long seed = 12345;
    for (int i = 4; i < argc; ++i) {
        std::string a = argv[i];
        bool has = i + 1 < argc;
        if (a == "--maxiter" && has) maxiter = std::atoi(argv[++i]);
        else if (a == "--tol" && has) tol = std::strtof(argv[++i], nullptr);
        else if (a == "--numMC" && has) numMC = std::atoi(argv[++i]);
        else if (a == "--precision" && has) {
            std::string v = argv[++i];
            if (v == "fp64") precision = GLOBE_PREC_FP64;
            else if (v == "mixed") precision = GLOBE_PREC_MIXED;
            else return fail("--precision must be fp64 or mixed");
        } else if (a == "--pcgTol" && has) pcg_tol = std::atof(argv[++i]);
        else if (a == "--device" && has) device = std::atoi(argv[++i]);
        else if (a == "--seed" && has) seed = std::strtoull(argv[++i], nullptr, 10);
        else if (a == "--probes" && has) probes_file = argv[++i];
        else if (a == "--geno" && has) geno = argv[++i];
        else if (a == "--separateSolves") fuse = 0;
        else if (a == "--digits" && has) digits = std::atoi(argv[++i]);
        else if (a == "--minMAF" && has) min_maf = std::strtof(argv[++i], nullptr);
        else if (a == "--maxMissingRate" && has) max_miss = std::strtof(argv[++i], nullptr);
        else {
            for (int q = 0; q < NVC; ++q)
                if (a == vcflag[q] && has) th[q] = std::strtof(argv[++i], nullptr);
        }
    }
    char err[1024] = {0};
    int64_t Nrec = 0;
    int32_t N = 0, p = 0;
#ifdef GLOBE_NO_TIME
    // every column but INDIV and PHENO is a covariate; the last one stands in for time,
    // which this model does not use (its time-effect components are zero)
    if (globe_read_records_no_time(input.c_str(), &Nrec, &N, &p, nullptr, nullptr, nullptr, err, sizeof err))
        return fail(err);
    if (p < 1) return fail("the record table needs at least one covariate column (e.g. an intercept)");
    std::vector<int32_t> indiv(Nrec);
    std::vector<double> X((size_t)Nrec * p), y(Nrec);
    if (globe_read_records_no_time(input.c_str(), &Nrec, &N, &p, indiv.data(), X.data(), y.data(), err, sizeof err))
        return fail(err);
    std::printf("Found N = %d indivuduals, \n      p = %d fixed effects, and\n      Nrec = %lld records in the "
                "input file.\n", N, p, (long long)Nrec);
    p -= 1;
#else
    if (globe_read_records(input.c_str(), &Nrec, &N, &p, nullptr, nullptr, nullptr, err, sizeof err)) return fail(err);
    std::vector<int32_t> indiv(Nrec);
    std::vector<double> X((size_t)Nrec * (p + 1)), y(Nrec);
    if (globe_read_records(input.c_str(), &Nrec, &N, &p, indiv.data(), X.data(), y.data(), err, sizeof err))
        return fail(err);
    std::printf("Found N = %d indivuduals, \n      p = %d fixed effects (in addition to TIME), and\n      Nrec = %lld "
                "records in the input file.\n", N, p, (long long)Nrec);
#endif
    std::vector<float> A;
    if (geno.empty()) {
        A.resize((size_t)N * (N + 1) / 2);
        if (globe_read_grm(grm.c_str(), N, A.data(), err, sizeof err)) return fail(err);
    }
    std::vector<double> probes;
    if (!probes_file.empty()) {
        FILE* f = std::fopen(probes_file.c_str(), "rb");
        if (!f) return fail("cannot open --probes file");
        double buf[4096];
        size_t got;
        while ((got = std::fread(buf, sizeof(double), 4096, f)) > 0) probes.insert(probes.end(), buf, buf + got);
        std::fclose(f);
    }
    globe_ctx* ctx = nullptr;
    if (globe_create(&ctx, device)) return fail(globe_last_error(nullptr));
    auto die = [&](const char* what) {
        std::fprintf(stderr, "Error (%s): %s\n", what, globe_last_error(ctx));
        globe_destroy(ctx);
        return EXIT_FAILURE;
    };
#ifdef GLOBE_NO_TIME
    if (globe_set_model(ctx, GLOBE_MODEL_NO_TIME)) return die("model");
#endif
    if (globe_load_records(ctx, Nrec, N, p, indiv.data(), X.data(), y.data())) return die("records");
    if (geno.empty()) {
        if (globe_load_grm(ctx, A.data(), N)) return die("GRM");
    } else {
        // streamed from disk in chunks (globe_load_bed_file)
        globe_bed_info info{};
        if (globe_load_bed_file(ctx, geno.c_str(), min_maf, max_miss, 0, nullptr, nullptr, nullptr, nullptr, nullptr,
                                &info))
            return die("genotypes");
        std::printf("%lld of %lld SNPs pass the MAF / missingness filter.\n", (long long)info.kept,
                    (long long)info.M);
    }
    std::printf("Input files read and processed successfully.\nRunning AI-REML...\n");
    globe_aireml_opts o{};
    o.maxiter = maxiter;
    o.tol = tol;
    o.numMC = numMC;
    for (int k = 0; k < 5; ++k) o.theta0[k] = th[k];
    o.pcg_tol = pcg_tol;
    o.pcg_maxit = 1000;
    o.precision = precision;
    o.mask = 0;
    o.seed = seed;
    o.fuse = fuse;
    o.digits = digits;
    o.probes = probes.empty() ? nullptr : probes.data();
    o.probes_len = (int64_t)probes.size();
    globe_aireml_result r{};
    std::string log = outp + ".log";
    if (globe_aireml_run(ctx, &o, log.c_str(), &r)) return die("AIREML");
    const char* nm[5] = {"   sig2e", "   sig2g", "  sig2b0", "  sigb01", "  sig2b1"};
    std::printf("Final variance components +- SEs (%d iterations%s):\n", r.iterations,
                r.converged ? ", converged" : "");
    for (int k = 0; k < NVC; ++k) std::printf("%s = %.9g +- %.9g\n", nm[k], r.theta[k], r.se[k]);
    globe_destroy(ctx);
    return 0;
}
