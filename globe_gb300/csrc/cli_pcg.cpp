// runPCGsolver -- drop-in for the reference program of the same name
// (PCGsolver.cpp:235-463): same flags, same inputs, same output files, with
// the solve on the GPU through the C ABI in include/globe.h.
//
// Extra flags (absent from the reference): --precision fp64|mixed,
// --pcgTol <v> (default 1e-5, PCGsolver.cpp:54), --pcgMaxIter <n> (1000),
// --device <id>, --save64 (also write <out>_*.f64.bin with float64 payloads),
// --digits <n> (with --precision mixed: base-32 digits per column, globe_set_digits).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "globe.h"

static void usage(const char* prog) {
    std::fprintf(stderr,
                 "Usage:\n%s --input <file> --output <prefix>  --sig2e <val> --sig2g <val> --sig2b0 <val> "
                 "--sigb01 <val> --sig2b1 <val>\n  EITHER:  --geno <plinkPrefix>\n      OR:  --grm <grmPrefix>\n"
                 " Optional:\n   [--debug] [--minMAF val] [--maxMissingRate val]\n"
                 "   [--precision fp64|mixed] [--pcgTol val] [--pcgMaxIter n] [--device id] [--save64] [--digits n]\n",
                 prog);
}

static bool parse_float(const std::string& s, float* out) {
    char* end = nullptr;
    float v = std::strtof(s.c_str(), &end);
    if (end == s.c_str()) return false;
    *out = v;
    return true;
}

static int fail(const char* msg) {
    std::fprintf(stderr, "[Error] %s\n", msg);
    return EXIT_FAILURE;
}

int main(int argc, char** argv) {
    if (argc < 2) {
        usage(argv[0]);
        return EXIT_FAILURE;
    }
    bool debug = false, save64 = false;
    float min_maf = 0.01f, max_miss = 0.2f;
    std::string geno, grm, input, output;
    float vc_f[5] = {0.1f, 0.1f, 0.1f, 0.1f, 0.1f};
    bool have[5] = {false, false, false, false, false};
    const char* vcflag[5] = {"--sig2e", "--sig2g", "--sig2b0", "--sigb01", "--sig2b1"};
    int precision = GLOBE_PREC_FP64, device = 0, maxit = 1000, digits = 0;
    double tol = 1e-5;
    bool have_in = false, have_out = false;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        auto next = [&](std::string* v) -> bool {
            if (i + 1 >= argc) {
                std::fprintf(stderr, "[Error] Flag %s expects an argument.\n", a.c_str());
                return false;
            }
            *v = argv[++i];
            return true;
        };
        std::string v;
        if (a == "--debug") {
            debug = true;
        } else if (a == "--save64") {
            save64 = true;
        } else if (a == "--minMAF" || a == "--maxMissingRate") {
            if (!next(&v)) return EXIT_FAILURE;
            float f;
            if (!parse_float(v, &f)) return fail(("cannot parse value of " + a).c_str());
            (a == "--minMAF" ? min_maf : max_miss) = f;
        } else if (a == "--geno") {
            if (!next(&geno)) return EXIT_FAILURE;
        } else if (a == "--grm") {
            if (!next(&grm)) return EXIT_FAILURE;
        } else if (a == "--input") {
            if (!next(&input)) return EXIT_FAILURE;
            have_in = true;
        } else if (a == "--output") {
            if (!next(&output)) return EXIT_FAILURE;
            have_out = true;
        } else if (a == "--precision") {
            if (!next(&v)) return EXIT_FAILURE;
            if (v == "fp64") precision = GLOBE_PREC_FP64;
            else if (v == "mixed") precision = GLOBE_PREC_MIXED;
            else return fail("--precision must be fp64 or mixed");
        } else if (a == "--pcgTol") {
            if (!next(&v)) return EXIT_FAILURE;
            tol = std::atof(v.c_str());
        } else if (a == "--pcgMaxIter") {
            if (!next(&v)) return EXIT_FAILURE;
            maxit = std::atoi(v.c_str());
        } else if (a == "--device") {
            if (!next(&v)) return EXIT_FAILURE;
            device = std::atoi(v.c_str());
        } else if (a == "--digits") {
            if (!next(&v)) return EXIT_FAILURE;
            digits = std::atoi(v.c_str());
        } else {
            int k = -1;
            for (int q = 0; q < 5; ++q)
                if (a == vcflag[q]) k = q;
            if (k < 0) {
                std::fprintf(stderr, "[Error] Unknown flag: %s\n", a.c_str());
                return EXIT_FAILURE;
            }
            if (!next(&v)) return EXIT_FAILURE;
            if (!parse_float(v, &vc_f[k])) return fail(("cannot parse value of " + a).c_str());
            have[k] = true;
        }
    }
    if (!have_in || !have_out || !have[0] || !have[1] || !have[2] || !have[3] || !have[4])
        return fail("Missing required flags.");
    if (min_maf < 0 || min_maf > 0.5f || max_miss < 0 || max_miss > 1.0f)
        return fail("Invalid MAF or missing rate thresholds.");
    if (geno.empty() == grm.empty())
        return fail("You must specify exactly one of:\n  --geno <plinkPrefix>\nOR\n  --grm  <grmPrefix>\nbut not both.");

    char err[1024] = {0};
    int64_t Nrec = 0;
    int32_t N = 0, p = 0;
    if (globe_read_records(input.c_str(), &Nrec, &N, &p, nullptr, nullptr, nullptr, err, sizeof err)) return fail(err);
    std::vector<int32_t> indiv(Nrec);
    std::vector<double> X((size_t)Nrec * (p + 1)), y(Nrec);
    if (globe_read_records(input.c_str(), &Nrec, &N, &p, indiv.data(), X.data(), y.data(), err, sizeof err))
        return fail(err);
    if (debug)
        std::printf("[checkInputs] Found:\n   N = %d unique individuals\n   p = %d fixed effects (not counting TIME)\n"
                    "   Nrec = %lld records total.\n", N, p, (long long)Nrec);
    globe_ctx* ctx = nullptr;
    if (globe_create(&ctx, device)) return fail(globe_last_error(nullptr));
    auto die = [&](const char* what) {
        std::fprintf(stderr, "[Error] %s: %s\n", what, globe_last_error(ctx));
        globe_destroy(ctx);
        return EXIT_FAILURE;
    };
    if (digits && globe_set_digits(ctx, digits)) return die("digits");
    if (globe_load_records(ctx, Nrec, N, p, indiv.data(), X.data(), y.data())) return die("records");
    if (!geno.empty()) {
        // streamed from disk in chunks (globe_load_bed_file): the file never sits whole in host memory
        globe_bed_info bi{};
        if (globe_load_bed_file(ctx, geno.c_str(), min_maf, max_miss, 0, nullptr, nullptr, nullptr, nullptr, nullptr,
                                &bi))
            return die("genotypes");
        const long long M = (long long)bi.M;
        std::printf("[prepGenotypeInput] Processed %lld / %lld SNPs.\n", M, M);
        if (debug) std::printf("[prepGenotypeInput] Filtered SNPs = %lld / %lld\n", (long long)bi.kept, M);
    } else {
        std::vector<float> A((size_t)N * (N + 1) / 2);
        if (globe_read_grm(grm.c_str(), N, A.data(), err, sizeof err)) {
            globe_destroy(ctx);
            return fail(err);
        }
        if (globe_load_grm(ctx, A.data(), N)) return die("GRM");
    }
    std::printf("[prepareAllInputs] Input prepared successfully.\n");
    const double vc[5] = {vc_f[0], vc_f[1], vc_f[2], vc_f[3], vc_f[4]};  // float values, as std::stof gives
    if (globe_set_vc(ctx, vc)) return die("variance components");
    globe_pcg_opts o{tol, maxit, GLOBE_RULE_PCGSOLVER, GLOBE_X0_ZERO, 0, precision};
    globe_pcg_info info{};
    std::vector<double> beta(p + 1), uhat(N), bhat(2 * (size_t)N);
    std::printf("[runPCG_multi] Starting PCG solver...\n");
    if (globe_mme(ctx, &o, beta.data(), uhat.data(), bhat.data(), nullptr, &info)) return die("solve");
    if (info.stagnated)
        std::printf("[runPCG_multi] Stalled (no significant improvement for 10 iters).\n");
    std::printf("[runPCG_multi] Converged at iteration %d\n", info.iters);
    struct Out {
        const char* suffix;
        const std::vector<double>* v;
    } outs[3] = {{"_beta", &beta}, {"_uhat", &uhat}, {"_bhat", &bhat}};
    for (auto& o2 : outs) {
        std::string fn = output + o2.suffix + ".bin";
        if (globe_save_vector_f32(fn.c_str(), o2.v->data(), (int32_t)o2.v->size()))
            std::fprintf(stderr, "[saveVector] Error writing file: %s\n", fn.c_str());
        else std::printf("[saveVector] Vector saved: %s\n", fn.c_str());
        if (save64) {
            std::string f64 = output + o2.suffix + ".f64.bin";
            if (globe_save_vector_f64(f64.c_str(), o2.v->data(), (int32_t)o2.v->size()))
                std::fprintf(stderr, "[saveVector] Error writing file: %s\n", f64.c_str());
        }
    }
    globe_destroy(ctx);
    std::printf("[main] Done.\n");
    return 0;
}
