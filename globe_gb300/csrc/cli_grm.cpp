// buildGRM -- writes the genetic relationship matrix of a PLINK fileset as
// <output_prefix>.grm.bin, the dense input of runPCGsolver --grm and
// runAIREML (readFullGRM, PCGsolver.cpp:778-809; readGRM,
// varCompEst.cpp:270-295), with the standardisation runPCGsolver --geno
// applies on the fly (PCGsolver.cpp:615-763, :826-842): the same MAF and
// missingness filter, A = Zs'Zs / M_kept.  The reference has no such program.
//
//   buildGRM <plink_prefix> <output_prefix> [--minMAF 0.01] [--maxMissingRate 0.2]
//            [--precision mixed|fp64] [--device <id>] [--chunkMB <n>]
//
// N is the number of lines of <plink_prefix>.fam; individual i of the matrix is
// line i of the .fam, which is the INDIV = i+1 of the record tables that use it.
// <output_prefix>.grm.id gets the FID and IID of each .fam line.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "globe.h"

static int fail(const char* msg) {
    std::fprintf(stderr, "Error: %s\n", msg);
    return EXIT_FAILURE;
}

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr,
                     "Usage: %s <plink_prefix> <output_prefix> [--minMAF <float>] [--maxMissingRate <float>] "
                     "[--precision mixed|fp64] [--device <int>] [--chunkMB <int>]\n",
                     argv[0]);
        return EXIT_FAILURE;
    }
    std::string geno = argv[1], outp = argv[2];
    float min_maf = 0.01f, max_miss = 0.2f;   // runPCGsolver's defaults (PCGsolver.cpp:34-35)
    int precision = GLOBE_PREC_MIXED, device = 0;
    long long chunk_mb = 0;
    for (int i = 3; i < argc; ++i) {
        std::string a = argv[i];
        bool has = i + 1 < argc;
        if (a == "--minMAF" && has) min_maf = std::strtof(argv[++i], nullptr);
        else if (a == "--maxMissingRate" && has) max_miss = std::strtof(argv[++i], nullptr);
        else if (a == "--precision" && has) {
            std::string v = argv[++i];
            if (v == "fp64") precision = GLOBE_PREC_FP64;
            else if (v == "mixed") precision = GLOBE_PREC_MIXED;
            else return fail("--precision must be fp64 or mixed");
        } else if (a == "--device" && has) device = std::atoi(argv[++i]);
        else if (a == "--chunkMB" && has) chunk_mb = std::atoll(argv[++i]);
        else return fail(("unknown argument " + a).c_str());
    }
    // individuals: the non-empty lines of the .fam
    std::vector<std::string> ids;
    {
        std::ifstream fam(geno + ".fam");
        if (!fam) return fail(("cannot open " + geno + ".fam").c_str());
        std::string line;
        while (std::getline(fam, line)) {
            std::istringstream ss(line);
            std::string fid, iid;
            if (!(ss >> fid)) continue;
            if (!(ss >> iid)) iid = fid;
            ids.push_back(fid + "\t" + iid);
        }
    }
    if (ids.empty()) return fail("the .fam file lists no individuals");
    const int32_t N = (int32_t)ids.size();
    auto t0 = std::chrono::steady_clock::now();
    globe_ctx* ctx = nullptr;
    if (globe_create(&ctx, device)) return fail(globe_last_error(nullptr));
    auto die = [&](const char* what) {
        std::fprintf(stderr, "Error (%s): %s\n", what, globe_last_error(ctx));
        globe_destroy(ctx);
        return EXIT_FAILURE;
    };
    if (globe_set_individuals(ctx, N)) return die("individuals");
    if (globe_set_precision(ctx, precision)) return die("precision");
    globe_bed_info info{};
    if (globe_load_bed_file(ctx, geno.c_str(), min_maf, max_miss, chunk_mb * (1ll << 20), nullptr, nullptr, nullptr,
                            nullptr, nullptr, &info))
        return die("genotypes");
    std::printf("Found N = %d individuals and M = %lld SNPs; %lld SNPs pass the MAF / missingness filter.\n", N,
                (long long)info.M, (long long)info.kept);
    std::vector<float> lt((size_t)N * ((size_t)N + 1) / 2);
    if (globe_grm_build(ctx, lt.data())) return die("GRM");
    globe_destroy(ctx);
    char err[1024] = {0};
    if (globe_write_grm(outp.c_str(), lt.data(), N, err, sizeof err)) return fail(err);
    {
        std::ofstream idf(outp + ".grm.id");
        for (const auto& s : ids) idf << s << "\n";
        if (!idf) return fail(("cannot write " + outp + ".grm.id").c_str());
    }
    const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("Wrote %s.grm.bin (%lld values, %s) in %.2f s.\n", outp.c_str(), (long long)lt.size(),
                precision == GLOBE_PREC_MIXED ? "tensor cores" : "FP64", sec);
    return 0;
}
