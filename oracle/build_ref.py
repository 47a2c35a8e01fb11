#!/usr/bin/env python3
"""Build the upstream GLOBE executables from their own sources, as test oracles.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports or runs what this
script makes; the tests use it to pin the C restatement in
``oracle/globe_oracle.c`` and to make the golden fixtures under
``tests/golden/``.

The reference tree is read in place (``REF`` below, default ``/root/reference``).
Patched variants are written to a scratch copy under ``/tmp`` (never into this
repository) and every binary goes to ``oracle/_ref/`` (git-ignored).  The
reference's own CMake build is not used: each program is one translation unit
plus ``src/utils.cpp`` with the vendored header-only Eigen, so ``g++`` is
called on those files directly.

Variants:

* ``runPCGsolver``        -- FP32 as shipped (``src/PCGsolver.cpp``).
* ``runPCGsolver_stats``  -- FP32 plus one print per SNP of the counts, the
  float ``maf`` and ``missRate`` (hex float, bit-exact) and the keep decision,
  inserted after ``PCGsolver.cpp:733`` (the ``missRate`` line).
* ``runPCGsolver64``      -- FP64: ``float``->``double`` over the sources, the
  Eigen aliases renamed, PCG tolerance 1e-13 (``PCGsolver.cpp:54``).
* ``runAIREML64``         -- FP64 ``src/varCompEst.cpp`` with (i) the normal
  draws of ``generate_standard_normal`` (``varCompEst.cpp:763-772``) read
  from the file named by ``GLOBE_PROBE_FILE`` (float64, consumed in call
  order), (ii) PCG tolerance ``GLOBE_REF_TOL`` (compile-time, default 1e-12)
  in place of the hard-coded 1e-5 (``:633,950,1025``), (iii) 17-digit
  printing.  Links the bundled NLopt, which is an x86-64 binary: this
  variant is skipped on other hosts.
* ``runAIREML``           -- FP32 as shipped (x86-64 only, bundled NLopt).
* ``runAIREML_reduced64`` -- FP64 ``src/varCompEst_reducedModel_noTime.cpp``
  (the reference's ``runAIREML_reducedModel``) with the same three patches as
  ``runAIREML64`` (x86-64 only, bundled NLopt).
"""
import os
import platform
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF = os.environ.get("GLOBE_REFERENCE_DIR", "/root/reference")
TMP = "/tmp/globe_ref_src"


def _read(p):
    with open(p) as f:
        return f.read()


def _write(p, s):
    os.makedirs(os.path.dirname(p), exist_ok=True)
    with open(p, "w") as f:
        f.write(s)


def _fp64(src):
    """Type substitution: every float becomes double, and the float Eigen types their double forms."""
    s = re.sub(r"\bfloat\b", "double", src)
    s = re.sub(r"Eigen::MatrixXf|\bMatrixXf\b", "MatT", s)
    s = re.sub(r"Eigen::VectorXf|\bVectorXf\b", "VecT", s)
    return s


def _patch_stats(src):
    anchor = "float missRate = (float)missing_count / (float)N;"
    assert anchor in src, "stats anchor not found"
    ins = anchor + (
        "\n        { bool _k = (maf >= maf_threshold && maf <= (1.0f - maf_threshold)"
        " && missRate <= missing_threshold);"
        ' std::printf("[snpstat] %zu %zu %zu %a %a %d\\n", snp_i, alt_count, missing_count,'
        " (double)maf, (double)missRate, (int)_k); }")
    return src.replace(anchor, ins)


def _grm_read_f32(s, old, dst, cnt):
    """The .grm.bin payload is float32 on disk; the double build must widen it."""
    assert old in s, old
    new = ("{ std::vector<float> _t(%s); file.read(reinterpret_cast<char*>(_t.data()), (%s) * sizeof(float));"
           " for (size_t _i = 0; _i < (size_t)(%s); ++_i) %s[_i] = _t[_i]; }" % (cnt, cnt, cnt, dst))
    return s.replace(old, new)


def _patch_pcg64(src):
    s = _fp64(src)
    s = _grm_read_f32(s, "file.read(reinterpret_cast<char*>(gData.GRM_lt.data()), nelt * sizeof(double));",
                      "gData.GRM_lt", "nelt")
    s = s.replace("double PCG_TOL = 1e-5f;", "double PCG_TOL = 1e-13;")
    assert "1e-13" in s
    return s


def _patch_aireml64(src):
    s = _fp64(src)
    s = _grm_read_f32(s, "file.read(reinterpret_cast<char*>(A_vecLT.data()), A_vecLT.size() * sizeof(double));",
                      "A_vecLT", "A_vecLT.size()")
    # probe injection: replace the body of generate_standard_normal
    pat = re.compile(r"VecT generate_standard_normal\(int dimension\) \{.*?\n\}", re.S)
    body = (
        "static FILE* g_probe_fp = nullptr;\n"
        "VecT generate_standard_normal(int dimension) {\n"
        "    if (!g_probe_fp) {\n"
        "        const char* fn = std::getenv(\"GLOBE_PROBE_FILE\");\n"
        "        if (!fn || !(g_probe_fp = std::fopen(fn, \"rb\"))) {\n"
        "            std::fprintf(stderr, \"GLOBE_PROBE_FILE missing\\n\"); std::exit(3); }\n"
        "    }\n"
        "    VecT z(dimension);\n"
        "    if (std::fread(z.data(), sizeof(double), dimension, g_probe_fp) != (size_t)dimension) {\n"
        "        std::fprintf(stderr, \"probe file exhausted\\n\"); std::exit(4); }\n"
        "    return z;\n"
        "}")
    s, n = pat.subn(lambda m: body, s)
    assert n == 1, "generate_standard_normal not found"
    s = s.replace("double tol = 1e-5;", "double tol = GLOBE_REF_TOL;")
    s = s.replace("Yvs, Vinv_Yvs, 1e-5, 1000, true, false", "Yvs, Vinv_Yvs, GLOBE_REF_TOL, 1000, true, false")
    s = s.replace("f_theta, Vinv_f_theta, 1e-5, 1000, false, true",
                  "f_theta, Vinv_f_theta, GLOBE_REF_TOL, 1000, false, true")
    assert s.count("GLOBE_REF_TOL") == 3, s.count("GLOBE_REF_TOL")
    anchor = "std::cout.rdbuf(&tee_streambuf);"
    assert anchor in s
    s = s.replace(anchor, anchor + "\n    std::cout << std::setprecision(17);")
    s = "#include <iomanip>\n#include <cstdio>\n#ifndef GLOBE_REF_TOL\n#define GLOBE_REF_TOL 1e-12\n#endif\n" + s
    return s


def _patch_reduced64(src):
    """The reduced model (no time effects) with runAIREML64's patches: probes from
    GLOBE_PROBE_FILE, PCG tolerance GLOBE_REF_TOL, 17-digit printing."""
    s = _fp64(src)
    s = _grm_read_f32(s, "file.read(reinterpret_cast<char*>(CohortData.A_vecLT.data()), nTri * sizeof(double));",
                      "CohortData.A_vecLT", "nTri")
    pat = re.compile(r"VecT generate_standard_normal\(int dimension\) \{.*?\n\}", re.S)
    body = (
        "static FILE* g_probe_fp = nullptr;\n"
        "VecT generate_standard_normal(int dimension) {\n"
        "    if (!g_probe_fp) {\n"
        "        const char* fn = std::getenv(\"GLOBE_PROBE_FILE\");\n"
        "        if (!fn || !(g_probe_fp = std::fopen(fn, \"rb\"))) {\n"
        "            std::fprintf(stderr, \"GLOBE_PROBE_FILE missing\\n\"); std::exit(3); }\n"
        "    }\n"
        "    VecT z(dimension);\n"
        "    if (std::fread(z.data(), sizeof(double), dimension, g_probe_fp) != (size_t)dimension) {\n"
        "        std::fprintf(stderr, \"probe file exhausted\\n\"); std::exit(4); }\n"
        "    return z;\n"
        "}")
    s, n = pat.subn(lambda m: body, s)
    assert n == 1, "generate_standard_normal not found"
    s = s.replace("double tol = 1e-5;", "double tol = GLOBE_REF_TOL;")
    s = s.replace("Yvs, Vinv_Yvs, 1e-5, 1000, true, false", "Yvs, Vinv_Yvs, GLOBE_REF_TOL, 1000, true, false")
    s = s.replace("f_theta, Vinv_f_theta, 1e-5, 1000, false, true",
                  "f_theta, Vinv_f_theta, GLOBE_REF_TOL, 1000, false, true")
    assert s.count("GLOBE_REF_TOL") == 3, s.count("GLOBE_REF_TOL")
    anchor = "std::cout.rdbuf(&tee_streambuf);"
    assert anchor in s
    s = s.replace(anchor, anchor + "\n    std::cout << std::setprecision(17);")
    s = "#include <iomanip>\n#include <cstdio>\n#ifndef GLOBE_REF_TOL\n#define GLOBE_REF_TOL 1e-12\n#endif\n" + s
    return s


def _compile(args):
    name, srcs, extra = args
    out = os.path.join(OUT, name)
    eigen = os.path.join(REF, "thirdParty", "eigen")
    cflags = [a for a in extra if not (a.startswith("-l") or a.startswith("-Wl"))]
    ldflags = [a for a in extra if a.startswith("-l") or a.startswith("-Wl")]
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-w", "-I", eigen] + cflags + srcs + ldflags + ["-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("failed to build %s:\n%s" % (name, r.stderr[-4000:]))
    return name


def main():
    if not os.path.isdir(os.path.join(REF, "src")):
        print("reference sources not present; oracle/_ref not built")
        return 0
    os.makedirs(OUT, exist_ok=True)
    if os.path.isdir(TMP):
        shutil.rmtree(TMP)
    src = os.path.join(REF, "src")
    pcg = _read(os.path.join(src, "PCGsolver.cpp"))
    vce = _read(os.path.join(src, "varCompEst.cpp"))
    red = _read(os.path.join(src, "varCompEst_reducedModel_noTime.cpp"))
    utc = _read(os.path.join(src, "utils.cpp"))
    uth = _read(os.path.join(src, "utils.hpp"))
    # FP32 stats variant
    _write(os.path.join(TMP, "f32s", "PCGsolver.cpp"), "#include <cstdio>\n" + _patch_stats(pcg))
    # FP64 variants (utils too: saveVector then writes float64 payloads)
    _write(os.path.join(TMP, "f64", "utils.hpp"), _fp64(uth))
    _write(os.path.join(TMP, "f64", "utils.cpp"), _fp64(utc))
    _write(os.path.join(TMP, "f64", "PCGsolver.cpp"), _patch_pcg64(pcg))
    _write(os.path.join(TMP, "f64", "varCompEst.cpp"), _patch_aireml64(vce))
    _write(os.path.join(TMP, "f64", "varCompEst_reduced.cpp"), _patch_reduced64(red))
    jobs = [
        ("runPCGsolver", [os.path.join(src, "PCGsolver.cpp"), os.path.join(src, "utils.cpp")], ["-I", src]),
        ("runPCGsolver_stats", [os.path.join(TMP, "f32s", "PCGsolver.cpp"), os.path.join(src, "utils.cpp")],
         ["-I", src]),
        ("runPCGsolver64", [os.path.join(TMP, "f64", "PCGsolver.cpp"), os.path.join(TMP, "f64", "utils.cpp")],
         ["-I", os.path.join(TMP, "f64")]),
    ]
    if platform.machine() in ("x86_64", "AMD64"):
        nl = os.path.join(REF, "thirdParty", "nlopt")
        nlf = ["-I", os.path.join(nl, "include"), "-L", os.path.join(nl, "lib64"), "-lnlopt",
               "-Wl,-rpath," + os.path.join(nl, "lib64")]
        jobs.append(("runAIREML64", [os.path.join(TMP, "f64", "varCompEst.cpp"),
                                     os.path.join(TMP, "f64", "utils.cpp")],
                     ["-I", os.path.join(TMP, "f64")] + nlf))
        jobs.append(("runAIREML", [os.path.join(src, "varCompEst.cpp"), os.path.join(src, "utils.cpp")],
                     ["-I", src] + nlf))
        jobs.append(("runAIREML_reduced64", [os.path.join(TMP, "f64", "varCompEst_reduced.cpp"),
                                             os.path.join(TMP, "f64", "utils.cpp")],
                     ["-I", os.path.join(TMP, "f64")] + nlf))
    with ThreadPoolExecutor(len(jobs)) as ex:
        for n in ex.map(_compile, jobs):
            print("built", os.path.join(OUT, n))
    return 0


if __name__ == "__main__":
    sys.exit(main())
