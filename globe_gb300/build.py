"""In-tree build of libglobe_gb300.so and the runPCGsolver / runAIREML programs.

nvcc compiles every translation unit for sm_103a only (one -gencode), in
parallel, into ``globe_gb300/_build``; the shared library lands in
``globe_gb300/`` and the command-line programs in ``globe_gb300/bin``.  The
bounds-checked debug library (``libglobe_gb300_bounds.so``, -DGLOBE_CHECK_BOUNDS)
is built beside it from the same sources.
"""
import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
# GLOBE_BUILD_TAG / GLOBE_NVCC_FLAGS build a variant library (e.g. other pipeline
# depths) next to the default one: lib<tag>.so, objects in _build_<tag>.
TAG = os.environ.get("GLOBE_BUILD_TAG", "")
EXTRA = os.environ.get("GLOBE_NVCC_FLAGS", "").split()
BIN = os.path.join(HERE, "bin")
# variants build() also makes: the bounds-checked debug library (globe_debug_bounds)
VARIANTS = {"bounds": ["-DGLOBE_CHECK_BOUNDS"]}


def lib_path(tag=TAG):
    return os.path.join(HERE, "libglobe_gb300%s.so" % ("_" + tag if tag else ""))


def _build_dir(tag):
    return os.path.join(HERE, "_build" + ("_" + tag if tag else ""))


LIB = lib_path()
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-I", os.path.join(ROOT, "include"), "-I", SRC,
          "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]
LIB_SOURCES = ["api.cu", "k_bed.cu", "k_records.cu", "k_records_df.cu", "k_grm_geno.cu", "k_grm_dense.cu", "k_tc_geno.cu",
               "solver.cu", "noalloc.cu", "ingest.cu", "k_grm_build.cu", "k_tc_dense.cu",
               "aireml.cpp", "io.cpp"]
# program -> (source, extra flags)
CLI = {"runPCGsolver": ("cli_pcg.cpp", []), "runAIREML": ("cli_aireml.cpp", []),
       "runAIREML_reducedModel": ("cli_aireml.cpp", ["-DGLOBE_NO_TIME"]), "buildGRM": ("cli_grm.cpp", [])}


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    return glob.glob(os.path.join(SRC, "*.cuh")) + glob.glob(os.path.join(SRC, "*.hpp")) + \
        [os.path.join(ROOT, "include", "globe.h")]


def _compile(src, build_dir, extra):
    obj = os.path.join(build_dir, os.path.basename(src) + ".o")
    if not _newer(obj, [src] + _headers()):
        return obj
    cmd = [NVCC] + COMMON + extra + (ARCH if src.endswith(".cu") else []) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-6000:]))
    if r.stderr.strip():
        sys.stderr.write(r.stderr)
    return obj


def _build_lib(tag, extra, workers):
    build_dir, lib = _build_dir(tag), lib_path(tag)
    os.makedirs(build_dir, exist_ok=True)
    srcs = [os.path.join(SRC, s) for s in LIB_SOURCES]
    with ThreadPoolExecutor(workers) as ex:
        objs = list(ex.map(lambda f: _compile(f, build_dir, extra), srcs))
    if _newer(lib, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"]
        subprocess.check_call(cmd)
    return lib


def build(verbose=True, variants=True):
    """The library (and, with no GLOBE_BUILD_TAG, the programs and the VARIANTS libraries)."""
    os.makedirs(BIN, exist_ok=True)
    workers = max(1, min(2 * len(LIB_SOURCES), os.cpu_count() or 4))
    jobs = [(TAG, EXTRA)] + ([(t, f) for t, f in VARIANTS.items()] if variants and not TAG else [])
    with ThreadPoolExecutor(len(jobs)) as ex:
        libs = list(ex.map(lambda j: _build_lib(j[0], j[1], workers), jobs))
    lib = libs[0]
    for name, (src, flags) in (CLI.items() if not TAG else []):
        s = os.path.join(SRC, src)
        exe = os.path.join(BIN, name)
        if os.path.exists(s) and _newer(exe, [s, lib] + _headers()):
            cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include")] + flags + [s, "-o", exe,
                   "-L", HERE, "-lglobe_gb300", "-Wl,-rpath,$ORIGIN/.."]
            subprocess.check_call(cmd)
    if verbose:
        for l in libs:
            print("built", l)
    return lib


if __name__ == "__main__":
    build()
