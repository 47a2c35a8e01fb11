#!/usr/bin/env python3
"""Make the golden fixtures in tests/golden/ by running the reference itself.

Run in a container that has the GLOBE sources (oracle/build_ref.py builds
them into oracle/_ref/).  Inputs are written with globe_gb300.synth from fixed
seeds; the reference programs' outputs are stored next to them:

* ``<case>.{txt,bed,bim,fam,grm.bin}``  -- inputs (record table, PLINK, GRM)
* ``<case>_ref.npz``                    -- reference outputs:
    stats_*   per-SNP counts / float32 maf / missing rate / keep from the FP32
              build with the per-SNP print (runPCGsolver_stats);
    f32_*     beta / uhat / bhat of the shipped FP32 build (--geno);
    geno64_*  beta / uhat / bhat of the float->double build (--geno, tol 1e-13);
    grm64_*   the same with --grm.
* ``aireml_small_ref.json`` -- runAIREML (float->double build, PCG tol 1e-12,
  probe draws injected from globe_gb300.synth.normal_stream(PROBE_SEED)):
  per-iteration gradients, AI matrices, steps, rho, accepted components.
* ``reduced_small.{txt,grm.bin}`` + ``reduced_small_ref.json`` -- the same for
  runAIREML_reducedModel (no time effects, components sig2e and sig2g; one
  record per individual; record table INDIV PHENO COV0 COV1 COV2).
* ``geno_small_grmf64_ref.npz`` -- beta / uhat / bhat of the float->double
  runPCGsolver --grm on the GRM of geno_small built by the oracle's
  orc_grm_build with the double allele frequency (the GPU builder's
  convention), next to geno64_* of the same program with --geno.

``python make_golden.py grm_build`` makes only the last fixture (from the
committed geno_small inputs).

Two fixtures at the benchmark configurations' sizes keep only the reference's
outputs: their inputs come from ``globe_gb300.synth.portable_cohort``, which
gives the same bytes on every platform, so the tests regenerate them and check
their SHA-256 against the fixture instead of reading committed copies.

* ``geno_2k_10k_ref.npz`` (``python make_golden.py portable_pcg``) -- the
  runPCGsolver --geno configuration: N=2,000 individuals, 3-10 records each
  (times U[0,5]), intercept + 2 covariates, M=10,000 SNPs, MAF U(0.05,0.5),
  1% missing.  stats_*, f32_* and geno64_* as above.
* ``aireml_dense_2k_ref.json`` (``python make_golden.py portable_aireml``) --
  the dense-GRM runAIREML configuration's structure at N=2,000: Poisson(5)+1
  records (times U[0,10]), a float32 .grm.bin from 5,000 SNPs (MAF
  U(0.01,0.5)), numMC=15, runAIREML64 with injected probes.
"""
import json
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from globe_gb300 import synth  # noqa: E402

sys.path.insert(0, os.path.dirname(HERE))
from helpers import portable_inputs  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")
VC = (0.6, 0.4, 0.4, 0.2, 0.2)
PROBE_SEED = 5
AIREML_NUMMC = 4
AIREML_MAXITER = 6

CASES = {
    # name: (seed, N, M, record dist, T, miss_rate, edge SNPs)
    "geno_small": (7, 203, 1000, ("uniform", 3, 10), 5.0, 0.01, True),
    "tiny": (3, 37, 64, ("uniform", 1, 4), 4.0, 0.05, True),
}


def _vec(fn):
    b = open(fn, "rb").read()
    n = int(np.frombuffer(b[:4], np.int32)[0])
    dt = np.float64 if len(b) - 4 == 8 * n else np.float32
    return np.frombuffer(b[4:], dt)[:n].copy()


def _vcargs(vc):
    return ["--sig2e", repr(vc[0]), "--sig2g", repr(vc[1]), "--sig2b0", repr(vc[2]), "--sigb01", repr(vc[3]),
            "--sig2b1", repr(vc[4])]


def make_pcg_case(name, seed, N, M, recs, T, miss, edge, tmp):
    coh = synth.simulate_cohort(seed, N, M, recs, T, miss_rate=miss, edge_snps=edge)
    pre = synth.write_cohort(HERE, name, coh, grm=True)
    out = {}
    r = subprocess.run([os.path.join(REF, "runPCGsolver_stats"), "--input", pre + ".txt", "--output",
                        os.path.join(tmp, name + "_s"), "--geno", pre] + _vcargs(VC),
                       capture_output=True, text=True, check=True)
    rows = [ln.split() for ln in r.stdout.splitlines() if ln.startswith("[snpstat]")]
    out["stats_alt"] = np.array([int(x[2]) for x in rows], np.int64)
    out["stats_miss"] = np.array([int(x[3]) for x in rows], np.int64)
    out["stats_maf"] = np.array([float.fromhex(x[4]) for x in rows], np.float32)
    out["stats_miss_rate"] = np.array([float.fromhex(x[5]) for x in rows], np.float32)
    out["stats_keep"] = np.array([int(x[6]) for x in rows], np.uint8)
    for tag, exe, src in (("f32", "runPCGsolver", ["--geno", pre]), ("geno64", "runPCGsolver64", ["--geno", pre]),
                          ("grm64", "runPCGsolver64", ["--grm", pre])):
        o = os.path.join(tmp, name + "_" + tag)
        subprocess.run([os.path.join(REF, exe), "--input", pre + ".txt", "--output", o] + src + _vcargs(VC),
                       capture_output=True, text=True, check=True)
        for v in ("beta", "uhat", "bhat"):
            out["%s_%s" % (tag, v)] = _vec("%s_%s.bin" % (o, v))
    np.savez_compressed(os.path.join(HERE, name + "_ref.npz"), **out)
    print(name, "N=%d Nrec=%d M=%d kept=%d" % (N, coh["Nrec"], M, int(out["stats_keep"].sum())))


def _floats(s):
    return [float(x) for x in s.split()]


def parse_aireml_log(text, nc=5):
    """Per-iteration blocks of the reference log (17-digit prints); nc components."""
    its = []
    for blk in re.split(r"\n-+ Iteration \d+ -+\n", text)[1:]:
        d = {"gradients": [_floats(m) for m in re.findall(r"Gradient:\s*([^\n]+)", blk)],
             "ai": [[_floats(l) for l in m.strip().split("\n")] for m in
                    re.findall(r"AI matrix: \n((?:[^\n]+\n){%d})" % nc, blk)],
             "steps": [_floats(m) for m in re.findall(r"Predicted step:\s*([^\n]+)", blk)],
             "nlopt": [int(m) for m in re.findall(r"NLopt result: (-?\d+)", blk)],
             "rho": [float(m) for m in re.findall(r"Rho: ([^\n]+)", blk)],
             "theta_new": [_floats(m) for m in re.findall(r"theta_new: ([^\n]+)", blk)],
             "delta_after": [float(m) for m in re.findall(r"Trust region radius: ([^\n]+)", blk)]}
        if nc == 5:
            m = re.search(r"Estimated variance components:\s*sig2e = ([^,]+), sig2g = ([^,]+), sig2b0 = ([^,]+), "
                          r"sigb01 = ([^,]+), sig2b1 = ([^\n]+)", blk)
        else:
            m = re.search(r"Estimated variance components:\s*sig2e = ([^,]+), sig2g = ([^\n]+)", blk)
        d["theta"] = [float(m.group(k)) for k in range(1, nc + 1)] if m else None
        its.append(d)
    fin = re.search(r"Final variance components[^\n]*\n((?:[^\n]+\n){%d})" % nc, text)
    final = []
    if fin:
        for ln in fin.group(1).strip().split("\n"):
            a, b = ln.split("=")[1].split("\xc2\xb1") if "\xc2\xb1" in ln else ln.split("=")[1].split("±")
            final.append([float(a), float(b)])
    return its, final


def make_aireml_case(tmp):
    name = "aireml_small"
    vc = (0.6, 0.4, 0.4, 0.05, 0.2)
    coh = synth.simulate_cohort(22, 300, 1500, ("poisson", 5), 10.0, maf_lo=0.01, miss_rate=0.0, vc=vc)
    pre = os.path.join(HERE, name)
    synth.write_record_table(pre + ".txt", coh)
    synth.write_grm_bin(pre, synth.grm_from_packed(coh["packed"], coh["N"]))
    per = AIREML_NUMMC * (3 * coh["N"] + coh["Nrec"])
    probe_file = os.path.join(tmp, "probes.bin")
    synth.normal_stream(PROBE_SEED, per * 200).tofile(probe_file)
    env = dict(os.environ, GLOBE_PROBE_FILE=probe_file)
    out = os.path.join(tmp, name)
    subprocess.run([os.path.join(REF, "runAIREML64"), pre + ".txt", pre, out, "--numMC", str(AIREML_NUMMC),
                    "--maxiter", str(AIREML_MAXITER)], env=env, capture_output=True, text=True, check=True)
    text = open(out + ".log", encoding="utf-8", errors="replace").read()
    its, final = parse_aireml_log(text)
    with open(os.path.join(HERE, name + "_ref.json"), "w") as f:
        json.dump({"numMC": AIREML_NUMMC, "maxiter": AIREML_MAXITER, "probe_seed": PROBE_SEED,
                   "pcg_tol": 1e-12, "theta0": [0.5, 0.30000001192092896, 0.20000000298023224,
                                                 0.10000000149011612, 0.10000000149011612],
                   "N": coh["N"], "Nrec": coh["Nrec"], "iterations": its, "final": final}, f, indent=1)
    print(name, "N=%d Nrec=%d iterations=%d" % (coh["N"], coh["Nrec"], len(its)))


def make_reduced_case(tmp):
    """runAIREML_reducedModel: y = X b + g + e, V = sig2g A + sig2e I, one record per individual."""
    name = "reduced_small"
    rng = np.random.default_rng(31)
    N, M = 300, 1500
    G = synth.simulate_genotypes(rng, M, N, 0.01, 0.5, 0.0)
    packed = synth.pack_genotypes(G)
    Gf = np.where(G < 0, 0, G).astype(np.float64)
    f = np.clip(Gf.mean(axis=1) / 2.0, 1e-3, 1 - 1e-3)
    Zs = (Gf - 2 * f[:, None]) / np.sqrt(2 * f * (1 - f))[:, None]
    s2e, s2g = 0.6, 0.4
    u = Zs.T @ rng.standard_normal(M) * np.sqrt(s2g / M)
    X = np.column_stack([np.ones(N)] + [np.round(rng.standard_normal(N) * 1024) / 1024 for _ in range(2)])
    y = X @ np.array([1.0, 0.5, -0.3]) + u + rng.standard_normal(N) * np.sqrt(s2e)
    y = np.round(y * 4096) / 4096
    pre = os.path.join(HERE, name)
    with open(pre + ".txt", "w") as fh:
        fh.write("INDIV PHENO COV0 COV1 COV2\n")
        for i in range(N):
            fh.write("%d %.10g %.10g %.10g %.10g\n" % (i + 1, y[i], X[i, 0], X[i, 1], X[i, 2]))
    synth.write_grm_bin(pre, synth.grm_from_packed(packed, N))
    per = AIREML_NUMMC * 2 * N
    probe_file = os.path.join(tmp, "probes_reduced.bin")
    synth.normal_stream(PROBE_SEED, per * 200).tofile(probe_file)
    env = dict(os.environ, GLOBE_PROBE_FILE=probe_file)
    out = os.path.join(tmp, name)
    subprocess.run([os.path.join(REF, "runAIREML_reduced64"), pre + ".txt", pre, out, "--numMC", str(AIREML_NUMMC),
                    "--maxiter", str(AIREML_MAXITER)], env=env, capture_output=True, text=True, check=True)
    text = open(out + ".log", encoding="utf-8", errors="replace").read()
    its, final = parse_aireml_log(text, nc=2)
    with open(os.path.join(HERE, name + "_ref.json"), "w") as fh:
        json.dump({"numMC": AIREML_NUMMC, "maxiter": AIREML_MAXITER, "probe_seed": PROBE_SEED,
                   "pcg_tol": 1e-12, "theta0": [0.5, 0.5], "N": N, "iterations": its, "final": final}, fh, indent=1)
    print(name, "N=%d iterations=%d" % (N, len(its)))


def make_grm_build_case(tmp):
    """The reference's FP64 runPCGsolver --grm on the oracle-built GRM (double allele
    frequency) of the committed geno_small inputs."""
    from oracle import oracle
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import golden_case
    c = golden_case("geno_small")
    lt = oracle.grm_build(c["packed"], c["N"], freq="f64")
    g = os.path.join(tmp, "geno_small_f64")
    synth.write_grm_bin(g, lt)
    o = os.path.join(tmp, "geno_small_grmf64")
    subprocess.run([os.path.join(REF, "runPCGsolver64"), "--input", c["prefix"] + ".txt", "--output", o,
                    "--grm", g] + _vcargs(VC), capture_output=True, text=True, check=True)
    out = {v: _vec("%s_%s.bin" % (o, v)) for v in ("beta", "uhat", "bhat")}
    np.savez_compressed(os.path.join(HERE, "geno_small_grmf64_ref.npz"), **out)
    print("geno_small_grmf64: reference --grm on the oracle-built GRM")


PORTABLE_PCG = dict(name="geno_2k_10k", seed=2001, N=2000, M=10000, recs=["uniform", 3, 10], T=5.0,
                    maf_lo=0.05, maf_hi=0.5, miss_rate=0.01)
PORTABLE_AIREML = dict(name="aireml_dense_2k", seed=2002, N=2000, M=5000, recs=["poisson", 5], T=10.0,
                       maf_lo=0.01, maf_hi=0.5, miss_rate=0.0, freq_levels=64, numMC=15, maxiter=50,
                       probe_seed=9, vc=[0.6, 0.4, 0.4, 0.2, 0.2])


def make_portable_pcg(tmp):
    spec = PORTABLE_PCG
    pre, coh = portable_inputs(spec, tmp)
    name = spec["name"]
    out = {}
    r = subprocess.run([os.path.join(REF, "runPCGsolver_stats"), "--input", pre + ".txt", "--output",
                        os.path.join(tmp, name + "_s"), "--geno", pre] + _vcargs(VC),
                       capture_output=True, text=True, check=True)
    rows = [ln.split() for ln in r.stdout.splitlines() if ln.startswith("[snpstat]")]
    out["stats_alt"] = np.array([int(x[2]) for x in rows], np.int64)
    out["stats_miss"] = np.array([int(x[3]) for x in rows], np.int64)
    out["stats_maf"] = np.array([float.fromhex(x[4]) for x in rows], np.float32)
    out["stats_miss_rate"] = np.array([float.fromhex(x[5]) for x in rows], np.float32)
    out["stats_keep"] = np.array([int(x[6]) for x in rows], np.uint8)
    for tag, exe in (("f32", "runPCGsolver"), ("geno64", "runPCGsolver64")):
        o = os.path.join(tmp, name + "_" + tag)
        subprocess.run([os.path.join(REF, exe), "--input", pre + ".txt", "--output", o, "--geno", pre] + _vcargs(VC),
                       capture_output=True, text=True, check=True)
        for v in ("beta", "uhat", "bhat"):
            out["%s_%s" % (tag, v)] = _vec("%s_%s.bin" % (o, v))
    out["spec"] = np.array(json.dumps(spec))
    out["sha256_txt"] = np.array(synth.file_sha256(pre + ".txt"))
    out["sha256_bed"] = np.array(synth.file_sha256(pre + ".bed"))
    np.savez_compressed(os.path.join(HERE, name + "_ref.npz"), **out)
    print(name, "N=%d Nrec=%d M=%d kept=%d" % (coh["N"], coh["Nrec"], spec["M"], int(out["stats_keep"].sum())))


def make_portable_aireml(tmp):
    spec = PORTABLE_AIREML
    pre, coh = portable_inputs(spec, tmp)
    name = spec["name"]
    per = spec["numMC"] * (3 * coh["N"] + coh["Nrec"])
    probe_file = os.path.join(tmp, name + "_probes.bin")
    synth.normal_stream(spec["probe_seed"], per * 120).tofile(probe_file)
    env = dict(os.environ, GLOBE_PROBE_FILE=probe_file)
    out = os.path.join(tmp, name)
    subprocess.run([os.path.join(REF, "runAIREML64"), pre + ".txt", pre, out, "--numMC", str(spec["numMC"]),
                    "--maxiter", str(spec["maxiter"])], env=env, capture_output=True, text=True, check=True)
    text = open(out + ".log", encoding="utf-8", errors="replace").read()
    its, final = parse_aireml_log(text)
    with open(os.path.join(HERE, name + "_ref.json"), "w") as f:
        json.dump({"spec": spec, "numMC": spec["numMC"], "maxiter": spec["maxiter"], "probe_seed": spec["probe_seed"],
                   "pcg_tol": 1e-12, "theta0": [0.5, 0.30000001192092896, 0.20000000298023224,
                                                 0.10000000149011612, 0.10000000149011612],
                   "N": coh["N"], "Nrec": coh["Nrec"], "sha256_txt": synth.file_sha256(pre + ".txt"),
                   "sha256_grm": synth.file_sha256(pre + ".grm.bin"), "iterations": its, "final": final}, f, indent=1)
    print(name, "N=%d Nrec=%d iterations=%d" % (coh["N"], coh["Nrec"], len(its)))


def main():
    if not os.path.exists(os.path.join(REF, "runPCGsolver64")):
        sys.exit("build the reference first: python oracle/build_ref.py")
    tmp = "/tmp/globe_golden"
    os.makedirs(tmp, exist_ok=True)
    if sys.argv[1:] == ["grm_build"]:
        make_grm_build_case(tmp)
        return
    if sys.argv[1:] == ["portable_pcg"]:
        make_portable_pcg(tmp)
        return
    if sys.argv[1:] == ["portable_aireml"]:
        make_portable_aireml(tmp)
        return
    for name, args in CASES.items():
        make_pcg_case(name, *args, tmp)
    if os.path.exists(os.path.join(REF, "runAIREML64")):
        make_aireml_case(tmp)
    if os.path.exists(os.path.join(REF, "runAIREML_reduced64")):
        make_reduced_case(tmp)
    make_grm_build_case(tmp)


if __name__ == "__main__":
    main()
