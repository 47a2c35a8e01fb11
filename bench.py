#!/usr/bin/env python3
"""Benchmark: block-PCG throughput (RHS x iterations / s) of the LGMM solve.

Workload (default ``--config precision``): the on-the-fly genotype GRM
configuration -- N = 100,000 individuals, M = 500,000 SNPs as 2-bit PLINK
codes (MAF ~ U(0.01, 0.5), 2% missing; ~12.5 GB in HBM), ~700,000 records
(Poisson(6)+1 per individual, times U[0,10]), intercept + 2 covariates + time,
right-hand sides [X y] (k = 5), components (0.6, 0.4, 0.4, 0.2, 0.2).
Synthetic: genotypes drawn on the GPU by a counter-based generator, records
by numpy from a fixed seed.

A step is one call of the block-PCG solve (globe_pcg_dev) capped at
``--iters`` iterations with the tolerance at 0 so every column stays active:
it performs ``k * iters`` RHS-iterations (each = one V.P product through the
GRM on the packed genotypes + the PCG vector updates).  ``value`` is the
device-resident throughput; ``e2e`` is the same through globe_pcg with pinned
host buffers (B copied in, X copied out inside the timed region).

The same run also reports AIREML time to converge (numMC=15, 32 for c5; tol 1e-3, same
probes for both precisions): ``aireml`` on this workload with the selected
precision, and ``aireml_mixed_vs_fp64`` on a smaller cohort (N=20k, M=20k)
where the plain FP64 path also finishes in seconds.  The phenotype's genetic
term is computed from the generated genotypes (``genetic_values``).

``aireml.parity`` checks the mixed path on this workload against plain FP64:
one gradient evaluation (fitMME, probe solves, AI matrix) in each precision at
the mixed AIREML estimate, same probes -- the MME outputs, gradient, AI matrix
and the Newton step they give.

``--impl reference`` times the reference algorithm on the host cores: the
FP32 OpenMP restatement of computeVx_multi with the reference's loop
structure (oracle/globe_oracle.c, orc_ref_vx_f32).  Each step runs one full
50,000-SNP compute chunk over all individuals; the value scales it to all
kept SNPs (one PCG iteration = one V.x) and the line says by what factor.

Multi-GPU: the path does not shard across GPUs in this design (one GPU per
solve); with torchrun each rank runs an independent replica and ``value`` is
the sum over ranks divided by the slowest rank's time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "PCG RHS*iters/s"
CONFIGS = {
    # name: N, M, record distribution, T, maf_lo, maf_hi, miss
    "precision": dict(N=100_000, M=500_000, recs=("poisson", 6), T=10.0, maf_lo=0.01, maf_hi=0.5, miss=0.02,
                      label="N=100k indiv, M=500k 2-bit SNPs, ~700k records, k=5 RHS ([X y])"),
    "mid": dict(N=100_000, M=50_000, recs=("poisson", 6), T=10.0, maf_lo=0.01, maf_hi=0.5, miss=0.02,
                label="N=100k indiv, M=50k 2-bit SNPs (1.25 GB), ~700k records, k=5 (profiling size)"),
    "small": dict(N=20_000, M=40_000, recs=("poisson", 6), T=10.0, maf_lo=0.01, maf_hi=0.5, miss=0.02,
                  label="N=20k indiv, M=40k SNPs, ~140k records, k=5"),
    # dense .grm.bin path: the GRM is built on the GPU from 50k synthetic SNPs (float32 packed lower triangle)
    "c2": dict(N=20_000, M=50_000, recs=("poisson", 5), T=10.0, maf_lo=0.01, maf_hi=0.5, miss=0.0, dense=True, k=16,
               label="N=20k indiv, ~120k records, dense float32 GRM (800 MB) from M=50k SNPs, k=16 RHS"),
    # batching shape: y + 64 probe-like columns as one 65-RHS block
    "c4": dict(N=200_000, M=300_000, recs=("fixed", 6), T=10.0, maf_lo=0.01, maf_hi=0.5, miss=0.02, k=65,
               label="N=200k indiv, M=300k 2-bit SNPs (15 GB), 1.2M records, k=65 RHS"),
    # biobank shape: 60 GB of packed genotypes, geometric record counts 1-200
    "c5": dict(N=400_000, M=600_000, recs=("geometric", 0.1, 1, 200), T=15.0, maf_lo=0.01, maf_hi=0.5, miss=0.02,
               numMC=32, label="N=400k indiv, M=600k 2-bit SNPs (60 GB), ~4M records (geometric 1-200), k=5 RHS"),
    "c1": dict(N=2_000, M=10_000, recs=("uniform", 3, 10), T=5.0, maf_lo=0.05, maf_hi=0.5, miss=0.01,
               label="N=2000 indiv, M=10k SNPs, ~13k records, k=5"),
}
VC = (0.6, 0.4, 0.4, 0.2, 0.2)
SEED = 20261203


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for nm, v in zip(names, r[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_records(cfg, seed=SEED, iid_genetic=True):
    """Record table of the workload.  iid_genetic=False leaves the genetic term
    out of y (it is added from the genotypes by genetic_values)."""
    from globe_gb300 import synth
    vc = VC if iid_genetic else (VC[0], 0.0, VC[2], VC[3], VC[4])
    coh = synth.simulate_cohort(seed, cfg["N"], 0, cfg["recs"], cfg["T"], vc=vc, exact_genetic=False)
    X = np.asfortranarray(np.column_stack([coh["cov"], coh["times"]]))
    return coh["indiv"].astype(np.int32), X, coh["y"], cfg["N"]


def genetic_values(torch, raw, M, N, s2g, seed, chunk=2048):
    """u = Zs' w sqrt(s2g / M_kept) from packed genotypes on the GPU (torch, chunks of SNPs):
    the genetic term of the simulated phenotype, zs standardised as the reference does
    (A1 frequency over non-missing samples, missing genotype -> 0, MAF/missingness filter)."""
    bps = (N + 3) // 4
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    w = torch.randn(M, generator=gen, device="cuda", dtype=torch.float32)
    lut = torch.tensor([2.0, 0.0, 1.0, 0.0], device="cuda")      # code -> A1 count, missing -> 0
    u = torch.zeros(N, dtype=torch.float64, device="cuda")
    kept = 0
    for s0 in range(0, M, chunk):
        b = raw[s0:s0 + chunk, :bps]
        codes = torch.stack([(b >> (2 * j)) & 3 for j in range(4)], dim=2).reshape(b.shape[0], bps * 4)[:, :N].long()
        g = lut[codes]
        nobs = (codes != 1).sum(1).clamp(min=1).float()
        f = g.sum(1) / (2.0 * nobs)
        miss = 1.0 - nobs / N
        keep = (f >= 0.01) & (f <= 0.99) & (miss <= 0.2)
        sd = torch.sqrt(2.0 * f * (1.0 - f)).clamp(min=1e-6)
        ww = torch.where(keep, w[s0:s0 + chunk] / sd, torch.zeros_like(sd))
        u += ((g - 2.0 * f[:, None]) * ww[:, None]).sum(0).double()
        kept += int(keep.sum())
    return (u * np.sqrt(s2g / max(kept, 1))).cpu().numpy()


GRM_BUILD = dict(N=20_000, M=50_000, maf_lo=0.01, maf_hi=0.5, miss=0.02)
GRM_KG, GRM_NMMA = 21, 192          # columns per tensor-core group and its MMA width (k_grm_build.cu)


def grm_build_bench(G, torch, hbm, bf16, peak_src, raw=None, cfg=GRM_BUILD, fp64=True, device=0):
    """globe_grm_build_dev (A = Zs'Zs / M_kept, float32 packed lower triangle) on the
    dense-GRM shape: tensor-core and FP64 builds, their agreement, and the tensor-core
    GEMM's issued FP8 rate.  Returns (record, lower triangle on the device)."""
    N, M = cfg["N"], cfg["M"]
    bps = (N + 3) // 4
    stride = (bps + 15) // 16 * 16
    cx = G.Context(device)
    cx.set_individuals(N)
    own = raw is None
    if own:
        raw = torch.empty((M, stride), dtype=torch.uint8, device="cuda")
        cx.synth_bed_dev(raw.data_ptr(), M, N, stride, SEED + 11, cfg["maf_lo"], cfg["maf_hi"], cfg["miss"])
    Mk = cx.load_bed_dev(raw.data_ptr(), M, stride)
    if own:
        del raw
    lt = torch.empty(N * (N + 1) // 2, dtype=torch.float32, device="cuda")
    rec = {"workload": "N=%d indiv, M=%d SNPs (%d kept) -> %.0f MB float32 packed lower triangle" % (
        N, M, Mk, N * (N + 1) / 2 * 4 / 1e6), "kept_snps": int(Mk)}
    cx.set_precision(G.PREC_MIXED)
    t0 = time.perf_counter()
    cx.grm_build_dev(lt.data_ptr())       # first call also lays out the individual-major tile-blocked codes
    cx.synchronize()
    rec["mixed_first_call_seconds"] = time.perf_counter() - t0
    reps = 3
    cx.prof_enable(True)
    t0 = time.perf_counter()
    for _ in range(reps):
        cx.grm_build_dev(lt.data_ptr())
    cx.synchronize()
    rec["mixed_seconds"] = (time.perf_counter() - t0) / reps
    nb, msb = cx.prof_query(G._lib.PROF_GRM_BUILD)
    ng, msg = cx.prof_query(G._lib.PROF_GRM_BUILD_GEMM)
    cx.prof_enable(False)
    rec["mixed_device_ms"] = msb / max(nb, 1)
    rec["gemm_share"] = msg / msb if msb else None
    # issued FP8 work: per group of 21 columns, the row tiles (256 rows) from its first column down,
    # 192 digit columns, K = the padded SNP count
    kpad = -(-((Mk + 3) // 4) // 32) * 32 * 4
    rows = sum(-(-(N - (j0 // 256) * 256) // 256) * 256 for j0 in range(0, N, GRM_KG))
    issued = 2.0 * rows * GRM_NMMA * kpad
    t_gemm = msg / 1000.0 / reps
    fp8_peak = 2.0 * bf16
    rec["tensor"] = {"kernel": "k_tc_gemm<192> (e4m3 x e4m3 -> f32, 9 digits per column)",
                     "issued_tflops": issued / t_gemm / 1e12, "peak_tflops": fp8_peak,
                     "frac": issued / t_gemm / 1e12 / fp8_peak,
                     "peak_source": "%s bf16 burst x 2 (FP8 dense rate)" % peak_src,
                     "useful_tflops": 2.0 * N * (N + 1) / 2 * Mk / (rec["mixed_device_ms"] / 1000.0) / 1e12}
    if fp64:
        ref = lt.clone()
        cx.set_precision(G.PREC_FP64)
        t0 = time.perf_counter()
        cx.grm_build_dev(lt.data_ptr())
        cx.synchronize()
        rec["fp64_seconds"] = time.perf_counter() - t0
        rec["speedup"] = rec["fp64_seconds"] / rec["mixed_seconds"]
        a = ref.view(torch.int32).to(torch.int64)
        b = lt.view(torch.int32).to(torch.int64)
        a = torch.where(a < 0, -(a & 0x7FFFFFFF), a)
        b = torch.where(b < 0, -(b & 0x7FFFFFFF), b)
        d = (a - b).abs()
        rec["mixed_vs_fp64_max_ulp"] = int(d.max())
        rec["mixed_vs_fp64_equal_fraction"] = float((d == 0).double().mean())
        lt = ref
    cx.close()
    return rec, lt


def cpu_reference_vx(indiv, X, packed_rows, maf_rows, N, k, rng):
    """One FP32 V.x of the reference's loop structure over the given SNP rows."""
    from oracle import oracle
    x = rng.standard_normal((len(indiv), k)).astype(np.float32)
    t0 = time.perf_counter()
    oracle.ref_vx_f32(indiv, X[:, -1], packed_rows, maf_rows, VC, x, N)
    return time.perf_counter() - t0


REF_CHUNK = 50_000      # SNPs per compute chunk of computeVx_multi (SNP_CHUNK_SIZE, PCGsolver.cpp:1135)


def chunk_rows(sample_rows, sample_maf, n=REF_CHUNK):
    """One reference compute chunk of n SNP rows: the sample rows repeated (the
    loop's cost does not depend on the genotype values)."""
    reps = -(-n // sample_rows.shape[0])
    rows = np.ascontiguousarray(np.tile(sample_rows, (reps, 1))[:n])
    return rows, np.ascontiguousarray(np.tile(sample_maf, reps)[:n])


def cpu_baseline(indiv, X, N, Mk, k, rows, maf, t_rec=None):
    """Time the reference algorithm on one full compute chunk (rows, maf: REF_CHUNK
    SNPs) and extrapolate to Mk SNPs.  Returns (RHS*iters/s, record, seconds of the
    chunk's V.x)."""
    rng = np.random.default_rng(1)
    if t_rec is None:
        t_rec = cpu_reference_vx(indiv, X, rows[:0], maf[:0], N, k, rng)
    t = cpu_reference_vx(indiv, X, rows, maf, N, k, rng)
    n = rows.shape[0]
    per_snp = max(t - t_rec, 1e-9) / n
    t_matvec = t_rec + per_snp * Mk
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    rec = {"value": k / t_matvec, "unit": "RHS*iters/s", "cores": threads, "kind": "port",
           "sample": ("FP32 reference-structure V.x (orc_ref_vx_f32, OpenMP) over one %d-SNP compute chunk x %d "
                      "individuals, k=%d: %.3f s (record ops %.3f s); scaled to all %d kept SNPs: %.2f s per PCG "
                      "iteration" % (n, N, k, t, t_rec, Mk, t_matvec)),
           "extrapolated_from": {"snps_timed": n, "snps_total": int(Mk), "factor": Mk / n,
                                 "chunk_seconds": t, "record_ops_seconds": t_rec}}
    return k / t_matvec, rec, t


def common_config(args, cfg, k, Nrec):
    """The workload keys both arms print under "config" (same keys, same values)."""
    return {"workload": args.config, "shape": cfg["label"], "seed": SEED, "rhs": k, "records": int(Nrec)}


AIREML_THETA0 = (0.5, 0.3, 0.2, 0.1, 0.1)
# base-32 digits per column in the AIREML solves (globe_set_digits): 6 digits round each
# right-hand side to ~2e-9 relative, far below the solves' own tolerance (1e-5)
AIREML_DIGITS = 6
AIREML_CMP = dict(N=20_000, M=20_000, recs=("poisson", 6), T=10.0, maf_lo=0.01, miss=0.02)


def aireml_compare(G):
    """AIREML to convergence with the mixed and the plain FP64 GRM product on one
    smaller cohort (N=20k, M=20k, genotype-linked y), same probes: time and agreement."""
    from globe_gb300 import synth
    c = AIREML_CMP
    coh = synth.simulate_cohort(SEED + 3, c["N"], c["M"], c["recs"], c["T"], maf_lo=c["maf_lo"], miss_rate=c["miss"])
    X = np.asfortranarray(np.column_stack([coh["cov"], coh["times"]]))
    out = {}
    for name, prec, nd in (("mixed", G.PREC_MIXED, AIREML_DIGITS), ("mixed9", G.PREC_MIXED, 9),
                           ("fp64", G.PREC_FP64, 0)):
        with G.Context(0) as cx:
            cx.load_records(coh["indiv"].astype(np.int32), X, coh["y"], c["N"])
            cx.load_bed(coh["packed"])
            cx.set_vc(G.as_float_vc(AIREML_THETA0))
            cx.synchronize()
            t0 = time.perf_counter()
            r = cx.aireml_run(theta0=AIREML_THETA0, maxiter=50, tol=1e-3, numMC=15, precision=prec, seed=SEED,
                              digits=nd)
            out[name] = (time.perf_counter() - t0, r)
    (tm, rm), (t9, r9), (tf, rf) = out["mixed"], out["mixed9"], out["fp64"]

    def diff(a):
        return float(np.max(np.abs(a["theta"] - rf["theta"]) / np.abs(rf["theta"])))
    return {"workload": "N=20k indiv, M=20k SNPs, ~140k records, numMC=15, tol 1e-3, same probes",
            "digits": AIREML_DIGITS, "mixed_seconds": tm, "fp64_seconds": tf, "speedup": tf / tm,
            "iterations": [rm["iterations"], rf["iterations"]], "max_rel_theta_diff": diff(rm),
            "mixed_9_digits": {"seconds": t9, "iterations": r9["iterations"], "max_rel_theta_diff": diff(r9)},
            "theta_fp64": [float(v) for v in rf["theta"]]}


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _gls(X, S):
    """beta = (X'V^-1X)^-1 X'V^-1y and V^-1 r = V^-1y - V^-1X beta from S = V^-1 [X y]."""
    p1 = X.shape[1]
    beta = np.linalg.solve(X.T @ S[:, :p1], X.T @ S[:, p1])
    return beta, S[:, p1] - S[:, :p1] @ beta


def headline_parity(G, ctx, theta, numMC, seed, X, y, tol=1e-5):
    """The mixed path against plain FP64 on the benchmark workload itself, at the mixed
    AIREML estimate theta.

    mme: the mixed solve of V [X y] to relative residual 1e-10; its residual under the FP64
    operator (b - V x with the FP64 GRM product); an FP64 solve continued from it to 1e-12;
    beta and V^-1 r (which u-hat and b-hat are linear in) from both.

    evaluation: one AIREML gradient evaluation in each precision with the same probes and
    fresh solves as runAIREML makes them (fitMME from x0 = Q^-1 b, the probe solves, the AI
    solve; PCG tolerance 1e-5).  Rounding separates the two Krylov paths; where the solves
    are ill-conditioned they may stop an iteration or two apart, each within the
    tolerance, and the gradients then differ at the level the tolerance allows.  From
    each, the Newton step p = AI^-1 g:
    the FP64 step's distance from the mixed one, relative to theta, is how far one FP64
    iteration from theta lands from the mixed iteration; the FP64 step's own size is how
    far theta is from the FP64 fixed point for these probes (Monte-Carlo noise at numMC)."""
    ctx.set_vc(theta)
    B = np.asfortranarray(np.column_stack([X, y]))
    t0 = time.perf_counter()
    Xm, im = ctx.pcg(B, tol=1e-10, rule=G.RULE_AIREML, precision=G.PREC_MIXED)
    t_m = time.perf_counter() - t0
    t0 = time.perf_counter()
    ctx.set_precision(G.PREC_FP64)
    try:
        R = B - ctx.vx(Xm)
    finally:
        ctx.set_precision(G.PREC_FP64)
    res = float(np.max(np.linalg.norm(R, axis=0) / np.linalg.norm(B, axis=0)))
    X64, i64 = ctx.pcg(B, X0=Xm, tol=1e-12, rule=G.RULE_AIREML, precision=G.PREC_FP64)
    t_f = time.perf_counter() - t0
    bm, rm = _gls(X, Xm)
    bf, rf = _gls(X, X64)
    mme = {"mixed_tol": 1e-10, "mixed_iterations": im["iters"], "fp64_residual_of_mixed": res,
           "fp64_continuation_tol": 1e-12, "fp64_iterations": i64["iters"],
           "beta_max_rel": _rel(bm, bf), "vinv_r_max_rel": _rel(rm, rf), "solution_max_rel": _rel(Xm, X64),
           "seconds": {"mixed": t_m, "fp64": t_f}}
    res_ev = {}
    for name, prec in (("mixed", G.PREC_MIXED), ("fp64", G.PREC_FP64)):
        ctx.set_vc(theta)
        ctx.synchronize()
        t0 = time.perf_counter()
        m = ctx.mme(tol=tol, rule=G.RULE_AIREML, x0mode=G.X0_PRECOND, precision=prec)
        g = ctx.aireml_grad(numMC, seed=seed, tol=tol, precision=prec)
        ai = ctx.aireml_ai(tol=tol, precision=prec)
        res_ev[name] = dict(seconds=time.perf_counter() - t0, mme=m, grad=g["grad"], ai=ai,
                            iters=[m["iters"], g["iters"]])
    mx, sf = res_ev["mixed"], res_ev["fp64"]
    th = np.asarray(theta, np.float64)
    p_m = np.linalg.solve(mx["ai"], mx["grad"])
    p_f = np.linalg.solve(sf["ai"], sf["grad"])
    ev = {"what": "one AIREML gradient evaluation at theta*, same probes (seed %d, numMC %d), PCG tol %g" % (
              seed, numMC, tol),
          "mme_max_rel": {v: _rel(mx["mme"][v], sf["mme"][v]) for v in ("beta", "uhat", "bhat")},
          "grad_max_rel": _rel(mx["grad"], sf["grad"]), "ai_max_rel": _rel(mx["ai"], sf["ai"]),
          "newton_step_diff_rel_theta": float(np.abs(p_m - p_f).max() / np.abs(th).max()),
          "fp64_newton_step_rel_theta": float(np.abs(p_f).max() / np.abs(th).max()),
          "iterations": {"mixed": mx["iters"], "fp64": sf["iters"]},
          "seconds": {"mixed": mx["seconds"], "fp64": sf["seconds"]}}
    return {"what": "mixed vs plain FP64 GPU on this workload at the mixed AIREML estimate theta*",
            "theta": [float(v) for v in th], "max_rel": max(mme["beta_max_rel"], mme["vinv_r_max_rel"]),
            "theta_check": ev["newton_step_diff_rel_theta"], "mme": mme, "evaluation": ev}


def aggregate_replicas(torch, t_ms, units, device):
    """Whole-job figures of independent replicas: the slowest rank's time and the
    units of all ranks (an initialised process group; any backend)."""
    import torch.distributed as dist
    tt = torch.tensor([float(t_ms)], device=device, dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    uu = torch.tensor([float(units)], device=device, dtype=torch.float64)
    dist.all_reduce(uu, op=dist.ReduceOp.SUM)
    return float(tt.item()), float(uu.item())


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def run_reference(args, cfg):
    """The reference algorithm on the host cores: each step times one full compute
    chunk (REF_CHUNK SNPs x all individuals, every record op) of the FP32 V.x and
    scales it to all kept SNPs (one PCG iteration = one V.x)."""
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    from globe_gb300 import synth
    from oracle import oracle
    oracle.build()
    indiv, X, y, N = make_records(cfg)
    k = int(cfg.get("k", 5))
    rng = np.random.default_rng(2)
    nsample = min(cfg["M"], 4096)
    G = synth.simulate_genotypes(rng, nsample, N, cfg["maf_lo"], cfg["maf_hi"], cfg["miss"])
    packed = synth.pack_genotypes(G)
    del G
    alt, miss, maf, _, keep = oracle.bed_stats(packed, N)
    Mk = int(round(cfg["M"] * keep.mean()))
    rows, mafc = chunk_rows(packed[keep], maf[keep], min(REF_CHUNK, Mk))
    t_rec = cpu_reference_vx(indiv, X, rows[:0], mafc[:0], N, k, np.random.default_rng(1))
    vals, secs = [], []
    for s in range(args.warmup + args.steps):
        v, rec, t = cpu_baseline(indiv, X, N, Mk, k, rows, mafc, t_rec=t_rec)
        if s >= args.warmup:
            vals.append(v)
            secs.append(t)
    value = float(np.mean(vals))
    rec["value"] = value
    line = {"metric": METRIC, "value": value, "unit": "RHS*iters/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * float(np.mean(secs)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": common_config(args, cfg, k, len(indiv)),
            "impl": "reference",
            "step": "one %d-SNP compute chunk of the V.x (ms_per_step is its measured time); value scales it to "
                    "all %d kept SNPs (extrapolated_from)" % (rows.shape[0], Mk),
            "extrapolated_from": rec["extrapolated_from"],
            "cpu_baseline": rec,
            "e2e": {"value": value, "unit": "RHS*iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_ours(args, cfg):
    import torch

    import globe_gb300 as G
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    device = local if world > 1 else 0
    torch.cuda.set_device(device)
    prec = G.PREC_MIXED if args.precision == "mixed" else G.PREC_FP64
    ctx = G.Context(device)
    if args.no_autotune:
        ctx.set_autotune(False)
    indiv, X, y, N = make_records(cfg, iid_genetic=False)
    Nrec = len(indiv)
    bps = (N + 3) // 4
    stride = (bps + 15) // 16 * 16
    M = cfg["M"]
    raw = torch.empty((M, stride), dtype=torch.uint8, device="cuda")
    ctx.synth_bed_dev(raw.data_ptr(), M, N, stride, SEED + 7919 * rank, cfg["maf_lo"], cfg["maf_hi"], cfg["miss"])
    y = y + genetic_values(torch, raw, M, N, VC[1], SEED + 1)[indiv]     # genotype-linked genetic term
    ctx.load_records(indiv, X, y, N)
    dense = bool(cfg.get("dense"))
    grm_rec = None
    if dense:
        # the dense input built on the GPU by globe_grm_build from the same genotypes
        hbm0, bf160, src0 = load_peaks()
        grm_rec, lt = grm_build_bench(G, torch, hbm0, bf160, src0, raw=raw, cfg=cfg, fp64=not args.no_fp64,
                                      device=device)
        Mk = grm_rec["kept_snps"]
        ctx.load_grm(lt.cpu().numpy(), N)
        del lt
        sample_rows = None
    else:
        Mk = ctx.load_bed_dev(raw.data_ptr(), M, stride)
        # a host copy of some kept-looking rows for the CPU baseline (rank 0)
        sample_rows = raw[: min(M, 4096)].cpu().numpy()[:, :bps].copy() if rank == 0 else None
    del raw
    torch.cuda.empty_cache()
    ctx.set_vc(G.as_float_vc(VC))
    k = int(cfg.get("k", 5))
    B = torch.empty((k, Nrec), dtype=torch.float64, device="cuda")      # column-major Nrec x k
    B[:4] = torch.from_numpy(np.ascontiguousarray(X.T)).cuda()
    B[4] = torch.from_numpy(y).cuda()
    if k > 5:                                                            # extra right-hand sides: probe-like columns
        B[5:] = torch.from_numpy(np.random.default_rng(SEED + 5).standard_normal((k - 5, Nrec))).cuda()
    Xs = torch.zeros_like(B)
    stream = torch.cuda.ExternalStream(ctx.stream)
    opts = dict(tol=0.0, maxit=args.iters, rule=G.RULE_AIREML, x0mode=G.X0_ZERO, precision=prec)

    def step_dev():
        return ctx.pcg_dev(B.data_ptr(), Xs.data_ptr(), k, **opts)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        step_dev()
    barrier()
    clocks = ClockSampler(device)
    clocks.start()
    ctx.prof_enable(True)
    launches0 = ctx.kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    ev0.record(stream)
    rhs_iters = 0
    for _ in range(args.steps):
        rhs_iters += step_dev()["rhs_iters"]
    ev1.record(stream)
    barrier()
    launches = ctx.kernel_launches() - launches0
    t_ms = ev0.elapsed_time(ev1)
    prof = {kind: ctx.prof_query(kind) for kind in (G._lib.PROF_GRM, G._lib.PROF_GRM_PASS1, G._lib.PROF_GRM_PASS2,
                                                    G._lib.PROF_PCG_ITER)}
    ctx.prof_enable(False)
    clk = clocks.stop()
    t_max = t_ms
    total_units = rhs_iters
    if world > 1:
        t_max, total_units = aggregate_replicas(torch, t_ms, rhs_iters, "cuda")
    value = total_units / (t_max / 1000.0)

    # The timed region above records CUDA events around every pass (the roofline's kernel
    # times), and profiling runs the PCG iterations as direct launches.  The same steps again
    # with profiling off replay each iteration as a CUDA graph (the library's default).
    barrier()
    ev0.record(stream)
    g_units = 0
    for _ in range(args.steps):
        g_units += step_dev()["rhs_iters"]
    ev1.record(stream)
    barrier()
    t_g = ev0.elapsed_time(ev1)
    if world > 1:
        t_g, g_units = aggregate_replicas(torch, t_g, g_units, "cuda")
    graphs_line = {"value": g_units / (t_g / 1000.0), "unit": "RHS*iters/s", "ms_per_step": t_g / args.steps,
                   "cuda_graphs": bool(ctx.get_graphs())}

    # e2e through the public API with pinned host buffers
    hB = torch.empty((k, Nrec), dtype=torch.float64, pin_memory=True)
    hB.copy_(B.cpu())
    hX = torch.empty_like(hB).pin_memory()
    nB, nX = hB.numpy(), hX.numpy()
    Bf, Xf = nB.T, nX.T          # Fortran-ordered views (Nrec x k)
    barrier()
    t0 = time.perf_counter()
    e2e_units = 0
    for _ in range(args.steps):
        Xout, info = ctx.pcg(Bf, out=Xf, **opts)
        e2e_units += info["rhs_iters"]
    barrier()
    t_e2e = time.perf_counter() - t0
    e2e = {"value": e2e_units / t_e2e, "unit": "RHS*iters/s", "h2d_bytes_per_step": int(8 * Nrec * k),
           "d2h_bytes_per_step": int(8 * Nrec * k)}

    # FP64-plain comparison on the same data (one iteration per step)
    fp64 = None
    if prec != G.PREC_FP64 and not args.no_fp64:
        o64 = dict(opts, precision=G.PREC_FP64, maxit=1)
        ctx.pcg_dev(B.data_ptr(), Xs.data_ptr(), k, **o64)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        u64 = 0
        for _ in range(2):
            u64 += ctx.pcg_dev(B.data_ptr(), Xs.data_ptr(), k, **o64)["rhs_iters"]
        e1.record(stream)
        barrier()
        t64 = e0.elapsed_time(e1)
        fp64 = {"value": u64 / (t64 / 1000.0), "unit": "RHS*iters/s", "ms_per_iteration": t64 / 2,
                "speedup_of_mixed": value / (u64 / (t64 / 1000.0))}

    # AIREML time to converge on this workload (genotype GRM, numMC from the config, tol 1e-3) -- replicas skip it
    aireml = None
    if not args.no_aireml and world == 1:
        numMC = int(cfg.get("numMC", 15))
        runs = {}
        for nd in ((AIREML_DIGITS, 9) if prec == G.PREC_MIXED and not dense else (0,)):
            barrier()
            t0 = time.perf_counter()
            r = ctx.aireml_run(theta0=AIREML_THETA0, maxiter=50, tol=1e-3, numMC=numMC, precision=prec, seed=SEED,
                               digits=nd)
            runs[nd] = (time.perf_counter() - t0, r)
        nd0 = next(iter(runs))
        t_air, r = runs[nd0]
        aireml = {"workload": args.config + " (same genetic source and records)",
                  "precision": args.precision, "digits": nd0 or None,
                  "seconds_to_converge": t_air, "converged": bool(r["converged"]), "iterations": r["iterations"],
                  "grad_evals": r["grad_evals"], "pcg_rhs_iters": r["pcg_rhs_iters"],
                  "theta": [float(v) for v in r["theta"]], "numMC": numMC, "tol": 1e-3}
        if not args.no_parity and prec == G.PREC_MIXED and not dense:
            aireml["parity"] = headline_parity(G, ctx, r["theta"], numMC, SEED + 99, X, y)
        if 9 in runs and nd0 != 9:
            t9, r9 = runs[9]
            aireml["nine_digits"] = {"seconds_to_converge": t9, "iterations": r9["iterations"],
                                     "max_rel_theta_diff": float(np.max(np.abs(r["theta"] - r9["theta"]) /
                                                                        np.abs(r9["theta"])))}

    # roofline of the dominant GRM kernel (one genotype pass per launch; the dense product per launch)
    hbm, bf16, peak_src = load_peaks()
    n1, ms1 = prof[G._lib.PROF_GRM_PASS1]
    n2, ms2 = prof[G._lib.PROF_GRM_PASS2]
    kernel_bytes = None
    if dense:
        if prec == G.PREC_MIXED:
            # k_tc_dense streams the 7 digit planes of A (full squares, rows padded to 128 / 256)
            npad = -(-N // 128) * 128
            kernel_bytes = (-(-7 * npad // 256) * 256) * npad
            dom = ("k_tc_dense (sig2g A Z, 7 e4m3 digit planes of A)", n1, ms1)
        else:
            ng, msg = prof[G._lib.PROF_GRM]
            dom = ("k_dense_f64 (sig2g A Z, packed lower triangle)", ng, msg)
        # algorithmic bytes: the packed float32 triangle once + the k right-hand sides in and out (FP64)
        bytes_per_launch = N * (N + 1) // 2 * 4 + 2 * N * k * 8
    else:
        tcname = "k_tc_gemm" if prec == G.PREC_MIXED else "k_geno"
        dom = (tcname + "(pass 2: Zs'w)", n2, ms2) if ms2 >= ms1 else (tcname + "(pass 1: Zs v)", n1, ms1)
        # algorithmic bytes of one pass: the packed genotypes once + the k right-hand sides in and out (FP32-equivalent)
        bytes_per_launch = Mk * bps + (N + Mk) * k * 4
    avg_s = dom[2] / 1000.0 / max(dom[1], 1)
    achieved = bytes_per_launch / avg_s / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tf):
        passname = "pass2" if "pass 2" in dom[0] else "pass1"
        traffic = json.load(open(tf)).get("%s:%s:%s:%s" % (args.config, args.precision, dom[0].split("(")[0].strip(),
                                                              passname))
    ngrm, msgrm = prof[G._lib.PROF_GRM]
    niter, msiter = prof[G._lib.PROF_PCG_ITER]
    roof = {"bound": "hbm", "kernel": dom[0], "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "peak_source": peak_src, "traffic": traffic,
            "bytes_per_launch": bytes_per_launch, "avg_launch_ms": avg_s * 1000.0, "launches": dom[1],
            "grm_product_share_of_iteration": (msgrm / msiter) if msiter else None,
            "pass_ms": {"pass1": ms1 / max(n1, 1), "pass2": ms2 / max(n2, 1)}}
    if dense:
        roof["fma_tflops_achieved"] = 2.0 * N * N * k / avg_s / 1e12    # N^2 k multiply-adds per product
    if kernel_bytes is not None:
        # the kernel's own HBM stream (digit planes) against the same peak
        roof["kernel_bytes_per_launch"] = kernel_bytes
        roof["kernel_stream_frac"] = kernel_bytes / avg_s / 1e9 / hbm
    line = {"metric": METRIC, "value": value, "unit": "RHS*iters/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": ("f64" if prec == G.PREC_FP64 else
                      "e4m3 x e4m3 -> f32 (exact digits of A and Z); PCG vectors in double-float f32 pairs, "
                      "scalars and dot products f64"),
            "data": "synthetic (GPU counter-based genotypes%s, seeded numpy records)" % (
                ", GRM built from them" if dense else ""),
            "config": common_config(args, cfg, k, Nrec),
            "run": {"precision": args.precision, "iters_per_step": args.iters, "kept_snps": Mk,
                    "l2": ("inputs larger than L2 (%s %.1f GB)" % (
                        ("dense GRM", N * (N + 1) / 2 * 4 / 1e9) if dense else ("packed genotypes", Mk * stride / 1e9))),
                    "parallelism": "replicas" if world > 1 else "single GPU",
                    "cuda_graphs": "off in the timed region (per-pass CUDA events); on in e2e and "
                                   "device_unprofiled"},
            "autotune": ctx.autotune_log(), "device_loop_solves": ctx.device_loop_runs(),
            "e2e": e2e, "roofline": roof, "clocks": clk, "gpu_launches": int(launches),
            "device_unprofiled": graphs_line}
    if fp64 is not None:
        line["fp64_plain"] = fp64
    if aireml is not None:
        line["aireml"] = aireml
    if rank == 0 and world == 1 and not args.no_aireml and prec != G.PREC_FP64 and not dense:
        line["aireml_mixed_vs_fp64"] = aireml_compare(G)
    if grm_rec is None and rank == 0 and world == 1 and not args.no_grm_build and prec != G.PREC_FP64:
        grm_rec, _ = grm_build_bench(G, torch, hbm, bf16, peak_src, fp64=not args.no_fp64)
    if grm_rec is not None:
        line["grm_build"] = grm_rec
    if rank == 0 and not args.no_cpu_baseline and not dense:
        from oracle import oracle
        alt, miss, maf, _, keep = oracle.bed_stats(sample_rows, N)
        rows, mafc = chunk_rows(sample_rows[keep], maf[keep], min(REF_CHUNK, Mk))
        del sample_rows
        v, rec, _ = cpu_baseline(indiv, X, N, Mk, k, rows, mafc)
        line["cpu_baseline"] = rec
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", choices=sorted(CONFIGS), default="precision")
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="mixed")
    ap.add_argument("--iters", type=int, default=0, help="PCG iterations per step (0: 10 mixed, 1 fp64)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the in-run FP64-plain comparison")
    ap.add_argument("--no-aireml", action="store_true", help="skip the AIREML time-to-converge runs")
    ap.add_argument("--no-grm-build", action="store_true", help="skip the GRM build (N=20k, M=50k) measurement")
    ap.add_argument("--no-autotune", action="store_true",
                    help="the cost model's split counts and groupings only (profiling captures a fixed launch sequence)")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the mixed-vs-FP64 evaluation at the AIREML estimate on this workload")
    args = ap.parse_args()
    cfg = CONFIGS[args.config]
    if args.iters <= 0:
        args.iters = 10 if args.precision == "mixed" else 1
    if args.impl == "reference":
        return run_reference(args, cfg)
    return run_ours(args, cfg)


if __name__ == "__main__":
    sys.exit(main())
