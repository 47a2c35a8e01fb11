"""Shared test helpers: golden cases, cohorts and comparison metrics."""
import json
import os

import numpy as np

from globe_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
VC = (0.6, 0.4, 0.4, 0.2, 0.2)
VC_F = tuple(float(np.float32(v)) for v in VC)   # as std::stof parses them


def rel(a, b):
    """max |a-b| / max |b|."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.abs(b).max()
    return float(np.abs(a - b).max() / (d if d > 0 else 1.0))


def read_bed_payload(prefix, N):
    raw = np.fromfile(prefix + ".bed", np.uint8)
    assert list(raw[:3]) == [0x6C, 0x1B, 0x01]
    bps = (N + 3) // 4
    M = (raw.size - 3) // bps
    return raw[3:3 + M * bps].reshape(M, bps)


def parse_records_py(path):
    """Independent numpy parse of the record table (named columns first)."""
    with open(path) as f:
        hdr = f.readline().split()
        rows = [l.split() for l in f if l.strip()]
    a = np.array(rows, dtype=np.float64)
    ci, cp, ct = hdr.index("INDIV"), hdr.index("PHENO"), hdr.index("TIMES")
    cov = [j for j in range(len(hdr)) if j not in (ci, cp, ct)]
    ids = a[:, ci].astype(int)
    N = len(set(ids.tolist()))
    X = np.column_stack([a[:, j] for j in cov] + [a[:, ct]])
    return (ids - 1).astype(np.int32), np.asfortranarray(X), a[:, cp].copy(), N


def golden_case(name):
    pre = os.path.join(GOLDEN, name)
    indiv, X, y, N = parse_records_py(pre + ".txt")
    d = dict(prefix=pre, indiv=indiv, X=X, y=y, N=N, Nrec=len(indiv))
    if os.path.exists(pre + ".bed"):
        d["packed"] = read_bed_payload(pre, N)
    if os.path.exists(pre + ".grm.bin"):
        d["grm"] = np.fromfile(pre + ".grm.bin", np.float32)
    ref = pre + "_ref.npz"
    if os.path.exists(ref):
        d["ref"] = dict(np.load(ref))
    js = pre + "_ref.json"
    if os.path.exists(js):
        d["ref"] = json.load(open(js))
    return d


def aireml_probes(case, n_evals):
    ref = case["ref"]
    per = ref["numMC"] * (3 * case["N"] + case["Nrec"])
    return synth.normal_stream(ref["probe_seed"], per * n_evals), per


def cohort(seed, N, M, recs=("uniform", 3, 10), T=5.0, miss=0.01, edge=False, maf_lo=0.05):
    coh = synth.simulate_cohort(seed, N, M, recs, T, maf_lo=maf_lo, miss_rate=miss, edge_snps=edge)
    coh["X"] = np.asfortranarray(np.column_stack([coh["cov"], coh["times"]]))
    return coh


def f32_ulps(a, b):
    """Distance in float32 units in the last place, elementwise."""
    def key(x):
        i = np.ascontiguousarray(x, np.float32).view(np.int32).astype(np.int64)
        return np.where(i < 0, -(i & 0x7FFFFFFF), i)
    return np.abs(key(a) - key(b))


def tc_digits(col, nd):
    """nd balanced base-32 digits of a column as k_digits forms them (rows: digit j), and the
    column's exponent e: I = round(x 2^-e 32^(nd-1)) with |x 2^-e| < 16."""
    col = np.asarray(col, np.float64)
    mx = np.abs(col).max()
    e = (np.frexp(mx)[1] - 4) if mx > 0 else -4
    I = np.rint(np.ldexp(col, 5 * (nd - 1) - e)).astype(np.int64)
    D = np.zeros((nd, len(col)))
    for j in range(nd - 1, 0, -1):
        d = ((I + 16) & 31) - 16
        D[j] = d
        I = (I - d) >> 5
    assert np.all(np.abs(I) <= 16)
    D[0] = I
    return D, e


def tc_product_emulation(G, f, inv, Z, scale, nd):
    """The tensor-core GRM product with nd digits per column, in exact arithmetic:
    G = kept genotypes (Mk x N, missing as 0), f / inv_std per SNP.  Pass 1 forms
    u = inv^2 (G d(Z) - 2 f sum Z), pass 2 out = scale (G' d(u) - sum 2 f u), where d()
    is the column rounded to nd base-32 digits."""
    G = np.asarray(G, np.float64)
    w = 32.0 ** -np.arange(nd)
    U = np.zeros((G.shape[0], Z.shape[1]))
    for c in range(Z.shape[1]):
        D, e = tc_digits(Z[:, c], nd)
        P = G @ D.T                                   # exact integers
        U[:, c] = inv ** 2 * (np.ldexp(P @ w, e) - 2 * f * Z[:, c].sum())
    out = np.zeros_like(Z, dtype=np.float64)
    for c in range(Z.shape[1]):
        D, e = tc_digits(U[:, c], nd)
        P = G.T @ D.T
        out[:, c] = scale * (np.ldexp(P @ w, e) - (2 * f * U[:, c]).sum())
    return out


def lt_to_full(lt, N):
    """The symmetric N x N matrix of a packed lower triangle (row-major, i >= j)."""
    A = np.zeros((N, N))
    A[np.tril_indices(N)] = np.asarray(lt, np.float64)
    return A + np.tril(A, -1).T


def dense_tc_emulation(A, Z, scale, nd, da=None):
    """The tensor-core dense GRM product in exact arithmetic: A rounded to the grid of its
    da = min(7, nd) digit planes (k_dense_digits: I = round(A 2^-e 32^(da-1)), max|A| 2^-e in
    [8, 16)), each column of Z to nd base-32 digits (k_digits); then one FP64 product."""
    A = np.asarray(A, np.float64)
    da = min(7, nd) if da is None else da
    mx = np.abs(A).max()
    e = (np.frexp(mx)[1] - 4) if mx > 0 else -4
    Ar = np.ldexp(np.rint(np.ldexp(A, 5 * (da - 1) - e)), e - 5 * (da - 1))
    w = 32.0 ** -np.arange(nd)
    Zr = np.zeros_like(np.asarray(Z, np.float64))
    for c in range(Zr.shape[1]):
        D, ez = tc_digits(Z[:, c], nd)
        Zr[:, c] = np.ldexp(D.T @ w, ez)
    return scale * (Ar @ Zr)


def portable_inputs(spec, outdir):
    """Write the inputs of a portable fixture (``spec`` as stored in it) under outdir:
    the record table and the PLINK trio, or the .grm.bin when the spec has
    ``freq_levels``.  Returns (prefix, cohort)."""
    kw = dict(maf_lo=spec["maf_lo"], maf_hi=spec["maf_hi"], miss_rate=spec["miss_rate"])
    if spec.get("freq_levels"):
        kw["freq_levels"] = spec["freq_levels"]
    if spec.get("vc"):
        kw["vc"] = tuple(spec["vc"])
    coh = synth.portable_cohort(spec["seed"], spec["N"], spec["M"], tuple(spec["recs"]), spec["T"], **kw)
    pre = os.path.join(outdir, spec["name"])
    synth.write_record_table(pre + ".txt", coh)
    if spec.get("freq_levels"):
        synth.write_grm_bin(pre, synth.portable_grm(coh["G"], coh["p_a1"]))
    else:
        synth.write_plink(pre, coh["packed"], coh["N"])
    return pre, coh


def portable_case(name, outdir):
    """A fixture at a benchmark configuration's size whose inputs are regenerated
    (globe_gb300.synth.portable_cohort) and checked byte for byte (SHA-256) against
    the inputs the reference ran on.  Same keys as :func:`golden_case`."""
    base = os.path.join(GOLDEN, name + "_ref")
    if os.path.exists(base + ".npz"):
        ref = dict(np.load(base + ".npz"))
        spec = json.loads(str(ref["spec"]))
        sums = {"txt": str(ref["sha256_txt"]), "bed": str(ref["sha256_bed"])}
    else:
        ref = json.load(open(base + ".json"))
        spec = ref["spec"]
        sums = {"txt": ref["sha256_txt"], "grm.bin": ref["sha256_grm"]}
    pre, coh = portable_inputs(spec, outdir)
    for ext, want in sums.items():
        got = synth.file_sha256(pre + "." + ext)
        assert got == want, "regenerated %s.%s differs from the reference's input" % (name, ext)
    indiv, X, y, N = parse_records_py(pre + ".txt")
    d = dict(prefix=pre, indiv=indiv, X=X, y=y, N=N, Nrec=len(indiv), ref=ref, spec=spec)
    if "bed" in sums:
        d["packed"] = read_bed_payload(pre, N)
    else:
        d["grm"] = np.fromfile(pre + ".grm.bin", np.float32)
    return d
