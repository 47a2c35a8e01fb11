"""Host-side mirror of GLOBE's interface over the C ABI.

``Context`` wraps one ``globe_ctx`` (one GPU, one stream).  ``run_pcg_solver``
and ``run_aireml`` mirror the reference's programs (same arguments, same
files); the C++ programs ``globe_gb300/bin/runPCGsolver``, ``runAIREML`` and
``runAIREML_reducedModel`` are the command-line drop-ins.  ``build_grm`` (and
the ``buildGRM`` program) writes the ``.grm.bin`` input from genotypes.
"""
import ctypes as C
import os

import numpy as np

from . import _lib as L
from ._lib import GlobeError, PcgInfo, PcgOpts

VC_NAMES = ("sig2e", "sig2g", "sig2b0", "sigb01", "sig2b1")


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


def _cols(a, rows):
    a = np.asarray(a, dtype=np.float64)
    if a.ndim == 1:
        a = a[:, None]
    assert a.shape[0] == rows, (a.shape, rows)
    return np.asfortranarray(a)


def as_float_vc(vc):
    """Components as the reference parses them (std::stof): float32 values."""
    return tuple(float(np.float32(v)) for v in vc)


class Context:
    def __init__(self, device=0):
        self._L = L.lib()
        h = C.c_void_p()
        rc = self._L.globe_create(C.byref(h), device)
        if rc != L.GLOBE_OK:
            raise GlobeError(rc, self._L.globe_last_error(None).decode())
        self.h = h
        self.N = self.Nrec = self.p = 0

    def close(self):
        if getattr(self, "h", None):
            self._L.globe_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, rc):
        if rc != L.GLOBE_OK:
            raise GlobeError(rc, self._L.globe_last_error(self.h).decode())

    # ---- state ----
    @property
    def stream(self):
        s = C.c_void_p()
        self._ck(self._L.globe_get_stream(self.h, C.byref(s)))
        return s.value

    def synchronize(self):
        self._ck(self._L.globe_synchronize(self.h))

    def prof_enable(self, on=True):
        self._ck(self._L.globe_prof_enable(self.h, int(on)))

    def prof_query(self, kind):
        n, ms = C.c_int64(), C.c_double()
        self._ck(self._L.globe_prof_query(self.h, kind, C.byref(n), C.byref(ms)))
        return n.value, ms.value

    def device_bytes(self):
        return int(self._L.globe_device_bytes(self.h))

    def kernel_launches(self):
        return int(self._L.globe_kernel_launches(self.h))

    # ---- inputs ----
    def load_records(self, indiv, X, y, N):
        indiv = np.ascontiguousarray(indiv, dtype=np.int32)
        X = np.asfortranarray(X, dtype=np.float64)
        y = np.ascontiguousarray(y, dtype=np.float64)
        Nrec, p1 = X.shape
        self._ck(self._L.globe_load_records(self.h, Nrec, N, p1 - 1, _p(indiv, C.c_int32), _p(X), _p(y)))
        self.N, self.Nrec, self.p = N, Nrec, p1 - 1

    def set_individuals(self, N):
        """Genotype-only context of N individuals (no record table), for grm_build."""
        self._ck(self._L.globe_set_individuals(self.h, N))
        self.N, self.Nrec, self.p = N, 0, 0

    def grm_build_dev(self, d_ptr):
        """grm_build into a device buffer of N(N+1)/2 float32 (globe_grm_build_dev)."""
        self._ck(self._L.globe_grm_build_dev(self.h, C.c_void_p(d_ptr)))

    def grm_build(self):
        """A = Zs'Zs / M_kept of the loaded genotypes as the float32 packed lower
        triangle (the .grm.bin payload), N(N+1)/2 values (globe_grm_build)."""
        out = np.empty(self.N * (self.N + 1) // 2, np.float32)
        self._ck(self._L.globe_grm_build(self.h, _p(out, C.c_float)))
        return out

    def load_bed(self, payload, min_maf=0.01, max_miss=0.2):
        """payload: (M, ceil(N/4)) uint8 .bed bytes without the magic."""
        payload = np.ascontiguousarray(payload, dtype=np.uint8)
        M = payload.shape[0]
        alt = np.zeros(M, np.int64)
        miss = np.zeros(M, np.int64)
        maf = np.zeros(M, np.float32)
        mr = np.zeros(M, np.float32)
        keep = np.zeros(M, np.uint8)
        info = L.BedInfo()
        self._ck(self._L.globe_load_bed(self.h, _p(payload, C.c_uint8), M, C.c_float(min_maf),
                                        C.c_float(max_miss), _p(alt, C.c_int64), _p(miss, C.c_int64),
                                        _p(maf, C.c_float), _p(mr, C.c_float), _p(keep, C.c_uint8),
                                        C.byref(info)))
        return dict(alt=alt, miss=miss, maf=maf, miss_rate=mr, keep=keep.astype(bool), kept=info.kept)

    def load_bed_file(self, prefix, min_maf=0.01, max_miss=0.2, chunk_bytes=0):
        """Stream <prefix>.bed from disk (globe_load_bed_file); same result as load_bed."""
        lib = self._L
        err = C.create_string_buffer(1024)
        M = C.c_int64()
        rc = lib.globe_bed_dims(prefix.encode(), self.N, C.byref(M), err, 1024)
        if rc:
            raise GlobeError(rc, err.value.decode())
        M = M.value
        alt = np.zeros(M, np.int64)
        miss = np.zeros(M, np.int64)
        maf = np.zeros(M, np.float32)
        mr = np.zeros(M, np.float32)
        keep = np.zeros(M, np.uint8)
        info = L.BedInfo()
        self._ck(lib.globe_load_bed_file(self.h, prefix.encode(), C.c_float(min_maf), C.c_float(max_miss),
                                         int(chunk_bytes), _p(alt, C.c_int64), _p(miss, C.c_int64),
                                         _p(maf, C.c_float), _p(mr, C.c_float), _p(keep, C.c_uint8), C.byref(info)))
        return dict(alt=alt, miss=miss, maf=maf, miss_rate=mr, keep=keep.astype(bool), kept=info.kept)

    def load_bed_dev(self, d_ptr, M, stride, min_maf=0.01, max_miss=0.2):
        info = L.BedInfo()
        self._ck(self._L.globe_load_bed_dev(self.h, C.c_void_p(d_ptr), M, stride, C.c_float(min_maf),
                                            C.c_float(max_miss), None, None, None, None, None, C.byref(info)))
        return info.kept

    def synth_bed_dev(self, d_ptr, M, N, stride, seed, maf_lo, maf_hi, miss_rate):
        self._ck(self._L.globe_synth_bed_dev(self.h, C.c_void_p(d_ptr), M, N, stride, seed, C.c_float(maf_lo),
                                             C.c_float(maf_hi), C.c_float(miss_rate)))

    def load_grm(self, grm_lt, N):
        g = np.ascontiguousarray(grm_lt, dtype=np.float32)
        assert g.size == N * (N + 1) // 2
        self._ck(self._L.globe_load_grm(self.h, _p(g, C.c_float), N))

    def set_precision(self, precision):
        self._ck(self._L.globe_set_precision(self.h, precision))

    def _probe_draws(self):
        """Normal draws per probe: Z1 (N), Z2 (2N, time effects only), Z3 (Nrec)."""
        no_time = self._L.globe_get_model(self.h) == L.MODEL_NO_TIME
        return (1 if no_time else 3) * self.N + self.Nrec

    def set_digits(self, nd):
        """Base-32 digits per column of the tensor-core product, 2..9 (default 9)."""
        self._ck(self._L.globe_set_digits(self.h, nd))

    def get_digits(self):
        return int(self._L.globe_get_digits(self.h))

    def set_graphs(self, on):
        """Replay the block-PCG iteration as a CUDA graph (default on; off while profiling)."""
        self._ck(self._L.globe_set_graphs(self.h, int(on)))

    def get_graphs(self):
        return bool(self._L.globe_get_graphs(self.h))

    def set_device_loop(self, on):
        """Run a solve's iterations after the first as one device-side loop (default on)."""
        self._ck(self._L.globe_set_device_loop(self.h, int(on)))

    def get_device_loop(self):
        return bool(self._L.globe_get_device_loop(self.h))

    def device_loop_runs(self):
        """Solves that ran their iterations as the device-side loop."""
        return int(self._L.globe_device_loop_runs(self.h))

    def set_record_df(self, on):
        """Run the record kernels of mixed-precision solves in double-float (default on)."""
        self._ck(self._L.globe_set_record_df(self.h, int(on)))

    def get_record_df(self):
        return bool(self._L.globe_get_record_df(self.h))

    def record_df_solves(self):
        """Solves that ran their record kernels in double-float."""
        return int(self._L.globe_record_df_solves(self.h))

    def set_autotune(self, on):
        """Time split counts and column groupings of the tensor-core product on first use (default on)."""
        self._ck(self._L.globe_set_autotune(self.h, int(on)))

    def get_autotune(self):
        return bool(self._L.globe_get_autotune(self.h))

    def autotune_log(self):
        """The autotuner's decisions (list of dicts)."""
        import json
        n = int(self._L.globe_autotune_log(self.h, None, 0))
        buf = C.create_string_buffer(n + 1)
        self._L.globe_autotune_log(self.h, buf, n + 1)
        return json.loads(buf.value.decode())

    def debug_force_splits(self, splits):
        """Test hook: every tensor-core genotype pass uses this split count (0 = off)."""
        self._ck(self._L.globe_debug_force_splits(self.h, int(splits)))

    def set_model(self, model):
        """MODEL_FULL (default) or MODEL_NO_TIME (components sig2e, sig2g only)."""
        self._ck(self._L.globe_set_model(self.h, model))

    def set_vc(self, vc):
        v = np.ascontiguousarray(vc, dtype=np.float64)
        self._ck(self._L.globe_set_vc(self.h, _p(v)))

    # ---- operators ----
    def grm_apply(self, Z):
        Z = _cols(Z, self.N)
        out = np.zeros_like(Z, order="F")
        self._ck(self._L.globe_grm_apply(self.h, _p(Z), _p(out), Z.shape[1]))
        return out

    def vx(self, x):
        x = _cols(x, self.Nrec)
        out = np.zeros_like(x, order="F")
        self._ck(self._L.globe_vx(self.h, _p(x), _p(out), x.shape[1]))
        return out

    def precond_apply(self, r):
        r = _cols(r, self.Nrec)
        z = np.zeros_like(r, order="F")
        self._ck(self._L.globe_precond_apply(self.h, _p(r), _p(z), r.shape[1]))
        return z

    def genetic_diag(self):
        d = np.zeros(self.N)
        self._ck(self._L.globe_genetic_diag(self.h, _p(d)))
        return d

    @staticmethod
    def opts(tol=1e-5, maxit=1000, rule=L.RULE_PCGSOLVER, x0mode=L.X0_ZERO, mask=False, precision=L.PREC_FP64):
        return PcgOpts(tol, maxit, rule, x0mode, int(bool(mask)), precision)

    @staticmethod
    def info_dict(info):
        return dict(iters=info.iters, inner_iters=info.inner_iters, rhs_iters=info.rhs_iters,
                    max_rel_res=info.max_rel_res, converged=bool(info.converged), stagnated=bool(info.stagnated))

    def pcg(self, B, X0=None, out=None, **kw):
        """Solve V X = B.  ``out``: optional Fortran-ordered float64 (Nrec x k)
        array that receives X (e.g. a pinned host buffer)."""
        B = _cols(B, self.Nrec)
        o = self.opts(**kw)
        if out is not None:
            assert out.shape == B.shape and out.dtype == np.float64 and out.flags.f_contiguous
            X = out
            if X0 is not None:
                X[...] = _cols(X0, self.Nrec)
        else:
            X = np.zeros_like(B, order="F") if X0 is None else _cols(X0, self.Nrec).copy(order="F")
        if X0 is not None:
            o.x0mode = L.X0_GIVEN
        info = PcgInfo()
        self._ck(self._L.globe_pcg(self.h, _p(B), _p(X), B.shape[1], C.byref(o), C.byref(info)))
        return X, self.info_dict(info)

    def pcg_dev(self, d_B, d_X, k, **kw):
        o = self.opts(**kw)
        info = PcgInfo()
        self._ck(self._L.globe_pcg_dev(self.h, C.c_void_p(d_B), C.c_void_p(d_X), k, C.byref(o), C.byref(info)))
        return self.info_dict(info)

    def mme(self, **kw):
        o = self.opts(**kw)
        info = PcgInfo()
        beta = np.zeros(self.p + 1)
        uhat = np.zeros(self.N)
        bhat = np.zeros(2 * self.N)
        vr = np.zeros(self.Nrec)
        self._ck(self._L.globe_mme(self.h, C.byref(o), _p(beta), _p(uhat), _p(bhat), _p(vr), C.byref(info)))
        return dict(beta=beta, uhat=uhat, bhat=bhat, vinv_r=vr, **self.info_dict(info))

    def aireml_grad(self, numMC, probes=None, seed=0, **kw):
        kw.setdefault("rule", L.RULE_AIREML)
        o = self.opts(**kw)
        info = PcgInfo()
        pr = None if probes is None else np.ascontiguousarray(probes, dtype=np.float64)
        if pr is not None:
            assert pr.size == numMC * self._probe_draws()
        fth = np.zeros((self.Nrec, 5), order="F")
        first, trace, grad = np.zeros(5), np.zeros(5), np.zeros(5)
        self._ck(self._L.globe_aireml_grad(self.h, _p(pr), numMC, C.c_uint64(seed), C.byref(o), _p(fth),
                                           _p(first), _p(trace), _p(grad), C.byref(info)))
        return dict(f_theta=fth, first=first, trace=trace, grad=grad, **self.info_dict(info))

    def aireml_eval(self, numMC, probes=None, seed=0, **kw):
        """MME + score with one block solve of [X y | probes] (globe_aireml_eval)."""
        kw.setdefault("rule", L.RULE_AIREML)
        o = self.opts(**kw)
        info = PcgInfo()
        pr = None if probes is None else np.ascontiguousarray(probes, dtype=np.float64)
        if pr is not None:
            assert pr.size == numMC * self._probe_draws()
        first, trace, grad = np.zeros(5), np.zeros(5), np.zeros(5)
        self._ck(self._L.globe_aireml_eval(self.h, _p(pr), numMC, C.c_uint64(seed), C.byref(o), _p(first),
                                           _p(trace), _p(grad), C.byref(info)))
        return dict(first=first, trace=trace, grad=grad, **self.info_dict(info))

    def aireml_ai(self, **kw):
        kw.setdefault("rule", L.RULE_AIREML)
        o = self.opts(**kw)
        info = PcgInfo()
        ai = np.zeros((5, 5), order="F")
        self._ck(self._L.globe_aireml_ai(self.h, C.byref(o), _p(ai), C.byref(info)))
        return np.array(ai)

    def aireml_run(self, theta0=(0.5, 0.3, 0.2, 0.1, 0.1), maxiter=50, tol=1e-3, numMC=15, pcg_tol=1e-5,
                   pcg_maxit=1000, precision=L.PREC_FP64, mask=False, seed=12345, probes=None, log_path=None,
                   fuse=True, digits=0):
        """digits: GLOBE_PREC_MIXED digits per column for this run (0: the context's, see set_digits)."""
        o = L.AiremlOpts()
        o.maxiter, o.tol, o.numMC = maxiter, tol, numMC
        for k in range(5):
            o.theta0[k] = theta0[k]
        o.pcg_tol, o.pcg_maxit, o.precision, o.mask, o.seed = pcg_tol, pcg_maxit, precision, int(mask), seed
        o.fuse = int(bool(fuse))
        o.digits = int(digits)
        pr = None
        if probes is not None:
            pr = np.ascontiguousarray(probes, dtype=np.float64)
            o.probes = _p(pr)
            o.probes_len = pr.size
        r = L.AiremlResult()
        self._ck(self._L.globe_aireml_run(self.h, C.byref(o), log_path.encode() if log_path else None, C.byref(r)))
        return dict(iterations=r.iterations, converged=bool(r.converged), theta=np.array(r.theta),
                    se=np.array(r.se), ai=np.array(r.ai).reshape(5, 5).T, grad=np.array(r.grad),
                    grad_evals=r.grad_evals, pcg_rhs_iters=r.pcg_rhs_iters)


def trust_region_step(theta, grad, ai, delta):
    """Solve oneIter_AIREML's step subproblem (varCompEst.cpp:1166-1199)."""
    th = np.ascontiguousarray(theta, np.float64)
    g = np.ascontiguousarray(grad, np.float64)
    A = np.asfortranarray(ai, np.float64).ravel(order="F").copy()
    p = np.zeros(5)
    st = C.c_int(0)
    rc = L.lib().globe_trust_region_step(_p(th), _p(g), _p(A), C.c_double(delta), _p(p), C.byref(st))
    if rc != L.GLOBE_OK:
        raise GlobeError(rc, "trust-region step")
    return p, st.value


def trust_region_step_no_time(theta, grad, ai, delta):
    """Step of the model without time effects (two components;
    varCompEst_reducedModel_noTime.cpp:782-830)."""
    th = np.ascontiguousarray(theta[:2], np.float64)
    g = np.ascontiguousarray(grad[:2], np.float64)
    A = np.asfortranarray(np.asarray(ai)[:2, :2], np.float64).ravel(order="F").copy()
    p = np.zeros(2)
    st = C.c_int(0)
    rc = L.lib().globe_trust_region_step_no_time(_p(th), _p(g), _p(A), C.c_double(delta), _p(p), C.byref(st))
    if rc != L.GLOBE_OK:
        raise GlobeError(rc, "trust-region step")
    return p, st.value


# ---- files ---------------------------------------------------------------

def read_records(path):
    """Record table (checkInputs + readInputData, PCGsolver.cpp:465-587).
    Returns indiv (0-based int32), X (Nrec x (p+1), time last), y, N."""
    lib = L.lib()
    err = C.create_string_buffer(1024)
    Nrec, N, p = C.c_int64(), C.c_int32(), C.c_int32()
    rc = lib.globe_read_records(path.encode(), C.byref(Nrec), C.byref(N), C.byref(p), None, None, None, err, 1024)
    if rc:
        raise GlobeError(rc, err.value.decode())
    indiv = np.zeros(Nrec.value, np.int32)
    X = np.zeros((Nrec.value, p.value + 1), order="F")
    y = np.zeros(Nrec.value)
    rc = lib.globe_read_records(path.encode(), C.byref(Nrec), C.byref(N), C.byref(p), _p(indiv, C.c_int32), _p(X),
                                _p(y), err, 1024)
    if rc:
        raise GlobeError(rc, err.value.decode())
    return indiv, X, y, N.value


def read_records_no_time(path):
    """Record table of the model without time effects: INDIV, PHENO and covariates
    in file order.  Returns indiv, X (Nrec x p), y, N."""
    lib = L.lib()
    err = C.create_string_buffer(1024)
    Nrec, N, p = C.c_int64(), C.c_int32(), C.c_int32()
    rc = lib.globe_read_records_no_time(path.encode(), C.byref(Nrec), C.byref(N), C.byref(p), None, None, None,
                                        err, 1024)
    if rc:
        raise GlobeError(rc, err.value.decode())
    indiv = np.zeros(Nrec.value, np.int32)
    X = np.zeros((Nrec.value, p.value), order="F")
    y = np.zeros(Nrec.value)
    rc = lib.globe_read_records_no_time(path.encode(), C.byref(Nrec), C.byref(N), C.byref(p), _p(indiv, C.c_int32),
                                        _p(X), _p(y), err, 1024)
    if rc:
        raise GlobeError(rc, err.value.decode())
    return indiv, X, y, N.value


def read_bed(prefix, N):
    lib = L.lib()
    err = C.create_string_buffer(1024)
    M = C.c_int64()
    rc = lib.globe_bed_dims(prefix.encode(), N, C.byref(M), err, 1024)
    if rc:
        raise GlobeError(rc, err.value.decode())
    payload = np.zeros((M.value, (N + 3) // 4), np.uint8)
    rc = lib.globe_read_bed(prefix.encode(), N, M.value, _p(payload, C.c_uint8), err, 1024)
    if rc:
        raise GlobeError(rc, err.value.decode())
    return payload


def read_grm(prefix, N):
    lib = L.lib()
    err = C.create_string_buffer(1024)
    g = np.zeros(N * (N + 1) // 2, np.float32)
    rc = lib.globe_read_grm(prefix.encode(), N, _p(g, C.c_float), err, 1024)
    if rc:
        raise GlobeError(rc, err.value.decode())
    return g


def write_grm(prefix, grm_lt, N):
    """<prefix>.grm.bin from the packed lower triangle (globe_write_grm)."""
    lib = L.lib()
    err = C.create_string_buffer(1024)
    g = np.ascontiguousarray(grm_lt, dtype=np.float32)
    assert g.size == N * (N + 1) // 2
    rc = lib.globe_write_grm(prefix.encode(), _p(g, C.c_float), N, err, 1024)
    if rc:
        raise GlobeError(rc, err.value.decode())


def read_vector(path):
    """saveVector layout (utils.cpp:18-34): int32 n, then n values (float32,
    or float64 for the .f64.bin files)."""
    b = open(path, "rb").read()
    n = int(np.frombuffer(b[:4], np.int32)[0])
    dt = np.float64 if len(b) - 4 == 8 * n else np.float32
    return np.frombuffer(b[4:], dt)[:n].copy()


def save_vector(path, v, f64=False):
    v = np.ascontiguousarray(v, np.float64)
    fn = L.lib().globe_save_vector_f64 if f64 else L.lib().globe_save_vector_f32
    rc = fn(path.encode(), _p(v), v.size)
    if rc:
        raise GlobeError(rc, "cannot write %s" % path)


def build_grm(geno, output, minMAF=0.01, maxMissingRate=0.2, precision=L.PREC_MIXED, device=0):
    """buildGRM: <output>.grm.bin of the PLINK fileset <geno> (N = lines of the .fam),
    the matrix runPCGsolver --geno applies.  Returns the packed lower triangle."""
    if not (0 <= minMAF <= 0.5 and 0 <= maxMissingRate <= 1):
        raise ValueError("Invalid MAF or missing rate thresholds.")
    with open(geno + ".fam") as f:
        N = sum(1 for line in f if line.split())
    with Context(device) as ctx:
        ctx.set_individuals(N)
        ctx.set_precision(precision)
        ctx.load_bed_file(geno, float(np.float32(minMAF)), float(np.float32(maxMissingRate)))
        lt = ctx.grm_build()
    write_grm(output, lt, N)
    return lt


def run_pcg_solver(input, output, sig2e, sig2g, sig2b0, sigb01, sig2b1, geno=None, grm=None, minMAF=0.01,
                   maxMissingRate=0.2, precision=L.PREC_FP64, pcg_tol=1e-5, pcg_maxit=1000, device=0, save64=False):
    """runPCGsolver (PCGsolver.cpp:235-306): writes <output>_beta/_uhat/_bhat.bin."""
    if (geno is None) == (grm is None):
        raise ValueError("exactly one of geno / grm")
    if not (0 <= minMAF <= 0.5 and 0 <= maxMissingRate <= 1):
        raise ValueError("Invalid MAF or missing rate thresholds.")
    indiv, X, y, N = read_records(input)
    with Context(device) as ctx:
        ctx.load_records(indiv, X, y, N)
        if geno is not None:
            ctx.load_bed(read_bed(geno, N), float(np.float32(minMAF)), float(np.float32(maxMissingRate)))
        else:
            ctx.load_grm(read_grm(grm, N), N)
        ctx.set_vc(as_float_vc((sig2e, sig2g, sig2b0, sigb01, sig2b1)))
        r = ctx.mme(tol=pcg_tol, maxit=pcg_maxit, rule=L.RULE_PCGSOLVER, x0mode=L.X0_ZERO, precision=precision)
    for nm in ("beta", "uhat", "bhat"):
        save_vector("%s_%s.bin" % (output, nm), r[nm])
        if save64:
            save_vector("%s_%s.f64.bin" % (output, nm), r[nm], f64=True)
    return r


def run_aireml(input_filename, grm_prefix, output_prefix, maxiter=50, tol=1e-3, numMC=15, sig2e=0.5, sig2g=0.3,
               sig2b0=0.2, sigb01=0.1, sig2b1=0.1, precision=L.PREC_FP64, pcg_tol=1e-5, seed=12345, probes=None,
               device=0):
    """runAIREML (varCompEst.cpp:1347-1500): writes <output_prefix>.log."""
    indiv, X, y, N = read_records(input_filename)
    with Context(device) as ctx:
        ctx.load_records(indiv, X, y, N)
        ctx.load_grm(read_grm(grm_prefix, N), N)
        return ctx.aireml_run(theta0=as_float_vc((sig2e, sig2g, sig2b0, sigb01, sig2b1)), maxiter=maxiter,
                              tol=float(np.float32(tol)), numMC=numMC, pcg_tol=pcg_tol, precision=precision,
                              seed=seed, probes=probes, log_path=output_prefix + ".log")
