"""ctypes wrapper of the C oracle (``oracle/globe_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``; never by the ``globe_gb300``
package.  ``build()`` compiles the oracle with gcc (OpenMP when available).
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libglobe_oracle.so")
SRC = os.path.join(HERE, "globe_oracle.c")

_dp = C.POINTER(C.c_double)
_fp = C.POINTER(C.c_float)


def build(force=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "globe_oracle.h"))):
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-fPIC", "-shared", SRC, "-o", LIB, "-lm"]
    subprocess.check_call(cmd)
    return LIB


class _Model(C.Structure):
    _fields_ = [("N", C.c_int32), ("Nrec", C.c_int64), ("p", C.c_int32),
                ("indiv", C.POINTER(C.c_int32)), ("X", _dp), ("y", _dp),
                ("geno", C.POINTER(C.c_uint8)), ("Mk", C.c_int64), ("stride", C.c_int64),
                ("f", _dp), ("inv_std", _dp), ("grm_lt", _fp), ("vc", C.c_double * 5)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.orc_bed_stats.restype = C.c_int64
        L.orc_create.restype = C.c_void_p
        for fn in ("orc_destroy", "orc_set_vc", "orc_grm_apply", "orc_genetic_diag", "orc_vx",
                   "orc_precond_build", "orc_precond_apply", "orc_pcg", "orc_mme",
                   "orc_aireml_grad", "orc_aireml_ai"):
            getattr(L, fn).argtypes = None
        _lib = L
    return _lib


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def bed_stats(packed, N, min_maf=0.01, max_miss=0.2):
    """Per-SNP (alt, miss, maf f32, miss_rate f32, keep) -- PCGsolver.cpp:700-743."""
    packed = np.ascontiguousarray(packed, dtype=np.uint8)
    M = packed.shape[0]
    alt = np.zeros(M, np.int64)
    miss = np.zeros(M, np.int64)
    maf = np.zeros(M, np.float32)
    mr = np.zeros(M, np.float32)
    keep = np.zeros(M, np.uint8)
    lib().orc_bed_stats(_p(packed, C.c_uint8), C.c_int64(M), C.c_int32(N), C.c_float(min_maf),
                        C.c_float(max_miss), _p(alt, C.c_int64), _p(miss, C.c_int64), _p(maf, C.c_float),
                        _p(mr, C.c_float), _p(keep, C.c_uint8))
    return alt, miss, maf, mr, keep.astype(bool)


def std_params(alt, miss, N):
    alt = np.ascontiguousarray(alt, np.int64)
    miss = np.ascontiguousarray(miss, np.int64)
    f = np.zeros(len(alt))
    inv = np.zeros(len(alt))
    lib().orc_std_params(_p(alt, C.c_int64), _p(miss, C.c_int64), C.c_int64(len(alt)), C.c_int32(N),
                         _p(f), _p(inv))
    return f, inv


def grm_build(packed, N, min_maf=0.01, max_miss=0.2, freq="f64"):
    """A = Zs'Zs / M_kept as the float32 packed lower triangle (orc_grm_build).
    freq "f64": the allele frequency and inverse std of the float->double
    reference build (std_params; what the product path uses).  freq "f32": the
    FP32 program's float maf (PCGsolver.cpp:728) widened to double, with
    inv_std = 1/sqrt(2f(1-f)) in double (1 when 2f(1-f) <= 1e-12)."""
    alt, miss, maf, _, keep = bed_stats(packed, N, min_maf, max_miss)
    kp = np.ascontiguousarray(np.asarray(packed, np.uint8)[keep])
    if freq == "f64":
        f, inv = std_params(alt[keep], miss[keep], N)
    else:
        f = maf[keep].astype(np.float64)
        den = 2 * f * (1 - f)
        inv = np.where(den > 1e-12, 1.0 / np.sqrt(np.where(den > 0, den, 1.0)), 1.0)
    lt = np.zeros(N * (N + 1) // 2, np.float32)
    lib().orc_grm_build(_p(kp, C.c_uint8), C.c_int64(kp.shape[0]), C.c_int64((N + 3) // 4), C.c_int32(N),
                        _p(f), _p(inv), _p(lt, C.c_float))
    return lt


class Solver:
    """One cohort + one genetic source (kept genotypes or dense packed GRM)."""

    def __init__(self, indiv, X, y, N, vc, packed=None, alt=None, miss=None, keep=None, grm_lt=None):
        self._keep = []
        indiv = np.ascontiguousarray(indiv, np.int32)
        X = np.asfortranarray(X, np.float64)
        y = np.ascontiguousarray(y, np.float64)
        m = _Model()
        m.N = N
        m.Nrec = len(indiv)
        m.p = X.shape[1] - 1
        m.indiv = _p(indiv, C.c_int32)
        m.X = _p(X)
        m.y = _p(y)
        self.N, self.Nrec, self.p = N, len(indiv), X.shape[1] - 1
        self._keep += [indiv, X, y]
        if packed is not None:
            if alt is None:
                alt, miss, _, _, keep = bed_stats(packed, N)
            kp = np.ascontiguousarray(packed[keep], np.uint8)
            f, inv = std_params(alt[keep], miss[keep], N)
            m.geno = _p(kp, C.c_uint8)
            m.Mk = kp.shape[0]
            m.stride = kp.shape[1] if kp.ndim == 2 else (N + 3) // 4
            m.f = _p(f)
            m.inv_std = _p(inv)
            self._keep += [kp, f, inv]
            self.f, self.inv_std, self.Mk = f, inv, kp.shape[0]
        else:
            g = np.ascontiguousarray(grm_lt, np.float32)
            m.grm_lt = _p(g, C.c_float)
            self._keep.append(g)
        for i in range(5):
            m.vc[i] = vc[i]
        self._m = m
        self.h = C.c_void_p(lib().orc_create(C.byref(m)))

    def __del__(self):
        try:
            lib().orc_destroy(self.h)
        except Exception:
            pass

    def set_vc(self, vc):
        a = np.ascontiguousarray(vc, np.float64)
        lib().orc_set_vc(self.h, _p(a))

    def grm_apply(self, Z):
        Z = np.asfortranarray(np.atleast_2d(Z.T).T, np.float64)
        out = np.zeros_like(Z, order="F")
        lib().orc_grm_apply(self.h, _p(Z), C.c_int(Z.shape[1]), _p(out))
        return out

    def genetic_diag(self):
        d = np.zeros(self.N)
        lib().orc_genetic_diag(self.h, _p(d))
        return d

    def vx(self, x):
        x = np.asfortranarray(np.atleast_2d(x.T).T, np.float64)
        out = np.zeros_like(x, order="F")
        lib().orc_vx(self.h, _p(x), C.c_int(x.shape[1]), _p(out))
        return out

    def precond_build(self):
        lib().orc_precond_build(self.h)

    def precond_apply(self, r):
        r = np.asfortranarray(np.atleast_2d(r.T).T, np.float64)
        z = np.zeros_like(r, order="F")
        lib().orc_precond_apply(self.h, _p(r), C.c_int(r.shape[1]), _p(z))
        return z

    def pcg(self, B, tol, maxit=1000, rule=0, x0mode=0, X0=None):
        B = np.asfortranarray(np.atleast_2d(B.T).T, np.float64)
        X = np.zeros_like(B, order="F") if X0 is None else np.asfortranarray(X0, np.float64).copy(order="F")
        it = lib().orc_pcg(self.h, _p(B), _p(X), C.c_int(B.shape[1]), C.c_double(tol), C.c_int(maxit),
                           C.c_int(rule), C.c_int(x0mode))
        return X, it

    def mme(self, tol, maxit=1000, rule=0, x0mode=0):
        beta = np.zeros(self.p + 1)
        uhat = np.zeros(self.N)
        bhat = np.zeros(2 * self.N)
        vr = np.zeros(self.Nrec)
        it = lib().orc_mme(self.h, C.c_double(tol), C.c_int(maxit), C.c_int(rule), C.c_int(x0mode),
                           _p(beta), _p(uhat), _p(bhat), _p(vr))
        return dict(beta=beta, uhat=uhat, bhat=bhat, vinv_r=vr, iters=it)

    def aireml_grad(self, probes, numMC, tol, maxit=1000):
        probes = np.ascontiguousarray(probes, np.float64)
        assert probes.size == numMC * (3 * self.N + self.Nrec)
        fth = np.zeros((self.Nrec, 5), order="F")
        first = np.zeros(5)
        trace = np.zeros(5)
        grad = np.zeros(5)
        it = lib().orc_aireml_grad(self.h, _p(probes), C.c_int(numMC), C.c_double(tol), C.c_int(maxit),
                                   _p(fth), _p(first), _p(trace), _p(grad))
        return dict(f_theta=fth, first=first, trace=trace, grad=grad, iters=it)

    def aireml_ai(self, fth, tol, maxit=1000):
        fth = np.asfortranarray(fth, np.float64)
        ai = np.zeros((5, 5), order="F")
        lib().orc_aireml_ai(self.h, _p(fth), C.c_double(tol), C.c_int(maxit), _p(ai))
        return np.array(ai)


def ref_vx_f32(indiv, times, packed_kept, maf_kept, vc, x, N):
    """FP32 V.x with the reference's loop structure (timing baseline)."""
    indiv = np.ascontiguousarray(indiv, np.int32)
    times = np.ascontiguousarray(times, np.float32)
    g = np.ascontiguousarray(packed_kept, np.uint8)
    maf = np.ascontiguousarray(maf_kept, np.float32)
    v = np.ascontiguousarray(vc, np.float32)
    x = np.asfortranarray(np.atleast_2d(x.T).T, np.float32)
    if x.shape[1] > 256:
        raise ValueError("the FP32 reference-structure port takes at most 256 columns")
    out = np.zeros_like(x, order="F")
    lib().orc_ref_vx_f32(C.c_int32(N), C.c_int64(len(indiv)), _p(indiv, C.c_int32), _p(times, C.c_float),
                         _p(g, C.c_uint8), C.c_int64(g.shape[0]), C.c_int64(g.shape[1]), _p(maf, C.c_float),
                         _p(v, C.c_float), _p(x, C.c_float), C.c_int(x.shape[1]), _p(out, C.c_float))
    return out
