"""C-ABI checks that need no GPU: every declared symbol is exported, the
host-only readers/writers follow the reference's formats and fail cleanly."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import globe_gb300 as G
from globe_gb300 import _lib
from helpers import GOLDEN, ROOT, golden_case, parse_records_py


def _declared():
    src = open(os.path.join(ROOT, "include", "globe.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(globe_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported():
    L = _lib.lib()
    names = _declared()
    assert len(names) >= 30
    for n in names:
        assert hasattr(L, n), n
    assert set(names) <= set(_lib.SIGNATURES), set(names) - set(_lib.SIGNATURES)


def test_create_fails_cleanly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(G.GlobeError) as e:
        G.Context(0)
    assert e.value.code in (-2, -1)


@pytest.mark.parametrize("name", ["geno_small", "tiny", "aireml_small"])
def test_read_records_matches_independent_parse(name):
    indiv, X, y, N = G.read_records(os.path.join(GOLDEN, name + ".txt"))
    i2, X2, y2, N2 = parse_records_py(os.path.join(GOLDEN, name + ".txt"))
    assert N == N2 and np.array_equal(indiv, i2) and np.array_equal(X, X2) and np.array_equal(y, y2)


def _write(tmp, text):
    p = os.path.join(tmp, "r.txt")
    open(p, "w").write(text)
    return p


def test_read_records_errors(tmp_path):
    t = str(tmp_path)
    with pytest.raises(G.GlobeError, match="Missing required columns"):
        G.read_records(_write(t, "INDIV PHENO C1\n1 2 3\n"))
    with pytest.raises(G.GlobeError, match="cannot parse"):
        G.read_records(_write(t, "INDIV PHENO TIMES C\n1 2 x 1\n"))
    with pytest.raises(G.GlobeError, match="outside"):
        G.read_records(_write(t, "INDIV PHENO TIMES C\n1 2 0 1\n2 2 0 1\n5 1 1 1\n"))
    with pytest.raises(G.GlobeError):
        G.read_records(os.path.join(t, "does_not_exist.txt"))
    # named columns anywhere: covariates keep file order, time is last
    indiv, X, y, N = G.read_records(_write(t, "C0 TIMES INDIV C1 PHENO\n1 0.5 1 7 2.5\n1 1.5 2 8 3.5\n"))
    assert N == 2 and list(indiv) == [0, 1]
    assert np.array_equal(X, [[1, 7, 0.5], [1, 8, 1.5]]) and np.array_equal(y, [2.5, 3.5])


def test_bed_and_grm_readers(tmp_path):
    c = golden_case("geno_small")
    pay = G.read_bed(c["prefix"], c["N"])
    assert np.array_equal(pay, c["packed"])
    g = G.read_grm(c["prefix"], c["N"])
    assert np.array_equal(g, c["grm"])
    t = str(tmp_path)
    pre = os.path.join(t, "x")
    open(pre + ".bim", "w").write("a\nb\n")
    open(pre + ".bed", "wb").write(bytes([0x6C, 0x1B, 0x00]) + bytes(10))
    with pytest.raises(G.GlobeError, match="individual-major"):
        G.read_bed(pre, 8)
    open(pre + ".bed", "wb").write(bytes([0x6C, 0x1C, 0x01]) + bytes(10))
    with pytest.raises(G.GlobeError, match="magic"):
        G.read_bed(pre, 8)
    open(pre + ".bed", "wb").write(bytes([0x6C, 0x1B, 0x01]) + bytes(3))
    with pytest.raises(G.GlobeError, match="need"):
        G.read_bed(pre, 8)      # 2 SNPs x 2 bytes needed
    open(pre + ".grm.bin", "wb").write(np.zeros(5, np.float32).tobytes())
    with pytest.raises(G.GlobeError, match="Error reading"):
        G.read_grm(pre, 4)      # needs 10 values


def test_save_vector_layout(tmp_path):
    v = np.array([1.5, -2.25, 3e-8])
    p = os.path.join(str(tmp_path), "v.bin")
    G.save_vector(p, v)
    b = open(p, "rb").read()
    assert np.frombuffer(b[:4], np.int32)[0] == 3 and len(b) == 4 + 12
    assert np.array_equal(G.read_vector(p), v.astype(np.float32))
    G.save_vector(p, v, f64=True)
    assert np.array_equal(G.read_vector(p), v)
