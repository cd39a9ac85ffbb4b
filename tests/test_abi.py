"""libtp3.so loads and exports every symbol include/tp3.h declares; its host-only
table builder agrees with the oracle.  No GPU calls."""
import os
import re

import numpy as np
import pytest

import tp3
from tp3 import _lib
from oracle import sh
from oracle.basis import enumerate_basis

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "tp3.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(tp3_[A-Za-z0-9_]+)\s*\(", txt)))


def test_header_symbols_exported():
    lib = tp3.load()
    syms = declared_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(_lib.SIGNATURES), "ctypes table out of sync with include/tp3.h"


def test_julia_shim_binds_declared_symbols():
    """Every ccall of the Julia shim names an entry point that include/tp3.h declares and
    libtp3.so exports, with as many argument types as the declaration has parameters."""
    shim = os.path.join(os.path.dirname(HEADER), "..", "threephotons.jl_gb300", "julia", "ThreePhotonsGB300.jl")
    src = open(shim).read()
    calls = re.findall(r"ccall\(\(:(tp3_[A-Za-z0-9_]+), libtp3\),\s*\w+,\s*\(([^)]*)\)", src)
    assert len(calls) == src.count("ccall(("), "a ccall the pattern does not parse"
    header = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    lib = tp3.load()
    for name, argtypes in calls:
        assert hasattr(lib, name), name
        m = re.search(r"\b" + name + r"\s*\(([^)]*)\)", header)
        assert m, name
        nparams = 0 if m.group(1).strip() in ("", "void") else len(m.group(1).split(","))
        nargs = len([a for a in argtypes.split(",") if a.strip()])
        assert nargs == nparams, (name, nargs, nparams)


def test_status_strings():
    for s in range(0, 10):
        assert _lib.status_string(s)
    assert tp3.load().tp3_version() >> 16 == 1


def test_library_3j_matches_golden(golden_sh):
    lib = tp3.load()
    for l1, l2, l3, m1, m2, m3, v in golden_sh["wigner3j"]:
        assert lib.tp3_wigner3j(l1, l2, l3, m1, m2, m3) == pytest.approx(v, abs=1e-15, rel=1e-13)


def test_library_sphPlm_matches_golden(golden_sh):
    lib = tp3.load()
    for l, m, th, v in golden_sh["sphPlm"]:
        assert lib.tp3_sphPlm(l, m, th) == pytest.approx(v, abs=1e-13)


@pytest.mark.parametrize("L,LMAX,N,K", [(8, 9, 16, 8), (12, 25, 16, 15), (18, 25, 32, 26)])
def test_library_basis_info(L, LMAX, N, K):
    import ctypes
    info = (ctypes.c_int64 * 8)()
    assert tp3.load().tp3_basis_info(L, LMAX, N, K, 0.0, 0.0, info) == 0
    expect = {8: (4583, 65), 12: (26263, 175), 18: (163153, 505)}[L]
    assert (info[0], info[1]) == expect
    assert info[2] == K * (K + 1) * (K + 2) // 6
    assert info[3] == 2 * N * N and info[4] * info[5] == info[3]
    assert info[6] == (L // 2 + 1) * (L + 1)


def test_basis_info_rejects_bad_lmax():
    import ctypes
    info = (ctypes.c_int64 * 8)()
    assert tp3.load().tp3_basis_info(8, 8, 16, 8, 0.0, 0.0, info) == _lib.TP3_ERR_ARG


def test_umat_matches_oracle():
    for l in range(0, 9):
        np.testing.assert_allclose(tp3.Umat(l), sh.Umat(l), atol=0)
