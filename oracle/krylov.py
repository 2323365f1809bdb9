"""ctypes wrapper of the C restatement of KrylovKitExp (oracle/lm_oracle_krylov.c).

TEST INFRASTRUCTURE / CPU BASELINE ONLY: used by the tests and by the CPU-baseline leg of
bench.py, never by the product library.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import scipy.sparse as sp

HERE = Path(__file__).resolve().parent
SRC = HERE / "lm_oracle_krylov.c"
LIB = HERE / "_build" / "liblmoracle.so"

_lib = None


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    cc = shutil.which("gcc") or "cc"
    tmp = LIB.with_suffix(".tmp.so")
    cmd = [cc, "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(str(LIB))
        lib.lmo_krylov_block.restype = C.c_int
        lib.lmo_krylov_block.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                         C.c_void_p, C.c_int64, C.c_int64, C.c_double, C.c_int, C.c_int]
        lib.lmo_max_threads.restype = C.c_int
        _lib = lib
    return _lib


class CSR:
    """CSR arrays of a sparse complex matrix kept alive for the C calls."""

    def __init__(self, H):
        A = sp.csr_matrix(H)
        A.sort_indices()
        self.n = A.shape[0]
        self.rowptr = np.ascontiguousarray(A.indptr, dtype=np.int64)
        self.col = np.ascontiguousarray(A.indices, dtype=np.int64)
        self.val = np.ascontiguousarray(A.data, dtype=np.complex128)


def krylov_expv_block(csr: CSR, dt: float, X: np.ndarray, tol: float = 1e-12, kdim: int = 30,
                      nthreads: int = 0) -> np.ndarray:
    """exp(-i dt H) X column by column (in place on a Fortran copy, returned)."""
    lib = load()
    Y = np.asfortranarray(X, dtype=np.complex128).copy(order="F")
    if Y.ndim == 1:
        Y = Y.reshape(-1, 1, order="F")
    n, m = Y.shape
    fails = lib.lmo_krylov_block(n, csr.rowptr.ctypes.data, csr.col.ctypes.data, csr.val.ctypes.data,
                                 float(dt), Y.ctypes.data, n, m, float(tol), int(kdim), int(nthreads))
    if fails != 0:
        raise RuntimeError(f"exponentiate did not converge for {fails} kets")
    return Y


def max_threads() -> int:
    return load().lmo_max_threads()
