"""General sparse Hamiltonians: other lattices and internal degrees of freedom.

The square-lattice path assembles H(t) on the device from the lattice and the field.  Any
other Hermitian operator that the reference's ``construct_operator`` builds
(src/operators/constructoperator.jl:4-47) -- HoneycombLattice, KagomeLattice, ``qwz`` and the
other zoo models, longer-range hopping -- enters as its ``SparseMatrixCSC`` (here a scipy CSC
matrix or the raw 1-based arrays) and is stored on the device as an ELL table.  The same
``ChebyshevGPU`` solver, ``Evolution`` driver, states and ``localdensity`` apply; the
currents are returned for every stored entry (``DensityCurrents(H, P)[i, j]``).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import weakref

import numpy as np

from . import _lib
from .device import default_context


class Sites:
    """The site set of a general Hamiltonian: N sites, optional coordinates (N x d)."""

    def __init__(self, N: int, coords=None, name: str = "Sites"):
        self.N = int(N)
        self.coords_ = None if coords is None else np.asarray(coords, dtype=np.float64)
        self.name = name

    def coords(self):
        return self.coords_

    def key(self):
        return ("sites", self.N, id(self))

    def __len__(self):
        return self.N

    def __repr__(self):
        return f"{self.name}({self.N} sites)"


def _csc_arrays(H):
    if isinstance(H, tuple):
        colptr, rowval, nzval = H
        return (np.ascontiguousarray(colptr, dtype=np.int64), np.ascontiguousarray(rowval, dtype=np.int64),
                np.ascontiguousarray(nzval, dtype=np.complex128))
    import scipy.sparse as sp
    M = sp.csc_matrix(H)
    M.sort_indices()
    return (M.indptr.astype(np.int64) + 1, M.indices.astype(np.int64) + 1,
            np.ascontiguousarray(M.data, dtype=np.complex128))


class _DeviceEll:
    """One lm_ell; values replaced in place when a new H(t) has the same pattern."""

    def __init__(self, ctx, n, colptr, rowval, nzval):
        self.ctx = ctx
        p = C.c_void_p()
        vals = np.ascontiguousarray(nzval).view(np.float64)
        ctx.check(ctx.lib.lm_ell_create_csc(ctx.handle, int(n), _lib.i64ptr(colptr), _lib.i64ptr(rowval),
                                            _lib.dptr(vals), C.byref(p)))
        self.handle = p
        self.values = np.array(nzval)
        weakref.finalize(self, ctx.lib.lm_ell_destroy, p)

    def ensure(self, nzval):
        if nzval is self.values or np.array_equal(nzval, self.values):
            return
        vals = np.ascontiguousarray(nzval, dtype=np.complex128)
        self.ctx.check(self.ctx.lib.lm_ell_set_values(self.handle, _lib.dptr(vals.view(np.float64))))
        self.values = vals.copy()


_cache: dict = {}


class SparseHamiltonian:
    """A Hermitian operator on ``sites`` given as a sparse matrix (scipy) or as the reference's
    CSC arrays (colptr, rowval, nzval), 1-based."""

    def __init__(self, sites: Sites, H):
        self.lattice = sites
        self.colptr, self.rowval, self.nzval = _csc_arrays(H)
        if len(self.colptr) != sites.N + 1:
            raise ValueError("matrix size does not match the site set")
        h = hashlib.sha1()
        h.update(self.colptr.tobytes())
        h.update(self.rowval.tobytes())
        self._pattern = (sites.N, h.hexdigest())

    @property
    def N(self):
        return self.lattice.N

    def __eq__(self, other):
        return (isinstance(other, SparseHamiltonian) and self._pattern == other._pattern
                and np.array_equal(self.nzval, other.nzval))

    __hash__ = None

    def device(self, ctx=None) -> _DeviceEll:
        ctx = ctx or default_context()
        key = (id(ctx), self._pattern)
        dh = _cache.get(key)
        if dh is None:
            if len(_cache) >= 8:
                _cache.pop(next(iter(_cache)))
            dh = _cache[key] = _DeviceEll(ctx, self.N, self.colptr, self.rowval, self.nzval)
        else:
            dh.ensure(self.nzval)
        return dh

    def bounds(self, ctx=None):
        ctx = ctx or default_context()
        dh = self.device(ctx)
        lo, hi = C.c_double(), C.c_double()
        ctx.check(ctx.lib.lm_ell_bounds(dh.handle, C.byref(lo), C.byref(hi)))
        return lo.value, hi.value

    def __repr__(self):
        return f"SparseHamiltonian({self.N}x{self.N}, nnz={len(self.rowval)}) on {self.lattice!r}"


def entry_currents(H: SparseHamiltonian, state) -> np.ndarray:
    """DensityCurrents(H, state)[i, j] = 2 Im(H[i,j] P[j,i]) (src/zoo/currents.jl:92-102) for every
    stored entry of H in CSC order (0 on the diagonal)."""
    ctx = state.ctx
    dh = H.device(ctx)
    out = np.empty(len(H.rowval), dtype=np.float64)
    ctx.check(ctx.lib.lm_ell_currents(dh.handle, state.handle, _lib.dptr(out)))
    return out
