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
from .observables import _CurrentsOps


class Sites:
    """The site set of a general Hamiltonian.  ``N`` is the matrix size (lattice sites times
    ``internal`` states per site, index = internal (site - 1) + alpha as in the reference's
    one-particle basis); optional coordinates, one row per site."""

    def __init__(self, N: int, coords=None, name: str = "Sites", internal: int = 1):
        self.N = int(N)
        self.internal = int(internal)
        if self.internal < 1 or self.N % self.internal:
            raise ValueError("internal must be a positive divisor of N")
        self.nsites = self.N // self.internal
        self.coords_ = None if coords is None else np.asarray(coords, dtype=np.float64)
        self.name = name

    def coords(self):
        return self.coords_

    def key(self):
        return ("sites", self.N, id(self))

    def __len__(self):
        return self.nsites

    def __repr__(self):
        if self.internal > 1:
            return f"{self.name}({self.nsites} sites x {self.internal} internal states)"
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


def _local_op(H: SparseHamiltonian, op):
    n = H.lattice.internal
    if op is None:
        return None
    O = np.asarray(op, dtype=np.complex128)
    if O.shape != (n, n):
        raise ValueError(f"operator must be {n}x{n}, the internal basis of the Hamiltonian")
    return np.ascontiguousarray(O.T).view(np.float64).ravel()  # column-major, interleaved


class SiteCurrents(_CurrentsOps):
    """DensityCurrents (src/zoo/currents.jl:81-102) or LocalOperatorCurrents (:150-184) of a
    state under a SparseHamiltonian.  One device pass gives the value of every stored entry of
    H (``lm_ell_op_currents``); ``curr[i, j]`` (1-based sites) is the sum over the entries of
    the (i, j) site block, which is the reference's ``getindex``."""

    def __init__(self, H: SparseHamiltonian, state, op=None):
        if H.lattice is not state.lattice and H.N != state.n:
            raise ValueError("Hamiltonian and state live on different site sets")
        self.hamiltonian = H
        self.state = state
        self.op = None if op is None else np.asarray(op, dtype=np.complex128)
        self._op_buf = _local_op(H, op)
        self._entries = None
        self._pairs = None

    @property
    def lattice(self):
        return self.hamiltonian.lattice

    def entry_values(self, out: np.ndarray = None) -> np.ndarray:
        """The contribution of every stored entry of H, in CSC order (0 inside a site block)."""
        if self._entries is None or out is not None:
            ctx = self.state.ctx
            dh = self.hamiltonian.device(ctx)
            vals = out if out is not None else np.empty(len(self.hamiltonian.rowval), dtype=np.float64)
            opp = None if self._op_buf is None else _lib.dptr(self._op_buf)
            ctx.check(ctx.lib.lm_ell_op_currents(dh.handle, self.state.handle, int(self.lattice.internal), opp,
                                                 _lib.dptr(vals)))
            if out is not None:
                return out
            self._entries = vals
        return self._entries

    bond_values = entry_values

    def site_pairs(self):
        """(src, dst, values): every ordered pair of distinct sites (1-based) with a stored
        block, and the summed current of that block."""
        if self._pairs is None:
            H = self.hamiltonian
            self._pairs = _aggregate_pairs(H, self.entry_values())
        return self._pairs

    def __getitem__(self, ij):
        if not isinstance(ij, tuple):
            return self.select(ij)
        i, j = ij
        src, dst, v = self.site_pairs()
        k = np.nonzero((src == i) & (dst == j))[0]
        return float(v[k[0]]) if len(k) else 0.0


def _entry_sites(H: SparseHamiltonian):
    n = H.lattice.internal
    cols = np.repeat(np.arange(H.N, dtype=np.int64), np.diff(H.colptr))
    return (H.rowval - 1) // n, cols // n


def _aggregate_pairs(H: SparseHamiltonian, entries):
    si, sj = _entry_sites(H)
    off = si != sj
    key = si[off] * H.lattice.nsites + sj[off]
    uk, inv = np.unique(key, return_inverse=True)
    vals = np.bincount(inv, weights=entries[off], minlength=len(uk))
    return uk // H.lattice.nsites + 1, uk % H.lattice.nsites + 1, vals


def LocalOperatorCurrents(H: SparseHamiltonian, state, op) -> SiteCurrents:
    """LocalOperatorCurrents(H, state, op) (src/zoo/currents.jl:150-170): currents of the local
    operator ``op`` (internal x internal) on a Hamiltonian with internal degrees of freedom."""
    if not isinstance(H, SparseHamiltonian) or H.lattice.internal < 2:
        raise ValueError("System expected to have internal degrees of freedom")
    return SiteCurrents(H, state, op)


def site_currents_matrix(curr: SiteCurrents):
    """Currents(curr) (src/currents.jl:223-237): curr[i, j] at [i, j] and -curr[i, j] at [j, i]
    for every site pair i > j, |value| < 1e-10 dropped; a scipy CSC matrix over the sites."""
    import scipy.sparse as sp
    src, dst, v = curr.site_pairs()
    lo = (src > dst) & (np.abs(v) >= 1e-10)
    r = np.concatenate([src[lo] - 1, dst[lo] - 1])
    c = np.concatenate([dst[lo] - 1, src[lo] - 1])
    d = np.concatenate([v[lo], -v[lo]])
    ns = curr.lattice.nsites
    return sp.csc_matrix((d, (r, c)), shape=(ns, ns))


def entry_currents(H: SparseHamiltonian, state) -> np.ndarray:
    """DensityCurrents(H, state)[i, j] = 2 Im(H[i,j] P[j,i]) (src/zoo/currents.jl:92-102) for every
    stored entry of H in CSC order (0 on the diagonal)."""
    ctx = state.ctx
    dh = H.device(ctx)
    out = np.empty(len(H.rowval), dtype=np.float64)
    ctx.check(ctx.lib.lm_ell_currents(dh.handle, state.handle, _lib.dptr(out)))
    return out
