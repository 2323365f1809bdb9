"""Readouts: ``localdensity`` and ``DensityCurrents`` computed on the device.

localdensity: src/operators/latticeutils.jl:41-45 (Re P[i,i]; |psi_i|^2 for a ket).
DensityCurrents: src/zoo/currents.jl:81-102, J_ij = 2 Im(H[i,j] P[j,i]).
Currents: src/currents.jl:223-255 (materialised, |J| < 1e-10 dropped).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .hamiltonian import Hamiltonian
from .lattice import LatticeValue, SquareLattice
from .states import DeviceState

CURRENTS_EPS = 1e-10  # src/currents.jl:4


def _site_sum(lattice, vals):
    n = getattr(lattice, "internal", 1)
    return vals if n == 1 else vals.reshape(-1, n).sum(axis=1)


def localdensity(state: DeviceState) -> LatticeValue:
    """Re P[i,i] summed over the internal states of every site (latticeutils.jl:44)."""
    out = np.empty(state.n, dtype=np.float64)
    state.ctx.check(state.ctx.lib.lm_localdensity(state.handle, _lib.dptr(out)))
    return LatticeValue(state.lattice, _site_sum(state.lattice, out))


def localdensity_into(state: DeviceState, out: np.ndarray) -> np.ndarray:
    """localdensity into a caller-owned float64 buffer (e.g. pinned memory)."""
    state.ctx.check(state.ctx.lib.lm_localdensity(state.handle, _lib.dptr(out)))
    return out


class _CurrentsOps:
    """The AbstractCurrents surface shared by every currents object (src/currents.jl:1-109):
    ``curr[i, j]`` on 1-based sites, ``curr[mask]`` -> SubCurrents, iteration over site pairs
    and ``len``."""

    def _n(self):
        return getattr(self.lattice, "nsites", self.lattice.N)

    def __len__(self):
        n = self._n()
        return n * (n - 1) // 2

    def __iter__(self):
        """((src, dst), value) for every pair i < j, oriented so that the value is >= 0
        (src/currents.jl:37-47)."""
        M = self._matrix()
        n = self._n()
        for i in range(1, n + 1):
            row = M[i - 1]
            for j in range(i + 1, n + 1):
                c = row[j - 1]
                yield ((i, j), c) if c > 0 else ((j, i), -c)

    def _matrix(self):
        """Dense antisymmetric matrix of curr[i, j] (small lattices; iteration)."""
        n = self._n()
        return np.array([[0.0 if i == j else self[i, j] for j in range(1, n + 1)] for i in range(1, n + 1)])

    def select(self, sel):
        from .lattice import site_indices
        return SubCurrents(self, site_indices(self.lattice, sel))


class DensityCurrents(_CurrentsOps):
    """Lazy density currents of ``state`` under ``H``; bond values come from one device pass.
    For a SparseHamiltonian this is a ``SiteCurrents`` (per stored entry, summed per site
    block)."""

    def __new__(cls, H, state):
        from .sparse import SiteCurrents, SparseHamiltonian
        if isinstance(H, SparseHamiltonian):
            return SiteCurrents(H, state)
        return super().__new__(cls)

    def __init__(self, H: Hamiltonian, state: DeviceState):
        if H.lattice != state.lattice:
            raise ValueError("Hamiltonian and state live on different lattices")
        self.hamiltonian = H
        self.state = state
        self._vals = None

    @property
    def lattice(self):
        return self.hamiltonian.lattice

    def bond_values(self, out: np.ndarray = None) -> np.ndarray:
        """J on every NearestNeighbor(1) bond, in the lattice's bond order."""
        if self._vals is None or out is not None:
            ctx = self.state.ctx
            dh = self.hamiltonian.device(ctx)
            nb = self.lattice.nbonds()
            vals = out if out is not None else np.empty(nb, dtype=np.float64)
            ctx.check(ctx.lib.lm_bond_currents(dh.handle, self.state.handle, _lib.dptr(vals)))
            if out is not None:
                return out
            self._vals = vals
        return self._vals

    def __getitem__(self, ij):
        """dc[i, j] for 1-based site indices (zero between non-adjacent sites); dc[mask] is a
        SubCurrents."""
        if not isinstance(ij, tuple):
            return self.select(ij)
        i, j = ij
        if i == j:
            return 0.0
        src, dst = self.lattice.bonds()
        v = self.bond_values()
        tot = 0.0
        for b in np.nonzero((src == i) & (dst == j))[0]:
            tot += v[b]
        for b in np.nonzero((src == j) & (dst == i))[0]:
            tot -= v[b]
        # a pair joined by two bonds carries the current of one matrix entry
        return tot / max(1, len(np.nonzero(((src == i) & (dst == j)) | ((src == j) & (dst == i)))[0]))


class SubCurrents(_CurrentsOps):
    """``curr[mask]`` (src/currents.jl:50-66): the same currents on a subset of the sites,
    indexed 1..n within the subset."""

    def __init__(self, parent, indices):
        self.parent = parent
        self.indices = np.asarray(indices, dtype=np.int64)
        self.lattice = _SubSites(parent.lattice, self.indices)

    def __getitem__(self, ij):
        if not isinstance(ij, tuple):
            return self.select(ij)
        i, j = ij
        return self.parent[int(self.indices[i - 1]), int(self.indices[j - 1])]

    def _matrix(self):
        M = _full_matrix(self.parent)
        if M is not None:
            idx = self.indices - 1
            return np.asarray(M[np.ix_(idx, idx)].todense() if hasattr(M, "todense") else M[np.ix_(idx, idx)])
        return super()._matrix()


class _SubSites:
    """The site subset a SubCurrents lives on."""

    def __init__(self, parent_lattice, indices):
        self.parent = parent_lattice
        self.indices = indices
        self.N = len(indices)
        self.nsites = len(indices)

    def coords(self):
        return self.parent.coords()[self.indices - 1]

    def __repr__(self):
        return f"{len(self.indices)}-site subset of {self.parent!r}"


def _full_matrix(curr):
    """Antisymmetric sparse matrix of every curr[i, j], when the object can give it without
    calling curr[i, j] pair by pair; else None."""
    if isinstance(curr, Currents):
        return curr.currents.tocsr()
    if isinstance(curr, DensityCurrents):
        return _bond_matrix(curr, drop=False).tocsr()
    from .sparse import SiteCurrents
    if isinstance(curr, SiteCurrents):
        import scipy.sparse as sp
        src, dst, v = curr.site_pairs()
        n = curr.lattice.nsites
        return sp.coo_matrix((v, (src - 1, dst - 1)), shape=(n, n)).tocsr()
    return None


def _bond_matrix(curr, drop=True):
    import scipy.sparse as sp
    lat = curr.lattice
    src, dst = lat.bonds()
    v = curr.bond_values()
    keep = np.abs(v) >= CURRENTS_EPS if drop else np.ones(len(v), dtype=bool)
    r = np.concatenate([src[keep] - 1, dst[keep] - 1])
    c = np.concatenate([dst[keep] - 1, src[keep] - 1])
    d = np.concatenate([v[keep], -v[keep]])
    m = sp.coo_matrix((d, (r, c)), shape=(lat.N, lat.N)).tocsc()
    m.sum_duplicates()
    return m


class Currents(_CurrentsOps):
    """Materialised antisymmetric currents (src/currents.jl:111-255): ``Currents(curr[, bonds])``
    from any currents object, or ``Currents(lattice)`` for an empty one."""

    def __init__(self, curr, bonds=None):
        import scipy.sparse as sp
        from .sparse import SiteCurrents, site_currents_matrix
        if isinstance(curr, (SquareLattice,)) or hasattr(curr, "nsites") and not hasattr(curr, "lattice"):
            n = getattr(curr, "nsites", curr.N)
            self.lattice = curr
            self.currents = sp.csc_matrix((n, n))
            return
        if isinstance(curr, SubCurrents):
            self.lattice = curr.lattice
            M = np.array(curr._matrix(), dtype=np.float64)
            n = M.shape[0]
            lo = np.tril(np.ones((n, n), dtype=bool), -1)
            keep = lo & (np.abs(M) >= CURRENTS_EPS)
            I, J = np.nonzero(keep)
            v = M[I, J]
            self.currents = sp.csc_matrix((np.concatenate([v, -v]), (np.concatenate([I, J]), np.concatenate([J, I]))),
                                          shape=(n, n))
            return
        if isinstance(curr, SiteCurrents):
            if bonds is not None:
                raise ValueError("bond subsets are defined for the square-lattice path only")
            self.lattice = curr.lattice
            self.currents = site_currents_matrix(curr)
            return
        self.lattice = curr.lattice
        self.currents = _bond_matrix(curr)

    @classmethod
    def _from_matrix(cls, lattice, m):
        c = object.__new__(cls)
        c.lattice = lattice
        c.currents = m.tocsc()
        return c

    def __getitem__(self, ij):
        if not isinstance(ij, tuple):
            return self.select(ij)
        i, j = ij
        return self.currents[i - 1, j - 1]

    def __setitem__(self, ij, value):
        """m[i, j] = v sets m[j, i] = -v (src/currents.jl:125-136); i == j is refused with a
        warning, as in the reference."""
        import warnings
        i, j = ij
        if i == j:
            if value != 0:
                warnings.warn("Attempt to assign nonzero current from site to self")
            return
        m = self.currents.tolil()
        m[i - 1, j - 1] = value
        m[j - 1, i - 1] = -value
        self.currents = m.tocsc()

    def _matrix(self):
        return self.currents.toarray()

    def toarray(self):
        return self.currents.toarray()

    # arithmetic of materialised currents on the same lattice (src/currents.jl:138-152)
    def __add__(self, other):
        return Currents._from_matrix(self.lattice, self.currents + other.currents)

    def __sub__(self, other):
        return Currents._from_matrix(self.lattice, self.currents - other.currents)

    def __mul__(self, k):
        return Currents._from_matrix(self.lattice, self.currents * float(k))

    __rmul__ = __mul__

    def __truediv__(self, k):
        return Currents._from_matrix(self.lattice, self.currents / float(k))

    def __neg__(self):
        return Currents._from_matrix(self.lattice, -self.currents)

    def zero(self):
        return Currents._from_matrix(self.lattice, self.currents * 0.0)

    def isapprox(self, other, rtol: float = 1.4901161193847656e-08):
        """``≈`` on the current matrices (Frobenius norm, relative)."""
        a = self.currents.toarray()
        b = other.currents.toarray() if isinstance(other, Currents) else np.asarray(other._matrix())
        return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b))


def currentsfrom(curr, src) -> LatticeValue:
    """``currentsfrom(curr, src)`` (src/currents.jl:78-89): for every site j, 0 inside ``src``,
    else the sum of curr[i, j] over i in ``src``."""
    from .lattice import site_indices
    lat = curr.lattice
    n = getattr(lat, "nsites", lat.N)
    src_i = [int(i) for i in site_indices(lat, src)]
    M = _full_matrix(curr)
    if M is not None:
        rows = np.asarray(M[np.array(src_i) - 1].sum(axis=0)).ravel()
        out = rows.copy()
    else:
        out = np.array([sum(curr[i, j] for i in src_i) for j in range(1, n + 1)], dtype=np.float64)
    out[np.array(src_i) - 1] = 0.0
    return LatticeValue(lat, out)


def currentsfromto(curr, src, dst=None) -> float:
    """currentsfromto(curr, src[, dst]) (src/currents.jl:104-109): the sum of curr[i, j] over
    i in ``src`` and j in ``dst`` (default: every other site); sites as 1-based indices or
    Bool masks."""
    from .lattice import site_indices
    ns = getattr(curr.lattice, "nsites", curr.lattice.N)
    src = [int(i) for i in site_indices(curr.lattice, src)]
    if dst is None:
        sset = set(src)
        dst = [j for j in range(1, ns + 1) if j not in sset]
    else:
        dst = [int(j) for j in site_indices(curr.lattice, dst)]
    M = _full_matrix(curr)
    if M is not None:
        return float(M[np.ix_(np.array(src) - 1, np.array(dst) - 1)].sum())
    return float(sum(curr[i, j] for i in src for j in dst))
