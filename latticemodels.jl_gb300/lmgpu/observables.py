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
from .lattice import LatticeValue
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


class DensityCurrents:
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
        """dc[i, j] for 1-based site indices (zero between non-adjacent sites)."""
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


class Currents:
    """Materialised antisymmetric currents on the bonds (src/currents.jl:223-255)."""

    def __init__(self, curr: DensityCurrents, bonds=None):
        import scipy.sparse as sp
        from .sparse import SiteCurrents, site_currents_matrix
        if isinstance(curr, SiteCurrents):
            if bonds is not None:
                raise ValueError("bond subsets are defined for the square-lattice path only")
            self.lattice = curr.lattice
            self.currents = site_currents_matrix(curr)
            return
        lat = curr.lattice
        src, dst = lat.bonds()
        v = curr.bond_values()
        keep = np.abs(v) >= CURRENTS_EPS
        r = np.concatenate([src[keep] - 1, dst[keep] - 1])
        c = np.concatenate([dst[keep] - 1, src[keep] - 1])
        d = np.concatenate([v[keep], -v[keep]])
        m = sp.coo_matrix((d, (r, c)), shape=(lat.N, lat.N)).tocsc()
        m.sum_duplicates()
        self.lattice = lat
        self.currents = m

    def __getitem__(self, ij):
        i, j = ij
        return self.currents[i - 1, j - 1]

    def toarray(self):
        return self.currents.toarray()


def currentsfromto(curr, src, dst=None) -> float:
    """currentsfromto(curr, src[, dst]) (src/currents.jl:104-109): the sum of curr[i, j] over
    i in ``src`` and j in ``dst`` (default: every other site); 1-based site indices."""
    ns = getattr(curr.lattice, "nsites", curr.lattice.N)
    src = [src] if np.ndim(src) == 0 else list(src)
    dst = [j for j in range(1, ns + 1) if j not in src] if dst is None else ([dst] if np.ndim(dst) == 0 else list(dst))
    if isinstance(curr, Currents):
        M = curr.currents.tocsr()
        return float(sum(M[i - 1, j - 1] for i in src for j in dst))
    return float(sum(curr[i, j] for i in src for j in dst))
