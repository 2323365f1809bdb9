"""Bravais lattices with a basis (HoneycombLattice, KagomeLattice, TriangularLattice) and their
nearest-neighbour tight-binding Hamiltonians, assembled on the device from the bond geometry.

Geometry as the reference builds it:
* unit cells (j1, j2), 1 <= j1 <= a, 1 <= j2 <= b, basis sites s = 1..nb, in the order of the
  Bravais pointers (j1, j2, s) (src/lattices/bravais/unitcell.jl:113-132), site coordinates
  j1 a1 + j2 a2 + b_s (src/zoo/lattices.jl:145-211 for the unit cells);
* nearest-neighbour translations from the shortest basis-to-basis distance over the unit-cell
  offsets C in {-2..2}^2 (detect_nnhops, src/lattices/bravais/nearestneighbor.jl:87-131): a
  translation (i => j, C) for i < j, or (C) for every basis index when i == j, counted once per
  direction (first nonzero component of C positive);
* bonds iterate the translations, then the sites in lattice order: site -> its destination
  (src/lattices/bravais/bonds.jl:87-98), routed through periodic boundaries along a a1
  ("axis1") and b a2 ("axis2") with the twist factor e^{i Theta} per wrap, the unwrapped
  destination kept for the field's line integral (src/core/boundaries.jl:251-289).

``tightbinding_hamiltonian(lat, [V]; t1, field)`` gives a ``LatticeHamiltonian``: H[i, j] =
t1 e^{i Theta n} e^{-2 pi i LI(r_i -> r_j)}, H[j, i] its conjugate and the on-site term, assembled
by the library (lm_ell_create_bonds, lm_ell_assemble) each time the field amplitudes or the
on-site term change.  It evolves, reads out and diagonalises like any general Hamiltonian.
"""
from __future__ import annotations

import ctypes as C
import math
import weakref
from collections import OrderedDict

import numpy as np

from . import _lib
from .device import default_context
from .fields import AbstractField, NoField
from .lattice import LatticeValue
from .sparse import SparseHamiltonian

_SQ3 = math.sqrt(3.0)
UNITCELLS = {
    # name: (unit vectors as columns, basis sites as columns)
    "TriangularLattice": (np.array([[1.0, 0.5], [0.0, _SQ3 / 2]]), np.array([[0.0], [0.0]])),
    "HoneycombLattice": (np.array([[1.0, 0.5], [0.0, _SQ3 / 2]]), np.array([[0.0, 0.5], [0.0, _SQ3 / 6]])),
    "KagomeLattice": (np.array([[1.0, 0.5], [0.0, _SQ3 / 2]]), np.array([[0.0, 0.5, 0.25], [0.0, 0.0, _SQ3 / 4]])),
}


def _offsets(depth: int):
    """CartesianIndex(-d, -d):CartesianIndex(d, d), the first index fastest."""
    return [(c1, c2) for c2 in range(-depth, depth + 1) for c1 in range(-depth, depth + 1)]


class BravaisLattice:
    """An a x b patch of a two-dimensional Bravais lattice with a basis."""

    def __init__(self, name: str, a: int, b: int, boundaries=None):
        if name not in UNITCELLS:
            raise ValueError(f"unknown lattice {name}")
        if a < 1 or b < 1:
            raise ValueError("lattice size must be positive")
        self.name = name
        self.a, self.b = int(a), int(b)
        self.T, self.basis = UNITCELLS[name]
        self.nb = self.basis.shape[1]
        self.N = self.nb * self.a * self.b
        self.internal = 1
        self.nsites = self.N
        per, tw = [False, False], [0.0, 0.0]
        for k, v in (boundaries or {}).items():
            ax = {"axis1": 0, "axis2": 1}.get(k)
            if ax is None:
                raise ValueError(f"unknown boundary {k!r}: axis1 (a * a1) or axis2 (b * a2)")
            if v is True:
                per[ax] = True
            elif v is False or v is None:
                continue
            else:
                per[ax] = True
                tw[ax] = float(v)
        self.periodic = tuple(per)
        self.twist = tuple(tw)
        j1, j2, s = np.meshgrid(np.arange(1, self.a + 1), np.arange(1, self.b + 1), np.arange(self.nb), indexing="ij")
        self._cells = np.stack([j1.ravel(), j2.ravel(), s.ravel()], axis=1)  # (N, 3), lattice order
        self._coords = (self.T @ self._cells[:, :2].T.astype(float)).T + self.basis[:, self._cells[:, 2]].T
        self._bonds = None

    def __len__(self):
        return self.N

    def __repr__(self):
        return f"{self.a}x{self.b} {self.name} ({self.N} sites)"

    def key(self):
        return ("bravais", self.name, self.a, self.b, self.periodic, self.twist)

    def coords(self) -> np.ndarray:
        return self._coords

    def index(self, j1, j2, s):
        """0-based site index of basis site s (1-based) in unit cell (j1, j2)."""
        return ((j1 - 1) * self.b + (j2 - 1)) * self.nb + (s - 1)

    def nn_translations(self):
        """(i, j, C) of the nearest-neighbour translations, i, j 1-based basis indices (0 = all)."""
        found = []  # (length, [translations])
        for C in _offsets(2):
            U = self.T @ np.array(C, dtype=float)
            for i in range(self.nb):
                for j in range(i, self.nb):
                    if i == j:
                        if i > 1:
                            continue
                        nz = [c for c in C if c != 0]
                        if not nz or nz[0] < 1:
                            continue
                    r = float(np.linalg.norm(U - self.basis[:, i] + self.basis[:, j]))
                    tr = (0, 0, C) if i == j else (i + 1, j + 1, C)
                    for ent in found:
                        if math.isclose(ent[0], r, rel_tol=1.5e-8):
                            if tr not in ent[1]:
                                ent[1].append(tr)
                            break
                    else:
                        found.append((r, [tr]))
        found.sort(key=lambda e: e[0])
        return found[0][1]

    def bonds(self):
        """Nearest-neighbour bonds: (src, dst) 1-based, (x1, y1, x2, y2) with the destination
        unwrapped, and the boundary factor (complex), in the reference's iteration order."""
        if self._bonds is not None:
            return self._bonds
        src, dst, xy, fac = [], [], [], []
        ext = (self.a, self.b)
        for (i, j, C) in self.nn_translations():
            for site in range(self.N):
                j1, j2, s = (int(v) for v in self._cells[site])
                if i and s + 1 != i:
                    continue
                t = (j - 1) if i else s
                d = [j1 + C[0], j2 + C[1]]
                f = 1.0 + 0.0j
                ok = True
                for ax in range(2):
                    L = ext[ax]
                    while d[ax] > L or d[ax] < 1:
                        if not self.periodic[ax]:
                            ok = False
                            break
                        step = -1 if d[ax] > L else 1
                        d[ax] += step * L
                        f *= complex(math.cos(self.twist[ax]), math.sin(self.twist[ax])) ** (-step)
                    if not ok:
                        break
                if not ok:
                    continue
                r1 = self._coords[site]
                r2 = self.T @ np.array([j1 + C[0], j2 + C[1]], dtype=float) + self.basis[:, t]
                src.append(site + 1)
                dst.append(self.index(d[0], d[1], t + 1) + 1)
                xy.append((r1[0], r1[1], r2[0], r2[1]))
                fac.append(f)
        self._bonds = (np.array(src, dtype=np.int64), np.array(dst, dtype=np.int64),
                       np.array(xy, dtype=np.float64).reshape(-1, 4), np.array(fac, dtype=np.complex128))
        return self._bonds

    def nbonds(self):
        return len(self.bonds()[0])


def HoneycombLattice(a: int, b: int, boundaries=None) -> BravaisLattice:
    """HoneycombLattice(a, b) (src/zoo/lattices.jl:145-151): two sites per unit cell at (0, 0)
    and (1/2, sqrt(3)/6), unit vectors (1, 0) and (1/2, sqrt(3)/2)."""
    return BravaisLattice("HoneycombLattice", a, b, boundaries)


def KagomeLattice(a: int, b: int, boundaries=None) -> BravaisLattice:
    """KagomeLattice(a, b) (src/zoo/lattices.jl:200-211): three sites per unit cell at (0, 0),
    (1/2, 0) and (1/4, sqrt(3)/4)."""
    return BravaisLattice("KagomeLattice", a, b, boundaries)


def TriangularLattice(a: int, b: int, boundaries=None) -> BravaisLattice:
    """TriangularLattice(a, b) (src/zoo/lattices.jl:136-143)."""
    return BravaisLattice("TriangularLattice", a, b, boundaries)


def _pattern(n: int, src, dst):
    """(colptr, rowval) 1-based of the stored pattern lm_ell_create_bonds builds: every
    diagonal entry and both entries of every bond, in CSC order."""
    rows = np.concatenate([np.arange(n), src - 1, dst - 1])
    cols = np.concatenate([np.arange(n), dst - 1, src - 1])
    key = np.unique(cols * n + rows)
    c, r = key // n, key % n
    colptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(colptr, c + 1, 1)
    return np.cumsum(colptr) + 1, r.astype(np.int64) + 1


class _DeviceBondEll:
    """One lm_ell built from the bonds of a lattice, with fixed field components."""

    def __init__(self, ctx, lat: BravaisLattice, t1: float, comps):
        self.ctx = ctx
        src, dst, xy, fac = lat.bonds()
        base = np.ascontiguousarray((t1 * fac).astype(np.complex128))
        xyc = np.ascontiguousarray(xy, dtype=np.float64)
        p = C.c_void_p()
        ctx.check(ctx.lib.lm_ell_create_bonds(ctx.handle, lat.N, len(src), _lib.i64ptr(np.ascontiguousarray(src)),
                                              _lib.i64ptr(np.ascontiguousarray(dst)), _lib.dptr(xyc),
                                              _lib.dptr(base.view(np.float64)), C.byref(p)))
        self.handle = p
        weakref.finalize(self, ctx.lib.lm_ell_destroy, p)
        for kind, px, py in comps:
            idx = C.c_int()
            ctx.check(ctx.lib.lm_ell_add_field(p, kind, px, py, C.byref(idx)))
        # the honeycomb in the reference's site order is a brick lattice: ComplexF32 kets then
        # step through the temporally blocked kernel (periodic axes need 3 or more cells)
        self.brick = (lat.name == "HoneycombLattice" and (not lat.periodic[0] or lat.a >= 3)
                      and (not lat.periodic[1] or lat.b >= 3))
        if self.brick:
            ctx.check(ctx.lib.lm_ell_set_layout(p, _lib.LM_LAYOUT_HONEYCOMB, lat.a, lat.b, int(lat.periodic[0]),
                                                int(lat.periodic[1])))
        self.onsite_ref = None
        self.amps = None

    def ensure(self, onsite, amps):
        ctx = self.ctx
        if onsite is not self.onsite_ref:
            ctx.check(ctx.lib.lm_ell_set_onsite(self.handle, None if onsite is None else _lib.dptr(onsite)))
            self.onsite_ref = onsite
            self.amps = None
        a = np.ascontiguousarray(amps, dtype=np.float64)
        if self.amps is None or not np.array_equal(a, self.amps):
            ctx.check(ctx.lib.lm_ell_assemble(self.handle, _lib.dptr(a) if len(a) else None, len(a)))
            self.amps = a.copy()


_cache: "OrderedDict[tuple, _DeviceBondEll]" = OrderedDict()


class LatticeHamiltonian(SparseHamiltonian):
    """Nearest-neighbour tight-binding Hamiltonian of a BravaisLattice, assembled on the device."""

    def __init__(self, lattice: BravaisLattice, t1=1.0, field: AbstractField = None, onsite=None):
        self.lattice = lattice
        self.t1 = float(t1)
        self.field = field if field is not None else NoField()
        for kind, px, py in self.field.components():
            if kind not in (_lib.LM_FIELD_LANDAU, _lib.LM_FIELD_SYMMETRIC, _lib.LM_FIELD_POINTFLUX_AXIAL,
                            _lib.LM_FIELD_POINTFLUX_SINGULAR):
                raise ValueError("unsupported field component")
        if onsite is not None:
            v = onsite.values if isinstance(onsite, LatticeValue) else onsite
            v = np.ascontiguousarray(v, dtype=np.float64)
            if v.shape != (lattice.N,):
                raise ValueError("on-site term must have one value per site")
            onsite = v
        self.onsite = onsite
        pat = getattr(lattice, "_csc_pattern", None)
        if pat is None:  # built once per lattice: h(t) makes a new Hamiltonian every step
            src, dst, _, _ = lattice.bonds()
            pat = lattice._csc_pattern = _pattern(lattice.N, src, dst)
        self.colptr, self.rowval = pat
        self.nzval = None
        self._pattern = ("bonds",) + lattice.key()

    def __eq__(self, other):
        if not isinstance(other, LatticeHamiltonian):
            return False
        if (self.lattice.key() != other.lattice.key() or self.t1 != other.t1 or self.field != other.field):
            return False
        if self.onsite is other.onsite:
            return True
        return self.onsite is not None and other.onsite is not None and np.array_equal(self.onsite, other.onsite)

    __hash__ = None

    def device(self, ctx=None) -> _DeviceBondEll:
        ctx = ctx or default_context()
        comps = tuple(self.field.components())
        key = (id(ctx), self.lattice.key(), self.t1, comps)
        dh = _cache.get(key)
        if dh is None:
            dh = _cache[key] = _DeviceBondEll(ctx, self.lattice, self.t1, comps)
            while len(_cache) > 8:
                _cache.popitem(last=False)
        else:
            _cache.move_to_end(key)
        dh.ensure(self.onsite, self.field.amplitudes())
        return dh

    def bond_entries(self):
        """Index of the stored entry H[src, dst] of every bond (CSC order)."""
        src, dst, _, _ = self.lattice.bonds()
        n = self.N
        cols = np.repeat(np.arange(n, dtype=np.int64), np.diff(self.colptr))
        key = cols * n + (self.rowval - 1)
        return np.searchsorted(key, (dst - 1) * n + (src - 1))

    def __repr__(self):
        return f"LatticeHamiltonian(t1={self.t1}, field={self.field!r}) on {self.lattice!r}"


def bravais_tightbinding(lattice: BravaisLattice, *args, t1=1, t2=0, t3=0, field=None) -> LatticeHamiltonian:
    """``tightbinding_hamiltonian(lat, [V]; t1, field)`` (src/operators/constructoperator.jl:190-194)
    for a BravaisLattice: nearest-neighbour hopping t1 and an optional on-site term."""
    if t2 != 0 or t3 != 0:
        raise NotImplementedError("t2/t3 hopping is not implemented by the GPU backend")
    onsite = None
    for a in args:
        if onsite is not None:
            raise NotImplementedError("only one on-site term is supported")
        onsite = a
    return LatticeHamiltonian(lattice, t1, field, onsite)
