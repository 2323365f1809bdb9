"""SquareLattice and LatticeValue: the host-side mirror of the reference's lattice types.

Site order, coordinates and bond iteration follow LatticeModels.jl exactly:
index = (x-1)*Ly + y (src/lattices/bravais/unitcell.jl:126-132), coordinates = lattice
coordinates (src/lattices/bravais/unitcell.jl:119-122), NearestNeighbor(1) bonds as
translations [1,0] then [0,1] (src/lattices/bravais/nearestneighbor.jl:97-131), boundary
routing by the axis translations (src/core/boundaries.jl:251-289).
"""
from __future__ import annotations

import ctypes as C
import math
import weakref

import numpy as np

from . import _lib
from .device import default_context


def _parse_boundaries(boundaries):
    """Accepts ``(:axis1 => true, :axis2 => θ)`` in Python form: pairs ("axis1", True|θ) or a dict."""
    per = [False, False]
    tw = [0.0, 0.0]
    if boundaries is None:
        return tuple(per), tuple(tw)
    items = boundaries.items() if isinstance(boundaries, dict) else boundaries
    if isinstance(items, tuple) and len(items) == 2 and isinstance(items[0], str):
        items = [items]
    for key, val in items:
        ax = {"axis1": 0, "axis2": 1, 1: 0, 2: 1, "x": 0, "y": 1}.get(key)
        if ax is None:
            raise ValueError(f"unknown boundary axis {key!r}")
        if isinstance(val, bool):
            if val:
                per[ax] = True
                tw[ax] = 0.0
        else:
            th = float(val)
            if not math.isfinite(th):
                raise ValueError("twist angle must be finite")
            per[ax] = True
            tw[ax] = th
    return tuple(per), tuple(tw)


class SquareLattice:
    """``SquareLattice(Lx, Ly; boundaries)`` (src/zoo/lattices.jl:131)."""

    def __init__(self, Lx: int, Ly: int, boundaries=None):
        if int(Lx) < 1 or int(Ly) < 1:
            raise ValueError("lattice sizes must be positive")
        self.Lx, self.Ly = int(Lx), int(Ly)
        self.periodic, self.twist = _parse_boundaries(boundaries)
        self._handles = {}
        self._bonds = None

    # -- basic properties ------------------------------------------------------------------
    @property
    def N(self) -> int:
        return self.Lx * self.Ly

    def __len__(self) -> int:
        return self.N

    def __eq__(self, other) -> bool:
        return (isinstance(other, SquareLattice) and self.Lx == other.Lx and self.Ly == other.Ly
                and self.periodic == other.periodic and self.twist == other.twist)

    def __hash__(self):
        return hash((self.Lx, self.Ly, self.periodic, self.twist))

    def key(self):
        return (self.Lx, self.Ly, self.periodic, self.twist)

    def __repr__(self):
        b = "" if not any(self.periodic) else f", periodic={self.periodic}, twist={self.twist}"
        return f"SquareLattice({self.Lx}, {self.Ly}{b})"

    def has_boundaries(self) -> bool:
        return any(self.periodic)

    def site_index(self, x: int, y: int) -> int:
        """1-based index of site (x, y)."""
        if not (1 <= x <= self.Lx and 1 <= y <= self.Ly):
            raise IndexError(f"site ({x}, {y}) is not on {self!r}")
        return (x - 1) * self.Ly + y

    def coords(self) -> np.ndarray:
        """N x 2 site coordinates (x, y), 1-based lattice coordinates."""
        x = np.repeat(np.arange(1, self.Lx + 1), self.Ly).astype(np.float64)
        y = np.tile(np.arange(1, self.Ly + 1), self.Lx).astype(np.float64)
        return np.stack([x, y], axis=1)

    # -- device handle ------------------------------------------------------------------------
    def handle(self, ctx=None):
        ctx = ctx or default_context()
        h = self._handles.get(id(ctx))
        if h is None:
            p = C.c_void_p()
            ctx.check(ctx.lib.lm_lattice_square(ctx.handle, self.Lx, self.Ly, int(self.periodic[0]),
                                                int(self.periodic[1]), self.twist[0], self.twist[1],
                                                C.byref(p)))
            h = p
            self._handles[id(ctx)] = h
            weakref.finalize(self, ctx.lib.lm_lattice_destroy, h)
        return h

    def nbonds(self) -> int:
        nbx = self.N if self.periodic[0] else (self.Lx - 1) * self.Ly
        nby = self.N if self.periodic[1] else self.Lx * (self.Ly - 1)
        return nbx + nby

    def bonds(self):
        """NearestNeighbor(1) bonds (src, dst), 1-based, in the reference's iteration order.

        Computed by the library on a host-only lattice handle (no GPU needed)."""
        if self._bonds is None:
            lib = _lib.load()
            p = C.c_void_p()
            _lib.check(None, lib.lm_lattice_square(None, self.Lx, self.Ly, int(self.periodic[0]),
                                                   int(self.periodic[1]), self.twist[0], self.twist[1],
                                                   C.byref(p)))
            try:
                n = lib.lm_lattice_nbonds(p)
                src = np.empty(n, dtype=np.int64)
                dst = np.empty(n, dtype=np.int64)
                _lib.check(None, lib.lm_lattice_bonds(p, _lib.i64ptr(src), _lib.i64ptr(dst)))
            finally:
                lib.lm_lattice_destroy(p)
            self._bonds = (src, dst)
        return self._bonds


class LatticeValue:
    """Values on the sites of a lattice (src/core/latticevalue.jl:91-92)."""

    def __init__(self, lattice: SquareLattice, values):
        self.lattice = lattice
        self.values = np.asarray(values)
        if self.values.shape[0] != getattr(lattice, "nsites", lattice.N):
            raise ValueError("value count does not match the lattice")

    def __getitem__(self, i):
        return self.values[i]

    def __len__(self):
        return len(self.values)

    def __array__(self, dtype=None, copy=None):
        return np.asarray(self.values, dtype=dtype)

    def __repr__(self):
        return f"LatticeValue{{{self.values.dtype}}} on {self.lattice!r}"

    # elementwise comparisons give Bool masks (x .< y in the reference)
    def _cmp(self, other, op):
        o = other.values if isinstance(other, LatticeValue) else other
        return LatticeValue(self.lattice, op(self.values, o))

    def __lt__(self, other):
        return self._cmp(other, np.less)

    def __le__(self, other):
        return self._cmp(other, np.less_equal)

    def __gt__(self, other):
        return self._cmp(other, np.greater)

    def __ge__(self, other):
        return self._cmp(other, np.greater_equal)


def coordvalues(lattice):
    """``coordvalues(l)`` (src/core/latticevalue.jl:95-100): one LatticeValue per coordinate."""
    xy = lattice.coords()
    return tuple(LatticeValue(lattice, xy[:, d].copy()) for d in range(xy.shape[1]))


def site_indices(lattice, sel) -> np.ndarray:
    """1-based site indices of a selection: a Bool LatticeValue or mask, an index, or indices
    (the reference's ``to_inds``)."""
    if isinstance(sel, LatticeValue):
        sel = sel.values
    a = np.asarray(sel)
    if a.dtype == bool:
        return np.nonzero(a)[0] + 1
    return np.atleast_1d(a).astype(np.int64)
