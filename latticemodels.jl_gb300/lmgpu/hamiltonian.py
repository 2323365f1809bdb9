"""Device Hamiltonians: ``tightbinding_hamiltonian`` with on-device H(t) assembly.

A ``Hamiltonian`` is a light value object (lattice, t1, field, on-site term).  Calling
``h(t)`` every step, as the reference's ``Evolution(t -> h(t), P_0)`` does, only creates a
new value object; the device tables are kept per (lattice, t1, field structure) and
re-assembled on the GPU when the field amplitudes or the on-site term change
(src/operators/constructoperator.jl:136-194, src/operators/builder.jl:274-309).
"""
from __future__ import annotations

import ctypes as C
import weakref
from collections import OrderedDict

import numpy as np

from . import _lib
from .device import default_context
from .fields import AbstractField, NoField, pbc_warning
from .lattice import LatticeValue, SquareLattice


class _DeviceHam:
    """One lm_ham: fixed (lattice, t1, field kinds/points); assembled per amplitude set."""

    def __init__(self, ctx, lattice: SquareLattice, t1: float, comps, auto_pbc: bool):
        self.ctx = ctx
        lib = ctx.lib
        p = C.c_void_p()
        ctx.check(lib.lm_ham_create(ctx.handle, lattice.handle(ctx), float(t1), C.byref(p)))
        self.handle = p
        self._fin = weakref.finalize(self, lib.lm_ham_destroy, p)
        for kind, px, py in comps:
            idx = C.c_int()
            ctx.check(lib.lm_ham_add_field(p, kind, px, py, 1 if auto_pbc else 0, C.byref(idx)))
        self.ncomp = len(comps)
        self.onsite_ref = None   # the on-site array currently uploaded (kept alive for identity)
        self.lattice = lattice

    def ensure(self, onsite, amps):
        ctx = self.ctx
        if onsite is not self.onsite_ref:
            if onsite is None:
                ctx.check(ctx.lib.lm_ham_set_onsite(self.handle, None))
            else:
                ctx.check(ctx.lib.lm_ham_set_onsite(self.handle, _lib.dptr(onsite)))
            self.onsite_ref = onsite
        a = np.ascontiguousarray(amps, dtype=np.float64)
        ctx.check(ctx.lib.lm_ham_assemble(self.handle, _lib.dptr(a) if len(a) else None, len(a)))


_cache: "OrderedDict[tuple, _DeviceHam]" = OrderedDict()
_CACHE_MAX = 8


def _device_ham(ctx, H: "Hamiltonian") -> _DeviceHam:
    key = (id(ctx), H.lattice.key(), H.t1, tuple(H.field.components()), H.auto_pbc_field)
    dh = _cache.get(key)
    if dh is None:
        dh = _DeviceHam(ctx, H.lattice, H.t1, H.field.components(), H.auto_pbc_field)
        _cache[key] = dh
        while len(_cache) > _CACHE_MAX:
            _cache.popitem(last=False)
    else:
        _cache.move_to_end(key)
    return dh


class Hamiltonian:
    """Tight-binding Hamiltonian value; ``.data`` semantics are provided by the device tables."""

    def __init__(self, lattice: SquareLattice, t1=1.0, field: AbstractField = None, onsite=None,
                 auto_pbc_field: bool = True):
        self.lattice = lattice
        self.t1 = float(t1)
        self.field = field if field is not None else NoField()
        if onsite is not None:
            v = onsite.values if isinstance(onsite, LatticeValue) else onsite
            v = np.ascontiguousarray(v, dtype=np.float64)
            if v.shape != (lattice.N,):
                raise ValueError("on-site term must have one value per site")
            if not np.all(np.isfinite(v)):
                raise ValueError("on-site term must be finite")
            onsite = v
        self.onsite = onsite
        self.auto_pbc_field = bool(auto_pbc_field)

    # `mat == old` of the reference's CachedExp cache (src/evolution.jl:87)
    def __eq__(self, other):
        if not isinstance(other, Hamiltonian):
            return False
        if (self.lattice != other.lattice or self.t1 != other.t1 or self.field != other.field
                or self.auto_pbc_field != other.auto_pbc_field):
            return False
        if self.onsite is other.onsite:
            return True
        if self.onsite is None or other.onsite is None:
            return False
        return bool(np.array_equal(self.onsite, other.onsite))

    __hash__ = None

    def __repr__(self):
        return f"Hamiltonian(dim={self.lattice.N}x{self.lattice.N}) on {self.lattice!r}, field={self.field!r}"

    @property
    def N(self):
        return self.lattice.N

    def device(self, ctx=None) -> _DeviceHam:
        """Assembles H on the device (cached) and returns the device object."""
        ctx = ctx or default_context()
        dh = _device_ham(ctx, self)
        dh.ensure(self.onsite, self.field.amplitudes())
        return dh

    def device_private(self, ctx=None) -> _DeviceHam:
        """A device Hamiltonian owned by the caller (not shared through the cache), assembled."""
        ctx = ctx or default_context()
        dh = _DeviceHam(ctx, self.lattice, self.t1, self.field.components(), self.auto_pbc_field)
        dh.ensure(self.onsite, self.field.amplitudes())
        return dh

    def csc(self, ctx=None):
        """The assembled matrix as the reference's CSC: (colptr, rowval) 1-based, nzval complex."""
        ctx = ctx or default_context()
        dh = self.device(ctx)
        nnz = C.c_int64()
        ctx.check(ctx.lib.lm_ham_nnz(dh.handle, C.byref(nnz)))
        colptr = np.empty(self.N + 1, dtype=np.int64)
        rowval = np.empty(nnz.value, dtype=np.int64)
        nz = np.empty(2 * nnz.value, dtype=np.float64)
        ctx.check(ctx.lib.lm_ham_csc(dh.handle, _lib.i64ptr(colptr), _lib.i64ptr(rowval), _lib.dptr(nz)))
        return colptr, rowval, nz[0::2] + 1j * nz[1::2]

    def bounds(self, ctx=None, method: str = "gershgorin", iters: int = 80, seed: int = 1):
        """Interval enclosing the spectrum: "gershgorin" (rigorous) or "lanczos" (FP64 Lanczos
        estimate, padded and clipped to the Gershgorin interval; tighter, for one-shot
        expansions such as kpm.dos or densitymatrix at T > 0)."""
        ctx = ctx or default_context()
        dh = self.device(ctx)
        lo, hi = C.c_double(), C.c_double()
        if method == "gershgorin":
            ctx.check(ctx.lib.lm_ham_bounds(dh.handle, C.byref(lo), C.byref(hi)))
        elif method == "lanczos":
            ctx.check(ctx.lib.lm_ham_lanczos_bounds(dh.handle, int(iters), int(seed), C.byref(lo), C.byref(hi)))
        else:
            raise ValueError("method must be gershgorin or lanczos")
        return lo.value, hi.value


def tightbinding_hamiltonian(lattice: SquareLattice, *args, t1=1, t2=0, t3=0, field=None,
                             auto_pbc_field=True) -> Hamiltonian:
    """``tightbinding_hamiltonian(lat, args...; t1, t2, t3, field)`` (constructoperator.jl:190-194).

    ``args`` may hold one on-site term (a LatticeValue or an array of N values), the
    ``LatticeValue => 1`` pair of the reference.  Next-nearest (t2) and third-neighbour (t3)
    hopping are outside this backend.
    """
    from .bravais import BravaisLattice, bravais_tightbinding
    if isinstance(lattice, BravaisLattice):  # HoneycombLattice, KagomeLattice, TriangularLattice
        return bravais_tightbinding(lattice, *args, t1=t1, t2=t2, t3=t3, field=field)
    if t2 != 0 or t3 != 0:
        raise NotImplementedError("t2/t3 hopping is not implemented by the GPU backend")
    onsite = None
    for a in args:
        if isinstance(a, (LatticeValue, np.ndarray, list, tuple)):
            if onsite is not None:
                raise NotImplementedError("only one on-site term is supported")
            onsite = a
        else:
            raise TypeError(f"cannot interpret {type(a).__name__} as a Hamiltonian term")
    f = field if field is not None else NoField()
    if auto_pbc_field:
        pbc_warning(f, lattice)
    return Hamiltonian(lattice, t1, f, onsite, auto_pbc_field)
