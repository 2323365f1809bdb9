"""Device states: a Ket, a block of kets, or a density matrix.

The reference evolves ``Ket``/``Operator`` data (src/evolution.jl:69-80).  A block of M kets
is the backend's batched state (P = sum_m w_m |psi_m><psi_m| for the readouts); it has no
single reference counterpart, the reference would hold M separate ``Ket`` states.
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import _lib
from .device import default_context
from .lattice import SquareLattice

_PREC = {"c64": _lib.LM_C64, "c32": _lib.LM_C32, "complex128": _lib.LM_C64, "complex64": _lib.LM_C32}
_NP = {_lib.LM_C64: np.complex128, _lib.LM_C32: np.complex64}


class DeviceState:
    """An lm_state plus the lattice it lives on."""

    def __init__(self, lattice: SquareLattice, data, kind: int, precision="c64", weights=None, ctx=None,
                 shape=None):
        ctx = ctx or default_context()
        self.ctx = ctx
        self.lattice = lattice
        self.kind = kind
        self.precision = _PREC[precision] if isinstance(precision, str) else int(precision)
        if data is None:  # allocation only (zero state)
            arr = None
            n, m = shape
        else:
            arr = np.asarray(data)
            if arr.ndim == 1:
                arr = arr.reshape(-1, 1)
            n, m = arr.shape
        if n != lattice.N:
            raise ValueError(f"state has {n} rows, the lattice has {lattice.N} sites")
        if kind == _lib.LM_DENSITY and m != n:
            raise ValueError("a density matrix must be square")
        self.n, self.m = n, m
        p = C.c_void_p()
        ctx.check(ctx.lib.lm_state_create(ctx.handle, n, m, kind, self.precision, C.byref(p)))
        self.handle = p
        self._fin = weakref.finalize(self, ctx.lib.lm_state_destroy, p)
        if arr is not None:
            self.upload(arr)
        self.weights = None
        self.compensated = False
        if weights is not None:
            self.set_weights(weights)

    def set_compensation(self, enable: bool = True):
        """Keep the FP32 rounding residual of every amplitude beside it (ComplexF32 kets that
        the x-streaming step takes: square lattices with Ly even and Lx >= 2K + 3, honeycomb
        lattices in the brick layout): the step then forms each new amplitude from the (value,
        residual) pair with error-free transformations, so a long FP32 run accumulates far less
        rounding.  Norms and renormalize read value + residual; the readouts and to_numpy read
        the FP32 value."""
        self.ctx.check(self.ctx.lib.lm_state_set_compensation(self.handle, int(bool(enable))))
        self.compensated = bool(enable)
        return self

    @property
    def dtype(self):
        return _NP[self.precision]

    def upload(self, arr):
        """Copies host data (n x m) into the device state (column-major)."""
        a = np.asarray(arr)
        if a.ndim == 1:
            a = a.reshape(-1, 1)
        a = np.asfortranarray(a, dtype=self.dtype)
        if a.shape != (self.n, self.m):
            raise ValueError("shape mismatch")
        self.ctx.check(self.ctx.lib.lm_state_upload(self.handle, a.ctypes.data_as(C.c_void_p), self.n))
        self._host_ref = a  # the copy is asynchronous: keep the buffer alive until the next sync

    def upload_from(self, a: np.ndarray):
        """Upload from a caller-owned Fortran-ordered buffer of the state's dtype (e.g. pinned)."""
        if a.dtype != self.dtype or not a.flags.f_contiguous or a.shape != (self.n, self.m):
            raise ValueError("upload_from needs an (n, m) Fortran-ordered array of the state's dtype")
        self.ctx.check(self.ctx.lib.lm_state_upload(self.handle, a.ctypes.data_as(C.c_void_p), self.n))

    def to_numpy(self) -> np.ndarray:
        out = np.empty((self.n, self.m), dtype=self.dtype, order="F")
        self.ctx.check(self.ctx.lib.lm_state_download(self.handle, out.ctypes.data_as(C.c_void_p), self.n))
        return out

    def set_weights(self, w):
        if w is None:
            self.ctx.check(self.ctx.lib.lm_state_set_weights(self.handle, None))
            self.weights = None
            return
        w = np.ascontiguousarray(w, dtype=np.float64)
        if w.shape != (self.m,):
            raise ValueError("one weight per ket")
        self.ctx.check(self.ctx.lib.lm_state_set_weights(self.handle, _lib.dptr(w)))
        self.weights = w

    def norms(self) -> np.ndarray:
        out = np.empty(self.m, dtype=np.float64)
        self.ctx.check(self.ctx.lib.lm_state_norms(self.handle, _lib.dptr(out)))
        return out

    def renormalize(self, target):
        t = np.ascontiguousarray(target, dtype=np.float64)
        if t.shape != (self.m,):
            raise ValueError("one target norm per ket")
        self.ctx.check(self.ctx.lib.lm_state_renormalize(self.handle, _lib.dptr(t)))

    def trace(self) -> float:
        out = C.c_double()
        self.ctx.check(self.ctx.lib.lm_trace(self.handle, C.byref(out)))
        return out.value

    def device_ptr(self):
        p = C.c_void_p()
        ld = C.c_int64()
        self.ctx.check(self.ctx.lib.lm_state_device_ptr(self.handle, C.byref(p), C.byref(ld)))
        return p.value, ld.value

    def copy(self):
        """Device-to-device copy (the copy Evolution makes at construction)."""
        c = object.__new__(type(self))
        DeviceState.__init__(c, self.lattice, None, self.kind, self.precision, self.weights, self.ctx,
                             shape=(self.n, self.m))
        if self.compensated:
            c.set_compensation(True)
        self.ctx.check(self.ctx.lib.lm_state_copy(c.handle, self.handle))
        return c

    def __repr__(self):
        kind = "DensityMatrix" if self.kind == _lib.LM_DENSITY else ("Ket" if self.m == 1 else f"KetBlock[{self.m}]")
        prec = "c64" if self.precision == _lib.LM_C64 else "c32"
        return f"{kind}({prec}) on {self.lattice!r}"


class Ket(DeviceState):
    def __init__(self, lattice, data, precision="c64", ctx=None):
        super().__init__(lattice, np.asarray(data).reshape(-1), _lib.LM_KETS, precision, None, ctx)



class KetBlock(DeviceState):
    """N x M block of kets (column m = ket m), optional weights w_m."""

    def __init__(self, lattice, data, weights=None, precision="c64", ctx=None, compensated=False):
        super().__init__(lattice, data, _lib.LM_KETS, precision, weights, ctx)
        if compensated:
            self.set_compensation(True)



class DensityMatrix(DeviceState):
    """N x N one-particle density matrix (the reference's ``Operator`` state)."""

    def __init__(self, lattice, data, precision="c64", ctx=None):
        # data None: an N x N zero matrix (filled on the device, e.g. by densitymatrix)
        super().__init__(lattice, data, _lib.LM_DENSITY, precision, None, ctx, shape=(lattice.N, lattice.N))



Operator = DensityMatrix
