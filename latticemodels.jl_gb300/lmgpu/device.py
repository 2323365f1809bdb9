"""Per-process device context (one CUDA device, one stream)."""
from __future__ import annotations

import ctypes as C
import threading

from . import _lib


class Context:
    """Owns an lm_ctx: the device, its stream and the library's error slot."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        rc = self.lib.lm_ctx_create(int(device), C.byref(h))
        if rc != _lib.LM_OK:
            raise _lib.LMError(rc, f"cannot create a CUDA context on device {device} "
                                   "(the lmgpu backend has no CPU fallback)")
        self.handle = h
        self.device = device

    def check(self, code):
        _lib.check(self.handle, code)

    def synchronize(self):
        self.check(self.lib.lm_ctx_synchronize(self.handle))

    def set_fused(self, on: bool):
        """Temporally blocked c32 step (default on) or one launch per Chebyshev order."""
        self.check(self.lib.lm_ctx_set_option(self.handle, _lib.LM_OPT_FUSED, 1 if on else 0))

    def set_stream_form(self, on: bool):
        """x-streaming form of the fused step where the lattice allows it (default on), or the
        region form; both give bit-identical results."""
        self.check(self.lib.lm_ctx_set_option(self.handle, _lib.LM_OPT_STREAM, 1 if on else 0))

    def set_kpm_doublefloat(self, on: bool):
        """KPM and Fermi-operator (lm_cheb_apply) recurrences in double-float (FP32 pairs, on the
        FP32 pipe; the default) or FP64; KPM moments agree to about 1e-15 mu_0."""
        self.check(self.lib.lm_ctx_set_option(self.handle, _lib.LM_OPT_KPM, 1 if on else 0))

    def set_resident_form(self, on: bool):
        """Lattice-resident form of a c32 batch's fused pass for lattices that fit on chip (the
        default), or the region form; both give bit-identical results.  Applies from the next
        batch update."""
        self.check(self.lib.lm_ctx_set_option(self.handle, _lib.LM_OPT_RESIDENT, 1 if on else 0))

    def stream_launches(self) -> int:
        """Fused steps that ran in the x-streaming form so far."""
        n = C.c_int64()
        self.check(self.lib.lm_ctx_stream_launches(self.handle, C.byref(n)))
        return n.value

    def set_timing(self, on: bool):
        self.check(self.lib.lm_ctx_set_timing(self.handle, 1 if on else 0))

    def reset_timing(self):
        self.check(self.lib.lm_ctx_reset_timing(self.handle))

    def timing(self):
        ms = C.c_double()
        ol = C.c_int64()
        la = C.c_int64()
        self.check(self.lib.lm_ctx_timing(self.handle, C.byref(ms), C.byref(ol), C.byref(la)))
        return ms.value, ol.value, la.value

    def stream_ptr(self) -> int:
        """The context's cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
        p = C.c_void_p()
        self.check(self.lib.lm_ctx_stream(self.handle, C.byref(p)))
        return p.value or 0

    def close(self):
        if self.handle:
            self.lib.lm_ctx_destroy(self.handle)
            self.handle = None


_default = None
_default_device = 0
_lock = threading.Lock()


def set_default_device(device: int) -> None:
    """Selects the CUDA device of the default context; call before the first device use."""
    global _default_device
    with _lock:
        if _default is not None and _default.device != device:
            raise RuntimeError("the default context already exists on another device")
        _default_device = int(device)


def default_context() -> Context:
    global _default
    with _lock:
        if _default is None:
            _default = Context(_default_device)
        return _default
