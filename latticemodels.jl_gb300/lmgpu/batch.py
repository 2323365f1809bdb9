"""Batches of independent lattices evolved in the same launches (``lm_batch_*``).

Hundreds of uneven lattices (each its own size, field, disorder and state) advance together:
every step is one fixed sequence of launches over the work items of all instances, replayed
from a CUDA graph; ``tune`` picks the pass shape with the library's autotuner.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import weakref
from pathlib import Path

import numpy as np

from . import _lib
from .device import default_context
from .hamiltonian import Hamiltonian
from .states import DeviceState

CONFIG_NAMES = {0: "fused (all orders per launch)", 1: "per-order, 2 kets/thread",
                2: "per-order, 4 kets/thread", 3: "per-order, 8 kets/thread"}


class Batch:
    def __init__(self, kind="density", precision="c32", tol=None, ctx=None):
        self.ctx = ctx or default_context()
        self.kind = _lib.LM_DENSITY if kind == "density" else _lib.LM_KETS
        self.precision = _lib.LM_C32 if precision in ("c32", _lib.LM_C32) else _lib.LM_C64
        if tol is None:
            tol = 1e-9 if self.precision == _lib.LM_C32 else 1e-12
        p = C.c_void_p()
        self.ctx.check(self.ctx.lib.lm_batch_create(self.ctx.handle, self.kind, self.precision, float(tol),
                                                    C.byref(p)))
        self.handle = p
        self._fin = weakref.finalize(self, self.ctx.lib.lm_batch_destroy, p)
        self.hams, self.states, self._dev = [], [], []

    def add(self, H: Hamiltonian, state: DeviceState) -> int:
        if state.kind != self.kind or state.precision != self.precision:
            raise ValueError("state kind/precision differ from the batch")
        dh = H.device_private(self.ctx)
        idx = C.c_int()
        self.ctx.check(self.ctx.lib.lm_batch_add(self.handle, dh.handle, state.handle, C.byref(idx)))
        self.hams.append(H)
        self.states.append(state)
        self._dev.append(dh)  # the batch refers to these device objects
        return idx.value

    def update(self, dt: float):
        self.ctx.check(self.ctx.lib.lm_batch_update(self.handle, float(dt)))

    def step(self):
        self.ctx.check(self.ctx.lib.lm_batch_step(self.handle))

    def set_graph(self, on: bool):
        self.ctx.check(self.ctx.lib.lm_batch_set_graph(self.handle, 1 if on else 0))

    def set_panel(self, width: int):
        """Run the per-order recurrence on column panels of ``width`` columns in place (0: off):
        no full-size recurrence buffers, for batches that would not fit otherwise."""
        self.ctx.check(self.ctx.lib.lm_batch_set_panel(self.handle, int(width)))

    def set_config(self, cfg: int):
        self.ctx.check(self.ctx.lib.lm_batch_set_config(self.handle, int(cfg)))

    def info(self):
        K, cfg, ninst = C.c_int(), C.c_int(), C.c_int()
        items = C.c_int64()
        self.ctx.check(self.ctx.lib.lm_batch_info(self.handle, C.byref(K), C.byref(cfg), C.byref(items),
                                                  C.byref(ninst)))
        return {"K": K.value, "config": cfg.value, "items": items.value, "instances": ninst.value}

    def tune(self, steps: int = 2, cache_file=None):
        """Times every eligible pass shape and keeps the fastest; the choice is remembered in
        ``cache_file`` (JSON, default $LMGPU_TUNE_FILE) keyed by the batch signature."""
        key = self.signature()
        path = cache_file or os.environ.get("LMGPU_TUNE_FILE")
        if path and Path(path).exists():
            try:
                cached = json.loads(Path(path).read_text()).get(key)
            except (OSError, ValueError):
                cached = None
            if cached is not None:
                self.set_config(int(cached["config"]))
                return cached
        ms = np.zeros(4)
        best = C.c_int()
        self.ctx.check(self.ctx.lib.lm_batch_tune(self.handle, int(steps), _lib.dptr(ms), C.byref(best)))
        res = {"config": best.value, "name": CONFIG_NAMES[best.value],
               "ms_per_step": {CONFIG_NAMES[c]: (float(ms[c]) if ms[c] >= 0 else None) for c in range(4)}}
        if path:
            try:
                data = json.loads(Path(path).read_text()) if Path(path).exists() else {}
            except (OSError, ValueError):
                data = {}
            data[key] = res
            Path(path).write_text(json.dumps(data, indent=1))
        return res

    def signature(self) -> str:
        sizes = sorted(s.n for s in self.states)
        return json.dumps({"kind": self.kind, "precision": self.precision, "K": self.info()["K"],
                           "instances": len(sizes), "N_total": int(sum(sizes)),
                           "N_max": int(max(sizes)) if sizes else 0})
