"""Gradients of a density loss through the Chebyshev evolution (hand-written adjoint).

Problem: kets psi_0 (N x M) evolved for `nsteps` steps of dt under
    H(t) = tightbinding_hamiltonian(l, V; field = PointFlux(B_j, point))
with B_j piecewise constant over intervals of `steps_per_interval` steps, and the loss
    L = sum_i (rho_i(T) - target_i)^2,   rho_i = sum_m |psi_im(T)|^2.
`loss_and_grad` returns L, dL/dV (N values) and dL/dB (one per interval).  The forward pass
keeps a checkpoint every `checkpoint_every` steps; the backward pass recomputes each segment
from its checkpoint and runs the adjoint kernels (lm_adjoint_step) step by step, propagating
the co-state with U^dagger.  The spectral interval of the propagator is fixed for the whole
problem, so every step is one polynomial in H and the discrete gradient is exact.

`EvolutionDensityLoss` wraps it as a torch.autograd.Function (the Python analogue of the
ChainRulesCore rrule a Julia caller would define).
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import _lib
from .device import default_context
from .fields import PointFlux
from .hamiltonian import Hamiltonian
from .lattice import SquareLattice
from .states import DeviceState


class DensityLossAdjoint:
    def __init__(self, lattice: SquareLattice, psi0, target, dt: float, nsteps: int, steps_per_interval: int,
                 flux_point, t1: float = 1.0, precision: str = "c32", checkpoint_every: int = 20,
                 bounds=None, tol=None, ctx=None):
        self.ctx = ctx or default_context()
        self.lattice = lattice
        self.psi0 = np.asfortranarray(psi0)
        self.N, self.M = self.psi0.shape
        self.target = np.ascontiguousarray(target, dtype=np.float64)
        self.dt = float(dt)
        self.nsteps = int(nsteps)
        self.spi = int(steps_per_interval)
        self.nint = (self.nsteps + self.spi - 1) // self.spi
        self.point = (float(flux_point[0]), float(flux_point[1]))
        self.t1 = float(t1)
        self.precision = precision
        self.prec_code = _lib.LM_C32 if precision == "c32" else _lib.LM_C64
        self.every = int(checkpoint_every)
        # The truncation error of a step is not unitary; over hundreds of steps a 1e-7 series
        # tail (K = 5 at a dt = 0.22) moves the density by ~4e-6, so FP32 takes one more order.
        self.tol = tol if tol is not None else (1e-9 if precision == "c32" else 1e-12)
        self.bounds = bounds
        lib = self.ctx.lib
        self._dh = None
        self.fwd = self._solver()
        self.bwd = self._solver()
        p = C.c_void_p()
        self.ctx.check(lib.lm_adjoint_create(self.ctx.handle, self.N, self.M, self.prec_code, self.nint, C.byref(p)))
        self.adj = p
        weakref.finalize(self, lib.lm_adjoint_destroy, p)

    def _solver(self):
        p = C.c_void_p()
        self.ctx.check(self.ctx.lib.lm_solver_create(self.ctx.handle, float(self.tol), C.byref(p)))
        weakref.finalize(self, self.ctx.lib.lm_solver_destroy, p)
        return p

    def set_bounds(self, emin, emax):
        self.bounds = (float(emin), float(emax))

    def _prepare(self, V):
        V = np.ascontiguousarray(V, dtype=np.float64)
        if self.bounds is None:  # Gershgorin enclosure of the initial parameters with a margin
            r = 4.0 * abs(self.t1)
            lo, hi = float(V.min()) - r, float(V.max()) + r
            pad = 0.05 * (hi - lo)
            self.bounds = (lo - pad, hi + pad)
        for s in (self.fwd, self.bwd):
            self.ctx.check(self.ctx.lib.lm_solver_set_bounds(s, self.bounds[0], self.bounds[1]))
        H = Hamiltonian(self.lattice, self.t1, PointFlux(0.0, self.point), V)
        if self._dh is None:
            self._dh = H.device_private(self.ctx)
        return V

    def _assemble(self, V, B):
        self._dh.ensure(V, [float(B)])

    def _new_state(self):
        st = DeviceState.__new__(DeviceState)
        DeviceState.__init__(st, self.lattice, None, _lib.LM_KETS, self.precision, None, self.ctx,
                             shape=(self.N, self.M))
        return st

    def _step(self, solver, V, B, dt, st):
        self._assemble(V, B)
        self.ctx.check(self.ctx.lib.lm_solver_update(solver, self._dh.handle, dt, 0))
        self.ctx.check(self.ctx.lib.lm_solver_step(solver, st.handle))

    def forward(self, V, B, keep_checkpoints=False):
        """Evolves psi_0; returns the final state (and the checkpoints)."""
        V = self._prepare(V)
        psi = self._new_state()
        psi.upload(self.psi0)
        cps = [psi.copy()] if keep_checkpoints else None
        for n in range(self.nsteps):
            self._step(self.fwd, V, B[n // self.spi], self.dt, psi)
            if keep_checkpoints and (n + 1) % self.every == 0 and n + 1 < self.nsteps:
                cps.append(psi.copy())
        return psi, cps

    def loss(self, V, B) -> float:
        psi, _ = self.forward(V, B)
        lam = self._new_state()
        out = C.c_double()
        self.ctx.check(self.ctx.lib.lm_adjoint_seed(self.adj, psi.handle, _lib.dptr(self.target), lam.handle,
                                                    C.byref(out)))
        return out.value

    def loss_and_grad(self, V, B):
        V = np.ascontiguousarray(V, dtype=np.float64)
        B = np.asarray(B, dtype=np.float64)
        if B.shape != (self.nint,):
            raise ValueError(f"need {self.nint} field amplitudes")
        lib, ctx = self.ctx.lib, self.ctx
        psi, cps = self.forward(V, B, keep_checkpoints=True)
        lam = self._new_state()
        out = C.c_double()
        ctx.check(lib.lm_adjoint_seed(self.adj, psi.handle, _lib.dptr(self.target), lam.handle, C.byref(out)))
        loss = out.value
        ctx.check(lib.lm_adjoint_reset(self.adj))
        seg_states = None
        for c in range(len(cps) - 1, -1, -1):
            n0 = c * self.every
            n1 = min(self.nsteps, n0 + self.every)
            # recompute psi_{n0} .. psi_{n1-1} from the checkpoint
            if seg_states is None:
                seg_states = [self._new_state() for _ in range(self.every)]
            ctx.check(lib.lm_state_copy(seg_states[0].handle, cps[c].handle))
            for n in range(n0, n1 - 1):
                k = n - n0
                ctx.check(lib.lm_state_copy(seg_states[k + 1].handle, seg_states[k].handle))
                self._step(self.fwd, V, B[n // self.spi], self.dt, seg_states[k + 1])
            for n in range(n1 - 1, n0 - 1, -1):
                j = n // self.spi
                self._assemble(V, B[j])
                ctx.check(lib.lm_solver_update(self.fwd, self._dh.handle, self.dt, 0))
                ctx.check(lib.lm_adjoint_step(self.adj, self.fwd, self._dh.handle, 0, j,
                                              seg_states[n - n0].handle, lam.handle))
                # lambda_n = U_n^dagger lambda_{n+1}
                self._step(self.bwd, V, B[j], -self.dt, lam)
        gV = np.empty(self.N)
        gB = np.empty(self.nint)
        ctx.check(lib.lm_adjoint_gradients(self.adj, _lib.dptr(gV), _lib.dptr(gB)))
        return loss, gV, gB


def _torch_function():
    import torch

    class EvolutionDensityLoss(torch.autograd.Function):
        """loss = EvolutionDensityLoss.apply(V, B, problem): FP64 tensors in, scalar loss out."""

        @staticmethod
        def forward(ctx, V, B, problem):
            loss, gV, gB = problem.loss_and_grad(V.detach().cpu().numpy(), B.detach().cpu().numpy())
            ctx.save_for_backward(torch.as_tensor(gV, dtype=V.dtype), torch.as_tensor(gB, dtype=B.dtype))
            return torch.as_tensor(loss, dtype=V.dtype)

        @staticmethod
        def backward(ctx, g):
            gV, gB = ctx.saved_tensors
            return g * gV, g * gB, None

    return EvolutionDensityLoss


def __getattr__(name):
    if name == "EvolutionDensityLoss":
        return _torch_function()
    raise AttributeError(name)
