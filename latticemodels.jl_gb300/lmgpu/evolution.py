"""Time evolution: the reference's ``Evolution`` driver and its ``EvolutionSolver`` plugin API,
with ``ChebyshevGPU`` as the device solver (src/evolution.jl:5-33, :183-298).
"""
from __future__ import annotations

import ctypes as C
import math
import weakref

import numpy as np

from . import _lib
from .device import default_context
from .hamiltonian import Hamiltonian
from .states import DeviceState


class EvolutionSolver:
    """Abstract solver (src/evolution.jl:5-25).

    Methods to implement: ``update_solver(H, dt, force=False)``, ``step(state, cache)`` and
    optionally ``evolution_cache(state)`` (returns None by default).
    """

    def update_solver(self, H, dt, force=False):
        raise NotImplementedError

    def step(self, state, cache):
        raise NotImplementedError

    def evolution_cache(self, state):
        return None


class ChebyshevGPU(EvolutionSolver):
    """Chebyshev propagator exp(-i H dt) on the GPU.

    ``tol`` is the truncation of the Chebyshev series (sum of the neglected |c_k|); by default
    1e-12 for ComplexF64 states and 1e-9 for ComplexF32 states.  The truncation error of a step
    is coherent (the same polynomial every step), so it adds up linearly: 1e-9 keeps 200-step
    runs within 1e-6 of FP64 on densities and currents, while 1e-7 (one order fewer, ~12 %
    faster) is enough for runs of a few tens of steps.  ``renorm_every`` > 0 rescales
    every ket to its initial FP64 norm every that many steps (for the FP32 form).
    """

    def __init__(self, hamiltonian=None, *, tol=None, precision=None, renorm_every=0, ctx=None):
        self.ctx = ctx or default_context()
        self.tol = tol
        self.precision = precision
        self.renorm_every = int(renorm_every)
        self._solvers = {}
        self._H = None
        self._dt = None
        self._force = False
        self._nsteps = {}

    def _tol_for(self, state: DeviceState):
        if self.tol is not None:
            return float(self.tol)
        return 1e-12 if state.precision == _lib.LM_C64 else 1e-9

    def _solver(self, tol):
        s = self._solvers.get(tol)
        if s is None:
            p = C.c_void_p()
            self.ctx.check(self.ctx.lib.lm_solver_create(self.ctx.handle, tol, C.byref(p)))
            s = p
            self._solvers[tol] = s
            weakref.finalize(self, self.ctx.lib.lm_solver_destroy, p)
        return s

    def update_solver(self, H: Hamiltonian, dt: float, force: bool = False):
        """update_solver!(solver, H, dt, force) (src/evolution.jl:83-92)."""
        from .sparse import SparseHamiltonian
        if not isinstance(H, (Hamiltonian, SparseHamiltonian)):
            raise TypeError("ChebyshevGPU evolves device Hamiltonians (tightbinding_hamiltonian, SparseHamiltonian)")
        self._H = H
        self._dt = float(dt)
        self._force = bool(force)

    def _prepare(self, state):
        tol = self._tol_for(state)
        s = self._solver(tol)
        dh = self._H.device(self.ctx)
        if isinstance(self._H, Hamiltonian):
            self.ctx.check(self.ctx.lib.lm_solver_update(s, dh.handle, self._dt, 1 if self._force else 0))
        else:  # a general sparse Hamiltonian (other lattices, internal degrees of freedom)
            self.ctx.check(self.ctx.lib.lm_ell_solver_update(s, dh.handle, self._dt, 1 if self._force else 0))
        return s

    def order(self, state=None):
        """(K, a, b) of the current propagator: K Chebyshev orders on [b - a, b + a]."""
        tol = 1e-12 if state is None else self._tol_for(state)
        s = self._solver(tol)
        K = C.c_int()
        a = C.c_double()
        b = C.c_double()
        self.ctx.check(self.ctx.lib.lm_solver_order(s, C.byref(K), C.byref(a), C.byref(b)))
        return K.value, a.value, b.value

    def evolution_cache(self, state):
        """FP64 reference norms for the periodic renormalisation of the FP32 form."""
        if self.renorm_every > 0 and state.kind == _lib.LM_KETS:
            return {"norms": state.norms()}
        return None

    def step(self, state: DeviceState, cache=None):
        """step!(solver, state, cache) (src/evolution.jl:69-78): psi <- U psi, P <- U P U^dagger."""
        if self._H is None:
            raise RuntimeError("update_solver must run before step")
        s = self._prepare(state)
        self.ctx.check(self.ctx.lib.lm_solver_step(s, state.handle))
        n = self._nsteps.get(id(state), 0) + 1
        self._nsteps[id(state)] = n
        if self.renorm_every > 0 and cache and n % self.renorm_every == 0:
            state.renormalize(cache["norms"])
        return state


class EvolutionTimestamp:
    """One yielded moment: H (evaluated at the start of the step), the states and t
    (src/evolution.jl:277-298).  Unpacks as ``P, H, t = moment``."""

    def __init__(self, H, states, t):
        self.H = H
        self.states = states
        self.t = t

    def __iter__(self):
        vals = list(self.states.values()) if isinstance(self.states, dict) else list(self.states)
        return iter(vals + [self.H, self.t])

    @property
    def state(self):
        vals = list(self.states.values()) if isinstance(self.states, dict) else list(self.states)
        if len(vals) != 1:
            raise ValueError("moment holds more than one state")
        return vals[0]

    def __getitem__(self, key):
        if isinstance(self.states, dict) and isinstance(key, str):
            return self.states[key]
        vals = list(self.states.values()) if isinstance(self.states, dict) else list(self.states)
        return vals[key]

    def __getattr__(self, name):
        st = self.__dict__.get("states")
        if isinstance(st, dict) and name in st:
            return st[name]
        raise AttributeError(name)


class Evolution:
    """``Evolution([solver, ]hamiltonian, states...; timedomain, namedstates...)``
    (src/evolution.jl:183-236).

    ``hamiltonian`` is a Hamiltonian or a function t -> Hamiltonian.  States are copied at
    construction (src/evolution.jl:190-194).  The object is a stateful iterator: calling it
    again continues from the current time.
    """

    def __init__(self, *args, timedomain=None, showprogress=False, **namedstates):
        args = list(args)
        if not args:
            raise TypeError("Evolution needs a Hamiltonian")
        if isinstance(args[0], EvolutionSolver):
            solver = args.pop(0)
        elif isinstance(args[0], type) and issubclass(args[0], EvolutionSolver):
            solver = args.pop(0)()
        else:
            solver = ChebyshevGPU()
        if not args:
            raise TypeError("Evolution needs a Hamiltonian")
        self.hamiltonian = args.pop(0)
        states = args
        if states and namedstates:
            raise ValueError("Do not use named and unnamed states together")
        if not states and not namedstates:
            raise ValueError("No states provided")
        self.solver = solver
        self.named = bool(namedstates)
        src = namedstates if namedstates else {i: s for i, s in enumerate(states)}
        self.states = {}
        for k, st in src.items():
            if not isinstance(st, DeviceState):
                raise TypeError(f"invalid state type: {type(st).__name__}")
            c = st.copy()
            self.states[k] = (c, solver.evolution_cache(c))
        self.time = 0.0
        self.timedomain = timedomain
        self.showprogress = showprogress

    def _eval_ham(self, t):
        h = self.hamiltonian
        return h(t) if callable(h) and not isinstance(h, Hamiltonian) else h

    def step(self, dt: float):
        """step!(evol, dt) (src/evolution.jl:238-250): returns H(t) at the start of the step."""
        if dt < -1e-15:
            raise ValueError("negative time step")
        t = self.time
        H = self._eval_ham(t)
        if abs(dt) < 1e-15:
            return H
        self.solver.update_solver(H, dt, False)
        for st, cache in self.states.values():
            self.solver.step(st, cache)
        self.time += dt
        return H

    def current_states(self):
        if self.named:
            return {k: v[0] for k, v in self.states.items()}
        return tuple(v[0] for v in self.states.values())

    def __call__(self, times, showprogress=False):
        return EvolutionIterator(self, list(times))

    def __iter__(self):
        if self.timedomain is None:
            raise TypeError("Evolution created without a timedomain; call it with the times")
        return iter(EvolutionIterator(self, list(self.timedomain)))


class EvolutionIterator:
    """Yields a moment per time; the first dt is times[0] - current time (src/evolution.jl:261-275)."""

    def __init__(self, evol: Evolution, times):
        self.evol = evol
        self.times = times

    def __len__(self):
        return len(self.times)

    def __iter__(self):
        ev = self.evol
        for i, ti in enumerate(self.times):
            dt = ti - self.times[i - 1] if i > 0 else ti - ev.time
            H = ev.step(dt)
            yield EvolutionTimestamp(H, ev.current_states(), float(ev.time))
