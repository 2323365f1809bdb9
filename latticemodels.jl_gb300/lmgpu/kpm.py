"""Density of states and local density of states by the kernel polynomial method.

The reference computes ``dos(eig, E; broaden)`` from a full eigensystem,
``imag(sum(1 ./ (E_n .- (E + i*broaden)))) / pi`` (src/greenfunction.jl:306), and ``ldos``
from a Green's function (src/greenfunction.jl:309-339).  Here the same Lorentzian-broadened
quantities come from Chebyshev moments computed on the GPU (``lm_kpm_moments``), with no
eigensystem.  The resolvent has an exact Chebyshev expansion: for z outside [-1, 1],

    1 / (z - x) = (1 / sqrt(z^2 - 1)) * sum_n (2 - delta_n0) rho^n T_n(x),  rho = z - sqrt(z^2 - 1), |rho| < 1,

so with mu_n = Tr T_n(H~), H~ = (H - b)/a and z~ = (E + i*broaden - b)/a,

    Tr (E + i*broaden - H)^{-1} = (1/a) (1/sqrt(z~^2 - 1)) sum_n (2 - delta_n0) mu_n rho^n,

and dos(E) = -Im of that / pi.  The series converges geometrically (|rho| < 1 for
broaden > 0); ``nmom`` is chosen so that the neglected tail is below ``tol`` relative to mu_0.
With the exact trace (the N unit vectors, the default up to ``exact_max`` sites) the result
matches the eigensystem formula to the series tolerance; above that a stochastic trace over
``nvec`` random phase vectors is used.
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib
from .device import default_context
from .hamiltonian import Hamiltonian
from .lattice import LatticeValue
from .states import DeviceState


def _bounds(H: Hamiltonian, ctx, pad=1e-3, method: str = "gershgorin"):
    lo, hi = H.bounds(ctx, method=method)
    w = hi - lo
    return lo - pad * w, hi + pad * w


def moments(H: Hamiltonian, nmom: int, vecs=None, per_site: bool = False, bounds=None, ctx=None):
    """Chebyshev moments mu_n = sum_v <v|T_n(H~)|v>, n < nmom, on [emin, emax] = ``bounds``
    (default: the Gershgorin enclosure, padded by 0.1 %).  ``vecs``: an (N, R) array of starting
    vectors or a c64 ket DeviceState; None means the N unit vectors (exact trace).  Returns
    (mu, (emin, emax)); mu has shape (nmom,) or, with ``per_site``, (ncols, nmom)."""
    ctx = ctx or default_context()
    emin, emax = bounds if bounds is not None else _bounds(H, ctx)
    dh = H.device(ctx)
    st = None
    if vecs is not None:
        if isinstance(vecs, DeviceState):
            st = vecs
        else:
            st = DeviceState(H.lattice, np.asarray(vecs, dtype=np.complex128), _lib.LM_KETS, "c64", None, ctx)
    ncols = (st.m if st is not None else H.lattice.N) if per_site else 1
    out = np.empty(ncols * nmom, dtype=np.float64)
    ctx.check(ctx.lib.lm_kpm_moments(dh.handle, float(emin), float(emax), int(nmom),
                                     st.handle if st is not None else None, 1 if per_site else 0, _lib.dptr(out)))
    mu = out.reshape(ncols, nmom) if per_site else out
    return mu, (emin, emax)


def _rho(E, broaden, a, b):
    z = (np.asarray(E, dtype=np.float64) + 1j * broaden - b) / a
    s = np.sqrt(z * z - 1)
    rho = z - s
    flip = np.abs(rho) > 1
    s = np.where(flip, -s, s)
    rho = z - s
    return rho, s


def order_for(E, broaden: float, bounds, tol: float = 1e-11, cap: int = 200000) -> int:
    """Number of moments whose neglected tail is below ``tol`` (relative) on the energy grid."""
    if not broaden > 0:
        raise ValueError("broaden must be positive")
    emin, emax = bounds
    a, b = 0.5 * (emax - emin), 0.5 * (emax + emin)
    rho, _ = _rho(np.atleast_1d(E), broaden, a, b)
    r = float(np.abs(rho).max())
    n = int(math.ceil(math.log(tol * (1 - r)) / math.log(r))) + 2
    return max(2, min(n, cap))


def resolvent_trace(mu, E, broaden: float, bounds):
    """sum of Tr (E + i*broaden - H)^{-1} from the moments (last axis of mu), per energy."""
    emin, emax = bounds
    a, b = 0.5 * (emax - emin), 0.5 * (emax + emin)
    E = np.atleast_1d(np.asarray(E, dtype=np.float64))
    rho, s = _rho(E, broaden, a, b)
    n = np.arange(np.shape(mu)[-1])
    w = np.where(n == 0, 1.0, 2.0)
    P = rho[:, None] ** n[None, :] * w[None, :]          # (nE, nmom)
    G = (P @ np.asarray(mu, dtype=np.complex128).T)       # (nE,) or (nE, ncols)
    return G / (a * (s[:, None] if G.ndim == 2 else s))


def dos(H: Hamiltonian, E, broaden: float = 0.1, *, tol: float = 1e-11, nmom=None, exact_max: int = 8192,
        nvec: int = 64, seed: int = 0, bounds: str = "gershgorin", ctx=None):
    """dos(H, E; broaden): Im sum_n 1/(E_n - E - i*broaden) / pi (src/greenfunction.jl:306)
    from device Chebyshev moments.  Returns a float for a scalar E, else an array.  bounds:
    "gershgorin" or "lanczos" (tighter interval, fewer moments)."""
    ctx = ctx or default_context()
    bounds = _bounds(H, ctx, method=bounds)
    nm = nmom or order_for(E, broaden, bounds, tol)
    vecs = None if H.lattice.N <= exact_max else _phase_vectors(H.lattice.N, nvec, seed)
    mu, bounds = moments(H, nm, vecs, False, bounds, ctx)
    scale = 1.0 if vecs is None else 1.0 / nvec  # E[<v|A|v>] = Tr A for random-phase v
    d = -np.imag(resolvent_trace(mu, E, broaden, bounds)) / math.pi * scale
    return float(d[0]) if np.ndim(E) == 0 else d


def ldos(H: Hamiltonian, E: float, broaden: float = 0.1, *, tol: float = 1e-11, nmom=None,
         bounds: str = "gershgorin", ctx=None) -> LatticeValue:
    """Local density of states at every site, Im sum_n |psi_n(i)|^2/(E_n - E - i*broaden) / pi,
    from the per-site moments of the N unit vectors (exact)."""
    ctx = ctx or default_context()
    bounds = _bounds(H, ctx, method=bounds)
    nm = nmom or order_for(E, broaden, bounds, tol)
    mu, bounds = moments(H, nm, None, True, bounds, ctx)
    g = resolvent_trace(mu, E, broaden, bounds)[0]
    return LatticeValue(H.lattice, -np.imag(g) / math.pi)


def _phase_vectors(N: int, R: int, seed: int):
    """R random-phase vectors e^{i theta} (seeded PCG64): E[v v^dagger] = I."""
    rng = np.random.default_rng(seed)
    return np.exp(2j * math.pi * rng.random((N, R)))
