"""``diagonalize`` / ``densitymatrix`` on the device (src/spectrum.jl:48-55, :226-257, :317-333).

Two routes to P = f(H) = sum_i f(E_i) |psi_i><psi_i|, both on the library's own kernels:
* T > 0 FermiDirac ensemble: the Chebyshev series of f on the spectral interval, applied to
  the identity (``lm_cheb_apply``): no eigensystem, O(K N^2) work for K terms, exact to the
  series tolerance.
* every other case (T = 0, BoseEinstein, the Gibbs state, fixed N) or on request: the device
  eigensystem (``lm_eigsys_*``: Householder tridiagonalisation, bisection, inverse
  iteration, all FP64) weighted by the reference's occupations.  At T = 0 "E == mu" means
  |E - mu| <= DEGENERATE_TOL max(1, |E|max): a level exactly degenerate at mu is occupied as a
  whole instead of being split by the rounding of its computed eigenvalues.
"""
from __future__ import annotations

import ctypes as C
import math
import weakref

import numpy as np

from . import _lib
from .device import default_context
from .hamiltonian import Hamiltonian
from .states import DensityMatrix, DeviceState, KetBlock

# relative width of "E == mu" at T = 0 (src/spectrum.jl:230-232)
DEGENERATE_TOL = 1e-12


class Eigensystem:
    """The eigensystem of a device Hamiltonian, ``diagonalize(H)`` (src/spectrum.jl:48-55,
    :108-116): ``values`` (ascending, host FP64), eigenvectors and weighted projectors computed
    on the device on demand."""

    def __init__(self, H, ctx=None):
        from .sparse import SparseHamiltonian
        ctx = ctx or default_context()
        self.ctx = ctx
        self.hamiltonian = H
        self.lattice = H.lattice
        dh = H.device(ctx)
        p = C.c_void_p()
        if isinstance(H, SparseHamiltonian):
            ctx.check(ctx.lib.lm_eigsys_create_ell(dh.handle, C.byref(p)))
        elif isinstance(H, Hamiltonian):
            ctx.check(ctx.lib.lm_eigsys_create(dh.handle, C.byref(p)))
        else:
            raise TypeError("diagonalize takes a device Hamiltonian (tightbinding_hamiltonian, SparseHamiltonian)")
        self.handle = p
        self._fin = weakref.finalize(self, ctx.lib.lm_eigsys_destroy, p)
        n = C.c_int64()
        ctx.check(ctx.lib.lm_eigsys_size(p, C.byref(n)))
        self.n = n.value
        self.values = np.empty(self.n, dtype=np.float64)
        ctx.check(ctx.lib.lm_eigsys_values(p, _lib.dptr(self.values)))

    def __len__(self):
        return self.n

    def vectors(self, first: int = 0, count=None, precision="c64") -> KetBlock:
        """Eigenvectors first .. first + count - 1 as the columns of a device ket block."""
        count = self.n - first if count is None else int(count)
        if first < 0 or count < 1 or first + count > self.n:
            raise ValueError("eigenvector range outside the spectrum")
        out = DeviceState(self.lattice, None, _lib.LM_KETS, precision, ctx=self.ctx, shape=(self.n, count))
        out.__class__ = KetBlock
        self.ctx.check(self.ctx.lib.lm_eigsys_vectors(self.handle, int(first), out.handle))
        return out

    def projector(self, weights, precision="c64") -> DensityMatrix:
        """sum_k w_k |v_k><v_k| as a device density matrix (weights in eigenvalue order)."""
        w = np.ascontiguousarray(weights, dtype=np.float64)
        if w.shape != (self.n,):
            raise ValueError("one weight per eigenvalue")
        out = DensityMatrix(self.lattice, None, precision, ctx=self.ctx)
        self.ctx.check(self.ctx.lib.lm_eigsys_projector(self.handle, _lib.dptr(w), out.handle))
        return out


def diagonalize(H) -> Eigensystem:
    """``diagonalize(H)``: the device eigensystem (values ascending, vectors on demand)."""
    return Eigensystem(H)


def densfun(T: float, mu: float, statistics: str = "FermiDirac", degenerate_tol: float = 0.0):
    """E -> (E - mu == T == 0) ? 1 : 1 / (exp((E - mu)/T) + s), s = +1 FermiDirac, -1
    BoseEinstein (src/spectrum.jl:230-232).  At T = 0 a level below mu gets 1/s, and "E == mu"
    means |E - mu| <= degenerate_tol."""
    sgn = 1.0 if statistics == "FermiDirac" else -1.0

    def f(E):
        d = E - mu
        if T == 0 and abs(d) <= degenerate_tol:
            return 1.0
        if T == 0:
            return 1.0 / sgn if d < 0 else 0.0
        z = d / T
        return 1.0 / (math.exp(z) + sgn) if z < 700 else 0.0
    return f


def chebyshev_coefficients(f, bounds, tol: float = 1e-13, max_nodes: int = 1 << 22):
    """Real Chebyshev coefficients c_n of x -> f(a x + b) on [-1, 1] ([b - a, b + a] = bounds),
    truncated where sum_{n >= K} |c_n| <= tol, from Chebyshev-Gauss nodes (a type-II DCT)."""
    from scipy.fft import dct
    emin, emax = bounds
    a, b = 0.5 * (emax - emin), 0.5 * (emax + emin)
    nodes = 4096
    while True:
        k = np.arange(nodes)
        x = np.cos(math.pi * (k + 0.5) / nodes)
        c = dct(f(a * x + b), type=2) / nodes
        c[0] *= 0.5
        tail = np.cumsum(np.abs(c)[::-1])[::-1]
        below = np.nonzero(tail <= tol)[0]
        if len(below) and below[0] <= nodes // 4:
            return c[: max(int(below[0]), 1)]
        if nodes >= max_nodes:
            raise ValueError("the Chebyshev series of f does not converge on the spectral interval")
        nodes *= 2


def fermi_occupation(mu: float, T: float):
    """FermiDirac f(E) = 1 / (exp((E - mu)/T) + 1) for T > 0 (src/spectrum.jl:230-232), vectorised."""
    return lambda E: 0.5 * (1.0 - np.tanh((np.asarray(E) - mu) / (2.0 * T)))


_STATISTICS = ("FermiDirac", "BoseEinstein")


def degenerate_tol(w) -> float:
    """Width of "E == mu" for the eigenvalues w: DEGENERATE_TOL max(1, |E|max)."""
    w = np.asarray(w, dtype=np.float64)
    return DEGENERATE_TOL * max(1.0, float(np.abs(w).max()) if len(w) else 1.0)


def occupations(w, mu=None, T: float = 0.0, N=None, statistics=None, tol=None) -> np.ndarray:
    """Weights f(E_i) of the eigenvalues ``w`` (ascending) that ``densitymatrix`` puts on the
    eigenvectors, following the reference's dispatch for a one-particle system
    (src/spectrum.jl:239-333):
    * ``N``: fixn_densitymatrix -- at T = 0 the Fermi sphere (the lowest N states) or, for
      BoseEinstein, N times the ground state; at T > 0 mu from the reference's Newton
      iteration on the eigenvalues (start 0, step (N_ev - N)/dN_ev, atol sqrt(eps));
    * ``mu`` or ``statistics``: ensemble_densitymatrix, densfun(T, mu, statistics);
    * neither: gibbs_densitymatrix -- the ground state at T = 0, else exp(-E/T)/Z (shifted by
      the lowest level, which gives the same weights without overflow)."""
    import warnings
    w = np.asarray(w, dtype=np.float64)
    stat = statistics or "FermiDirac"
    if stat not in _STATISTICS:
        raise ValueError("statistics must be FermiDirac or BoseEinstein")
    if N is not None:
        if mu is not None:
            raise ValueError("cannot specify both N and μ")
        N = int(N)
        occ = np.zeros(len(w))
        if abs(T) < 1e-10:
            if stat == "BoseEinstein":
                occ[0] = N
                return occ
            if len(w) < N:
                raise ValueError(f"cannot build Fermi sphere with {N} particles: only {len(w)} bands present")
            if N < len(w) and math.isclose(w[N - 1], w[N], rel_tol=math.sqrt(np.finfo(float).eps)):
                warnings.warn("degenerate levels on the Fermi sphere")
            occ[:N] = 1.0
            return occ
        newmu = 0.0
        sgn = 1.0 if stat == "FermiDirac" else -1.0
        for _ in range(1000):
            z = np.minimum((w - newmu) / T, 700.0)
            ez = np.exp(z)
            n_ev = np.sum(np.where(z >= 700.0, 0.0, 1.0 / (ez + sgn)))
            dn_ev = np.sum(np.where(z >= 700.0, 0.0, -ez / T / (ez + sgn) ** 2))
            dmu = (n_ev - N) / dn_ev
            if abs(dmu) < math.sqrt(np.finfo(float).eps):
                f = densfun(T, newmu, stat)
                return np.array([f(e) for e in w])
            newmu += dmu
        raise ValueError("did not converge")
    if mu is not None or statistics is not None:
        f = densfun(T, 0.0 if mu is None else mu, stat, degenerate_tol(w) if tol is None else tol)
        return np.array([f(e) for e in w])
    occ = np.zeros(len(w))
    if abs(T) < 1e-10:
        occ[0] = 1.0
        return occ
    occ = np.exp(-(w - w[0]) / T)
    return occ / occ.sum()


def densitymatrix(H, mu=None, T: float = 0.0, *, N=None, statistics=None, precision="c64",
                  method: str = "auto", tol: float = 1e-13, bounds: str = "gershgorin") -> DensityMatrix:
    """``densitymatrix(H; mu, T, N, statistics)`` of a one-particle system (src/spectrum.jl:239-333;
    the dispatch is ``occupations``).  The FermiDirac ensemble at T > 0 runs the Chebyshev
    Fermi operator on the device (``lm_cheb_apply``) unless method="eigh"; every other case
    weights the device eigensystem (``diagonalize``).  bounds: the spectral interval of the
    Chebyshev route, "gershgorin" or "lanczos" (tighter: fewer terms)."""
    from .sparse import SparseHamiltonian
    if method not in ("auto", "chebyshev", "eigh"):
        raise ValueError("method must be auto, chebyshev or eigh")
    if N is not None and mu is not None:
        raise ValueError("cannot specify both N and μ")
    stat = statistics or "FermiDirac"
    if stat not in _STATISTICS:
        raise ValueError("statistics must be FermiDirac or BoseEinstein")
    fermi_ensemble = N is None and (mu is not None or statistics is not None) and stat == "FermiDirac"
    if method == "chebyshev" and not (fermi_ensemble and T > 0 and isinstance(H, Hamiltonian)):
        raise ValueError("the Chebyshev route covers the FermiDirac ensemble at T > 0 of a square-lattice "
                         "Hamiltonian (the T = 0 occupation is a step)")
    if fermi_ensemble and T > 0 and method != "eigh" and isinstance(H, Hamiltonian):
        mu = 0.0 if mu is None else mu
        ctx = default_context()
        lo, hi = H.bounds(ctx, method=bounds)
        pad = 1e-3 * (hi - lo)
        bounds = (lo - pad, hi + pad)
        coef = np.ascontiguousarray(chebyshev_coefficients(fermi_occupation(mu, T), bounds, tol))
        out = DensityMatrix(H.lattice, None, precision, ctx=ctx)
        dh = H.device(ctx)
        ctx.check(ctx.lib.lm_cheb_apply(dh.handle, float(bounds[0]), float(bounds[1]), _lib.dptr(coef), len(coef),
                                        None, out.handle))
        return out
    if not isinstance(H, (Hamiltonian, SparseHamiltonian)):
        raise TypeError("densitymatrix takes a device Hamiltonian (tightbinding_hamiltonian, SparseHamiltonian)")
    eig = Eigensystem(H)
    return eig.projector(occupations(eig.values, mu, T, N, statistics), precision)
