"""``diagonalize`` / ``densitymatrix`` on the device (src/spectrum.jl:48-55, :226-257, :317-333).

Two routes to P = f(H) = sum_i f(E_i) |psi_i><psi_i| with the FermiDirac occupation f:
* T > 0: the Chebyshev series of f on the spectral interval, applied to the identity by the
  library's own stencil kernels (``lm_cheb_apply``): no eigensystem, O(K N^2) work for K
  terms, exact to the series tolerance.
* T = 0 (a step function, whose series does not converge), or on request: the dense
  Hermitian eigensolver cuSOLVER (through torch.linalg.eigh on the GPU), with the reference's
  occupation rule (E == mu counts as occupied).
Both run on the GPU only (no host eigensolver).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .device import default_context
from .hamiltonian import Hamiltonian
from .states import DensityMatrix


def _torch_cuda():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("densitymatrix runs on the GPU and no CUDA device is available")
    return torch


def _dense_on_device(H: Hamiltonian, torch):
    colptr, rowval, nz = H.csc()
    N = H.N
    cols = np.repeat(np.arange(N), np.diff(colptr))
    rows = rowval - 1
    idx = torch.as_tensor(np.stack([rows, cols]), device="cuda")
    vals = torch.as_tensor(nz, device="cuda")
    return torch.sparse_coo_tensor(idx, vals, (N, N)).to_dense()


def diagonalize(H: Hamiltonian):
    """Eigenvalues (ascending, FP64 host array) and eigenvectors (device tensor)."""
    torch = _torch_cuda()
    A = _dense_on_device(H, torch)
    w, V = torch.linalg.eigh(A)
    return w.cpu().numpy(), V


def densfun(T: float, mu: float, statistics: str = "FermiDirac"):
    """E -> (E - mu == T == 0) ? 1 : 1 / (exp((E - mu)/T) + s), s = +1 FermiDirac, -1
    BoseEinstein (src/spectrum.jl:230-232).  At T = 0 a level below mu gets 1/s."""
    sgn = 1.0 if statistics == "FermiDirac" else -1.0

    def f(E):
        d = E - mu
        if d == 0 and T == 0:
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


def occupations(w, mu=None, T: float = 0.0, N=None, statistics=None) -> np.ndarray:
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
        f = densfun(T, 0.0 if mu is None else mu, stat)
        return np.array([f(e) for e in w])
    occ = np.zeros(len(w))
    if abs(T) < 1e-10:
        occ[0] = 1.0
        return occ
    occ = np.exp(-(w - w[0]) / T)
    return occ / occ.sum()


def densitymatrix(H: Hamiltonian, mu=None, T: float = 0.0, *, N=None, statistics=None, precision="c64",
                  method: str = "auto", tol: float = 1e-13, bounds: str = "gershgorin") -> DensityMatrix:
    """``densitymatrix(H; mu, T, N, statistics)`` of a one-particle system (src/spectrum.jl:239-333;
    the dispatch is ``occupations``).  The FermiDirac ensemble at T > 0 runs the Chebyshev
    Fermi operator on the device (``lm_cheb_apply``) unless method="eigh"; every other case
    weights the device eigensystem (cuSOLVER).  bounds: the spectral interval of the
    Chebyshev route, "gershgorin" or "lanczos" (tighter: fewer terms)."""
    if method not in ("auto", "chebyshev", "eigh"):
        raise ValueError("method must be auto, chebyshev or eigh")
    if N is not None and mu is not None:
        raise ValueError("cannot specify both N and μ")
    stat = statistics or "FermiDirac"
    if stat not in _STATISTICS:
        raise ValueError("statistics must be FermiDirac or BoseEinstein")
    fermi_ensemble = N is None and (mu is not None or statistics is not None) and stat == "FermiDirac"
    if method == "chebyshev" and not (fermi_ensemble and T > 0):
        raise ValueError("the Chebyshev route covers the FermiDirac ensemble at T > 0 (the T = 0 occupation "
                         "is a step)")
    if fermi_ensemble and T > 0 and method != "eigh":
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
    torch = _torch_cuda()
    w, V = diagonalize(H)
    occ = torch.as_tensor(occupations(w, mu, T, N, statistics), device="cuda", dtype=torch.float64)
    P = (V * occ) @ V.conj().T
    if precision == "c32":
        P = P.to(torch.complex64)
    # the library's layout is column-major: a row-major copy of P^T holds P column-major
    Pc = P.transpose(0, 1).contiguous()
    torch.cuda.current_stream().synchronize()
    ctx = default_context()
    out = DensityMatrix(H.lattice, None, precision, ctx=ctx)
    ctx.check(ctx.lib.lm_state_upload(out.handle, C.c_void_p(Pc.data_ptr()), H.lattice.N))
    ctx.synchronize()  # Pc stays alive until the device copy is done
    return out
