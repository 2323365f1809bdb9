"""``diagonalize`` / ``densitymatrix`` on the device (src/spectrum.jl:48-55, :226-257, :317-333).

The dense Hermitian eigensolver is cuSOLVER (through torch.linalg.eigh on the GPU); the
occupation f(E) and the projector V f(E) V^dagger follow the reference.  This produces the
input P_0 of the evolution path; it runs on the GPU only (no host eigensolver).
"""
from __future__ import annotations

import math

import numpy as np

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


def densfun(T: float, mu: float):
    """FermiDirac occupation; at T = 0, E == mu counts as occupied (src/spectrum.jl:230-232)."""
    def f(E):
        d = E - mu
        if d == 0 and T == 0:
            return 1.0
        if T == 0:
            return 1.0 if d < 0 else 0.0
        z = d / T
        return 1.0 / (math.exp(z) + 1.0) if z < 700 else 0.0
    return f


def densitymatrix(H: Hamiltonian, mu: float = 0.0, T: float = 0.0, precision="c64") -> DensityMatrix:
    """``densitymatrix(H; mu, T)`` for a one-particle system with FermiDirac statistics."""
    torch = _torch_cuda()
    w, V = diagonalize(H)
    f = densfun(T, mu)
    occ = torch.as_tensor(np.array([f(e) for e in w]), device="cuda", dtype=torch.float64)
    P = (V * occ) @ V.conj().T
    return DensityMatrix(H.lattice, P.cpu().numpy(), precision)
