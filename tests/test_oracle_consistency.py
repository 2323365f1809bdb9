"""Internal consistency of the oracle's helpers (CPU): the vectorised Hamiltonian against the
scalar restatement, the occupation derivative, the Bessel sequence, the honeycomb model, the
entry currents against the bond currents, and the exact loss gradient against finite
differences.  These are the pieces the GPU parity tests take as ground truth."""
import math

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import lm_oracle as o

GEOMS = [(5, 4, (False, False)), (6, 6, (True, True)), (7, 3, (True, False)), (4, 5, (False, True))]


@pytest.mark.parametrize("Lx,Ly,per", GEOMS)
@pytest.mark.parametrize("B", [None, 0.07])
@pytest.mark.parametrize("with_onsite", [False, True])
def test_vectorised_hamiltonian_equals_scalar(Lx, Ly, per, B, with_onsite):
    lat = o.SquareLattice(Lx, Ly, periodic=per)
    V = o.anderson_disorder(lat.N, 1.0, 11) if with_onsite else None
    field = None if B is None else o.LandauGauge(B)
    Hs, bonds, vals = o.tightbinding_hamiltonian(lat, field=field, onsite=V, return_bonds=True)
    Hf, src, dst, val = o.tightbinding_hamiltonian_fast(lat, field=field, onsite=V)
    assert abs(sp.csr_matrix(Hs) - sp.csr_matrix(Hf)).max() <= 1e-14
    # the same bonds (1-based source, destination) with the same values, in any order
    scalar = {(bd.src, bd.dst): v for bd, v in zip(bonds, vals)}
    fast = {(int(a), int(b)): v for a, b, v in zip(src, dst, val)}
    assert scalar.keys() == fast.keys()
    assert max(abs(scalar[k] - fast[k]) for k in scalar) <= 1e-14


@pytest.mark.parametrize("statistics", ["FermiDirac", "BoseEinstein"])
def test_occupation_derivative_is_the_energy_derivative(statistics):
    """ddensfun is df/dE = -e^z / T / (e^z + s)^2 as the reference writes it (src/spectrum.jl:233-235)."""
    T, mu, h = 0.3, 0.1, 1e-6
    f, df = o.densfun(T, mu, statistics), o.ddensfun(T, mu, statistics)
    for E in (0.25, 0.45, 1.3, 3.0):  # above mu: BoseEinstein stays finite
        fd = (f(E + h) - f(E - h)) / (2 * h)
        assert abs(df(E) - fd) <= 1e-7 * max(1.0, abs(fd))


def test_bessel_sequence():
    x = 2.7
    J = o.bessel_j_seq(x, 40)
    assert abs(o.bessel_j_seq(0.0, 3)[0] - 1.0) <= 1e-15 and np.all(o.bessel_j_seq(0.0, 3)[1:] == 0.0)
    for k in range(1, 39):  # J_{k-1} + J_{k+1} = (2k / x) J_k
        assert abs(J[k - 1] + J[k + 1] - 2 * k / x * J[k]) <= 1e-14
    assert abs(J[0] + 2 * J[2::2].sum() - 1.0) <= 1e-14  # 1 = J_0 + 2 sum J_2k


@pytest.mark.parametrize("a,b", [(3, 4), (5, 2)])
@pytest.mark.parametrize("B", [0.0, 0.1])
def test_honeycomb_model(a, b, B):
    H, coords = o.honeycomb_hamiltonian(a, b, B=B)
    H = sp.csr_matrix(H)
    N = 2 * a * b
    assert H.shape == (N, N) and coords.shape == (N, 2)
    assert abs(H - H.conj().T).max() <= 1e-15
    offdiag = H - sp.diags(H.diagonal())
    assert offdiag.nnz == 2 * (3 * a * b - a - b)  # open honeycomb: 3ab - a - b bonds
    # every bond joins the two sublattices at distance 1/sqrt(3)
    rows, cols = offdiag.nonzero()
    assert np.all(rows % 2 != cols % 2)
    d = np.linalg.norm(coords[rows] - coords[cols], axis=1)
    assert np.allclose(d, 1 / math.sqrt(3), atol=1e-12)
    # bipartite: the spectrum is symmetric about 0 with or without the field
    w = np.linalg.eigvalsh(H.toarray())
    assert np.allclose(w, -w[::-1], atol=1e-12)


@pytest.mark.parametrize("Lx,Ly,per", GEOMS)
def test_entry_currents_match_bond_currents(Lx, Ly, per):
    lat = o.SquareLattice(Lx, Ly, periodic=per)
    H = o.tightbinding_hamiltonian(lat, field=o.LandauGauge(0.07), onsite=o.anderson_disorder(lat.N, 1.0, 3))
    X = o.random_kets(lat.N, 5, 2)
    bonds = o.nn_bonds(lat)
    src = np.array([bd.src for bd in bonds])
    dst = np.array([bd.dst for bd in bonds])
    J = o.bond_currents(H, X, src, dst)
    C = o.csc_currents(H, X)
    Hc = sp.csc_matrix(H)
    Hc.sort_indices()
    cols = np.repeat(np.arange(Hc.shape[1]), np.diff(Hc.indptr))
    entry = {(r, c): v for r, c, v in zip(Hc.indices, cols, C)}
    for s, t, j in zip(src - 1, dst - 1, J):
        if s == t:
            continue
        if (Lx == 2 and per[0]) or (Ly == 2 and per[1]):
            continue  # a 2-site ring adds both bonds into one entry
        assert abs(entry[(s, t)] - j) <= 1e-14 and abs(entry[(t, s)] + j) <= 1e-14
    assert all(v == 0.0 for (r, c), v in entry.items() if r == c)


def _loss(lat, psi0, V, B, target, dt, nsteps, spi, point):
    psi = np.asarray(psi0, dtype=np.complex128)
    for n in range(nsteps):
        H = o.tightbinding_hamiltonian(lat, 1.0, field=o.PointFlux(B[n // spi], point), onsite=V).toarray()
        w, U = np.linalg.eigh(H)
        psi = U @ (np.exp(-1j * dt * w)[:, None] * (U.conj().T @ psi))
    rho = (np.abs(psi) ** 2).sum(axis=1)
    return float(((rho - target) ** 2).sum())


def test_exact_loss_gradient_matches_finite_differences():
    """The adjoint tests' reference gradient (Frechet derivatives of the step exponentials)
    against central differences of the loss, evolved with an eigendecomposition."""
    lat = o.SquareLattice(3, 3)
    rng = np.random.default_rng(4)
    psi0 = o.random_kets(lat.N, 2, 5)
    psi0 /= np.linalg.norm(psi0, axis=0)
    V = rng.uniform(-0.5, 0.5, lat.N)
    B = np.array([0.15, 0.3])
    target = rng.uniform(0.0, 0.4, lat.N)
    dt, nsteps, spi, point = 0.3, 4, 2, (2.5, 2.5)
    loss, gV, gB = o.density_loss_gradient_exact(lat, psi0, V, B, target, dt, nsteps, spi, point)
    assert abs(loss - _loss(lat, psi0, V, B, target, dt, nsteps, spi, point)) <= 1e-13
    h = 1e-6
    for i in (0, 4, 8):
        e = np.zeros(lat.N)
        e[i] = h
        fd = (_loss(lat, psi0, V + e, B, target, dt, nsteps, spi, point)
              - _loss(lat, psi0, V - e, B, target, dt, nsteps, spi, point)) / (2 * h)
        assert abs(gV[i] - fd) <= 1e-7 * max(1.0, abs(fd))
    for k in range(len(B)):
        e = np.zeros(len(B))
        e[k] = h
        fd = (_loss(lat, psi0, V, B + e, target, dt, nsteps, spi, point)
              - _loss(lat, psi0, V, B - e, target, dt, nsteps, spi, point)) / (2 * h)
        assert abs(gB[k] - fd) <= 1e-7 * max(1.0, abs(fd))
