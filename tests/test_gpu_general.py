"""General sparse Hamiltonians (lm_ell_*): HoneycombLattice and the qwz model (two internal
states per site) built by the oracle, evolved on the device against the exact exponent."""
import numpy as np
import pytest

from oracle import lm_oracle as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lm():
    import lmgpu
    lmgpu.default_context()
    return lmgpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def models():
    V = o.anderson_disorder(2 * 7 * 6, 1.0, 21)
    Hh, coords = o.honeycomb_hamiltonian(7, 6, B=0.04, onsite=V)
    Hq = o.qwz_hamiltonian(6, 5, m=np.linspace(-1.5, 1.5, 30))
    return [("honeycomb", Hh, coords), ("qwz", Hq, None)]


@pytest.mark.parametrize("idx", [0, 1])
@pytest.mark.parametrize("precision", ["c64", "c32"])
def test_ket_steps_and_currents(lm, idx, precision):
    name, Ho, coords = models()[idx]
    N = Ho.shape[0]
    sites = lm.Sites(N, coords, name)
    H = lm.SparseHamiltonian(sites, Ho)
    X = o.random_kets(N, 5, 3)
    st = lm.KetBlock(sites, X, precision=precision)
    s = lm.ChebyshevGPU()
    dt = 0.15
    s.update_solver(H, dt)
    for _ in range(4):
        s.step(st)
    Y = X
    for _ in range(4):
        Y = o.expm_multiply(Ho, dt, Y)
    got = st.to_numpy().astype(np.complex128)
    assert rel(got, Y) <= (1e-10 if precision == "c64" else 2e-6)
    rho = lm.localdensity(st).values
    assert np.abs(rho - (np.abs(got) ** 2).sum(axis=1)).max() <= 1e-12 * rho.max()
    J = lm.entry_currents(H, st)
    Jref = o.csc_currents(Ho, got)
    assert np.abs(J - Jref).max() <= 1e-12 * np.abs(Jref).max()


@pytest.mark.parametrize("idx", [0, 1])
def test_density_matrix_step(lm, idx):
    name, Ho, coords = models()[idx]
    N = Ho.shape[0]
    sites = lm.Sites(N, coords, name)
    H = lm.SparseHamiltonian(sites, Ho)
    P0, _, _ = o.densitymatrix(Ho, mu=0.1)
    st = lm.DensityMatrix(sites, P0)
    s = lm.ChebyshevGPU()
    s.update_solver(H, 0.2)
    for _ in range(3):
        s.step(st)
    U = o.expm_exact(Ho, 0.2)
    P = P0
    for _ in range(3):
        P = U @ P @ U.conj().T
    assert rel(st.to_numpy(), P) <= 1e-10
    assert abs(st.trace() - np.trace(P0).real) <= 1e-11 * np.trace(P0).real
    J = lm.entry_currents(H, st)
    assert np.abs(J - o.csc_currents(Ho, P, is_density=True)).max() <= 1e-12


def test_time_dependent_values_through_evolution(lm):
    """H(t) on a fixed pattern (the Landau field ramps): Evolution with the left-endpoint H
    of every step against the oracle stepping the same matrices."""
    a, b = 5, 4
    N = 2 * a * b
    _, coords = o.honeycomb_hamiltonian(a, b)
    sites = lm.Sites(N, coords, "honeycomb")
    Bt = lambda t: 0.02 + 0.05 * t
    h = lambda t: lm.SparseHamiltonian(sites, o.honeycomb_hamiltonian(a, b, B=Bt(t))[0])
    X = o.random_kets(N, 3, 8)
    ev = lm.Evolution(lm.ChebyshevGPU(), h, lm.KetBlock(sites, X))
    times = [0.1 * k for k in range(1, 6)]
    Y = X
    t0 = 0.0
    for moment, t in zip(ev(times), times):
        Y = o.expm_multiply(o.honeycomb_hamiltonian(a, b, B=Bt(t0))[0], t - t0, Y)
        t0 = t
        assert rel(moment.state.to_numpy(), Y) <= 1e-10


def test_rejects_non_hermitian(lm):
    import scipy.sparse as sp
    M = sp.random(12, 12, density=0.3, random_state=1, format="csc") * (1 + 1j)
    with pytest.raises(lm.LMError):
        lm.SparseHamiltonian(lm.Sites(12), M).device()
