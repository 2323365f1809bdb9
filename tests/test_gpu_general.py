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


SZ = np.array([[1, 0], [0, -1]])
OPS = [None, SZ, np.array([[1, 0], [0, 0]]), np.array([[0.3, 1 - 2j], [1 + 2j, -0.5]])]


def qwz_setup(lm):
    """qwz(SquareLattice(4, 4), field=LandauGauge(0.1)) with the field-free ground state
    (test/test_currents.jl:1-9)."""
    H0 = o.qwz_hamiltonian(4, 4).toarray()
    H1 = o.qwz_hamiltonian(4, 4, field=o.LandauGauge(0.1))
    gs = np.linalg.eigh(H0)[1][:, 0]
    sites = lm.Sites(32, None, "qwz", internal=2)
    return H1, gs, sites, lm.SparseHamiltonian(sites, H1)


@pytest.mark.parametrize("kind", ["ket", "density"])
@pytest.mark.parametrize("precision", ["c64", "c32"])
def test_local_operator_currents(lm, kind, precision):
    H1, gs, sites, H = qwz_setup(lm)
    if kind == "ket":
        st = lm.KetBlock(sites, gs[:, None], precision=precision)
        ref_state, kw = gs, {}
    else:
        P = np.outer(gs, gs.conj())
        st = lm.DensityMatrix(sites, P, precision=precision)
        ref_state, kw = P, {"is_density": True}
    tol = 1e-13 if precision == "c64" else 1e-6
    for op in OPS:
        curr = lm.LocalOperatorCurrents(H, st, op) if op is not None else lm.DensityCurrents(H, st)
        ent = curr.entry_values()
        ref = o.entry_op_currents(H1, ref_state, 2, op, **kw)
        assert np.abs(ent - ref).max() <= tol * max(np.abs(ref).max(), 1e-3)
        M = lm.Currents(curr).currents
        Mref = o.site_currents_matrix(H1, ref_state, 2, op, **kw)
        assert abs(M - Mref).max() <= tol * max(abs(Mref).max(), 1e-3)
        src, dst, v = curr.site_pairs()
        pairs = o.site_currents(H1, ref_state, 2, op, **kw)
        for a, b, x in zip(src, dst, v):
            assert abs(x - pairs[(a - 1, b - 1)]) <= tol * max(np.abs(v).max(), 1e-3)
            assert curr[a, b] == x
    # test/test_currents.jl:88-93 through the device: Heisenberg identity at l[6]
    spin = lm.Currents(lm.LocalOperatorCurrents(H, st, SZ))
    Hd = H1.toarray()
    S = np.zeros_like(Hd)
    S[10:12, 10:12] = SZ
    dt = (gs.conj() @ (1j * (Hd @ S - S @ Hd)) @ gs).real
    assert abs(lm.currentsfromto(spin, 6) - dt) <= (1e-12 if precision == "c64" else 1e-6)


def test_internal_density_and_evolved_currents(lm):
    """An evolved weighted ket block: localdensity sums the internal states of a site
    (src/operators/latticeutils.jl:44), the spin currents follow the state."""
    H1, gs, sites, H = qwz_setup(lm)
    X = o.random_kets(32, 4, 9)
    w = np.array([0.1, 0.2, 0.3, 0.4])
    st = lm.KetBlock(sites, X, weights=w)
    s = lm.ChebyshevGPU()
    s.update_solver(H, 0.1)
    for _ in range(5):
        s.step(st)
    Y = X
    for _ in range(5):
        Y = o.expm_multiply(H1, 0.1, Y)
    rho = lm.localdensity(st).values
    assert rho.shape == (16,)
    ref = o.localdensity(Y, w).reshape(16, 2).sum(axis=1)
    assert np.abs(rho - ref).max() <= 1e-11
    ent = lm.LocalOperatorCurrents(H, st, SZ).entry_values()
    # the readout is exact in FP64; the 5 propagator steps (1e-12 each) set the tolerance
    assert np.abs(ent - o.entry_op_currents(H1, st.to_numpy(), 2, SZ, weights=w)).max() <= 1e-14
    ref = o.entry_op_currents(H1, Y, 2, SZ, weights=w)
    assert np.abs(ent - ref).max() <= 1e-11 * np.abs(ref).max()


def test_timesequence_ring_general(lm):
    """TimeSequence(moment_currents / moment_density) over a general Hamiltonian: the ring
    holds the per-entry currents and the site densities, equal to the synchronous calls."""
    H1, gs, sites, H = qwz_setup(lm)
    X = o.random_kets(32, 3, 2)
    times = [0.1 * k for k in range(1, 12)]
    ev = lambda: lm.Evolution(lm.ChebyshevGPU(), lambda t: H, lm.KetBlock(sites, X))
    tc = lm.TimeSequence(lm.moment_currents, ev()(times))
    td = lm.TimeSequence(lm.moment_density, ev()(times))
    sync_c, sync_d = [], []
    for m in ev()(times):
        sync_c.append(lm.DensityCurrents(m.H, m.state).entry_values().copy())
        sync_d.append(lm.localdensity(m.state).values)
    assert len(tc) == len(sync_c) == len(td)
    for (t, v), ref in zip(tc, sync_c):
        assert np.array_equal(v, ref)
    for (t, v), ref in zip(td, sync_d):
        assert np.array_equal(v.values, ref)


def test_local_operator_rejects(lm):
    H1, gs, sites, H = qwz_setup(lm)
    st = lm.KetBlock(sites, gs[:, None])
    with pytest.raises(ValueError):
        lm.LocalOperatorCurrents(H, st, np.eye(3))
    Hh, coords = o.honeycomb_hamiltonian(3, 3)
    hs = lm.Sites(18, coords, "honeycomb")
    with pytest.raises(ValueError):
        lm.LocalOperatorCurrents(lm.SparseHamiltonian(hs, Hh), lm.KetBlock(hs, o.random_kets(18, 1, 0)), np.eye(1))


@pytest.mark.parametrize("timedomain", [False, True])
def test_timedeps_evolution_qwz(lm, timedomain):
    """The reference's own evolution test through the device (test/test_timedeps.jl:42-68):
    qwz(SquareLattice(10, 10)) with two internal states per site, psi = the ground state of the
    dense H, ts = 0:0.1:10 through Evolution(ChebyshevGPU, H, psi); psi.data[2] (1-based: site
    1, second internal state) of every moment against exp(-i 0.1 H) applied step by step, with
    the reference's bar: Julia's `≈ atol=1e-10` on the vector of values, i.e. norm <= 1e-10."""
    Hs = o.qwz_hamiltonian(10, 10)
    Hd = Hs.toarray()
    psi = np.linalg.eigh(Hd)[1][:, 0]
    ts = [round(0.1 * k, 10) for k in range(101)]
    correct_ev = o.expm_exact(Hd, 0.1)
    correct, p = [], psi.copy()
    for _ in ts:
        correct.append(p[1])
        p = correct_ev @ p
    sites = lm.Sites(200, None, "qwz", internal=2)
    H = lm.SparseHamiltonian(sites, Hs)
    if timedomain:  # `for st in Evolution(solver, Hs, psi, timedomain=ts)`
        ev = lm.Evolution(lm.ChebyshevGPU(), H, lm.Ket(sites, psi), timedomain=ts)
        vals = [m.state.to_numpy()[1, 0] for m in ev]
    else:           # `for state in Evolution(solver, Hs, psi)(ts)`
        ev = lm.Evolution(lm.ChebyshevGPU(), H, lm.Ket(sites, psi))
        vals = [m[0].to_numpy()[1, 0] for m in ev(ts)]
    assert len(vals) == 101
    assert np.linalg.norm(np.array(vals) - np.array(correct)) <= 1e-10
