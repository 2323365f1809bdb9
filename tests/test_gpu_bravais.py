"""Bravais lattices on the device: H(t) of HoneycombLattice, KagomeLattice and
TriangularLattice assembled by the library from the bond geometry (lm_ell_create_bonds,
lm_ell_assemble) and evolved, read out and diagonalised through the general sparse path,
against the oracle's hard-coded restatements (src/zoo/lattices.jl:136-211)."""
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


CASES = [("HoneycombLattice", 6, 5), ("KagomeLattice", 5, 4), ("TriangularLattice", 7, 5)]
ORACLE = {"HoneycombLattice": o.honeycomb_hamiltonian, "KagomeLattice": o.kagome_hamiltonian,
          "TriangularLattice": o.triangular_hamiltonian}


def fields(lm, kind):
    if kind == "landau":
        return o.LandauGauge(0.04), lm.LandauGauge(0.04)
    return o.PointFlux(0.25, (2.6, 1.9)), lm.PointFlux(0.25, (2.6, 1.9))


@pytest.mark.parametrize("name,a,b", CASES)
@pytest.mark.parametrize("kind", ["landau", "pointflux"])
@pytest.mark.parametrize("precision", ["c64", "c32"])
def test_ket_evolution_and_currents(lm, name, a, b, kind, precision):
    lat = lm.BravaisLattice(name, a, b)
    of, lf = fields(lm, kind)
    V = o.anderson_disorder(lat.N, 1.0, 7)
    Ho, _ = ORACLE[name](a, b, field=of, onsite=V)
    H = lm.tightbinding_hamiltonian(lat, V, field=lf)
    X = o.random_kets(lat.N, 4, 5)
    st = lm.KetBlock(lat, X, precision=precision)
    s = lm.ChebyshevGPU()
    s.update_solver(H, 0.1)
    for _ in range(4):
        s.step(st)
    Y = o.expm_multiply(Ho, 0.4, X)
    got = st.to_numpy().astype(np.complex128)
    assert rel(got, Y) <= (1e-10 if precision == "c64" else 2e-6)
    # DensityCurrents(H, P)[i, j] per site pair, and in the lattice's bond order
    curr = lm.DensityCurrents(H, st)
    src, dst, v = curr.site_pairs()
    Pref = o.csc_currents(Ho, got)
    ref = {}
    Hc = Ho.tocsc()
    cols = np.repeat(np.arange(lat.N), np.diff(Hc.indptr))
    for r, c, x in zip(Hc.indices, cols, Pref):
        if r != c:
            ref[(r + 1, c + 1)] = ref.get((r + 1, c + 1), 0.0) + x
    tol = 1e-12 if precision == "c64" else 1e-6
    scale = max(abs(x) for x in ref.values())
    for i, j, x in zip(src, dst, v):
        assert abs(x - ref[(int(i), int(j))]) <= tol * scale
    bsrc, bdst, _, _ = lat.bonds()
    bv = curr.entry_values()[H.bond_entries()]
    for i, j, x in zip(bsrc, bdst, bv):
        assert abs(x - ref[(int(i), int(j))]) <= tol * scale


@pytest.mark.parametrize("name,a,b", CASES)
def test_time_dependent_field_assembled_on_device(lm, name, a, b):
    """h(t) = tightbinding_hamiltonian(lat, V; field = PointFlux(B(t), p)): every step the
    library re-assembles H from the bonds on the device; Evolution with the left-endpoint H of
    every step against the oracle stepping the same matrices."""
    lat = lm.BravaisLattice(name, a, b)
    V = o.anderson_disorder(lat.N, 0.8, 3)
    Bt = lambda t: 0.05 + 0.3 * t
    p = (2.6, 1.9)
    h = lambda t: lm.tightbinding_hamiltonian(lat, V, field=lm.PointFlux(Bt(t), p))
    X = o.random_kets(lat.N, 3, 8)
    ev = lm.Evolution(lm.ChebyshevGPU(), h, lm.KetBlock(lat, X))
    times = [0.1 * k for k in range(1, 7)]
    Y, t0 = X, 0.0
    for moment, t in zip(ev(times), times):
        Ho, _ = ORACLE[name](a, b, field=o.PointFlux(Bt(t0), p), onsite=V)
        Y = o.expm_multiply(Ho, t - t0, Y)
        t0 = t
        assert rel(moment.state.to_numpy(), Y) <= 1e-10


def test_periodic_twisted_honeycomb(lm):
    per, tw = (True, True), (0.3, -0.7)
    lat = lm.HoneycombLattice(6, 4, boundaries={"axis1": tw[0], "axis2": tw[1]})
    V = o.anderson_disorder(lat.N, 1.0, 9)
    Ho, _ = o.honeycomb_hamiltonian_periodic(6, 4, per, tw, field=o.LandauGauge(0.03), onsite=V)
    H = lm.tightbinding_hamiltonian(lat, V, field=lm.LandauGauge(0.03))
    X = o.random_kets(lat.N, 3, 4)
    st = lm.KetBlock(lat, X)
    s = lm.ChebyshevGPU()
    s.update_solver(H, 0.15)
    for _ in range(3):
        s.step(st)
    assert rel(st.to_numpy(), o.expm_multiply(Ho, 0.45, X)) <= 1e-10
    eig = lm.diagonalize(H)
    w = np.linalg.eigvalsh(Ho.toarray())
    assert np.abs(eig.values - w).max() <= 1e-13 * max(1.0, np.abs(w).max())


def test_densitymatrix_on_kagome(lm):
    """densitymatrix(h; mu) at T = 0 of a kagome Hamiltonian (flat band at E = 2 t1 away from
    mu): the device eigensystem against the oracle's LAPACK projector."""
    lat = lm.KagomeLattice(5, 4)
    of, lf = fields(lm, "pointflux")
    Ho, _ = o.kagome_hamiltonian(5, 4, field=of)
    H = lm.tightbinding_hamiltonian(lat, field=lf)
    w = np.linalg.eigvalsh(Ho.toarray())
    Pref, _, _ = o.densitymatrix(Ho, mu=0.3, degenerate_tol=1e-12 * max(1.0, np.abs(w).max()))
    P = lm.densitymatrix(H, mu=0.3).to_numpy()
    assert rel(P, Pref) <= 1e-10
