"""Readout kernels (localdensity, bond currents, column norms, trace) against numpy FP64 sums
of the same device data: c64 data to 1e-13, c32 data (double-float accumulation) to 1e-12."""
import numpy as np
import pytest

from oracle import lm_oracle as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lm():
    import lmgpu
    lmgpu.default_context()
    return lmgpu


CASES = [(16, 16, (True, True)), (7, 9, (False, False)), (33, 5, (True, False)), (2, 6, (True, True))]


@pytest.mark.parametrize("Lx,Ly,per", CASES)
@pytest.mark.parametrize("precision", ["c64", "c32"])
@pytest.mark.parametrize("weighted", [False, True])
def test_ket_block_readouts(lm, Lx, Ly, per, precision, weighted):
    ol = o.SquareLattice(Lx, Ly, periodic=per)
    b = {"axis1": per[0], "axis2": per[1]}
    ll = lm.SquareLattice(Lx, Ly, boundaries={k: v for k, v in b.items() if v})
    V = o.anderson_disorder(ol.N, 1.0, 5)
    Ho = o.tightbinding_hamiltonian(ol, field=o.LandauGauge(0.05), onsite=V)
    Hl = lm.tightbinding_hamiltonian(ll, V, field=lm.LandauGauge(0.05))
    M = 37
    X = o.random_kets(ol.N, M, 6)
    st = lm.KetBlock(ll, X, precision=precision)
    Xd = st.to_numpy().astype(np.complex128)  # exactly the device data
    w = np.random.default_rng(7).uniform(0.1, 2.0, M) if weighted else None
    if weighted:
        st.set_weights(w)
    ww = w if weighted else np.ones(M)
    rho = (np.abs(Xd) ** 2 * ww).sum(axis=1)
    tol = 1e-13 if precision == "c64" else 1e-12
    got = lm.localdensity(st).values
    assert np.abs(got - rho).max() <= tol * np.abs(rho).max()
    src, dst = zip(*[(bd.src, bd.dst) for bd in o.nn_bonds(ol)])
    J = o.bond_currents(Ho, Xd, np.asarray(src), np.asarray(dst), weights=ww)
    Jg = lm.DensityCurrents(Hl, st).bond_values()
    assert np.abs(Jg - J).max() <= tol * max(np.abs(J).max(), 1e-300) * 10
    nrm = np.linalg.norm(Xd, axis=0)
    assert np.abs(st.norms() - nrm).max() <= tol * nrm.max()


@pytest.mark.parametrize("precision", ["c64", "c32"])
def test_density_matrix_readouts(lm, precision):
    L = 9
    ol = o.SquareLattice(L, L)
    ll = lm.SquareLattice(L, L)
    Ho = o.tightbinding_hamiltonian(ol, field=o.PointFlux(0.2, (4.5, 4.5)))
    Hl = lm.tightbinding_hamiltonian(ll, field=lm.PointFlux(0.2, (4.5, 4.5)))
    P0, _, _ = o.densitymatrix(Ho, mu=0.0)
    st = lm.DensityMatrix(ll, P0, precision=precision)
    Pd = st.to_numpy().astype(np.complex128)
    assert np.array_equal(lm.localdensity(st).values, Pd.diagonal().real)
    src, dst = zip(*[(bd.src, bd.dst) for bd in o.nn_bonds(ol)])
    J = o.bond_currents(Ho, Pd, np.asarray(src), np.asarray(dst), is_density=True)
    assert np.abs(lm.DensityCurrents(Hl, st).bond_values() - J).max() <= 1e-14
    assert abs(st.trace() - Pd.diagonal().real.sum()) <= 1e-13


def test_subcurrents_and_currentsfrom_on_device_values(lm):
    """DensityCurrents of a device state: Currents(dc)[x .< y] == Currents(dc[x .< y]) against
    the oracle's materialised currents on the same subset, and currentsfrom /
    currentsfromto (test/test_currents.jl:11-62)."""
    L = 6
    ol = o.SquareLattice(L, L)
    ll = lm.SquareLattice(L, L)
    Ho = o.tightbinding_hamiltonian(ol, field=o.LandauGauge(0.1))
    Hl = lm.tightbinding_hamiltonian(ll, field=lm.LandauGauge(0.1))
    P0, _, _ = o.densitymatrix(o.tightbinding_hamiltonian(ol), mu=0.1)
    st = lm.DensityMatrix(ll, P0)
    dc = lm.DensityCurrents(Hl, st)
    ref = o.currents_matrix(Ho, P0, is_density=True).toarray()  # all pairs, |J| < 1e-10 dropped
    x, y = lm.coordvalues(ll)
    mask = x < y
    idx = np.nonzero(mask.values)[0]
    m1 = lm.Currents(dc)[mask]
    m2 = lm.Currents(dc[mask])
    assert np.abs(np.asarray(m1._matrix()) - ref[np.ix_(idx, idx)]).max() <= 1e-13
    assert np.abs(m2.toarray() - ref[np.ix_(idx, idx)]).max() <= 1e-13
    site = 8
    cf = lm.currentsfrom(dc, site).values
    want = ref[site - 1].copy()
    want[site - 1] = 0.0
    assert np.abs(cf - want).max() <= 1e-13
    assert abs(lm.currentsfromto(dc, site) - want.sum()) <= 1e-13


@pytest.mark.parametrize("M", [128, 300, 1000])
@pytest.mark.parametrize("weighted", [False, True])
def test_ket_sliced_density_readout(lm, M, weighted):
    """With 64 or more kets a small lattice's density readout splits the kets over a second grid
    axis (one wave of blocks) and adds the per-slice planes in slice order: the sum stays within
    1e-12 of numpy's FP64 sum of the device data and is bit-identical from call to call, and the
    ring readout gives the same bits."""
    lat = lm.SquareLattice(16, 16, boundaries={"axis1": True, "axis2": True})
    X = o.random_kets(lat.N, M, 9)
    st = lm.KetBlock(lat, X, precision="c32")
    Xd = st.to_numpy().astype(np.complex128)
    ww = np.ones(M)
    if weighted:
        ww = np.random.default_rng(3).uniform(0.1, 2.0, M)
        st.set_weights(ww)
    rho = (np.abs(Xd) ** 2 * ww).sum(axis=1)
    got = lm.localdensity(st).values
    assert np.abs(got - rho).max() <= 1e-12 * rho.max()
    assert np.array_equal(lm.localdensity(st).values, got)
    ring = lm.timesequence.ReadoutRing(lat.N, 2)
    _, vals = ring.wait(ring.push_density(st, 0.0))
    assert np.array_equal(vals, got)


@pytest.mark.parametrize("Lx,Ly,per", [(16, 16, (True, True)), (12, 8, (False, False)), (3, 4, (True, False)),
                                       (2, 12, (True, True))])
@pytest.mark.parametrize("M", [300, 1000])
@pytest.mark.parametrize("weighted", [False, True])
def test_sliced_vector_currents_readout(lm, Lx, Ly, per, M, weighted):
    """c32 bond currents with Ly % 4 == 0 take the kernel with four sites per lane, and with
    64 or more kets the kets split into slices added in slice order: within 1e-12 of numpy's
    FP64 sums of the same device data (open, periodic and 2-site periodic axes), the same bits
    from call to call and through the ring."""
    ol = o.SquareLattice(Lx, Ly, periodic=per)
    b = {"axis1": per[0], "axis2": per[1]}
    ll = lm.SquareLattice(Lx, Ly, boundaries={k: v for k, v in b.items() if v})
    V = o.anderson_disorder(ol.N, 1.0, 5)
    Ho = o.tightbinding_hamiltonian(ol, field=o.LandauGauge(0.05), onsite=V)
    Hl = lm.tightbinding_hamiltonian(ll, V, field=lm.LandauGauge(0.05))
    st = lm.KetBlock(ll, o.random_kets(ol.N, M, 6), precision="c32")
    Xd = st.to_numpy().astype(np.complex128)
    ww = np.ones(M)
    if weighted:
        ww = np.random.default_rng(7).uniform(0.1, 2.0, M)
        st.set_weights(ww)
    src, dst = zip(*[(bd.src, bd.dst) for bd in o.nn_bonds(ol)])
    J = o.bond_currents(Ho, Xd, np.asarray(src), np.asarray(dst), weights=ww)
    Jg = lm.DensityCurrents(Hl, st).bond_values()
    assert np.abs(Jg - J).max() <= 1e-11 * max(np.abs(J).max(), 1e-300)
    assert np.array_equal(lm.DensityCurrents(Hl, st).bond_values(), Jg)
    ring = lm.timesequence.ReadoutRing(len(Jg), 2)
    _, vals = ring.wait(ring.push_currents(Hl, st, 0.0))
    assert np.array_equal(vals, Jg)
