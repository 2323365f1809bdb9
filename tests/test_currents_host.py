"""Host logic of the currents surface (src/currents.jl): materialised Currents, SubCurrents,
iteration, currentsfrom / currentsfromto and arithmetic, restating the reference's "Basics",
"materialized" and "Subcurrents" testsets (test/test_currents.jl:11-62) on currents the
oracle computes.  No GPU: the values enter through Currents' matrix constructor."""
import warnings

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import lm_oracle as o


@pytest.fixture(scope="module")
def lm():
    import lmgpu
    return lmgpu


@pytest.fixture(scope="module")
def case(lm):
    """SquareLattice(4, 4), density currents of the field-free ground-state projector under a
    Landau field (the reference's setup uses qwz; this is the scalar lattice)."""
    ol = o.SquareLattice(4, 4)
    H0 = o.tightbinding_hamiltonian(ol).toarray()
    H1 = o.tightbinding_hamiltonian(ol, field=o.LandauGauge(0.1)).toarray()
    w, v = np.linalg.eigh(H0)
    P = v[:, :7] @ v[:, :7].conj().T
    M = np.array([[0.0 if i == j else o.density_current(H1, P, i, j) for j in range(16)] for i in range(16)])
    lat = lm.SquareLattice(4, 4)
    return lat, H1, P, M


def full(lm, lat, M):
    return lm.Currents._from_matrix(lat, sp.csc_matrix(M))


def test_iteration_and_length(lm, case):
    lat, H1, P, M = case
    c = full(lm, lat, M)
    n = 0
    for (a, b), v in c:
        assert v == pytest.approx(c[a, b])
        assert v >= 0
        n += 1
    assert n == len(c) == 16 * 15 // 2


def test_materialised_set_and_arithmetic(lm, case):
    l2 = lm.SquareLattice(1, 2)
    m = lm.Currents(l2)
    m[1, 2] = 2
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        m[1, 1] = 1
    assert any("site to self" in str(x.message) for x in w)
    assert np.array_equal(m.toarray(), [[0, 2], [-2, 0]])
    lat, H1, P, M = case
    mc = full(lm, lat, M)
    assert (mc + mc).isapprox(2 * mc + mc.zero())
    assert np.abs((mc - mc).toarray()).max() == 0
    assert np.allclose((mc / 4).toarray(), M / 4)


def test_subcurrents(lm, case):
    """Currents(dc)[x .< y] == Currents(dc[x .< y]) (test/test_currents.jl:54-62)."""
    lat, H1, P, M = case
    x, y = lm.coordvalues(lat)
    mask = x < y
    dc = full(lm, lat, M)
    m1 = dc[mask]
    m2 = lm.Currents(dc[mask])
    idx = np.nonzero(mask.values)[0]
    sub = M[np.ix_(idx, idx)]
    assert np.allclose(np.asarray(m1._matrix()), sub)
    ref = np.where(np.abs(sub) >= 1e-10, sub, 0.0)
    assert np.allclose(m2.toarray(), np.tril(ref, -1) - np.tril(ref, -1).T)
    assert m2.isapprox(m1)
    assert m1[1, 2] == pytest.approx(M[idx[0], idx[1]])


def test_currentsfrom_and_fromto(lm, case):
    lat, H1, P, M = case
    dc = full(lm, lat, M)
    site = 6
    cf = lm.currentsfrom(dc, site).values
    ref = M[site - 1].copy()
    ref[site - 1] = 0
    assert np.allclose(cf, ref)
    assert lm.currentsfromto(dc, site) == pytest.approx(ref.sum())
    # Heisenberg identity for the density at site 6 (test/test_currents.jl:22-26):
    # currentsfromto(dc, site) = d rho_site / dt = <i [H, n_site]>
    n = np.zeros((16, 16))
    n[site - 1, site - 1] = 1
    dt = np.trace(P @ (1j * (H1 @ n - n @ H1))).real
    assert lm.currentsfromto(dc, site) == pytest.approx(dt, abs=1e-12)
    x, y = lm.coordvalues(lat)
    assert lm.currentsfromto(dc, x < y, x >= y) == pytest.approx(M[np.ix_(np.nonzero((x < y).values)[0],
                                                                         np.nonzero((x >= y).values)[0])].sum())
