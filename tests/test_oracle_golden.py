"""Pins the CPU oracle against the known-answer values held by LatticeModels.jl's own tests and
doctests (the reference is Julia and cannot run here).  CPU only."""
import math

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import lm_oracle as o


# --- site order (src/core/latticevalue.jl:66-81 doctest) ---------------------------------
def test_site_order_doctest():
    l3 = o.SquareLattice(3, 3)
    assert [p[1] for p in l3.pointers] == [1, 2, 3, 1, 2, 3, 1, 2, 3]
    l2 = o.SquareLattice(2, 2)
    assert [p[0] for p in l2.pointers] == [1, 1, 2, 2]
    assert l3.site_index(2, 3) == 6


# --- nnz counts (src/spectrum.jl:96, src/operators/builder.jl:213 doctests) ---------------
def test_nnz_doctests():
    assert o.tightbinding_hamiltonian(o.SquareLattice(4, 4)).nnz == 48
    assert o.tightbinding_hamiltonian(o.SquareLattice(5, 5), field=o.LandauGauge(0.1)).nnz == 80


# --- 4x4 spectrum (src/spectrum.jl:102-105 doctest) ---------------------------------------
def test_spectrum_4x4_doctest():
    w = np.linalg.eigvalsh(o.tightbinding_hamiltonian(o.SquareLattice(4, 4)).toarray())
    assert round(w[0], 5) == -3.23607 and round(w[-1], 5) == 3.23607


# --- line integrals (test/test_field.jl:23-38) ---------------------------------------------
def test_line_integrals():
    p1, p2 = (1.0, 2.0), (3.0, 4.0)
    la = o.LandauGauge(0.1)
    assert math.isclose(la.line_integral(p1, p2), o.line_integral_trapezoid(la, p1, p2, 100), rel_tol=1e-12)
    sym = o.SymmetricGauge(0.1)
    assert math.isclose(sym.line_integral(p1, p2), o.line_integral_trapezoid(sym, p1, p2, 1), rel_tol=1e-12)
    assert math.isclose(sym.line_integral(p1, p2), o.line_integral_trapezoid(sym, p1, p2, 100), rel_tol=1e-12)
    flx = o.PointFlux(0.1)
    assert abs(o.line_integral_trapezoid(flx, p1, p2, 1000) - flx.line_integral(p1, p2)) < 1e-8
    tot = o.FieldSum((flx, sym))
    num = o.line_integral_trapezoid(flx, p1, p2, 1000) + o.line_integral_trapezoid(sym, p1, p2, 1000)
    assert abs(num - tot.line_integral(p1, p2)) < 1e-8


# --- point fluxes (test/test_field.jl:43-66) ------------------------------------------------
def test_point_fluxes():
    p1, p2 = (0.0, 0.0), (4.0, 0.0)
    pf1 = o.PointFlux(0.1, (1, 2))
    pf2 = o.PointFlux(0.1, (3, 4))
    ps1 = o.PointFluxes([0.1, 0.1], [(1, 2), (3, 4)], "singular")
    ps3 = o.PointFluxes([0.1, 0.1], [(1, 2), (3, 4)])
    assert abs(o.FieldSum((pf1, pf2)).line_integral(p1, p2) - ps3.line_integral(p1, p2)) < 1e-8
    assert abs(ps1.line_integral(p1, p2) - 0.2) < 1e-8


# --- flux replication counts (test/test_field.jl:80-97) -------------------------------------
def test_flux_replication_counts():
    lnb = o.SquareLattice(5, 5)
    lwb = o.SquareLattice(5, 5, periodic=(True, True))
    flx = o.PointFlux(0.1, (0.5, 0.5), "singular")
    flxs = o.periodic_fluxes(lnb, flx)
    assert flxs.points == o.periodic_fluxes(lwb, flx).points
    assert isinstance(o.adapt_field(flx, lnb), o.PointFlux)
    assert len(o.adapt_field(flxs, lnb).points) == 25
    assert len(o.adapt_field(flx, lwb).points) == 9
    assert len(o.adapt_field(flxs, lwb).points) == 9 * 25


# --- field application (test/test_field.jl:99-109) ------------------------------------------
def test_apply_field_equivalence():
    l = o.SquareLattice(10, 10)
    H1 = o.tightbinding_hamiltonian(l, field=o.LandauGauge(0.1)).toarray()
    H3 = o.tightbinding_hamiltonian(l).toarray()
    c = l.coords
    for i in range(l.N):  # apply_field! (src/operators/latticeutils.jl:101-110)
        for j in range(l.N):
            if H3[i, j] != 0:
                H3[i, j] *= np.exp(-2j * np.pi * o.LandauGauge(0.1).line_integral(c[i], c[j]))
    assert np.allclose(H1, H3, atol=1e-14)


# --- gauge invariance (test/test_operators.jl:211-213, TB instead of QWZ) -------------------
def test_gauge_invariance_spectrum():
    l = o.SquareLattice(5, 5)
    d1 = np.linalg.eigvalsh(o.tightbinding_hamiltonian(l, field=o.PointFlux(0.1, (3.5, 3.5))).toarray())
    d2 = np.linalg.eigvalsh(o.tightbinding_hamiltonian(l, field=o.PointFlux(0.1, (3.5, 3.5), "singular")).toarray())
    assert np.allclose(d1, d2, atol=1e-12)


# --- currents identities (test/test_currents.jl:11-32; TB instead of QWZ) --------------------
def _currents_setup():
    l = o.SquareLattice(4, 4)
    H0 = o.tightbinding_hamiltonian(l)
    H1 = o.tightbinding_hamiltonian(l, field=o.LandauGauge(0.1)).toarray()
    P, w, V = o.densitymatrix(H0, mu=0.0)
    return l, H1, P, V


def test_currents_antisymmetry_and_heisenberg():
    l, H1, P, V = _currents_setup()
    s1, s2 = 5, 10  # l[6], l[11] (0-based)
    dc = lambda i, j: o.density_current(H1, P, i, j)
    assert dc(s1, s2) == -dc(s2, s1)
    assert abs(dc(s1, s1)) <= np.finfo(float).eps
    nbrs = [s1 + 4, s1 + 1, s1 - 4, s1 - 1]  # +x, +y, -x, -y
    n_s = np.zeros((l.N, l.N)); n_s[s1, s1] = 1
    dens_dt = np.trace(1j * (H1 @ n_s - n_s @ H1) @ P)
    assert abs(sum(dc(s1, t) for t in nbrs) - dens_dt) < 1e-12
    assert abs(sum(dc(s1, t) for t in range(l.N) if t != s1) - dens_dt) < 1e-12


def test_currents_ket_vs_projector():
    l, H1, P, V = _currents_setup()
    gs = V[:, 0]
    src = np.arange(1, l.N + 1).repeat(l.N); dst = np.tile(np.arange(1, l.N + 1), l.N)
    m = src != dst
    c1 = o.bond_currents(H1, gs, src[m], dst[m])
    c2 = o.bond_currents(H1, np.outer(gs, gs.conj()), src[m], dst[m], is_density=True)
    assert np.allclose(c1, c2, atol=1e-14)


# --- von Neumann identity (test/test_operators.jl:35-42) -------------------------------------
def test_von_neumann_identity():
    l = o.SquareLattice(10, 10)
    H1 = o.tightbinding_hamiltonian(l, field=o.LandauGauge(0.1)).toarray()
    P, _, _ = o.densitymatrix(o.tightbinding_hamiltonian(l), mu=0.0)
    site = 10
    n_s = np.zeros((l.N, l.N)); n_s[site, site] = 1
    dens_dt = np.trace(1j * (H1 @ n_s - n_s @ H1) @ P)
    dts = o.localdensity(-1j * (H1 @ P - P @ H1))
    assert abs(dens_dt - dts[site]) < 1e-12


# --- densitymatrix (test/test_operators.jl:226-236) -------------------------------------------
def test_densitymatrix_groundstate_and_trace():
    l = o.SquareLattice(5, 5)
    H = o.tightbinding_hamiltonian(l)
    w, V = o.diagonalize(H)
    P, _, _ = o.densitymatrix(H, mu=w[0] + 1e-9)  # only the ground state occupied
    assert np.allclose(P, np.outer(V[:, 0], V[:, 0].conj()), atol=1e-12)
    P0, w0, _ = o.densitymatrix(H, mu=0.0)
    assert abs(np.trace(P0).real - np.sum(w0 <= 0)) < 1e-10


# --- evolution vs exact exponent (test/test_timedeps.jl:42-68) ---
def test_evolution_matches_exact_exponent():
    l = o.SquareLattice(10, 10)
    Hs = o.tightbinding_hamiltonian(l, field=o.LandauGauge(0.1))
    Hd = Hs.toarray()
    w, V = np.linalg.eigh(Hd)
    psi = V[:, 0]
    ts = np.round(np.arange(0, 10.0 + 1e-9, 0.1), 10)
    U = o.expm_exact(Hd, 0.1)
    correct, p = [], psi.copy()
    for _ in ts:
        correct.append(p[1]); p = U @ p
    val1 = [st[1] for _, st, _ in o.evolve(lambda t: Hs, psi, ts, o.OracleCachedExpSolver(threshold=1e-12))]
    from oracle import krylov
    csr = krylov.CSR(Hs)
    kv, p = [], psi.copy()
    for i, t in enumerate(ts):
        if i > 0:
            p = krylov.krylov_expv_block(csr, 0.1, p)[:, 0]
        kv.append(p[1])
    assert np.allclose(val1, correct, atol=1e-10)
    assert np.allclose(kv, correct, atol=1e-10)


def test_timedeps_evolution_qwz():
    """The reference's own evolution test, restated exactly (test/test_timedeps.jl:42-68):
    qwz(SquareLattice(10, 10)) (two internal states per site), psi = groundstate(dense H),
    ts = 0:0.1:10; psi.data[2] (1-based: site 1, second internal state) of KrylovKitExp and of
    CachedExp(threshold = 1e-12) against exp(-i 0.1 H) applied step by step, atol 1e-10."""
    Hs = o.qwz_hamiltonian(10, 10)
    Hd = Hs.toarray()
    w, V = np.linalg.eigh(Hd)
    psi = V[:, 0]
    ts = np.round(np.arange(0, 10.0 + 1e-9, 0.1), 10)
    correct_ev = o.expm_exact(Hd, 0.1)
    correct, p = [], psi.copy()
    for _ in ts:
        correct.append(p[1])
        p = correct_ev @ p
    from oracle import krylov
    csr = krylov.CSR(Hs)
    val1, p = [], psi.copy()
    for i, _ in enumerate(ts):
        if i > 0:
            p = krylov.krylov_expv_block(csr, 0.1, p)[:, 0]
        val1.append(p[1])
    val2 = [st[1] for _, st, _ in o.evolve(lambda t: Hs, psi, ts, o.OracleCachedExpSolver(threshold=1e-12))]
    assert len(val1) == len(val2) == len(correct) == 101
    # Julia's `a ≈ b atol=1e-10` on vectors is norm(a - b) <= 1e-10 (rtol is 0 once atol is set)
    assert np.linalg.norm(np.array(val1) - correct) <= 1e-10
    assert np.linalg.norm(np.array(val2) - correct) <= 1e-10


def test_evolution_iterator_semantics():
    """First moment has dt = 0 and returns the initial state; H is the left endpoint."""
    l = o.SquareLattice(3, 3)
    seen = []
    def h(t):
        seen.append(t)
        return o.tightbinding_hamiltonian(l, field=o.LandauGauge(0.1 * t))
    psi = np.zeros(l.N, complex); psi[0] = 1
    moments = list(o.evolve(h, psi, [0.0, 0.5, 1.0], o.OracleCachedExpSolver(exact=True)))
    assert np.array_equal(moments[0][1], psi)
    assert seen == [0.0, 0.0, 0.5]
    assert [m[2] for m in moments] == [0.0, 0.5, 1.0]
    with pytest.raises(ValueError):
        list(o.evolve(h, psi, [0.0, -0.5], o.OracleCachedExpSolver(exact=True)))


def test_cachedexp_default_threshold_gap():
    """The reference's default exponent stops at max|term| <= 1e-10; it is not exact."""
    l = o.SquareLattice(10, 10)
    H = o.tightbinding_hamiltonian(l, field=o.PointFlux(0.2, (5.5, 5.5)))
    U = o.expm_exact(H, 0.1)
    P10 = o.cachedexp(H, 0.1)
    P14 = o.cachedexp(H, 0.1, threshold=1e-14)
    assert abs(P14 - U).max() < 1e-13
    assert 1e-14 < abs(P10 - U).max() < 1e-9


def test_pbc_bond_routing_and_twist():
    l = o.SquareLattice(3, 4, periodic=(True, True), twist=(0.0, 0.7))
    b = o.nn_bonds(l)
    assert len(b) == 2 * l.N
    wrapped_y = [x for x in b if x.r2[1] > 4]
    assert all(abs(x.factor - np.exp(0.7j)) < 1e-15 for x in wrapped_y)
    assert all(x.factor == 1 for x in b if x.r2[1] <= 4)
    H = o.tightbinding_hamiltonian(l, field=o.LandauGauge(0.05))
    assert abs(H - H.conj().T).max() == 0
