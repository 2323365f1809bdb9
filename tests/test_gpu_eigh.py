"""The device eigensystem (lm_eigsys_*): diagonalize and densitymatrix on the library's own
FP64 kernels, against the oracle's LAPACK eigensystem (src/spectrum.jl:48-55, :226-257).

Bars: eigenvalues within 1e-13 |H|, residuals |H v - E v| and orthonormality within 1e-12;
the T = 0 projector within 1e-10 (relative Frobenius) of the oracle's, with "E == mu" read as
|E - mu| <= 1e-12 max(1, |E|max) on both sides, so that a level exactly degenerate at mu is
occupied as a whole (the reference's exact test splits it by the eigensolver's rounding).
"""
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


def square_case(lm, Lx, Ly, per=(False, False), tw=(0.0, 0.0), field=None, W=0.0, seed=0):
    ol = o.SquareLattice(Lx, Ly, periodic=per, twist=tw)
    b = {}
    for ax, name in enumerate(("axis1", "axis2")):
        if per[ax]:
            b[name] = float(tw[ax]) if tw[ax] else True
    ll = lm.SquareLattice(Lx, Ly, boundaries=b)
    V = o.anderson_disorder(ol.N, W, seed) if W else None
    of = lf = None
    if field is not None:
        kind, amp = field
        if kind == "landau":
            of, lf = o.LandauGauge(amp), lm.LandauGauge(amp)
        else:
            pt = ((Lx + 1) / 2.0, (Ly + 1) / 2.0)
            of, lf = o.PointFlux(amp, pt), lm.PointFlux(amp, pt)
    Ho = o.tightbinding_hamiltonian(ol, field=of, onsite=V)
    Hl = lm.tightbinding_hamiltonian(ll, *([V] if V is not None else []), field=lf)
    return Ho, Hl


CASES = {
    "10x10-open-degenerate": dict(Lx=10, Ly=10),
    "8x8-pointflux-disorder": dict(Lx=8, Ly=8, field=("pf", 0.2), W=2.0, seed=3),
    "2x3-periodic-twisted": dict(Lx=2, Ly=3, per=(True, True), tw=(0.3, 0.0), field=("landau", 0.1)),
    "2x2-periodic-double-bonds": dict(Lx=2, Ly=2, per=(True, True), field=("landau", 0.05)),
    "1x5-chain": dict(Lx=1, Ly=5, W=1.0, seed=1),
    "1x1": dict(Lx=1, Ly=1, W=1.0, seed=2),
    "17x13-periodic-landau-disorder": dict(Lx=17, Ly=13, per=(True, True), field=("landau", 0.03), W=1.0, seed=4),
}


@pytest.mark.parametrize("name", list(CASES))
def test_eigensystem_square(lm, name):
    Ho, Hl = square_case(lm, **CASES[name])
    Hd = Ho.toarray()
    wref = np.linalg.eigvalsh(Hd)
    eig = lm.diagonalize(Hl)
    hn = max(1.0, np.abs(wref).max())
    assert np.abs(eig.values - wref).max() <= 1e-13 * hn
    V = eig.vectors().to_numpy()
    n = len(wref)
    assert np.linalg.norm(Hd @ V - V * eig.values) <= 1e-12 * hn * np.sqrt(n)
    assert np.abs(V.conj().T @ V - np.eye(n)).max() <= 1e-12
    # a sub-range in ComplexF32 holds the same vectors rounded
    if n >= 4:
        V32 = eig.vectors(1, 2, precision="c32").to_numpy()
        assert np.abs(V32 - V[:, 1:3]).max() <= 1e-7


@pytest.mark.parametrize("which", ["honeycomb", "qwz"])
def test_eigensystem_general(lm, which):
    """General sparse Hamiltonians (lm_ell): the dense assembly adds the stored entries."""
    if which == "honeycomb":
        Ho, coords = o.honeycomb_hamiltonian(5, 4, B=0.04, onsite=o.anderson_disorder(40, 1.0, 5))
        sites = lm.Sites(Ho.shape[0], coords, "honeycomb")
    else:
        Ho = o.qwz_hamiltonian(5, 4, m=np.linspace(-1.5, 1.5, 20))
        sites = lm.Sites(Ho.shape[0], None, "qwz", internal=2)
    H = lm.SparseHamiltonian(sites, Ho)
    Hd = Ho.toarray()
    wref = np.linalg.eigvalsh(Hd)
    eig = lm.diagonalize(H)
    assert np.abs(eig.values - wref).max() <= 1e-13 * max(1.0, np.abs(wref).max())
    V = eig.vectors().to_numpy()
    assert np.linalg.norm(Hd @ V - V * eig.values) <= 1e-12 * np.linalg.norm(Hd)
    P = lm.densitymatrix(H, mu=0.1).to_numpy()
    Pref, _, _ = o.densitymatrix(Ho, mu=0.1, degenerate_tol=1e-12 * max(1.0, np.abs(wref).max()))
    assert rel(P, Pref) <= 1e-10


def test_zero_temperature_config1_degenerate(lm):
    """P_0 = densitymatrix(h(0), mu = 0) of the plain reference run: SquareLattice(10, 10), open,
    no field at t = 0, so E = 0 is exactly 10-fold degenerate (2 cos(pi m/11) + 2 cos(pi n/11) = 0
    for m + n = 11): all of it is occupied, 45 + 10 = 55 states."""
    Ho, Hl = square_case(lm, 10, 10)
    wref = np.linalg.eigvalsh(Ho.toarray())
    tol = 1e-12 * max(1.0, np.abs(wref).max())
    assert np.sum(np.abs(wref) <= tol) == 10
    Pref, _, _ = o.densitymatrix(Ho, mu=0.0, degenerate_tol=tol)
    P = lm.densitymatrix(Hl, mu=0.0)
    assert rel(P.to_numpy(), Pref) <= 1e-10
    assert abs(P.trace() - 55.0) <= 1e-10
    # and with the field switched on (B = 0.2): no level at mu, the two rules agree
    Ho2, Hl2 = square_case(lm, 10, 10, field=("pf", 0.2))
    P2 = lm.densitymatrix(Hl2, mu=0.0).to_numpy()
    Pexact, _, _ = o.densitymatrix(Ho2, mu=0.0)
    assert rel(P2, Pexact) <= 1e-10


@pytest.mark.parametrize("L", [16, 48])
def test_zero_temperature_batching_lattice(lm, L):
    """An instance of the batching workload (open LxL, PointFlux at the centre, disorder):
    P_0 = densitymatrix(h, mu = 0) against the oracle's LAPACK projector."""
    Ho, Hl = square_case(lm, L, L, field=("pf", 0.17), W=1.7, seed=L)
    Pref, w, _ = o.densitymatrix(Ho, mu=0.0, degenerate_tol=1e-12 * max(1.0, np.abs(np.linalg.eigvalsh(Ho.toarray())).max()))
    P = lm.densitymatrix(Hl, mu=0.0)
    assert rel(P.to_numpy(), Pref) <= 1e-10
    assert abs(P.trace() - np.trace(Pref).real) <= 1e-9


def test_zero_temperature_96_properties(lm):
    """The largest batching lattice, SquareLattice(96, 96) open with PointFlux(0.2) at the
    centre and disorder U[-0.75, 0.75] (N = 9216).  LAPACK on the host takes minutes here, so
    the projector is held to properties that fix it uniquely -- Hermitian, idempotent,
    commuting with H, with trace the number of levels at or below mu (from the eigenvalues,
    checked against a Sturm count of the oracle's matrix would need the same O(N^3)) -- and
    compared with an independent FP64 eigensolver on the same GPU (cuSOLVER through torch,
    used here only as a checker)."""
    torch = pytest.importorskip("torch")
    Ho, Hl = square_case(lm, 96, 96, field=("pf", 0.2), W=1.5, seed=96)
    eig = lm.diagonalize(Hl)
    tol = 1e-12 * max(1.0, np.abs(eig.values).max())
    nocc = int(np.sum(eig.values <= tol))
    P = eig.projector((eig.values <= tol).astype(float)).to_numpy()
    Pt = torch.as_tensor(P, device="cuda")
    Ht = torch.as_tensor(Ho.toarray(), device="cuda")
    n2 = float(torch.linalg.norm(Pt))
    assert float(torch.linalg.norm(Pt - Pt.conj().T)) <= 1e-13 * n2
    assert float(torch.linalg.norm(Pt @ Pt - Pt)) <= 1e-10 * n2
    assert float(torch.linalg.norm(Ht @ Pt - Pt @ Ht)) <= 1e-10 * n2
    assert abs(float(torch.trace(Pt).real) - nocc) <= 1e-8
    w_t, V_t = torch.linalg.eigh(Ht)
    w_t = w_t.cpu().numpy()
    assert np.abs(eig.values - w_t).max() <= 1e-12 * max(1.0, np.abs(w_t).max())
    Vo = V_t[:, :nocc]
    Pref = Vo @ Vo.conj().T
    assert float(torch.linalg.norm(Pt - Pref)) <= 1e-10 * float(torch.linalg.norm(Pref))
