"""Device Chebyshev moments (lm_kpm_moments) against the oracle's plain recurrence, and the
KPM dos / ldos against the reference's eigensystem formula (src/greenfunction.jl:306)."""
import numpy as np
import pytest

from oracle import lm_oracle as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lm():
    import lmgpu
    lmgpu.default_context()
    return lmgpu


def case(lm, L, per, field):
    ol = o.SquareLattice(L, L, periodic=(per, per))
    b = {"axis1": True, "axis2": True} if per else {}
    ll = lm.SquareLattice(L, L, boundaries=b)
    V = o.anderson_disorder(L * L, 1.5, 11)
    if field == "pf":
        Ho = o.tightbinding_hamiltonian(ol, field=o.PointFlux(0.25, (L / 2 + 0.5, L / 2 + 0.5)), onsite=V)
        Hl = lm.tightbinding_hamiltonian(ll, V, field=lm.PointFlux(0.25, (L / 2 + 0.5, L / 2 + 0.5)))
    else:
        Ho = o.tightbinding_hamiltonian(ol, field=o.LandauGauge(0.05), onsite=V)
        Hl = lm.tightbinding_hamiltonian(ll, V, field=lm.LandauGauge(0.05))
    return ol, Ho, Hl


@pytest.mark.parametrize("L,per,field", [(9, False, "pf"), (12, True, "landau"), (16, False, "landau")])
def test_moments_match_oracle(lm, L, per, field):
    ol, Ho, Hl = case(lm, L, per, field)
    bounds = lm.kpm._bounds(Hl, lm.default_context())
    nm = 301
    mu, _ = lm.kpm.moments(Hl, nm, bounds=bounds)
    ref = o.kpm_moments(Ho, *bounds, nm)
    assert np.abs(mu - ref).max() <= 1e-11 * ref[0]
    mus, _ = lm.kpm.moments(Hl, 40, per_site=True, bounds=bounds)
    refs = o.kpm_moments(Ho, *bounds, 40, per_column=True)
    assert np.abs(mus - refs).max() <= 1e-12
    R = o.random_kets(ol.N, 7, 5)
    muv, _ = lm.kpm.moments(Hl, 101, vecs=R, bounds=bounds)
    refv = o.kpm_moments(Ho, *bounds, 101, vecs=R)
    assert np.abs(muv - refv).max() <= 1e-11 * abs(refv[0])


@pytest.mark.parametrize("L,per,field", [(9, False, "pf"), (12, True, "landau"), (16, False, "landau")])
def test_doublefloat_moments_match_oracle(lm, L, per, field):
    """LM_OPT_KPM = 1 (the default): the recurrence in double-float (FP32 pairs) keeps the
    moments within the FP64 path's tolerances against the oracle, and within 1e-12 mu_0 of the
    device FP64 moments (LM_OPT_KPM = 0)."""
    ol, Ho, Hl = case(lm, L, per, field)
    ctx = lm.default_context()
    bounds = lm.kpm._bounds(Hl, ctx)
    nm = 301
    R = o.random_kets(ol.N, 7, 5)
    try:
        ctx.set_kpm_doublefloat(False)
        mu64, _ = lm.kpm.moments(Hl, nm, bounds=bounds)
        muv64, _ = lm.kpm.moments(Hl, 101, vecs=R, bounds=bounds)
        ref = o.kpm_moments(Ho, *bounds, nm)
        assert np.abs(mu64 - ref).max() <= 1e-11 * ref[0]
    finally:
        ctx.set_kpm_doublefloat(True)
    mu, _ = lm.kpm.moments(Hl, nm, bounds=bounds)
    mus, _ = lm.kpm.moments(Hl, 40, per_site=True, bounds=bounds)
    muv, _ = lm.kpm.moments(Hl, 101, vecs=R, bounds=bounds)
    ref = o.kpm_moments(Ho, *bounds, nm)
    assert np.abs(mu - ref).max() <= 1e-11 * ref[0]
    assert np.abs(mu - mu64).max() <= 1e-12 * ref[0]
    refs = o.kpm_moments(Ho, *bounds, 40, per_column=True)
    assert np.abs(mus - refs).max() <= 1e-12
    refv = o.kpm_moments(Ho, *bounds, 101, vecs=R)
    assert np.abs(muv - refv).max() <= 1e-11 * abs(refv[0])
    assert np.abs(muv - muv64).max() <= 1e-12 * abs(refv[0])


@pytest.mark.parametrize("broaden", [0.05, 0.2])
def test_dos_ldos_match_eigensystem(lm, broaden):
    ol, Ho, Hl = case(lm, 14, False, "pf")
    w, U = np.linalg.eigh(Ho.toarray())
    E = np.linspace(-4.8, 4.8, 25)
    d = lm.kpm.dos(Hl, E, broaden)
    ref = o.dos_eigensystem(w, E, broaden)
    assert np.abs(d - ref).max() <= 1e-9 * ref.max()
    ld = lm.kpm.ldos(Hl, 0.7, broaden).values
    lref = o.ldos_eigensystem(w, U, 0.7, broaden)
    assert np.abs(ld - lref).max() <= 1e-9 * lref.max()


def test_stochastic_trace_estimates_dos(lm):
    ol, Ho, Hl = case(lm, 20, True, "landau")
    w = np.linalg.eigvalsh(Ho.toarray())
    E = np.linspace(-3, 3, 7)
    d = lm.kpm.dos(Hl, E, 0.3, exact_max=0, nvec=256, seed=1)
    ref = o.dos_eigensystem(w, E, 0.3)
    # random-phase trace estimator: relative error ~ 1/sqrt(N * nvec)
    assert np.abs(d - ref).max() <= 0.02 * ref.max()


def test_bounds_must_enclose_spectrum(lm):
    _, _, Hl = case(lm, 8, False, "pf")
    with pytest.raises(lm.LMError):
        lm.kpm.moments(Hl, 200, bounds=(-1.0, 1.0))


@pytest.mark.parametrize("mu,T", [(0.0, 0.1), (0.5, 0.3), (-1.0, 0.05)])
@pytest.mark.parametrize("precision", ["c64", "c32"])
def test_fermi_operator_densitymatrix(lm, mu, T, precision):
    """densitymatrix(H; mu, T > 0) from the Chebyshev series of the occupation on the device
    against the oracle's eigensystem projector (src/spectrum.jl:226-257)."""
    ol, Ho, Hl = case(lm, 12, False, "pf")
    Pref, _, _ = o.densitymatrix(Ho, mu=mu, T=T)
    P = lm.densitymatrix(Hl, mu=mu, T=T, precision=precision)
    Pd = P.to_numpy().astype(np.complex128)
    err = np.linalg.norm(Pd - Pref) / np.linalg.norm(Pref)
    assert err <= (1e-11 if precision == "c64" else 1e-6), err
    assert abs(P.trace() - np.trace(Pref).real) <= (1e-10 if precision == "c64" else 1e-5) * np.trace(Pref).real


def test_fermi_operator_low_temperature_doublefloat(lm):
    """T = 0.005 on the 12 x 12 PointFlux lattice: the Fermi function's Chebyshev series runs to
    about ten thousand terms, so the recurrence's rounding has the longest run to build up.  The
    double-float recurrence (LM_OPT_KPM = 1, about 48 significant bits) against the FP64 one
    (LM_OPT_KPM = 0) and both against the oracle's eigensystem projector
    (src/spectrum.jl:226-257) at the FP64 route's 1e-11 bar."""
    from lmgpu.spectrum import chebyshev_coefficients, fermi_occupation
    ol, Ho, Hl = case(lm, 12, False, "pf")
    mu, T = 0.1, 0.005
    ctx = lm.default_context()
    lo, hi = Hl.bounds(ctx)
    pad = 1e-3 * (hi - lo)
    K = len(chebyshev_coefficients(fermi_occupation(mu, T), (lo - pad, hi + pad), 1e-13))
    Pref, _, _ = o.densitymatrix(Ho, mu=mu, T=T)
    try:
        ctx.set_kpm_doublefloat(False)
        P64 = lm.densitymatrix(Hl, mu=mu, T=T).to_numpy()
    finally:
        ctx.set_kpm_doublefloat(True)
    Pdf = lm.densitymatrix(Hl, mu=mu, T=T).to_numpy()
    r = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    gaps = {"K": K, "df_vs_fp64": r(Pdf, P64), "fp64_vs_oracle": r(P64, Pref), "df_vs_oracle": r(Pdf, Pref)}
    print("low-T Fermi operator (12x12, T = 0.005):", gaps)
    assert K >= 2000, gaps
    assert gaps["fp64_vs_oracle"] <= 1e-11, gaps
    assert gaps["df_vs_oracle"] <= 1e-11, gaps
    assert gaps["df_vs_fp64"] <= 1e-11, gaps


@pytest.mark.parametrize("precision", ["c64", "c32"])
def test_zero_temperature_densitymatrix(lm, precision):
    """densitymatrix(H; mu) at T = 0: the device eigensystem (cuSOLVER) and the projector
    stay on the device and go into the state without a host round trip; against the oracle's
    eigh projector (src/spectrum.jl:226-257).  mu sits between levels."""
    ol, Ho, Hl = case(lm, 12, False, "pf")
    w = np.linalg.eigvalsh(Ho.toarray())
    mu = 0.5 * (w[70] + w[71])
    Pref, _, _ = o.densitymatrix(Ho, mu=mu)
    P = lm.densitymatrix(Hl, mu=mu, precision=precision)
    Pd = P.to_numpy().astype(np.complex128)
    err = np.linalg.norm(Pd - Pref) / np.linalg.norm(Pref)
    assert err <= (1e-12 if precision == "c64" else 1e-6), err
    assert abs(P.trace() - 71) <= (1e-10 if precision == "c64" else 1e-4)


def test_cheb_apply_on_kets_matches_dense_function(lm):
    """lm_cheb_apply on a ket block: f(H) X for f = exp(-(E - 0.3)^2) against the dense oracle."""
    import ctypes as C
    ol, Ho, Hl = case(lm, 10, True, "landau")
    w, U = np.linalg.eigh(Ho.toarray())
    f = lambda E: np.exp(-(np.asarray(E) - 0.3) ** 2)
    X = o.random_kets(ol.N, 5, 9)
    ref = (U * f(w)) @ (U.conj().T @ X)
    ctx = lm.default_context()
    lo, hi = Hl.bounds(ctx)
    coef = lm.spectrum.chebyshev_coefficients(f, (lo, hi), 1e-14)
    st = lm.KetBlock(Hl.lattice, X)
    out = lm.KetBlock(Hl.lattice, np.zeros_like(X))
    ctx.check(ctx.lib.lm_cheb_apply(Hl.device(ctx).handle, lo, hi, coef.ctypes.data_as(C.POINTER(C.c_double)),
                                    len(coef), st.handle, out.handle))
    assert np.linalg.norm(out.to_numpy() - ref) <= 1e-12 * np.linalg.norm(ref)


@pytest.mark.parametrize("L,per,field", [(9, False, "pf"), (20, True, "landau"), (31, False, "landau")])
def test_lanczos_bounds_enclose_spectrum(lm, L, per, field):
    """FP64 Lanczos bounds (lm_ham_lanczos_bounds) enclose the exact spectrum, sit inside the
    Gershgorin interval and close to the exact extremes."""
    ol, Ho, Hl = case(lm, L, per, field)
    w = np.linalg.eigvalsh(Ho.toarray())
    ctx = lm.default_context()
    glo, ghi = Hl.bounds(ctx)
    lo, hi = Hl.bounds(ctx, method="lanczos")
    assert glo <= lo <= w[0] and w[-1] <= hi <= ghi
    assert (hi - lo) <= 1.05 * (w[-1] - w[0])


def test_densitymatrix_with_lanczos_bounds(lm):
    ol, Ho, Hl = case(lm, 12, False, "pf")
    Pref, _, _ = o.densitymatrix(Ho, mu=0.2, T=0.1)
    P = lm.densitymatrix(Hl, mu=0.2, T=0.1, bounds="lanczos").to_numpy()
    assert np.linalg.norm(P - Pref) <= 1e-11 * np.linalg.norm(Pref)


def test_dos_with_lanczos_bounds(lm):
    ol, Ho, Hl = case(lm, 14, False, "pf")
    w = np.linalg.eigvalsh(Ho.toarray())
    E = np.linspace(-4, 4, 9)
    d = lm.kpm.dos(Hl, E, 0.1, bounds="lanczos")
    assert np.abs(d - o.dos_eigensystem(w, E, 0.1)).max() <= 1e-9 * d.max()


@pytest.mark.parametrize("kw", [dict(), dict(T=0.3), dict(N=20), dict(N=20, T=0.2),
                                dict(mu=-3.5, T=0.4, statistics="BoseEinstein")],
                         ids=["gibbs-T0", "gibbs-T", "fermi-sphere", "fixed-N", "bose-ensemble"])
def test_densitymatrix_dispatch_on_device(lm, kw):
    """densitymatrix(H; ...) without mu (the Gibbs state), with N (Fermi sphere, fixed N at
    T > 0) and with BoseEinstein statistics: the device eigensystem weighted by the reference's
    occupations, against the oracle (src/spectrum.jl:239-333).  Disorder lifts degeneracies."""
    ol = o.SquareLattice(8, 8)
    ll = lm.SquareLattice(8, 8)
    V = o.anderson_disorder(64, 1.5, 11)
    Ho = o.tightbinding_hamiltonian(ol, field=o.PointFlux(0.2, (4.5, 4.5)), onsite=V)
    Hl = lm.tightbinding_hamiltonian(ll, V, field=lm.PointFlux(0.2, (4.5, 4.5)))
    Pref = o.densitymatrix_dispatch(Ho, **kw)
    P = lm.densitymatrix(Hl, **kw).to_numpy()
    assert np.abs(P - Pref).max() <= 1e-12 * max(1.0, np.abs(Pref).max())
