"""The KPM resolvent series of lmgpu.kpm (host arithmetic) against the eigensystem formula of
the reference's dos (src/greenfunction.jl:306), with the oracle's moments: no GPU needed."""
import numpy as np
import pytest

from oracle import lm_oracle as o
from lmgpu import kpm


@pytest.mark.parametrize("broaden", [0.05, 0.1, 0.3])
def test_dos_and_ldos_series_match_eigensystem(broaden):
    ol = o.SquareLattice(8, 8)
    V = o.anderson_disorder(64, 1.0, 3)
    H = o.tightbinding_hamiltonian(ol, field=o.PointFlux(0.2, (4.5, 4.5)), onsite=V)
    w, U = np.linalg.eigh(H.toarray())
    bounds = (w.min() - 0.05, w.max() + 0.05)
    E = np.linspace(-4.5, 4.5, 37)
    nm = kpm.order_for(E, broaden, bounds, 1e-12)
    mu = o.kpm_moments(H, *bounds, nm)
    d = -np.imag(kpm.resolvent_trace(mu, E, broaden, bounds)) / np.pi
    ref = o.dos_eigensystem(w, E, broaden)
    assert np.abs(d - ref).max() <= 1e-10 * ref.max()
    mus = o.kpm_moments(H, *bounds, nm, per_column=True)
    ld = -np.imag(kpm.resolvent_trace(mus, 0.3, broaden, bounds)[0]) / np.pi
    lref = o.ldos_eigensystem(w, U, 0.3, broaden)
    assert np.abs(ld - lref).max() <= 1e-10 * lref.max()
    assert abs(ld.sum() - o.dos_eigensystem(w, 0.3, broaden)[0]) <= 1e-10 * ld.sum()


def test_order_grows_as_broadening_shrinks():
    b = (-5.0, 5.0)
    assert kpm.order_for(0.0, 0.01, b) > kpm.order_for(0.0, 0.1, b) > kpm.order_for(0.0, 1.0, b)
    with pytest.raises(ValueError):
        kpm.order_for(0.0, 0.0, b)


@pytest.mark.parametrize("mu,T", [(0.0, 0.1), (0.5, 0.3), (-1.0, 0.05)])
def test_fermi_series_coefficients(mu, T):
    """The truncated Chebyshev series of the FermiDirac occupation (src/spectrum.jl:230-232)
    reproduces it to the requested tolerance on the whole interval."""
    pytest.importorskip("scipy")
    from lmgpu import spectrum
    f = spectrum.fermi_occupation(mu, T)
    b = (-5.3, 5.1)
    c = spectrum.chebyshev_coefficients(f, b, 1e-13)
    x = np.linspace(-1, 1, 2001)
    a, m = 0.5 * (b[1] - b[0]), 0.5 * (b[1] + b[0])
    assert np.abs(np.polynomial.chebyshev.chebval(x, c) - f(a * x + m)).max() <= 2e-13
    # against the oracle's scalar occupation
    fo = o.densfun(T, mu)
    E = np.linspace(-5, 5, 11)
    assert np.allclose(f(E), [fo(e) for e in E], rtol=0, atol=1e-15)
