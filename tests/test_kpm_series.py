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
