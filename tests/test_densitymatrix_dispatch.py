"""densitymatrix's keyword dispatch (src/spectrum.jl:239-333): the host occupations of
``lmgpu.spectrum.occupations`` against the oracle's restatement, for the Fermi sphere, the
BoseEinstein condensate, fixed N at T > 0 (Newton iteration for mu), the FermiDirac and
BoseEinstein ensembles and the Gibbs state.  No GPU: the eigensystem is numpy's."""
import warnings

import numpy as np
import pytest

from oracle import lm_oracle as o

CASES = [dict(N=5), dict(N=5, T=0.3), dict(T=0.3), dict(), dict(mu=0.2), dict(mu=0.2, T=0.1),
         dict(mu=-4.0, T=0.3, statistics="BoseEinstein"), dict(N=3, statistics="BoseEinstein"),
         dict(statistics="FermiDirac", T=0.2), dict(N=25)]


@pytest.fixture(scope="module")
def system():
    H = o.tightbinding_hamiltonian(o.SquareLattice(5, 5), field=o.LandauGauge(0.1),
                                   onsite=o.anderson_disorder(25, 1.0, 3))
    return H, o.diagonalize(H)


@pytest.mark.parametrize("kw", CASES, ids=[",".join(f"{k}={v}" for k, v in c.items()) or "gibbs-T0" for c in CASES])
def test_occupations_match_the_reference_dispatch(system, kw):
    from lmgpu.spectrum import occupations
    H, (w, V) = system
    P = (V * occupations(w, **kw)) @ V.conj().T
    Pref = o.densitymatrix_dispatch(H, **kw)
    assert np.abs(P - Pref).max() <= 1e-14


def test_particle_numbers(system):
    from lmgpu.spectrum import occupations
    H, (w, V) = system
    assert occupations(w, N=7).sum() == 7
    assert abs(occupations(w, N=7, T=0.2).sum() - 7) <= 1e-7
    assert abs(occupations(w, T=0.5).sum() - 1) <= 1e-14          # Gibbs: Tr P = 1
    assert occupations(w, N=4, statistics="BoseEinstein")[0] == 4   # condensate


def test_errors_and_warnings(system):
    from lmgpu.spectrum import occupations
    H, (w, V) = system
    with pytest.raises(ValueError):
        occupations(w, N=3, mu=0.1)
    with pytest.raises(ValueError):
        occupations(w, N=26)
    with pytest.raises(ValueError):
        occupations(w, mu=0.0, statistics="Boltzmann")
    wd = np.array([-1.0, 0.0, 0.0, 1.0])
    with warnings.catch_warnings(record=True) as rec:
        warnings.simplefilter("always")
        occupations(wd, N=2)
    assert any("degenerate levels" in str(r.message) for r in rec)
