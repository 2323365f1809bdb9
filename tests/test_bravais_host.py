"""Host-side geometry of the Bravais lattices (HoneycombLattice, KagomeLattice,
TriangularLattice): the library's nearest-neighbour detection from distances (detect_nnhops,
src/lattices/bravais/nearestneighbor.jl:87-131) and its boundary routing give the oracle's
hard-coded bond sets, phases and twists (no GPU: the Hamiltonian is formed here from the bond
list as the device assembly forms it)."""
import math

import numpy as np
import pytest

from oracle import lm_oracle as o


def dense_from_bonds(lat, field):
    src, dst, xy, fac = lat.bonds()
    H = np.zeros((lat.N, lat.N), complex)
    for s, d, r, f in zip(src, dst, xy, fac):
        li = 0.0 if field is None else field.line_integral((float(r[0]), float(r[1])), (float(r[2]), float(r[3])))
        v = f * np.exp(-2j * math.pi * li)
        H[s - 1, d - 1] += v
        H[d - 1, s - 1] += np.conj(v)
    return H


@pytest.mark.parametrize("name,fn,a,b", [("HoneycombLattice", o.honeycomb_hamiltonian, 5, 4),
                                         ("KagomeLattice", o.kagome_hamiltonian, 4, 3),
                                         ("TriangularLattice", o.triangular_hamiltonian, 5, 4)])
@pytest.mark.parametrize("field", [None, "landau", "pointflux"])
def test_open_lattices_match_oracle(name, fn, a, b, field):
    import lmgpu
    lat = lmgpu.BravaisLattice(name, a, b)
    fld = {None: None, "landau": o.LandauGauge(0.05), "pointflux": o.PointFlux(0.3, (2.1, 1.7))}[field]
    Ho, coords = fn(a, b, field=fld)
    assert np.array_equal(coords, lat.coords())  # site order and coordinates
    assert np.abs(dense_from_bonds(lat, fld) - Ho.toarray()).max() <= 1e-15


@pytest.mark.parametrize("per,tw", [((True, True), (0.3, -0.7)), ((True, False), (0.0, 0.0)),
                                    ((False, True), (0.0, 0.4))])
def test_periodic_honeycomb_routing_and_twist(per, tw):
    import lmgpu
    bnd = {"axis1": (tw[0] if tw[0] else True) if per[0] else False,
           "axis2": (tw[1] if tw[1] else True) if per[1] else False}
    lat = lmgpu.HoneycombLattice(4, 3, boundaries=bnd)
    fld = o.LandauGauge(0.07)
    Ho, _ = o.honeycomb_hamiltonian_periodic(4, 3, per, tw, field=fld)
    assert np.abs(dense_from_bonds(lat, fld) - Ho.toarray()).max() <= 1e-15
    if per == (True, True):
        assert lat.nbonds() == 3 * 4 * 3   # every A site has its three neighbours


def test_nn_translations_follow_the_reference_detection():
    import lmgpu
    # honeycomb: A -> B at distance 1/sqrt(3) in three cells; kagome: six basis pairs at 1/2;
    # triangular: three all-basis translations at 1
    assert sorted(lmgpu.HoneycombLattice(2, 2).nn_translations()) == [(1, 2, (-1, 0)), (1, 2, (0, -1)), (1, 2, (0, 0))]
    assert len(lmgpu.KagomeLattice(2, 2).nn_translations()) == 6
    assert sorted(lmgpu.TriangularLattice(2, 2).nn_translations()) == [(0, 0, (0, 1)), (0, 0, (1, -1)), (0, 0, (1, 0))]
