"""HoneycombLattice ComplexF32 kets through the temporally blocked x-streaming kernel.

In the reference's site order ((j1, j2, s) -> 2((j1-1) b + j2 - 1) + s - 1, basis [0, 0] and
[1/2, sqrt(3)/6]: src/lattices/bravais/unitcell.jl:113-132, src/zoo/lattices.jl:145-160) the
honeycomb is an a x 2b "brick" lattice whose unit cells are the streaming kernel's site pairs
(lm_ell_set_layout, LM_LAYOUT_HONEYCOMB).  Bars: against the oracle's exact exponent on its own
restatement of the lattice (FP32 bar 3e-6), against the general per-order ELL path of the same
matrix (the two FP32 forms agree to 2e-6), for every series order K the kernel takes, open and
periodic (twisted) boundaries; and the layout is refused for matrices that are not honeycomb
nearest-neighbour bonds.
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


def oracle_h(a, b, per, tw, field, V):
    if per == (False, False):
        return o.honeycomb_hamiltonian(a, b, field=field, onsite=V)[0]
    return o.honeycomb_hamiltonian_periodic(a, b, periodic=per, twist=tw, field=field, onsite=V)[0]


CASES = [
    # a, b, periodic, twist, dt (K grows with dt), kets
    (20, 14, (False, False), (0.0, 0.0), 0.05, 5),
    (24, 16, (True, True), (0.0, 0.0), 0.1, 4),
    (19, 9, (True, False), (0.7, 0.0), 0.2, 3),
    (17, 23, (False, True), (0.0, -0.4), 0.3, 2),
    (32, 40, (True, True), (0.3, 0.9), 0.02, 6),
    (20, 1, (False, False), (0.0, 0.0), 0.05, 3),   # one cell high: a single lane pair per column
    (21, 2, (True, False), (0.0, 0.0), 0.05, 2),
    (15, 33, (False, False), (0.0, 0.0), 0.05, 2),  # a = 2K + 3 at K = 6: the smallest streaming a
]


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}x{c[1]}-{c[4]}" for c in CASES])
def test_brick_step_vs_oracle_and_ell(lm, case):
    a, b, per, tw, dt, M = case
    bnd = {}
    for ax, name in enumerate(("axis1", "axis2")):
        if per[ax]:
            bnd[name] = tw[ax] if tw[ax] else True
    lat = lm.HoneycombLattice(a, b, boundaries=bnd)
    V = o.anderson_disorder(lat.N, 1.5, a * 100 + b)
    Ho = oracle_h(a, b, per, tw, o.LandauGauge(0.03), V)
    H = lm.tightbinding_hamiltonian(lat, V, field=lm.LandauGauge(0.03))
    X = o.random_kets(lat.N, M, 9)
    ctx = lm.default_context()
    st = lm.KetBlock(lat, X, precision="c32")
    s = lm.ChebyshevGPU()
    s.update_solver(H, dt)
    n0 = ctx.stream_launches()
    for _ in range(3):
        s.step(st)
    K = s.order(st)[0]
    assert ctx.stream_launches() - n0 == (3 if a >= 2 * K + 3 and K <= 6 else 0), K
    # the same matrix through the general per-order ELL path
    He = lm.SparseHamiltonian(lm.Sites(lat.N, None, "honeycomb"), Ho)
    se = lm.KetBlock(He.lattice, X, precision="c32")
    s2 = lm.ChebyshevGPU()
    s2.update_solver(He, dt)
    for _ in range(3):
        s2.step(se)
    Y = X
    for _ in range(3):
        Y = o.expm_multiply(Ho, dt, Y)
    got = st.to_numpy().astype(np.complex128)
    assert rel(got, Y) <= 3e-6, (K, rel(got, Y))
    assert rel(got, se.to_numpy().astype(np.complex128)) <= 2e-6, K


def test_brick_time_dependent_field(lm):
    """h(t) with a Landau amplitude that changes every step: the brick planes are rebuilt from
    the re-assembled ELL values at every update."""
    a, b, dt, n = 20, 12, 0.05, 5
    lat = lm.HoneycombLattice(a, b)
    V = o.anderson_disorder(lat.N, 1.0, 4)
    Bt = lambda t: 0.01 + 0.2 * t
    X = o.random_kets(lat.N, 3, 2)
    ctx = lm.default_context()
    n0 = ctx.stream_launches()
    ev = lm.Evolution(lm.ChebyshevGPU(), lambda t: lm.tightbinding_hamiltonian(lat, V, field=lm.LandauGauge(Bt(t))),
                      lm.KetBlock(lat, X, precision="c32"))
    times = [dt * (k + 1) for k in range(n)]
    Y, t0 = X, 0.0
    for moment, t in zip(ev(times), times):
        Ho = o.honeycomb_hamiltonian(a, b, field=o.LandauGauge(Bt(t0)), onsite=V)[0]
        Y = o.expm_multiply(Ho, t - t0, Y)
        t0 = t
        assert rel(moment.state.to_numpy().astype(np.complex128), Y) <= 3e-6
    assert ctx.stream_launches() - n0 == n


def test_layout_refusals(lm):
    from lmgpu import _lib as L
    ctx = lm.default_context()
    lib = ctx.lib
    # a Kagome matrix is not honeycomb nearest-neighbour bonds
    Hk, _ = o.kagome_hamiltonian(6, 5)
    H = lm.SparseHamiltonian(lm.Sites(Hk.shape[0], None, "kagome"), Hk)
    dh = H.device(ctx)
    assert lib.lm_ell_set_layout(dh.handle, L.LM_LAYOUT_HONEYCOMB, 9, 5, 0, 0) == L.LM_ERR_ARG  # 90 = 2ab
    # wrong cell counts, and periodic axes of fewer than 3 cells
    Hh = o.honeycomb_hamiltonian(6, 5)[0]
    H2 = lm.SparseHamiltonian(lm.Sites(Hh.shape[0], None, "honeycomb"), Hh)
    d2 = H2.device(ctx)
    assert lib.lm_ell_set_layout(d2.handle, L.LM_LAYOUT_HONEYCOMB, 5, 6, 0, 0) == L.LM_ERR_ARG
    assert lib.lm_ell_set_layout(d2.handle, L.LM_LAYOUT_HONEYCOMB, 6, 5, 0, 0) == L.LM_OK
    assert lib.lm_ell_set_layout(d2.handle, L.LM_LAYOUT_NONE, 0, 0, 0, 0) == L.LM_OK
    assert lib.lm_ell_set_layout(d2.handle, L.LM_LAYOUT_HONEYCOMB, 6, 5, 1, 0) == L.LM_OK  # open bonds only: fine
    assert lib.lm_ell_set_layout(d2.handle, L.LM_LAYOUT_HONEYCOMB, 2, 15, 1, 0) == L.LM_ERR_ARG
