"""Host-side logic of the library and the Python mirror; needs no GPU."""
import ctypes as C

import numpy as np
import pytest

from oracle import lm_oracle as o


def test_library_exports_every_header_symbol(lib):
    import lmgpu._lib as L
    names = L.header_functions()
    assert len(names) >= 35
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the ctypes table covers the same set
    assert sorted(L.SIGNATURES) == names


@pytest.mark.parametrize("Lx,Ly,per,tw", [
    (1, 1, (False, False), (0, 0)), (1, 7, (False, False), (0, 0)), (4, 4, (False, False), (0, 0)),
    (3, 5, (True, False), (0, 0)), (5, 3, (False, True), (0, 0.3)), (2, 2, (True, True), (0, 0)),
    (2, 3, (True, True), (0.1, 0.2)), (16, 12, (True, True), (0, 0)), (7, 1, (True, False), (0, 0))])
def test_bond_order_bit_exact(Lx, Ly, per, tw):
    import lmgpu
    ol = o.SquareLattice(Lx, Ly, periodic=per, twist=tw)
    ob = o.nn_bonds(ol)
    ll = lmgpu.SquareLattice(Lx, Ly, boundaries={"axis1": tw[0] if per[0] and tw[0] else per[0],
                                                 "axis2": tw[1] if per[1] and tw[1] else per[1]})
    src, dst = ll.bonds()
    assert len(src) == len(ob) == ll.nbonds()
    assert np.array_equal(src, [b.src for b in ob])
    assert np.array_equal(dst, [b.dst for b in ob])
    assert np.array_equal(ll.coords(), ol.coords)


def test_periodic_axis_of_length_one_rejected(lib):
    import lmgpu._lib as L
    p = C.c_void_p()
    rc = lib.lm_lattice_square(None, 1, 4, 1, 0, 0.0, 0.0, C.byref(p))
    assert rc == L.LM_ERR_NOTSUP


def test_null_arguments_rejected(lib):
    import lmgpu._lib as L
    assert lib.lm_lattice_square(None, 0, 4, 0, 0, 0.0, 0.0, C.byref(C.c_void_p())) == L.LM_ERR_ARG
    assert lib.lm_lattice_square(None, 3, 4, 0, 0, 0.0, 0.0, None) == L.LM_ERR_ARG
    assert lib.lm_solver_step(None, None) == L.LM_ERR_ARG
    assert lib.lm_localdensity(None, None) == L.LM_ERR_ARG
    assert lib.lm_chebyshev_plan(-1.0, 1e-12, 0, C.byref(C.c_int()), None) == L.LM_ERR_ARG


@pytest.mark.parametrize("x,tol", [(0.0, 1e-12), (0.25, 1e-12), (0.55, 1e-12), (0.25, 1e-7),
                                   (3.0, 1e-12), (40.0, 1e-10), (250.0, 1e-12)])
def test_chebyshev_plan_vs_scipy(lib, x, tol):
    from scipy.special import jv
    K = C.c_int()
    assert lib.lm_chebyshev_plan(x, tol, 0, C.byref(K), None) == 0
    K = K.value
    coef = np.zeros(2 * (K + 1))
    assert lib.lm_chebyshev_plan(x, tol, K + 1, C.byref(C.c_int()), coef.ctypes.data_as(C.POINTER(C.c_double))) == 0
    c = coef[0::2] + 1j * coef[1::2]
    k = np.arange(K + 1)
    ref = np.where(k == 0, 1.0, 2.0) * (-1j) ** k * jv(k, x)
    assert np.allclose(c, ref, atol=1e-15 * max(1.0, x / 10), rtol=1e-12)  # Miller normalisation sum
    # K is the smallest order (>= 2) whose neglected tail is below tol
    tail = lambda kk: 2 * np.sum(np.abs(jv(np.arange(kk + 1, kk + 200), x)))
    assert tail(K) <= tol * 1.0001
    assert K == 2 or tail(K - 1) > tol * 0.9999


def test_chebyshev_series_matches_exact_exponent():
    """The coefficient convention (with the e^{-ib dt} phase) reproduces exp(-iH dt)."""
    l = o.SquareLattice(6, 5)
    V = o.anderson_disorder(l.N, 2.0, 7)
    H = o.tightbinding_hamiltonian(l, field=o.PointFlux(0.3, (3.5, 2.5)), onsite=V)
    X = o.random_kets(l.N, 3, 1)
    lo, hi = V.min() - 4, V.max() + 4
    a = (hi - lo) / 2
    from scipy.special import jv
    K = 2
    while 2 * np.sum(np.abs(jv(np.arange(K + 1, K + 80), a * 0.1))) > 1e-13:
        K += 1
    Y = o.chebyshev_expv(H, 0.1, X, lo, hi, K)
    assert np.abs(Y - o.expm_exact(H, 0.1) @ X).max() < 1e-12


def test_evolution_driver_semantics_with_fake_solver(monkeypatch):
    """Evolution/EvolutionIterator call order and times, without a GPU (src/evolution.jl:238-275)."""
    import lmgpu
    from lmgpu import evolution as E
    from lmgpu.states import DeviceState

    class FakeState(DeviceState):
        def __init__(self):
            self.steps = []
        def copy(self):
            c = FakeState(); c.steps = list(self.steps); return c

    calls = []

    class FakeSolver(E.EvolutionSolver):
        def update_solver(self, H, dt, force=False):
            calls.append(("update", H, dt))
        def step(self, state, cache):
            state.steps.append(calls[-1][2])

    hs = []
    def h(t):
        hs.append(t)
        return ("H", t)

    s0 = FakeState()
    ev = lmgpu.Evolution(FakeSolver(), h, s0)
    moments = list(ev([0.0, 0.1, 0.3]))
    assert [m.t for m in moments] == [0.0, 0.1, 0.3]
    assert hs == [0.0, 0.0, 0.1]                       # left-endpoint H, first call at dt = 0
    assert [c[2] for c in calls] == [0.1, pytest.approx(0.2)]
    assert moments[1].H == ("H", 0.0)                   # moment k carries H(t_{k-1})
    assert s0.steps == []                               # the state was copied
    P, H, t = moments[2]
    assert t == 0.3 and H == ("H", 0.1)
    # stateful: calling again continues from the current time
    more = list(ev([0.4]))
    assert more[0].t == pytest.approx(0.4)
    with pytest.raises(ValueError):
        list(ev([0.2]))                                 # negative time step
    with pytest.raises(ValueError):
        lmgpu.Evolution(FakeSolver(), h, s0, P=s0)     # named and unnamed together
    with pytest.raises(ValueError):
        lmgpu.Evolution(FakeSolver(), h)                # no states
    named = lmgpu.Evolution(FakeSolver(), h, P=FakeState())
    m = list(named([0.0, 0.1]))[-1]
    assert isinstance(m["P"], FakeState) and isinstance(m.P, FakeState)
