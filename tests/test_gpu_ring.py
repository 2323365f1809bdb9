"""The readout ring (lm_ring_*) behind TimeSequence(moment_density / moment_currents, ev(times)):
identical values to synchronous per-moment readouts, wrap-around, and its error paths."""
import ctypes as C

import numpy as np
import pytest

from oracle import lm_oracle as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lm():
    import lmgpu
    lmgpu.default_context()
    return lmgpu


def evolution(lm, precision):
    L = 12
    lat = lm.SquareLattice(L, L)
    V = o.anderson_disorder(L * L, 1.0, 3)
    h = lambda t: lm.tightbinding_hamiltonian(lat, V, field=lm.PointFlux(0.05 * t, (6.5, 6.5)))
    X = o.random_kets(L * L, 6, 4)
    st = lm.KetBlock(lat, X, precision=precision)
    return lm.Evolution(lm.ChebyshevGPU(), h, st)


@pytest.mark.parametrize("precision", ["c64", "c32"])
@pytest.mark.parametrize("nslots", [3, 32])
def test_ring_matches_synchronous_readouts(lm, precision, nslots):
    times = [0.1 * k for k in range(1, 15)]
    ev = evolution(lm, precision)
    ref_rho, ref_J, ref_t = [], [], []
    for m in ev(times):
        ref_rho.append(lm.localdensity(m.state).values.copy())
        ref_J.append(lm.DensityCurrents(m.H, m.state).bond_values().copy())
        ref_t.append(m.t)
    ev_a = evolution(lm, precision)
    ts_rho = lm.TimeSequence(lm.moment_density, ev_a(times), nslots=nslots)
    ev_b = evolution(lm, precision)
    ts_J = lm.TimeSequence(lm.moment_currents, ev_b, times, nslots=nslots)
    assert ts_rho.times == ref_t and ts_J.times == ref_t
    for a, b in zip(ts_rho.values, ref_rho):
        assert np.array_equal(a.values, b)
    for a, b in zip(ts_J.values, ref_J):
        assert np.array_equal(a, b)
    # a generic f takes the synchronous path with the same values
    ev_c = evolution(lm, precision)
    ts_g = lm.TimeSequence(lambda m: lm.localdensity(m.state).values.sum(), ev_c(times))
    np.testing.assert_allclose(ts_g.values, [r.sum() for r in ref_rho], rtol=1e-12)


def test_ring_entry_lifetime(lm):
    ctx = lm.default_context()
    lat = lm.SquareLattice(5, 5)
    st = lm.KetBlock(lat, o.random_kets(25, 2, 1), precision="c64")
    ring = lm.ReadoutRing(25, nslots=2, ctx=ctx)
    s0 = ring.push_density(st, 0.0)
    s1 = ring.push_density(st, 1.0)
    t, v = ring.wait(s1)
    assert t == 1.0 and np.allclose(v, lm.localdensity(st).values)
    assert ring.ready(s0)
    ring.push_density(st, 2.0)  # overwrites entry 0
    with pytest.raises(lm.LMError):
        ring.wait(s0)
    with pytest.raises(lm.LMError):
        ring.wait(ring.head)  # not pushed yet
    with pytest.raises(lm.LMError):
        lm.ReadoutRing(10, nslots=2, ctx=ctx).push_density(st, 0.0)  # slot shorter than N


def test_onsite_buffer_is_free_after_the_call(lm):
    """lm_ham_set_onsite copies the caller's array during the call: overwriting a pinned
    buffer right after it returns does not change the assembled H."""
    torch = pytest.importorskip("torch")
    ctx = lm.default_context()
    lib = ctx.lib
    lat = lm.SquareLattice(64, 64)
    N = lat.N
    V = np.random.default_rng(0).uniform(-1, 1, N)
    pin = torch.empty(N, dtype=torch.float64, pin_memory=True)
    pin.numpy()[:] = V
    ham = C.c_void_p()
    ctx.check(lib.lm_ham_create(ctx.handle, lat.handle(ctx), 1.0, C.byref(ham)))
    try:
        for _ in range(3):
            ctx.check(lib.lm_ham_set_onsite(ham, pin.numpy().ctypes.data_as(C.POINTER(C.c_double))))
            pin.numpy()[:] = 1e6  # the caller reuses its buffer at once
            ctx.check(lib.lm_ham_assemble(ham, None, 0))
            pin.numpy()[:] = V
        nnz = C.c_int64()
        ctx.check(lib.lm_ham_nnz(ham, C.byref(nnz)))
        colptr = np.empty(N + 1, dtype=np.int64)
        rowval = np.empty(nnz.value, dtype=np.int64)
        nz = np.empty(2 * nnz.value)
        ctx.check(lib.lm_ham_csc(ham, colptr.ctypes.data_as(C.POINTER(C.c_int64)),
                                 rowval.ctypes.data_as(C.POINTER(C.c_int64)),
                                 nz.ctypes.data_as(C.POINTER(C.c_double))))
        diag = np.zeros(N)
        for j in range(N):
            for p in range(colptr[j] - 1, colptr[j + 1] - 1):
                if rowval[p] - 1 == j:
                    diag[j] = nz[2 * p]
        np.testing.assert_array_equal(diag, V)
    finally:
        lib.lm_ham_destroy(ham)
