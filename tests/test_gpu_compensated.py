"""Compensated ComplexF32 kets (lm_state_set_compensation): the x-streaming Chebyshev step
keeps each amplitude as an FP32 value plus the residual of its rounding, stored as a bfloat16
pair (8 significant bits of the residual, about 32 of the amplitude).

Bars: against the oracle's exact exponent (scipy expm_multiply on its own restatement of the
Hamiltonian, src/evolution.jl:69-80 applied step by step) the compensated block stays within
the FP32 form's bar; over the plain-method length (400 steps of dt = 0.05 on the periodic
256 x 256 Landau lattice) its local densities and bond currents stay within 1e-6 of the FP64
run of the same kets, and its error is below the plain FP32 form's.  Paths that cannot carry
the residual refuse a compensated state with LM_ERR_NOTSUP instead of dropping it.
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


def pair(lm, Lx, Ly, per):
    ol = o.SquareLattice(Lx, Ly, periodic=per)
    b = {name: True for ax, name in enumerate(("axis1", "axis2")) if per[ax]}
    return ol, lm.SquareLattice(Lx, Ly, boundaries=b)


CASES = [
    (32, 32, True, True, 0.05, 4, "landau"),
    (40, 18, True, False, 0.02, 3, "landau"),    # open y: uniform columns without the y seam
    (17, 64, False, True, 0.05, 5, "landau"),    # open x
    (30, 40, False, False, 0.02, 3, "pointflux"),  # complex x-hops (per-site planes, K <= 5)
    (26, 32, True, True, 0.02, 2, "symmetric"),    # complex hops on both axes, periodic
]


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}x{c[1]}-{c[6]}" for c in CASES])
def test_compensated_step_vs_oracle(lm, case):
    Lx, Ly, px, py, dt, M, fk = case
    ol, ll = pair(lm, Lx, Ly, (px, py))
    V = o.anderson_disorder(ol.N, 2.0, Lx + Ly)
    if fk == "landau":
        fo, fl = o.LandauGauge(0.02), lm.LandauGauge(0.02)
    elif fk == "symmetric":
        fo, fl = o.SymmetricGauge(0.015), lm.SymmetricGauge(0.015)
    else:
        pt = (Lx / 2 + 0.5, Ly / 2 + 0.5)
        fo, fl = o.PointFlux(0.3, pt), lm.PointFlux(0.3, pt)
    Ho = o.tightbinding_hamiltonian(ol, field=fo, onsite=V)
    Hl = lm.tightbinding_hamiltonian(ll, V, field=fl)
    X = o.random_kets(ol.N, M, 5)
    ctx = lm.default_context()
    out = {}
    for comp in (False, True):
        st = lm.KetBlock(ll, X, precision="c32", compensated=comp)
        s = lm.ChebyshevGPU()
        s.update_solver(Hl, dt)
        n0 = ctx.stream_launches()
        for _ in range(4):
            s.step(st)
        assert ctx.stream_launches() - n0 == 4
        out[comp] = st
    Y = X
    for _ in range(4):
        Y = o.expm_multiply(Ho, dt, Y)
    e_plain = rel(out[False].to_numpy().astype(np.complex128), Y)
    e_comp = rel(out[True].to_numpy().astype(np.complex128), Y)
    assert e_comp <= 3e-6, e_comp
    assert e_plain <= 3e-6, e_plain
    # the FP64 norms of value + residual hold the unitary evolution's norms closer than FP32
    assert np.abs(out[True].norms() - np.linalg.norm(X, axis=0)).max() <= 1e-7


def test_compensated_honeycomb_brick(lm):
    """A compensated ket block on a HoneycombLattice: the brick layout of the streaming kernel
    carries the residual; against the oracle's exact exponent, and below the FP32 form's error
    over 60 steps."""
    a, b, dt, M, steps = 20, 16, 0.05, 3, 60
    lat = lm.HoneycombLattice(a, b, boundaries={"axis1": True, "axis2": True})
    V = o.anderson_disorder(lat.N, 1.0, 13)
    Ho = o.honeycomb_hamiltonian_periodic(a, b, field=o.LandauGauge(0.03), onsite=V)[0]
    H = lm.tightbinding_hamiltonian(lat, V, field=lm.LandauGauge(0.03))
    X = o.random_kets(lat.N, M, 14)
    ctx = lm.default_context()
    errs = {}
    for comp in (False, True):
        st = lm.KetBlock(lat, X, precision="c32", compensated=comp)
        s = lm.ChebyshevGPU()
        s.update_solver(H, dt)
        n0 = ctx.stream_launches()
        for _ in range(steps):
            s.step(st)
        assert ctx.stream_launches() - n0 == steps
        errs[comp] = st.to_numpy().astype(np.complex128)
    Y = o.expm_multiply(Ho, dt * steps, X)
    e_plain, e_comp = rel(errs[False], Y), rel(errs[True], Y)
    assert e_comp <= 3e-6 and e_comp < e_plain, (e_plain, e_comp)


def test_compensated_copy_upload_renormalize(lm):
    """A copy carries the residual (the copy steps exactly like the original); an upload
    clears it (stepping after a re-upload repeats the first step bit for bit); renormalize
    reaches the target norms on value + residual."""
    ol, ll = pair(lm, 24, 16, (True, True))
    V = o.anderson_disorder(ol.N, 2.0, 9)
    Hl = lm.tightbinding_hamiltonian(ll, V, field=lm.LandauGauge(0.03))
    X = o.random_kets(ol.N, 3, 10)
    s = lm.ChebyshevGPU()
    s.update_solver(Hl, 0.05)
    a = lm.KetBlock(ll, X, precision="c32", compensated=True)
    s.step(a)
    first = a.to_numpy()
    s.step(a)
    b = a.copy()
    assert b.compensated
    s.step(a)
    s.step(b)
    assert np.array_equal(a.to_numpy(), b.to_numpy())
    a.upload(X)
    s.step(a)
    assert np.array_equal(a.to_numpy(), first)
    a.renormalize(np.full(3, 2.0))
    assert np.abs(a.norms() - 2.0).max() <= 1e-10  # the residual keeps ~9 bits below the FP32 ulp
    a.set_compensation(False)
    assert not a.compensated
    s.step(a)  # the plain form again


def test_compensated_refusals(lm):
    from lmgpu import _lib as L
    ctx = lm.default_context()
    ol, ll = pair(lm, 24, 24, (True, True))
    V = o.anderson_disorder(ol.N, 1.0, 3)
    X = o.random_kets(ol.N, 2, 4)
    # an odd number of rows: no x-streaming form, so no compensated step
    ol3, ll3 = pair(lm, 24, 25, (True, True))
    V3 = o.anderson_disorder(ol3.N, 1.0, 3)
    H3 = lm.tightbinding_hamiltonian(ll3, V3, field=lm.LandauGauge(0.02))
    st3 = lm.KetBlock(ll3, o.random_kets(ol3.N, 2, 4), precision="c32", compensated=True)
    s = lm.ChebyshevGPU()
    s.update_solver(H3, 0.05)
    with pytest.raises(L.LMError) as e:
        s.step(st3)
    assert e.value.code == L.LM_ERR_NOTSUP
    st = lm.KetBlock(ll, X, precision="c32", compensated=True)
    # ComplexF64 kets and density matrices have no residual plane
    with pytest.raises(L.LMError):
        lm.KetBlock(ll, X, precision="c64", compensated=True)
    dm = lm.DensityMatrix(ll, None, precision="c32")
    with pytest.raises(L.LMError):
        dm.set_compensation(True)
    # with the fused step switched off the per-order path refuses it
    Hl = lm.tightbinding_hamiltonian(ll, V, field=lm.LandauGauge(0.02))
    s.update_solver(Hl, 0.05)
    ctx.set_fused(False)
    try:
        with pytest.raises(L.LMError) as e:
            s.step(st)
        assert e.value.code == L.LM_ERR_NOTSUP
    finally:
        ctx.set_fused(True)
    s.step(st)


def test_compensated_time_dependent_h_through_evolution(lm):
    """Evolution over h(t) with a Landau amplitude and an on-site term that change every step
    (the e2e loop of the kets workload) on a compensated block: the coefficient planes are
    rebuilt every step and the residual is carried across the updates; against the oracle
    stepping the same left-endpoint Hamiltonians with the exact exponent."""
    L, M, dt, n = 32, 4, 0.05, 6
    ol, ll = pair(lm, L, L, (True, True))
    V = o.anderson_disorder(ol.N, 2.0, 21)
    Bt = lambda t: 0.01 * (1.0 + 0.1 * np.sin(t))
    Vt = lambda t: V + 0.05 * np.sin(0.5 * t)
    X = o.random_kets(ol.N, M, 22)
    st = lm.KetBlock(ll, X, precision="c32", compensated=True)
    ev = lm.Evolution(lm.ChebyshevGPU(), lambda t: lm.tightbinding_hamiltonian(ll, Vt(t), field=lm.LandauGauge(Bt(t))),
                      st)
    assert ev.current_states()[0].compensated
    times = [dt * (k + 1) for k in range(n)]
    Y, t0 = X, 0.0
    for moment, t in zip(ev(times), times):
        Ho = o.tightbinding_hamiltonian(ol, field=o.LandauGauge(Bt(t0)), onsite=Vt(t0))
        Y = o.expm_multiply(Ho, t - t0, Y)
        t0 = t
        assert rel(moment.state.to_numpy().astype(np.complex128), Y) <= 3e-6


def test_compensated_plain_config_400_steps(lm):
    """The plain-method lattice at its full length: SquareLattice(256, 256) periodic, Landau
    0.01, Anderson U[-1, 1], 64 complex-Gaussian kets, 400 steps of dt = 0.05 at tol 1e-9 with
    the norm correction every 20 steps, against the FP64 run of the same kets."""
    L, M, steps, dt = 256, 64, 400, 0.05
    lat = lm.SquareLattice(L, L, boundaries={"axis1": True, "axis2": True})
    V = np.random.default_rng(1).uniform(-1, 1, size=lat.N)
    H = lm.tightbinding_hamiltonian(lat, V, field=lm.LandauGauge(0.01))
    X = o.random_kets(lat.N, M, 2)

    def run(st, tol):
        solver = lm.ChebyshevGPU(tol=tol, renorm_every=20)
        cache = solver.evolution_cache(st)
        solver.update_solver(H, dt)
        for _ in range(steps):
            solver.step(st, cache)
        return st

    s64 = run(lm.KetBlock(lat, X, precision="c64"), None)
    r64 = lm.localdensity(s64).values
    J64 = lm.DensityCurrents(H, s64).bond_values()
    del s64
    errs = {}
    for comp in (False, True):
        st = run(lm.KetBlock(lat, X, precision="c32", compensated=comp), 1e-9)
        errs[comp] = {"density": rel(lm.localdensity(st).values, r64),
                      "currents": rel(lm.DensityCurrents(H, st).bond_values(), J64)}
        del st
    print("400 steps, 256^2, 64 kets: plain", errs[False], "compensated", errs[True])
    assert errs[True]["density"] <= 1e-6, errs
    assert errs[True]["currents"] <= 1e-6, errs
    assert errs[True]["currents"] < errs[False]["currents"], errs
