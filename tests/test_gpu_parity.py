"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Bars: bit-exact site/bond indexing and CSC structure; H values to 1e-15 (the device evaluates
sin/cos/acos with CUDA's functions); FP64 evolution to <= 1e-10 relative Frobenius error
against the exact exponent; particle number to 1e-12; the FP32 form to <= 1e-6 relative error
against FP64 on densities and currents.
"""
import math

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import lm_oracle as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lm():
    import lmgpu
    lmgpu.default_context()  # fails loudly without a GPU or without the library
    return lmgpu


def rel(a, b):
    a = np.asarray(a); b = np.asarray(b)
    d = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (d if d > 0 else 1.0)


def pair(lm, Lx, Ly, per=(False, False), tw=(0.0, 0.0)):
    b = {}
    for ax, name in enumerate(("axis1", "axis2")):
        if per[ax]:
            b[name] = float(tw[ax]) if tw[ax] else True
    return o.SquareLattice(Lx, Ly, periodic=per, twist=tw), lm.SquareLattice(Lx, Ly, boundaries=b)


def field_pair(lm, spec):
    """spec: list of (kind, amp, point, gauge) -> (oracle field, lmgpu field)."""
    of, lf = [], []
    for kind, amp, pt, gauge in spec:
        if kind == "landau":
            of.append(o.LandauGauge(amp)); lf.append(lm.LandauGauge(amp))
        elif kind == "sym":
            of.append(o.SymmetricGauge(amp)); lf.append(lm.SymmetricGauge(amp))
        else:
            of.append(o.PointFlux(amp, pt, gauge)); lf.append(lm.PointFlux(amp, pt, gauge))
    if not of:
        return None, None
    if len(of) == 1:
        return of[0], lf[0]
    return o.FieldSum(tuple(of)), lm.FieldSum(lf)


def csc_of(lmH):
    colptr, rowval, nz = lmH.csc()
    N = len(colptr) - 1
    return sp.csc_matrix((nz, rowval - 1, colptr - 1), shape=(N, N)), colptr, rowval


ASSEMBLY_CASES = [
    (10, 10, (False, False), (0, 0), [("pf", 0.2, (5.5, 5.5), "axial")], False),
    (5, 5, (False, False), (0, 0), [("landau", 0.1, None, None)], False),
    (16, 12, (True, True), (0, 0), [("landau", 0.01, None, None)], True),
    (9, 7, (True, True), (0, 0), [("pf", 0.3, (4.5, 3.5), "axial")], False),
    (9, 7, (True, False), (0, 0), [("pf", 0.3, (4.5, 3.5), "singular")], True),
    (6, 8, (False, True), (0, 0.7), [("sym", 0.05, None, None)], True),
    (7, 7, (False, False), (0, 0), [("landau", 0.05, None, None), ("pf", 0.4, (3.5, 4.5), "axial")], True),
    (2, 5, (True, True), (0.3, 0), [("landau", 0.1, None, None)], True),
    (1, 9, (False, False), (0, 0), [], True),
    (8, 8, (False, False), (0, 0), [("pf", 0.25, (4.0, 4.0), "axial")], False),  # flux on a site
]


@pytest.mark.parametrize("Lx,Ly,per,tw,fspec,onsite", ASSEMBLY_CASES)
def test_assembly_matches_oracle(lm, Lx, Ly, per, tw, fspec, onsite):
    ol, ll = pair(lm, Lx, Ly, per, tw)
    of, lf = field_pair(lm, fspec)
    V = o.anderson_disorder(ol.N, 2.0, 11) if onsite else None
    Ho = o.tightbinding_hamiltonian(ol, field=of, onsite=V)
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        Hl = lm.tightbinding_hamiltonian(ll, *( [V] if V is not None else []), field=lf)
    Hg, colptr, rowval = csc_of(Hl)
    # structure bit-exact (same stored entries as the reference's CSC)
    assert np.array_equal(colptr - 1, Ho.indptr)
    assert np.array_equal(rowval - 1, Ho.indices)
    assert np.abs(Hg.data - Ho.data).max() <= 1e-15 * max(1.0, np.abs(Ho.data).max())


def test_nnz_doctests_on_device(lm):
    H = lm.tightbinding_hamiltonian(lm.SquareLattice(4, 4))
    assert csc_of(H)[0].nnz == 48
    H = lm.tightbinding_hamiltonian(lm.SquareLattice(5, 5), field=lm.LandauGauge(0.1))
    assert csc_of(H)[0].nnz == 80


def _step_case(lm, Lx, Ly, per, fspec, M, dt, precision="c64", seed=3):
    ol, ll = pair(lm, Lx, Ly, per)
    of, lf = field_pair(lm, fspec)
    V = o.anderson_disorder(ol.N, 2.0, seed)
    Ho = o.tightbinding_hamiltonian(ol, field=of, onsite=V)
    Hl = lm.tightbinding_hamiltonian(ll, V, field=lf)
    X = o.random_kets(ol.N, M, seed + 1)
    st = lm.KetBlock(ll, X, precision=precision)
    solver = lm.ChebyshevGPU()
    solver.update_solver(Hl, dt)
    solver.step(st)
    Y = st.to_numpy()
    Yo = o.expm_multiply(Ho, dt, X)
    return Y, Yo, solver, st


@pytest.mark.parametrize("Lx,Ly,per,M", [(12, 10, (False, False), 5), (16, 16, (True, True), 8),
                                         (33, 17, (True, False), 3), (7, 300, (False, True), 1)])
def test_ket_step_fp64(lm, Lx, Ly, per, M):
    Y, Yo, _, _ = _step_case(lm, Lx, Ly, per, [("landau", 0.01, None, None)], M, 0.05)
    assert rel(Y, Yo) <= 1e-12


def test_ket_step_pointflux_large_dt(lm):
    Y, Yo, solver, st = _step_case(lm, 10, 10, (False, False), [("pf", 0.2, (5.5, 5.5), "axial")], 4, 1.7)
    K, a, b = solver.order(st)
    assert K > 10
    assert rel(Y, Yo) <= 1e-11


def test_backward_step_round_trip(lm):
    ol, ll = pair(lm, 20, 20, (True, True))
    V = o.anderson_disorder(ol.N, 2.0, 5)
    Hl = lm.tightbinding_hamiltonian(ll, V, field=lm.LandauGauge(0.02))
    X = o.random_kets(ol.N, 6, 9)
    st = lm.KetBlock(ll, X)
    s = lm.ChebyshevGPU()
    for dt in (0.05, 0.05, 0.05):
        s.update_solver(Hl, dt); s.step(st)
    for dt in (-0.05, -0.05, -0.05):
        s.update_solver(Hl, dt); s.step(st)
    assert rel(st.to_numpy(), X) <= 1e-12


def test_density_matrix_step_fp64(lm):
    ol, ll = pair(lm, 10, 10)
    Ho = o.tightbinding_hamiltonian(ol, field=o.PointFlux(0.13, (5.5, 5.5)))
    Hl = lm.tightbinding_hamiltonian(ll, field=lm.PointFlux(0.13, (5.5, 5.5)))
    P0, _, _ = o.densitymatrix(o.tightbinding_hamiltonian(ol), mu=0.0)
    st = lm.DensityMatrix(ll, P0)
    s = lm.ChebyshevGPU()
    s.update_solver(Hl, 0.1)
    s.step(st)
    U = o.expm_exact(Ho, 0.1)
    Pref = U @ P0 @ U.conj().T
    assert rel(st.to_numpy(), Pref) <= 1e-12
    assert abs(st.trace() - np.trace(P0).real) <= 1e-12 * max(1, abs(np.trace(P0)))


def test_config1_full_evolution(lm):
    """SquareLattice(10,10), open, PointFlux(B(t),(5.5,5.5)) with B ramped 0 -> 0.2 over
    tau = 10, dt = 0.1 to t = 20 (200 steps), dense P_0 at mu = 0; localdensity and currents
    every step against the oracle evolved with the exact exponent."""
    ol, ll = pair(lm, 10, 10)
    tau = 10.0
    B = lambda t: 0.2 * min(t, tau) / tau
    h_o = lambda t: o.tightbinding_hamiltonian(ol, field=o.PointFlux(B(t), (5.5, 5.5)))
    h_l = lambda t: lm.tightbinding_hamiltonian(ll, field=lm.PointFlux(B(t), (5.5, 5.5)))
    P0, _, _ = o.densitymatrix(h_o(0.0), mu=0.0)  # the shared P_0 (degenerate E = 0 fixed here)
    times = [round(0.1 * k, 10) for k in range(201)]
    src, dst = ll.bonds()
    # truncation 1e-14: the per-step series error stays below the 1e-12 particle-number bar
    ev = lm.Evolution(lm.ChebyshevGPU(tol=1e-14), h_l, lm.DensityMatrix(ll, P0))
    orc = o.evolve(h_o, P0, times, o.OracleCachedExpSolver(exact=True))
    tr0 = np.trace(P0).real
    worst = {"P": 0.0, "rho": 0.0, "J": 0.0, "tr": 0.0}
    Js, Jos = [], []
    for k, (mom, (Ho, Po, to)) in enumerate(zip(ev(times), orc)):
        P, H, t = mom
        assert t == pytest.approx(to, abs=1e-12)
        if k % 20 == 0 or k == 200:
            worst["P"] = max(worst["P"], rel(P.to_numpy(), Po))
        rho = lm.localdensity(P).values
        Js.append(lm.DensityCurrents(H, P).bond_values())
        Jos.append(o.bond_currents(Ho, Po, src, dst, is_density=True))
        worst["rho"] = max(worst["rho"], rel(rho, o.localdensity(Po)))
        worst["tr"] = max(worst["tr"], abs(P.trace() - tr0))
    # the currents vanish exactly while B(t) = 0, so their relative Frobenius error is taken
    # over the whole (moments x bonds) series
    worst["J"] = rel(np.array(Js), np.array(Jos))
    print("config1 worst errors:", worst)
    assert worst["P"] <= 1e-10, worst
    assert worst["rho"] <= 1e-10, worst
    assert worst["J"] <= 1e-10, worst
    assert worst["tr"] <= 1e-12 * tr0, worst


def test_ket_block_readouts_match_projector(lm):
    """Currents/densities of a weighted ket block equal those of P = sum w |psi><psi|."""
    ol, ll = pair(lm, 9, 8, (True, False))
    Hl = lm.tightbinding_hamiltonian(ll, field=lm.LandauGauge(0.07))
    Ho = o.tightbinding_hamiltonian(ol, field=o.LandauGauge(0.07))
    X = o.random_kets(ol.N, 7, 2)
    w = np.linspace(0.2, 1.0, 7)
    st = lm.KetBlock(ll, X, weights=w)
    P = (X * w) @ X.conj().T
    src, dst = ll.bonds()
    assert rel(lm.localdensity(st).values, o.localdensity(P)) <= 1e-14
    assert rel(lm.DensityCurrents(Hl, st).bond_values(), o.bond_currents(Ho, P, src, dst, is_density=True)) <= 1e-13
    dm = lm.DensityMatrix(ll, P)
    assert rel(lm.DensityCurrents(Hl, dm).bond_values(), lm.DensityCurrents(Hl, st).bond_values()) <= 1e-13
    assert abs(st.trace() - np.trace(P).real) <= 1e-12


def test_fp32_form_error_vs_fp64(lm):
    """Chosen form: c32 recurrence with FP64 coefficients/reductions, against the FP64 run."""
    ol, ll = pair(lm, 48, 48, (True, True))
    V = o.anderson_disorder(ol.N, 2.0, 21)
    Hl = lm.tightbinding_hamiltonian(ll, V, field=lm.LandauGauge(0.01))
    X = o.random_kets(ol.N, 64, 4, kind="phase")
    s64 = lm.KetBlock(ll, X, precision="c64")
    s32 = lm.KetBlock(ll, X, precision="c32")
    solver = lm.ChebyshevGPU(renorm_every=10)
    ev64 = lm.Evolution(solver, Hl, s64)
    ev32 = lm.Evolution(solver, Hl, s32)
    times = [0.05 * k for k in range(101)]
    for _ in ev64(times):
        pass
    for _ in ev32(times):
        pass
    a64 = ev64.current_states()[0]
    a32 = ev32.current_states()[0]
    r64, r32 = lm.localdensity(a64).values, lm.localdensity(a32).values
    J64 = lm.DensityCurrents(Hl, a64).bond_values()
    J32 = lm.DensityCurrents(Hl, a32).bond_values()
    assert rel(r32, r64) <= 1e-6
    assert rel(J32, J64) <= 1e-5  # currents are differences of nearby amplitudes
    assert np.abs(a32.norms() - 1).max() <= 1e-6


def test_edge_cases(lm):
    # single ket on a 1 x N chain, t1 = 0 evolution is a pure phase
    ol, ll = pair(lm, 1, 37)
    V = o.anderson_disorder(37, 2.0, 1)
    H0 = lm.Hamiltonian(ll, 0.0, None, V)
    x = o.random_kets(37, 1, 1)[:, 0]
    st = lm.Ket(ll, x)
    s = lm.ChebyshevGPU()
    s.update_solver(H0, 0.3)
    s.step(st)
    assert rel(st.to_numpy()[:, 0], np.exp(-0.3j * V) * x) <= 1e-12
    # N not a multiple of the block size, M not a multiple of the ket tile
    Y, Yo, _, _ = _step_case(lm, 13, 11, (False, True), [("landau", 0.03, None, None)], 7, 0.2)
    assert rel(Y, Yo) <= 1e-12
    # two-site periodic axis (both bonds join the same pair)
    Y, Yo, _, _ = _step_case(lm, 2, 9, (True, True), [("landau", 0.1, None, None)], 3, 0.1)
    assert rel(Y, Yo) <= 1e-12
    # dt = 0 in the iterator yields the initial state untouched
    ev = lm.Evolution(lambda t: H0, lm.Ket(ll, x))
    m0 = next(iter(ev([0.0])))
    assert np.array_equal(m0.state.to_numpy()[:, 0], x)
    # errors are reported, not silently ignored
    small = lm.KetBlock(lm.SquareLattice(3, 3), np.zeros((9, 2)))
    s.update_solver(lm.tightbinding_hamiltonian(lm.SquareLattice(4, 4)), 0.1)
    with pytest.raises(lm.LMError):
        s.step(small)  # state and lattice sizes differ
    with pytest.raises(ValueError):
        small.renormalize(np.ones(1))


@pytest.mark.parametrize("precision", ["c64", "c32"])
@pytest.mark.parametrize("n", [1000, 1001])
def test_renormalize(lm, precision, n):
    """lm_state_renormalize rescales every ket to its target FP64 norm without waiting for the
    device; the target buffer is copied during the call (overwriting it afterwards changes
    nothing).  Even n takes the 16-byte site-pair path for c32."""
    lat = lm.SquareLattice(n, 1)
    X = o.random_kets(n, 37, 5)
    st = lm.KetBlock(lat, X, precision=precision)
    target = np.linspace(0.5, 2.0, 37)
    keep = target.copy()
    st.renormalize(target)
    target[:] = 7.0
    got = st.norms()
    tol = 1e-14 if precision == "c64" else 1e-6
    assert np.abs(got - keep).max() <= tol * keep.max()
    ref = X / np.linalg.norm(X, axis=0) * keep
    assert rel(st.to_numpy().astype(np.complex128), ref) <= (1e-14 if precision == "c64" else 1e-6)


FUSED_CASES = [
    (256, 256, (True, True), [("landau", 0.01, None, None)], 11, 0.05),
    (10, 10, (False, False), [("pf", 0.2, (5.5, 5.5), "axial")], 9, 0.1),
    (1, 37, (False, False), [], 3, 0.05),
    (2, 9, (True, True), [("landau", 0.1, None, None)], 8, 0.05),
    (70, 45, (False, True), [("pf", 0.3, (35.5, 20.5), "singular")], 17, 0.08),
    (23, 130, (True, False), [("sym", 0.02, None, None)], 5, 0.12),
    (40, 40, (True, True), [("landau", 0.03, None, None)], 4, 0.4),   # K > 8: per-order path
]


@pytest.mark.parametrize("Lx,Ly,per,fspec,M,dt", FUSED_CASES)
def test_fused_c32_step(lm, Lx, Ly, per, fspec, M, dt):
    """The temporally blocked c32 step agrees with the per-order c32 path and with FP64."""
    ol, ll = pair(lm, Lx, Ly, per)
    of, lf = field_pair(lm, fspec)
    V = o.anderson_disorder(ol.N, 2.0, 13)
    Ho = o.tightbinding_hamiltonian(ol, field=of, onsite=V)
    Hl = lm.tightbinding_hamiltonian(ll, V, field=lf)
    X = o.random_kets(ol.N, M, 17)
    ctx = lm.default_context()
    outs = {}
    try:
        for fused in (True, False):
            ctx.set_fused(fused)
            st = lm.KetBlock(ll, X, precision="c32")
            s = lm.ChebyshevGPU()
            s.update_solver(Hl, dt)
            s.step(st)
            outs[fused] = st.to_numpy().astype(np.complex128)
    finally:
        ctx.set_fused(True)
    Yo = o.expm_multiply(Ho, dt, X)
    assert rel(outs[True], Yo) <= 2e-6
    assert rel(outs[False], Yo) <= 2e-6
    assert rel(outs[True], outs[False]) <= 2e-6


@pytest.mark.parametrize("fused", [True, False])
def test_fp32_long_run_keeps_norm(lm, fused):
    """400 FP32 steps with no renormalisation.  The step carries second FP32 words for its
    scalar constants (e^{-ib dt} c_0, e^{-ib dt}, c_1), so their rounding does not compound;
    without them the norms drift by ~1e-5 here.  The on-site offset 0.7 makes e^{-ib dt} a
    full complex phase."""
    L, M, dt, nsteps = 64, 16, 0.05, 400
    ol, ll = pair(lm, L, L)
    rng = np.random.default_rng(21)
    V = rng.uniform(-0.1, 0.1, L * L) + 0.7
    Hl = lm.tightbinding_hamiltonian(ll, V, field=lm.PointFlux(0.1, (32.5, 32.5)))
    X = o.random_kets(ol.N, M, 22)
    X /= np.linalg.norm(X, axis=0)
    ctx = lm.default_context()
    try:
        ctx.set_fused(fused)
        s32, s64 = lm.ChebyshevGPU(tol=1e-9), lm.ChebyshevGPU(tol=1e-13)
        st32 = lm.KetBlock(ll, X, precision="c32")
        st64 = lm.KetBlock(ll, X, precision="c64")
        s32.update_solver(Hl, dt)
        s64.update_solver(Hl, dt)
        for _ in range(nsteps):
            s32.step(st32)
            s64.step(st64)
    finally:
        ctx.set_fused(True)
    n32 = st32.norms()
    n64 = st64.norms()
    rho32 = lm.localdensity(st32).values
    rho64 = lm.localdensity(st64).values
    print(f"fused={fused}: max |norm-1| c32 {np.abs(n32 - 1).max():.2e} c64 {np.abs(n64 - 1).max():.2e}, "
          f"density rel {rel(rho32, rho64):.2e}")
    assert np.abs(n64 - 1).max() <= 1e-12
    assert np.abs(n32 - 1).max() <= 5e-7
    assert rel(rho32, rho64) <= 1e-6


@pytest.mark.parametrize("form", ["c32-fused", "c32-per-order", "c64", "c64-density"])
def test_real_x_hops_bit_identical(lm, form):
    """Landau-gauge x-hops are real, so the kernels skip their imaginary parts (the fused c32
    step and the per-order kernels of either precision).  Adding a zero point flux keeps H
    identical but forces the general (complex x-hop) kernels: the two results must agree bit
    for bit, kets and density matrices (whose row pass uses conj(H))."""
    L, M, dt = (16, 24, 0.05) if form == "c64-density" else (64, 24, 0.05)
    ll = lm.SquareLattice(L, L, boundaries={"axis1": True, "axis2": True})
    V = o.anderson_disorder(L * L, 2.0, 31)
    X = o.random_kets(L * L, M, 32)
    P = X @ X.conj().T / M
    ctx = lm.default_context()
    outs = []
    try:
        ctx.set_fused(form != "c32-per-order")
        for field in (lm.LandauGauge(0.02),
                      lm.FieldSum([lm.LandauGauge(0.02), lm.PointFlux(0.0, (10.5, 20.5), "singular")])):
            H = lm.tightbinding_hamiltonian(ll, V, field=field)
            if form == "c64-density":
                st = lm.DensityMatrix(ll, P)
            else:
                st = lm.KetBlock(ll, X, precision="c64" if form == "c64" else "c32")
            s = lm.ChebyshevGPU()
            s.update_solver(H, dt)
            for _ in range(3):
                s.step(st)
            outs.append(st.to_numpy())
    finally:
        ctx.set_fused(True)
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("tw", [(0.7, 0.0), (0.0, 1.3), (0.4, -0.9)])
def test_fused_twisted_boundaries(lm, tw):
    """Twisted periodic axes (complex seam hops, so the general x-hop kernel) through the fused
    c32 step, against the per-order path and the exact exponent; Landau field included."""
    ol, ll = pair(lm, 48, 70, (True, True), tw)
    V = o.anderson_disorder(ol.N, 1.0, 19)
    Ho = o.tightbinding_hamiltonian(ol, field=o.LandauGauge(0.02), onsite=V)
    Hl = lm.tightbinding_hamiltonian(ll, V, field=lm.LandauGauge(0.02))
    X = o.random_kets(ol.N, 6, 23)
    ctx = lm.default_context()
    outs = {}
    try:
        for fused in (True, False):
            ctx.set_fused(fused)
            st = lm.KetBlock(ll, X, precision="c32")
            s = lm.ChebyshevGPU()
            s.update_solver(Hl, 0.07)
            for _ in range(2):
                s.step(st)
            outs[fused] = st.to_numpy().astype(np.complex128)
    finally:
        ctx.set_fused(True)
    Y = o.expm_multiply(Ho, 0.07, o.expm_multiply(Ho, 0.07, X))
    assert rel(outs[True], Y) <= 2e-6
    assert rel(outs[True], outs[False]) <= 2e-6


STREAM_CASES = [
    # (Lx, Ly, periodic x, periodic y, field, dt, kets): K from the FP32 default tolerance
    (64, 64, True, True, "landau", 0.05, 24),     # K = 6, real x-hops, 2 strips
    (256, 256, True, True, "landau", 0.05, 5),    # the benchmark lattice, 5 strips, 2 x segments
    (47, 130, False, False, "landau", 0.05, 9),   # open, uneven edge strips
    (40, 70, True, False, "pointflux", 0.03, 7),  # complex x-hops (K <= 5)
    (33, 64, False, True, "pointflux", 0.03, 3),
    (20, 200, True, True, "landau", 0.05, 1),     # one ket, many strips
    (24, 128, True, True, "landau", 0.05, 7),     # 3 strips on a 128-row ring
    (16, 512, True, True, "landau", 0.05, 3),     # 10 strips on a 512-row ring
    (30, 128, False, False, "landau", 0.05, 5),   # open y, edge strips on both edges
    (21, 256, False, True, "pointflux", 0.03, 4), # complex hops on a periodic y axis
    (19, 1024, True, True, "landau", 0.05, 2),    # a tall ring
    (40, 64, True, True, "pointflux", 0.03, 5),   # periodic 64 rows, complex hops: strips
    (41, 30, False, False, "landau", 0.05, 5),    # Ly < 64 open: lanes outside the lattice
    (33, 50, True, False, "landau", 0.05, 3),
    (15, 64, True, True, "landau", 0.05, 6),      # Lx = 2K + 3 (K = 6): the smallest streaming Lx
    (14, 64, True, True, "landau", 0.05, 6),      # Lx = 2K + 2: region form
    (20, 2, True, True, "landau", 0.05, 5),       # a 2-row periodic ring (both y-bonds join one pair)
    (18, 4, False, True, "landau", 0.05, 4),      # a 4-row periodic ring, open x
    (64, 31, True, True, "landau", 0.05, 4),      # odd Ly: region form only
    (12, 64, True, True, "landau", 0.05, 4),      # Lx < 2K + 3: region form only
]


@pytest.mark.parametrize("case", STREAM_CASES, ids=[f"{c[0]}x{c[1]}-{c[4]}-M{c[6]}" for c in STREAM_CASES])
def test_stream_form_bit_identical_to_region(lm, case):
    """The x-streaming form of the fused step performs every site-order with the same FMAs as
    the region form, so three steps agree bit for bit; both against the exact exponent."""
    Lx, Ly, px, py, fk, dt, M = case
    ol, ll = pair(lm, Lx, Ly, (px, py))
    V = o.anderson_disorder(ol.N, 1.0, 41)
    if fk == "landau":
        fo, fl = o.LandauGauge(0.02), lm.LandauGauge(0.02)
    else:
        pt = (Lx / 2 + 0.5, Ly / 2 + 0.5)
        fo, fl = o.PointFlux(0.3, pt), lm.PointFlux(0.3, pt)
    Ho = o.tightbinding_hamiltonian(ol, field=fo, onsite=V)
    Hl = lm.tightbinding_hamiltonian(ll, V, field=fl)
    X = o.random_kets(ol.N, M, 42)
    ctx = lm.default_context()
    outs = {}
    eligible = Ly % 2 == 0
    try:
        for form in (True, False):
            ctx.set_stream_form(form)
            st = lm.KetBlock(ll, X, precision="c32")
            s = lm.ChebyshevGPU()
            s.update_solver(Hl, dt)
            n0 = ctx.stream_launches()
            for _ in range(3):
                s.step(st)
            ran = ctx.stream_launches() - n0
            if form:
                K = s.order(st)[0]
                expect = eligible and Lx >= 2 * K + 3 and K <= (6 if fk == "landau" else 5)
                assert ran == (3 if expect else 0)
            else:
                assert ran == 0
            outs[form] = st.to_numpy()
    finally:
        ctx.set_stream_form(True)
    assert np.array_equal(outs[True], outs[False])
    Y = X
    for _ in range(3):
        Y = o.expm_multiply(Ho, dt, Y)
    assert rel(outs[True].astype(np.complex128), Y) <= 3e-6


def test_stream_form_follows_time_dependent_h(lm):
    """H(t) changes every step (Landau field ramp and on-site term): the streaming kernel's packed
    coefficient planes must be rebuilt for every new H.  c32 kets through Evolution against the
    oracle stepping the same left-endpoint Hamiltonians with the exact exponent."""
    L, M, dt, nsteps = 32, 6, 0.05, 6
    ol, ll = pair(lm, L, L, (True, True))
    rng = np.random.default_rng(77)
    Vs = [rng.uniform(-1, 1, L * L) for _ in range(nsteps)]
    B = lambda t: 0.005 + 0.02 * t
    k_of = lambda t: min(int(round(t / dt)), nsteps - 1)
    h_l = lambda t: lm.tightbinding_hamiltonian(ll, Vs[k_of(t)], field=lm.LandauGauge(B(t)))
    h_o = lambda t: o.tightbinding_hamiltonian(ol, field=o.LandauGauge(B(t)), onsite=Vs[k_of(t)])
    X = o.random_kets(ol.N, M, 78)
    ctx = lm.default_context()
    n0 = ctx.stream_launches()
    ev = lm.Evolution(lm.ChebyshevGPU(), h_l, lm.KetBlock(ll, X, precision="c32"))
    times = [dt * k for k in range(1, nsteps + 1)]
    Y = X
    t0 = 0.0
    for moment, t in zip(ev(times), times):
        Y = o.expm_multiply(h_o(t0), t - t0, Y)
        t0 = t
        assert rel(moment.state.to_numpy().astype(np.complex128), Y) <= 5e-6
    assert ctx.stream_launches() - n0 == nsteps


def _random_stream_cases(n, seed=2026):
    rng = np.random.default_rng(seed)
    cases = []
    for _ in range(n):
        Lx = int(rng.integers(15, 70))
        Ly = int(rng.integers(2, 140))
        px, py = bool(rng.integers(0, 2)), bool(rng.integers(0, 2))
        tw = (float(rng.uniform(-1, 1)) if (px and rng.random() < 0.3) else 0.0,
              float(rng.uniform(-1, 1)) if (py and rng.random() < 0.3) else 0.0)
        fk = ["landau", "pointflux", "sym"][int(rng.integers(0, 3))]
        dt = float(rng.choice([0.01, 0.02, 0.035, 0.05]))
        M = int(rng.integers(1, 12))
        cases.append((Lx, Ly, px, py, tw, fk, dt, M))
    return cases


@pytest.mark.parametrize("case", _random_stream_cases(16), ids=lambda c: f"{c[0]}x{c[1]}-{c[5]}")
def test_stream_form_random_geometries(lm, case):
    """Seeded random shapes, boundaries (with twists), fields and step sizes (so K = 2..6): the
    fused step in its streaming form (where eligible) and in its region form agree bit for bit,
    and both follow the exact exponent."""
    Lx, Ly, px, py, tw, fk, dt, M = case
    ol, ll = pair(lm, Lx, Ly, (px, py), tw)
    V = o.anderson_disorder(ol.N, 1.0, Lx * 1000 + Ly)
    if fk == "landau":
        fo, fl = o.LandauGauge(0.02), lm.LandauGauge(0.02)
    elif fk == "sym":
        fo, fl = o.SymmetricGauge(0.015), lm.SymmetricGauge(0.015)
    else:
        pt = (Lx / 2 + 0.3, Ly / 2 + 0.7)
        fo, fl = o.PointFlux(0.25, pt), lm.PointFlux(0.25, pt)
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        Ho = o.tightbinding_hamiltonian(ol, field=fo, onsite=V)
        Hl = lm.tightbinding_hamiltonian(ll, V, field=fl)
    X = o.random_kets(ol.N, M, 3)
    ctx = lm.default_context()
    outs = {}
    try:
        for form in (True, False):
            ctx.set_stream_form(form)
            st = lm.KetBlock(ll, X, precision="c32")
            s = lm.ChebyshevGPU()
            s.update_solver(Hl, dt)
            for _ in range(2):
                s.step(st)
            outs[form] = st.to_numpy()
    finally:
        ctx.set_stream_form(True)
    assert np.array_equal(outs[True], outs[False])
    Y = o.expm_multiply(Ho, dt, o.expm_multiply(Ho, dt, X))
    assert rel(outs[True].astype(np.complex128), Y) <= 3e-6
