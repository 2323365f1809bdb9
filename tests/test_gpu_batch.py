"""Batches of uneven lattices (lm_batch_*) against the oracle and against single-lattice steps."""
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
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def instance(lm, L, B, W, seed, per=False):
    """One instance of the batching workload: LxL lattice, point flux through the plaquette
    centre nearest the lattice centre, Anderson disorder of width W."""
    rng = np.random.default_rng(seed)
    V = rng.uniform(-W / 2, W / 2, size=L * L)
    pt = (L // 2 + 0.5, L // 2 + 0.5)
    ol = o.SquareLattice(L, L, periodic=(per, per))
    ll = lm.SquareLattice(L, L, boundaries={"axis1": per, "axis2": per})
    gauge = "singular" if per else "axial"
    Ho = o.tightbinding_hamiltonian(ol, field=o.PointFlux(B, pt, gauge), onsite=V)
    Hl = lm.tightbinding_hamiltonian(ll, V, field=lm.PointFlux(B, pt, gauge))
    return ol, ll, Ho, Hl


SIZES = [5, 8, 11, 16, 23, 7, 30]


@pytest.mark.parametrize("precision,graph", [("c64", True), ("c32", True), ("c32", False)])
def test_batch_density_matrices(lm, precision, graph):
    rng = np.random.default_rng(4)
    batch = lm.Batch("density", precision)
    batch.set_graph(graph)
    refs = []
    for i, L in enumerate(SIZES):
        ol, ll, Ho, Hl = instance(lm, L, rng.uniform(0, 0.3), rng.uniform(0, 3), 100 + i)
        P0, _, _ = o.densitymatrix(Ho, mu=0.0)
        st = lm.DensityMatrix(ll, P0, precision=precision)
        batch.add(Hl, st)
        refs.append((Ho, P0, st))
    batch.update(0.1)
    info = batch.info()
    assert info["instances"] == len(SIZES)
    assert info["config"] == (0 if precision == "c32" else 2)
    steps = 4
    for _ in range(steps):
        batch.step()
    tol = 1e-10 if precision == "c64" else 5e-6
    for Ho, P0, st in refs:
        U = o.expm_exact(Ho, 0.1)
        P = P0
        for _ in range(steps):
            P = U @ P @ U.conj().T
        assert rel(st.to_numpy(), P) <= tol
        assert abs(st.trace() - np.trace(P0).real) <= (1e-11 if precision == "c64" else 2e-5) * np.trace(P0).real


def test_batch_ket_blocks_fused_vs_per_order(lm):
    rng = np.random.default_rng(9)
    outs = {}
    for cfg in (0, 2, 3):
        batch = lm.Batch("kets", "c32")
        sts = []
        for i, L in enumerate([12, 40, 65, 9]):
            ol, ll, Ho, Hl = instance(lm, L, 0.1 + 0.05 * i, 1.0, 200 + i, per=(i % 2 == 0))
            X = o.random_kets(ol.N, 5 + i, 300 + i)
            st = lm.KetBlock(ll, X, precision="c32")
            batch.add(Hl, st)
            sts.append((Ho, X, st))
        batch.update(0.05)
        batch.set_config(cfg)
        for _ in range(3):
            batch.step()
        outs[cfg] = [st.to_numpy().astype(np.complex128) for _, _, st in sts]
        for Ho, X, st in sts:
            Y = X
            for _ in range(3):
                Y = o.expm_multiply(Ho, 0.05, Y)
            assert rel(st.to_numpy().astype(np.complex128), Y) <= 3e-6
    for a, b in zip(outs[0], outs[2]):
        assert rel(a, b) <= 3e-6
    for a, b in zip(outs[2], outs[3]):
        assert rel(a, b) <= 1e-6


def test_batch_graph_replay_is_deterministic(lm):
    res = []
    for graph in (True, False):
        batch = lm.Batch("kets", "c32")
        batch.set_graph(graph)
        sts = []
        for i, L in enumerate([33, 17, 50]):
            _, ll, _, Hl = instance(lm, L, 0.2, 2.0, 400 + i)
            st = lm.KetBlock(ll, o.random_kets(L * L, 20, 500 + i), precision="c32")
            batch.add(Hl, st)
            sts.append(st)
        batch.update(0.1)
        for _ in range(5):
            batch.step()
        res.append([s.to_numpy() for s in sts])
    for a, b in zip(*res):
        assert np.array_equal(a, b)


def test_batch_tuner_leaves_states_untouched(lm, tmp_path):
    batch = lm.Batch("density", "c32")
    sts = []
    for i, L in enumerate([10, 21, 14]):
        ol, ll, Ho, Hl = instance(lm, L, 0.15, 1.5, 600 + i)
        P0, _, _ = o.densitymatrix(Ho, mu=0.0)
        st = lm.DensityMatrix(ll, P0, precision="c32")
        batch.add(Hl, st)
        sts.append((Ho, P0, st))
    batch.update(0.1)
    before = [st.to_numpy().copy() for _, _, st in sts]
    res = batch.tune(steps=2, cache_file=str(tmp_path / "tune.json"))
    assert res["config"] in (0, 1, 2, 3)
    assert res["ms_per_step"][lm.batch.CONFIG_NAMES[0]] is not None
    for b0, (_, _, st) in zip(before, sts):
        assert np.array_equal(b0, st.to_numpy())
    # the cache file answers the second time without timing
    assert batch.tune(cache_file=str(tmp_path / "tune.json"))["config"] == res["config"]
    batch.step()
    for Ho, P0, st in sts:
        U = o.expm_exact(Ho, 0.1)
        assert rel(st.to_numpy(), U @ P0 @ U.conj().T) <= 2e-6


def test_batch_rejects_mismatches(lm):
    batch = lm.Batch("density", "c32")
    ll = lm.SquareLattice(4, 4)
    H = lm.tightbinding_hamiltonian(ll)
    with pytest.raises(ValueError):
        batch.add(H, lm.KetBlock(ll, np.ones((16, 2)), precision="c32"))
    with pytest.raises(lm.LMError):
        batch.update(0.1)  # empty batch


@pytest.mark.parametrize("precision", ["c64", "c32"])
@pytest.mark.parametrize("dt", [0.1, 0.13])
def test_panelled_batch_is_bit_identical(lm, precision, dt):
    """Column panels (in place, panel scratch, in-place conjugate transposes) give exactly the
    per-order results of the full-buffer path, for even and odd K, and match the oracle."""
    rng = np.random.default_rng(12)
    outs = []
    for panel in (0, 7):
        batch = lm.Batch("density", precision)
        batch.set_config(2)
        batch.set_panel(panel)
        sts = []
        for i, L in enumerate([5, 8, 11, 3]):
            ol, ll, Ho, Hl = instance(lm, L, 0.1 + 0.05 * i, 1.5, 700 + i)
            P0, _, _ = o.densitymatrix(Ho, mu=0.0)
            st = lm.DensityMatrix(ll, P0, precision=precision)
            batch.add(Hl, st)
            sts.append((Ho, P0, st))
        batch.update(dt)
        for _ in range(3):
            batch.step()
        outs.append([st.to_numpy() for _, _, st in sts])
        if panel:
            for Ho, P0, st in sts:
                U = o.expm_exact(Ho, dt)
                P = P0
                for _ in range(3):
                    P = U @ P @ U.conj().T
                assert rel(st.to_numpy(), P) <= (1e-10 if precision == "c64" else 5e-6)
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


def test_panelled_ket_batch(lm):
    rng = np.random.default_rng(13)
    batch = lm.Batch("kets", "c64")
    batch.set_panel(4)
    sts = []
    for i, L in enumerate([9, 14]):
        ol, ll, Ho, Hl = instance(lm, L, 0.2, 1.0, 800 + i)
        X = o.random_kets(ol.N, 10 + i, 900 + i)
        st = lm.KetBlock(ll, X)
        batch.add(Hl, st)
        sts.append((Ho, X, st))
    batch.update(0.07)
    for _ in range(2):
        batch.step()
    for Ho, X, st in sts:
        Y = o.expm_multiply(Ho, 0.07, o.expm_multiply(Ho, 0.07, X))
        assert rel(st.to_numpy(), Y) <= 1e-10
