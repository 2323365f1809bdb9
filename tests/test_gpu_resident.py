"""The lattice-resident form of a c32 batch's fused pass (csrc/lmgpu_resident.cu).

A lattice of up to 4608 sites runs on one CTA (smaller ones several kets per CTA), one of up to
9216 sites on a cluster of two CTAs.  Bars: bit-identical to the region form (the kernel
repeats its per-site operation order) on every geometry class, open, periodic and twisted; the
oracle's exact exponent (c32 bar 5e-6, as for the other fused forms), including Chebyshev orders
above the region form's limit of 8 and lattices on a cluster; density matrices (U P U^dagger).
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
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def instance(lm, Lx, Ly, B, W, seed, per=(False, False), twist=(0.0, 0.0)):
    """Lx x Ly lattice with a point flux through the plaquette nearest the centre and Anderson
    disorder of width W (the batching workload's instances, any shape and boundary)."""
    rng = np.random.default_rng(seed)
    V = rng.uniform(-W / 2, W / 2, size=Lx * Ly)
    pt = (Lx // 2 + 0.5, Ly // 2 + 0.5)
    ol = o.SquareLattice(Lx, Ly, periodic=per, twist=twist)
    bnd = {}
    for ax, name in enumerate(("axis1", "axis2")):
        if per[ax]:
            bnd[name] = twist[ax] if twist[ax] else True
    ll = lm.SquareLattice(Lx, Ly, boundaries=bnd)
    gauge = "singular" if any(per) else "axial"
    Ho = o.tightbinding_hamiltonian(ol, field=o.PointFlux(B, pt, gauge), onsite=V)
    Hl = lm.tightbinding_hamiltonian(ll, V, field=lm.PointFlux(B, pt, gauge))
    return ol, ll, Ho, Hl


# (Lx, Ly, periodic, twist, kets): one CTA with several kets per CTA, one CTA, a cluster of two,
# open, periodic (Lx a multiple of 3, Ly of 4) and twisted, ragged block edges
GEOMS = [
    (16, 16, (False, False), (0.0, 0.0), 30),
    (5, 9, (False, False), (0.0, 0.0), 40),
    (24, 20, (True, True), (0.0, 0.0), 17),
    (30, 28, (True, False), (0.3, 0.0), 9),
    (41, 52, (False, True), (0.0, -0.2), 6),
    (66, 66, (False, False), (0.0, 0.0), 3),
    (67, 67, (False, False), (0.0, 0.0), 3),
    (96, 96, (False, False), (0.0, 0.0), 2),
    (81, 92, (True, True), (0.4, 0.7), 2),
    (1, 30, (False, False), (0.0, 0.0), 5),
    (30, 1, (False, False), (0.0, 0.0), 5),
]


def ket_batch(lm, dt, geoms=GEOMS, seed=5):
    rng = np.random.default_rng(seed)
    batch = lm.Batch("kets", "c32")
    insts = []
    for i, (Lx, Ly, per, tw, M) in enumerate(geoms):
        ol, ll, Ho, Hl = instance(lm, Lx, Ly, rng.uniform(0, 0.3), rng.uniform(0, 3), 500 + i, per, tw)
        X = o.random_kets(ol.N, M, 600 + i)
        st = lm.KetBlock(ll, X, precision="c32")
        batch.add(Hl, st)
        insts.append((Ho, X, st))
    batch.update(dt)
    return batch, insts


def run(lm, resident, dt, steps, geoms=GEOMS):
    ctx = lm.default_context()
    ctx.set_resident_form(resident)
    try:
        batch, insts = ket_batch(lm, dt, geoms)
        assert batch.info()["config"] == 0
        for _ in range(steps):
            batch.step()
        return batch, insts, [st.to_numpy() for _, _, st in insts]
    finally:
        ctx.set_resident_form(True)


@pytest.mark.parametrize("dt", [0.02, 0.08])
def test_resident_is_bit_identical_to_region_form(lm, dt):
    _, _, a = run(lm, True, dt, 3)
    _, _, b = run(lm, False, dt, 3)
    for i, (x, y) in enumerate(zip(a, b)):
        assert np.array_equal(x, y), (GEOMS[i], float(np.abs(x - y).max()))


@pytest.mark.parametrize("dt", [0.1, 0.45])
def test_resident_vs_oracle(lm, dt):
    """dt = 0.45 needs K > 8: only the resident form takes it in one fused pass."""
    batch, insts, outs = run(lm, True, dt, 2)
    K = batch.info()["K"]
    if dt > 0.4:
        assert K > 8, K
    for (Ho, X, _), got in zip(insts, outs):
        Y = X
        for _ in range(2):
            Y = o.expm_multiply(Ho, dt, Y)
        assert rel(got.astype(np.complex128), Y) <= 5e-6, K


def test_resident_density_matrices(lm):
    """U P U^dagger with P = densitymatrix(h, mu = 0): column pass, conjugate transpose, column pass.
    The 70 x 70 lattice (4900 sites) runs on a cluster of two CTAs; it is compared with the region
    form bit for bit, the smaller ones also with the oracle's exact exponent."""
    rng = np.random.default_rng(8)
    insts = []
    for i, (L, per) in enumerate([(12, True), (19, False), (36, True), (44, False), (70, False)]):
        ol, ll, Ho, Hl = instance(lm, L, L, rng.uniform(0, 0.3), rng.uniform(0, 3), 700 + i, (per, per))
        P0, _, _ = o.densitymatrix(Ho, mu=0.0)
        insts.append((Ho, Hl, ll, P0))
    outs = {}
    for resident in (True, False):
        lm.default_context().set_resident_form(resident)
        try:
            batch = lm.Batch("density", "c32")
            sts = []
            for Ho, Hl, ll, P0 in insts:
                st = lm.DensityMatrix(ll, P0, precision="c32")
                batch.add(Hl, st)
                sts.append(st)
            batch.update(0.1)
            for _ in range(3):
                batch.step()
            outs[resident] = [st.to_numpy() for st in sts]
        finally:
            lm.default_context().set_resident_form(True)
    for (Ho, Hl, ll, P0), got in zip(insts, outs[True]):
        if Ho.shape[0] > 2500:
            continue
        U = o.expm_exact(Ho, 0.1)
        P = P0
        for _ in range(3):
            P = U @ P @ U.conj().T
        assert rel(got, P) <= 5e-6
    for x, y in zip(outs[True], outs[False]):
        assert np.array_equal(x, y)


def test_resident_mixed_with_region_form_and_graph_replay(lm):
    """Instances that do not fit (97 x 97; a periodic axis that is not a multiple of the block)
    run in the region form in the same pass; a graph replay repeats the direct launches bit for
    bit."""
    geoms = [(97, 97, (False, False), (0.0, 0.0), 2), (23, 22, (True, True), (0.0, 0.0), 4),
             (20, 31, (False, False), (0.0, 0.0), 9), (70, 40, (False, False), (0.0, 0.0), 3)]
    res = {}
    for graph in (True, False):
        batch, insts = ket_batch(lm, 0.08, geoms, seed=11)
        batch.set_graph(graph)
        for _ in range(3):
            batch.step()
        res[graph] = [st.to_numpy() for _, _, st in insts]
        for (Ho, X, st), got in zip(insts, res[graph]):
            Y = X
            for _ in range(3):
                Y = o.expm_multiply(Ho, 0.08, Y)
            assert rel(got.astype(np.complex128), Y) <= 5e-6
    for x, y in zip(res[True], res[False]):
        assert np.array_equal(x, y)
