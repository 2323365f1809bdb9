"""Currents with internal degrees of freedom in the oracle: the identities of the reference's
"Operator currents" testset (test/test_currents.jl:76-93) on qwz(SquareLattice(4, 4),
field=LandauGauge(0.1)) with the ground state of the field-free model, and the per-entry
split that the device kernel computes, summed back to the reference's per-pair formula by the
host aggregation of ``lmgpu.sparse``."""
import numpy as np
import pytest

from oracle import lm_oracle as o

SZ = np.array([[1, 0], [0, -1]])
UP = np.array([[1, 0], [0, 0]])
DN = np.array([[0, 0], [0, 1]])


@pytest.fixture(scope="module")
def qwz():
    H0 = o.qwz_hamiltonian(4, 4).toarray()
    H1 = o.qwz_hamiltonian(4, 4, field=o.LandauGauge(0.1))
    w, v = np.linalg.eigh(H0)
    return H1, v[:, 0]


def test_qwz_builder_placement():
    """H[i, i+x] = [1 -i; -i -1]/2 (the term as written, bond (site, destination)), H[i+x, i]
    its adjoint; m sigma_z on site."""
    H = o.qwz_hamiltonian(3, 3, m=0.7).toarray()
    i, j = 0, 3  # (1,1) -> (2,1): x step, index (x-1) Ly + y
    assert np.allclose(H[2 * i:2 * i + 2, 2 * j:2 * j + 2], np.array([[1, -1j], [-1j, -1]]) / 2)
    assert np.allclose(H[2 * j:2 * j + 2, 2 * i:2 * i + 2], (np.array([[1, -1j], [-1j, -1]]) / 2).conj().T)
    assert np.allclose(H[2 * i:2 * i + 2, 2 * 1:2 * 1 + 2], np.array([[1, -1], [1, -1]]) / 2)  # y step
    assert np.allclose(H[0:2, 0:2], 0.7 * SZ)
    assert np.allclose(H, H.conj().T)


def test_operator_current_identities(qwz):
    H1, gs = qwz
    dc = o.site_currents_matrix(H1, gs, 2)
    ident = o.site_currents_matrix(H1, gs, 2, np.eye(2))
    up = o.site_currents_matrix(H1, gs, 2, UP)
    dn = o.site_currents_matrix(H1, gs, 2, DN)
    spin = o.site_currents_matrix(H1, gs, 2, SZ)
    assert abs(ident - dc).max() <= 1e-14
    assert abs(up + dn - dc).max() <= 1e-14
    assert abs(up - dn - spin).max() <= 1e-14
    assert abs(spin).max() > 1e-3


def test_heisenberg_identity(qwz):
    """currentsfromto(spin_curr, l[6]) = <gs| i [H, sigma_z (x) |6><6|] |gs> (test_currents.jl:88-93),
    and the same for the density."""
    H1, gs = qwz
    H = H1.toarray()
    site = 5
    for op in (SZ, np.eye(2)):
        S = np.zeros_like(H)
        S[2 * site:2 * site + 2, 2 * site:2 * site + 2] = op
        dt = (gs.conj() @ (1j * (H @ S - S @ H)) @ gs).real
        M = o.site_currents_matrix(H1, gs, 2, op)
        assert abs(o.currentsfromto(M, site) - dt) <= 1e-12
        assert abs(dt) > 1e-4


@pytest.mark.parametrize("op", [None, SZ, UP, np.array([[0.3, 1 - 2j], [1 + 2j, -0.5]])])
@pytest.mark.parametrize("kind", ["ket", "block", "density"])
def test_entry_split_sums_to_pairs(qwz, op, kind):
    import sys
    sys.path.insert(0, "latticemodels.jl_gb300")
    from lmgpu import sparse as lsp
    H1, gs = qwz
    rng = np.random.default_rng(4)
    if kind == "ket":
        state, kw = gs, {}
    elif kind == "block":
        state, kw = o.random_kets(H1.shape[0], 3, 5), {"weights": [0.5, 1.0, 2.0]}
    else:
        X = rng.standard_normal((32, 32)) + 1j * rng.standard_normal((32, 32))
        state, kw = X @ X.conj().T / 64, {"is_density": True}
    ent = o.entry_op_currents(H1, state, 2, op, **kw)
    pairs = o.site_currents(H1, state, 2, op, **kw)
    H = lsp.SparseHamiltonian(lsp.Sites(32, None, "qwz", internal=2), H1)
    src, dst, vals = lsp._aggregate_pairs(H, ent)
    got = {(int(a) - 1, int(b) - 1): v for a, b, v in zip(src, dst, vals)}
    assert set(got) == set(pairs)
    for key, v in pairs.items():
        assert abs(got[key] - v) <= 1e-14 * max(1.0, abs(v))
