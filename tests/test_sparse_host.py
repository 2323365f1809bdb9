"""Host logic of the general sparse path (no GPU): Sites with internal states,
SparseHamiltonian construction from scipy matrices and from the reference's 1-based CSC
arrays, pattern identity and value equality, and the per-site-pair aggregation of entry
currents (src/zoo/currents.jl:92-102, :170-184)."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import lm_oracle as o


@pytest.fixture(scope="module")
def lm():
    import lmgpu
    return lmgpu


def test_sites_internal(lm):
    s = lm.Sites(32, None, "qwz", internal=2)
    assert (s.N, s.nsites, len(s)) == (32, 16, 16)
    with pytest.raises(ValueError):
        lm.Sites(33, None, "bad", internal=2)
    with pytest.raises(ValueError):
        lm.Sites(8, None, "bad", internal=0)


def test_sparse_hamiltonian_inputs_and_equality(lm):
    H = o.qwz_hamiltonian(3, 4, field=o.LandauGauge(0.1))
    sites = lm.Sites(24, None, "qwz", internal=2)
    a = lm.SparseHamiltonian(sites, H)
    b = lm.SparseHamiltonian(sites, o.csc_arrays(H))   # the reference's 1-based CSC arrays
    assert np.array_equal(a.colptr, b.colptr) and np.array_equal(a.rowval, b.rowval)
    assert a == b
    c = lm.SparseHamiltonian(sites, H * 2.0)            # same pattern, other values
    assert c._pattern == a._pattern and not (c == a)
    with pytest.raises(ValueError):
        lm.SparseHamiltonian(lm.Sites(10), H)


def test_pair_aggregation_matches_reference_getindex(lm):
    """Entry shares (the device kernel's output, computed here by the oracle) summed per site
    block by the host give LocalOperatorCurrents(H, P, op)[i, j]."""
    from lmgpu import sparse as lsp
    H = o.qwz_hamiltonian(3, 3, m=np.linspace(-1, 1, 9), field=o.LandauGauge(0.2))
    X = o.random_kets(18, 4, 9)
    op = np.array([[0.5, 1j], [-1j, -0.25]])
    ent = o.entry_op_currents(H, X, 2, op)
    Hs = lsp.SparseHamiltonian(lsp.Sites(18, None, "qwz", internal=2), H)
    src, dst, vals = lsp._aggregate_pairs(Hs, ent)
    P = X @ X.conj().T
    for a, b, v in zip(src, dst, vals):
        assert abs(v - o.local_operator_current(H, P, 2, op, a - 1, b - 1)) <= 1e-14
    # every stored inter-site block appears exactly once
    A = sp.coo_matrix(H)
    blocks = {(r // 2 + 1, c // 2 + 1) for r, c in zip(A.row, A.col) if r // 2 != c // 2}
    assert set(zip(src.tolist(), dst.tolist())) == blocks
