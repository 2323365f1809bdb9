"""State uploads (lm_state_upload) from pageable, pinned and padded host buffers: ordered after
the work already queued on the state, exact round trips."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lm():
    import lmgpu
    lmgpu.default_context()
    return lmgpu


def big_block(N, M, seed):
    rng = np.random.default_rng(seed)
    X = np.empty((N, M), dtype=np.complex64, order="F")
    for c in range(0, M, 64):
        c1 = min(M, c + 64)
        X[:, c:c1] = rng.standard_normal((N, c1 - c), dtype=np.float32) + 1j * rng.standard_normal((N, c1 - c), dtype=np.float32)
    return X


@pytest.mark.parametrize("source", ["pageable", "pinned", "padded"])
def test_upload_round_trip_and_order(lm, source):
    """272 MiB of c32 kets.  The upload is queued right behind a Chebyshev step on the same
    state, so it must wait for that step; the download then returns exactly the uploaded values.
    'padded' passes a host leading dimension larger than n."""
    import torch
    lat = lm.SquareLattice(256, 256, boundaries={"axis1": True, "axis2": True})
    N, M = lat.N, 544
    X0 = big_block(N, M, 1)
    X1 = big_block(N, M, 2)
    st = lm.KetBlock(lat, X0, precision="c32")
    H = lm.tightbinding_hamiltonian(lat, field=lm.LandauGauge(0.01))
    s = lm.ChebyshevGPU(tol=1e-9)
    s.update_solver(H, 0.1)
    s.step(st)  # queued, still running when the upload below is issued
    if source == "pageable":
        st.upload(X1)
    elif source == "pinned":
        pin = torch.empty((M, N), dtype=torch.complex64, pin_memory=True)
        Xp = pin.numpy().T
        Xp[:] = X1
        st.upload_from(Xp)
    else:
        Xpad = np.zeros((N + 8, M), dtype=np.complex64, order="F")
        Xpad[:N] = X1
        st.ctx.check(st.ctx.lib.lm_state_upload(st.handle, Xpad.ctypes.data_as(C.c_void_p), N + 8))
    got = st.to_numpy()
    assert np.array_equal(got, X1)
