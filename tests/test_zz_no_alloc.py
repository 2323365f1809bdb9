"""The allocation-free step, lm_solver_step_noalloc, against the regular lm_solver_step.

Hosts whose device memory belongs to another allocator, or that may not allocate after
start-up, advance their own ket blocks with lm_solver_step_noalloc: its recurrence buffers
live in a static device array instead of memory the library allocates.  It must give the
regular step's results, call after call, for even and odd Chebyshev orders (an odd order
leaves the result in the static array and copies it back) and for blocks whose leading
dimension is larger than the number of sites.  This file is collected last on purpose.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _setup():
    import lmgpu
    ctx = lmgpu.default_context()
    lat = lmgpu.SquareLattice(24, 20, boundaries={"axis1": True})
    rng = np.random.default_rng(1)
    V = rng.uniform(-1, 1, lat.N)
    H = lmgpu.tightbinding_hamiltonian(lat, V, field=lmgpu.LandauGauge(0.03))
    M = 6
    X = rng.standard_normal((lat.N, M)) + 1j * rng.standard_normal((lat.N, M))
    X /= np.linalg.norm(X, axis=0)
    return lmgpu, ctx, lat, H, X


def _time_steps_by_parity(lmgpu, H, probe):
    """Two time steps whose Chebyshev orders are even and odd, for the probe state's tolerance."""
    found = {}
    for dt in np.linspace(0.02, 0.4, 39):
        s = lmgpu.ChebyshevGPU()
        s.update_solver(H, float(dt))
        s._prepare(probe)
        K = s.order(probe)[0]
        found.setdefault(K % 2, (float(dt), K))
        if len(found) == 2:
            return found
    raise AssertionError(f"no time step with both order parities: {found}")


# ComplexF64: both paths run the same per-order kernels; ComplexF32: the regular step runs the
# temporally blocked kernel, so the two agree to FP32 rounding (the fused-test bar)
TOLS = {"c64": 1e-13, "c32": 2e-6}


@pytest.mark.parametrize("precision", ["c64", "c32"])
def test_noalloc_step_matches_regular_step(precision):
    lmgpu, ctx, lat, H, X = _setup()
    from lmgpu import _lib as L
    lib = ctx.lib
    M = X.shape[1]
    probe = lmgpu.KetBlock(lat, X, precision=precision)
    for parity, (dt, K) in sorted(_time_steps_by_parity(lmgpu, H, probe).items()):
        ref = lmgpu.KetBlock(lat, X, precision=precision)   # regular step, library-owned scratch
        dut = lmgpu.KetBlock(lat, X, precision=precision)   # only used as a caller-owned buffer
        solver = lmgpu.ChebyshevGPU()
        solver.update_solver(H, dt)
        handle = solver._prepare(ref)                        # the lm_solver for this precision
        assert solver.order(ref)[0] % 2 == parity
        ptr, ld = dut.device_ptr()
        for _ in range(2):                                   # two calls in a row
            solver.step(ref)
            ctx.check(lib.lm_solver_step_noalloc(handle, ptr, lat.N, M, ld, dut.precision))
            assert rel(dut.to_numpy(), ref.to_numpy()) <= TOLS[precision], (dt, K)
        # blocks beyond the static scratch are refused before any device work
        rc = lib.lm_solver_step_noalloc(handle, ptr, lat.N, 1 << 20, ld, dut.precision)
        assert rc == L.LM_ERR_ARG


@pytest.mark.parametrize("precision", ["c64", "c32"])
def test_noalloc_step_padded_block(precision):
    """A caller-owned block with ld > n (rows n..ld-1 of every column are padding): the step
    must address columns by ld, match the regular step, and leave the padding untouched."""
    import torch
    lmgpu, ctx, lat, H, X = _setup()
    lib = ctx.lib
    n, M = X.shape
    ld = n + 13
    tdt = torch.complex128 if precision == "c64" else torch.complex64
    probe = lmgpu.KetBlock(lat, X, precision=precision)
    for parity, (dt, K) in sorted(_time_steps_by_parity(lmgpu, H, probe).items()):
        ref = lmgpu.KetBlock(lat, X, precision=precision)
        solver = lmgpu.ChebyshevGPU()
        solver.update_solver(H, dt)
        handle = solver._prepare(ref)
        host = np.full((M, ld), 7.0 + 7.0j, dtype=np.complex128)   # padding sentinel
        host[:, :n] = X.T
        buf = torch.from_numpy(host).to(dtype=tdt, device="cuda:0")  # column m at buf[m], stride ld
        torch.cuda.synchronize()
        for _ in range(2):
            solver.step(ref)
            ctx.check(lib.lm_solver_step_noalloc(handle, buf.data_ptr(), n, M, ld, ref.precision))
            ctx.synchronize()
            got = buf.cpu().numpy()
            assert rel(got[:, :n].T, ref.to_numpy()) <= TOLS[precision], (dt, K)
            assert np.all(got[:, n:] == np.complex64(7.0 + 7.0j)), "padding rows were written"
