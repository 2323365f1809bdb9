"""The allocation-free step, lm_solver_step_noalloc, against the regular lm_solver_step.

Hosts whose device memory belongs to another allocator, or that may not allocate after
start-up, advance their own ket blocks with lm_solver_step_noalloc: its recurrence buffers
live in a static device array instead of memory the library allocates.  It must give the
regular step's results, call after call.  This file is collected last on purpose.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_noalloc_step_matches_regular_step():
    import lmgpu
    from lmgpu import _lib as L

    ctx = lmgpu.default_context()
    lib = ctx.lib
    lat = lmgpu.SquareLattice(24, 20, boundaries={"axis1": True})
    rng = np.random.default_rng(1)
    V = rng.uniform(-1, 1, lat.N)
    H = lmgpu.tightbinding_hamiltonian(lat, V, field=lmgpu.LandauGauge(0.03))
    M = 6
    X = rng.standard_normal((lat.N, M)) + 1j * rng.standard_normal((lat.N, M))
    X /= np.linalg.norm(X, axis=0)
    # ComplexF64: both paths run the same per-order kernels; ComplexF32: the regular step runs
    # the temporally blocked kernel, so the two agree to FP32 rounding (the fused-test bar)
    for precision, tol in (("c64", 1e-13), ("c32", 2e-6)):
        ref = lmgpu.KetBlock(lat, X, precision=precision)   # regular step, library-owned scratch
        dut = lmgpu.KetBlock(lat, X, precision=precision)   # only used as a caller-owned buffer
        solver = lmgpu.ChebyshevGPU()
        solver.update_solver(H, 0.07)
        handle = solver._prepare(ref)                        # the lm_solver for this precision
        ptr, ld = dut.device_ptr()
        for _ in range(2):                                   # two calls in a row
            solver.step(ref)
            ctx.check(lib.lm_solver_step_noalloc(handle, ptr, lat.N, M, ld, dut.precision))
            assert rel(dut.to_numpy(), ref.to_numpy()) <= tol
        # blocks beyond the static scratch are refused before any device work
        rc = lib.lm_solver_step_noalloc(handle, ptr, lat.N, 1 << 20, ld, dut.precision)
        assert rc == L.LM_ERR_ARG
