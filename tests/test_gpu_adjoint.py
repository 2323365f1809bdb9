"""Adjoint gradients against an FP64 dense-exponential reference (small case) and against
central finite differences of the FP64 forward (the differentiation workload)."""
import math

import numpy as np
import pytest

from oracle import lm_oracle as o

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lm():
    import lmgpu
    lmgpu.default_context()
    return lmgpu


def bump(lat_coords, center, sigma):
    r2 = ((lat_coords - np.asarray(center)) ** 2).sum(axis=1)
    return 0.5 + 0.2 * np.exp(-r2 / (2 * sigma ** 2))


def oracle_loss(L, psi0, V, B, target, dt, nsteps, spi, point):
    """Loss of the same evolution with the exact dense exponential (FP64)."""
    ol = o.SquareLattice(L, L)
    psi = psi0.astype(np.complex128)
    for n in range(nsteps):
        H = o.tightbinding_hamiltonian(ol, field=o.PointFlux(B[n // spi], point), onsite=V)
        psi = o.expm_exact(H, dt) @ psi
    rho = (np.abs(psi) ** 2).sum(axis=1)
    return float(((rho - target) ** 2).sum())


def test_adjoint_matches_dense_exponential_gradient(lm):
    L, M, dt, nsteps, spi = 6, 3, 0.05, 12, 4
    point = (3.5, 3.5)
    rng = np.random.default_rng(2)
    V = rng.uniform(-0.1, 0.1, L * L)
    B = np.array([0.1, 0.15, 0.05])
    ol = o.SquareLattice(L, L)
    H0 = o.tightbinding_hamiltonian(ol, field=o.PointFlux(B[0], point), onsite=V)
    w, Vec = np.linalg.eigh(H0.toarray())
    psi0 = Vec[:, :M]
    target = bump(ol.coords, (2.5, 4.0), 1.5)
    lat = lm.SquareLattice(L, L)
    prob = lm.adjoint.DensityLossAdjoint(lat, psi0, target, dt, nsteps, spi, point, precision="c64",
                                         checkpoint_every=5)
    loss, gV, gB = prob.loss_and_grad(V, B)
    assert abs(loss - oracle_loss(L, psi0, V, B, target, dt, nsteps, spi, point)) <= 1e-12 * max(1.0, loss)
    ref_loss, ref_V, ref_B = o.density_loss_gradient_exact(ol, psi0, V, B, target, dt, nsteps, spi, point)
    assert abs(ref_loss - loss) <= 1e-12 * max(1.0, loss)
    scale_V = np.abs(ref_V).max()
    scale_B = np.abs(ref_B).max()
    print("dense-exponential reference: max |dV| rel", np.abs(gV - ref_V).max() / scale_V,
          "max |dB| rel", np.abs(gB - ref_B).max() / scale_B)
    assert np.abs(gV - ref_V).max() <= 1e-9 * scale_V
    assert np.abs(gB - ref_B).max() <= 1e-9 * scale_B
    # the FP32 adjoint against the same reference
    p32 = lm.adjoint.DensityLossAdjoint(lat, psi0, target, dt, nsteps, spi, point, precision="c32",
                                        checkpoint_every=5)
    _, gV32, gB32 = p32.loss_and_grad(V, B)
    assert np.abs(gV32 - ref_V).max() <= 1e-4 * scale_V
    assert np.abs(gB32 - ref_B).max() <= 1e-4 * scale_B


def test_adjoint_torch_function(lm):
    torch = pytest.importorskip("torch")
    L, M = 5, 2
    ol = o.SquareLattice(L, L)
    w, Vec = np.linalg.eigh(o.tightbinding_hamiltonian(ol).toarray())
    prob = lm.adjoint.DensityLossAdjoint(lm.SquareLattice(L, L), Vec[:, :M], np.full(L * L, 0.1), 0.05, 6, 3,
                                         (2.5, 2.5), precision="c64")
    V = torch.zeros(L * L, dtype=torch.float64, requires_grad=True)
    B = torch.full((2,), 0.1, dtype=torch.float64, requires_grad=True)
    loss = lm.adjoint.EvolutionDensityLoss.apply(V, B, prob)
    loss.backward()
    _, gV, gB = prob.loss_and_grad(V.detach().numpy(), B.detach().numpy())
    assert np.allclose(V.grad.numpy(), gV) and np.allclose(B.grad.numpy(), gB)


def test_differentiation_workload_fd(lm):
    """SquareLattice(64,64) open, M = 2048 lowest eigenstates, V ~ U[-0.1,0.1], 50 flux
    intervals of 8 steps (init 0.1) through (32.5, 32.5), T = 20 (400 steps of 0.05),
    checkpoint every 20 steps, FP32 forward + adjoint; gradient against FP64 central
    differences (h = 1e-4) on 32 random parameters (24 potentials, 8 flux amplitudes).

    Bar: every checked component within 1e-5 of the finite difference, relative to
    max(|fd_i|, RMS of its group's gradient).  The floor matters only for components far below
    their group's typical size (one potential gradient here is below 5e-4 against an RMS of
    0.024): the FP32 error is about the same in absolute terms for every component, so such a
    component would otherwise report that error divided by its own small size.  The FP64
    adjoint is held to 1e-6 of FD with no floor, which shows that the FD reference itself is
    good to that level and that the remaining error is the FP32 arithmetic's."""
    L, M, dt, nsteps, spi = 64, 2048, 0.05, 400, 8
    point = (32.5, 32.5)
    rng = np.random.default_rng(5)
    V = rng.uniform(-0.1, 0.1, L * L)
    B = np.full(50, 0.1)
    ol = o.SquareLattice(L, L)
    lat = lm.SquareLattice(L, L)
    # the M lowest eigenstates of h(V0) from the library's eigensystem
    psi0 = lm.diagonalize(lm.tightbinding_hamiltonian(lat, V, field=lm.PointFlux(B[0], point))).vectors(0, M).to_numpy()
    c = rng.uniform(20, 44, size=2)
    target = bump(ol.coords, c, 6.0)
    p32 = lm.adjoint.DensityLossAdjoint(lat, psi0, target, dt, nsteps, spi, point, precision="c32")
    loss32, gV, gB = p32.loss_and_grad(V, B)
    p64 = lm.adjoint.DensityLossAdjoint(lat, psi0, target, dt, nsteps, spi, point, precision="c64",
                                        bounds=p32.bounds)
    h = 1e-4
    iv = rng.choice(L * L, size=24, replace=False)
    ib = rng.choice(50, size=8, replace=False)
    _, gV64, gB64 = p64.loss_and_grad(V, B)  # the FP64 adjoint separates FP32 error from FD error
    fd, g32, g64 = [], [], []
    for i in iv:
        e = np.zeros(L * L); e[i] = h
        fd.append((p64.loss(V + e, B) - p64.loss(V - e, B)) / (2 * h))
        g32.append(gV[i]); g64.append(gV64[i])
    for j in ib:
        e = np.zeros(50); e[j] = h
        fd.append((p64.loss(V, B + e) - p64.loss(V, B - e)) / (2 * h))
        g32.append(gB[j]); g64.append(gB64[j])
    fd, g32, g64 = np.array(fd), np.array(g32), np.array(g64)
    # floor: the RMS of the group's FP64 adjoint gradient (4096 potentials, 50 flux amplitudes)
    floor = np.concatenate([np.full(len(iv), np.sqrt(np.mean(gV64 ** 2))), np.full(len(ib), np.sqrt(np.mean(gB64 ** 2)))])
    err32 = np.abs(g32 - fd) / np.maximum(np.abs(fd), floor)
    err64 = np.abs(g64 - fd) / np.maximum(np.abs(fd), 1e-300)
    err3264 = np.abs(g32 - g64) / np.maximum(np.abs(g64), floor)
    np.set_printoptions(precision=3, linewidth=200)
    print(f"differentiation workload: loss {loss32:.6e}; |gV| {np.linalg.norm(gV64):.3e}, |gB| {np.linalg.norm(gB64):.3e}")
    print("  |fd|            ", np.abs(fd))
    print("  c32 vs fd       ", err32)
    print("  c64 vs fd       ", err64)
    print(f"  max/median: c32-fd {err32.max():.3e}/{np.median(err32):.3e}  c64-fd {err64.max():.3e}/"
          f"{np.median(err64):.3e}  c32-c64 {err3264.max():.3e}")
    assert err64.max() <= 1e-6   # measured 1.05e-7
    assert err32.max() <= 1e-5   # measured 1.4e-6 against the floored scale
