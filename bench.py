#!/usr/bin/env python
"""Throughput of the LatticeModels.jl evolution hot path on GB300, in ket-steps/s.

Workload (the plain-method-at-GPU-scale configuration): SquareLattice(256, 256) with periodic
boundaries on both axes, hopping t1 = 1, uniform Landau-gauge field of 0.01 flux quanta per
plaquette, Anderson on-site disorder U[-1, 1], a block of M = 2048 complex-Gaussian normalised
kets, dt = 0.05.  One bench step advances the whole ket block by dt through the Chebyshev
propagator (ket-steps = M per step).

  value     chosen form: ComplexF32 recurrence, FP64 coefficients and reductions, tol 1e-9
  plain     ComplexF64 recurrence, tol 1e-12 (reported beside it)
  e2e       the same metric through the public API (Evolution + ChebyshevGPU + localdensity)
            with host buffers: the ket block uploaded from pinned memory, every step a
            time-dependent H(t) input (on-site term uploaded from pinned memory, assembled on
            the device) and the local densities downloaded to pinned memory.

``--impl reference`` times the CPU restatement of the reference's KrylovKitExp step (C,
OpenMP over kets, all host threads) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "latticemodels.jl_gb300"))
sys.path.insert(0, str(ROOT))

METRIC = "ket-steps/s at <=1e-6 rel err vs FP64: chosen vs plain form, 1xGB300"
LX = LY = 256
M_KETS = 2048
DT = 0.05
B_FIELD = 0.01
W_DISORDER = 2.0
SEED = 20261203
WORKLOAD_FMT = ("SquareLattice({L},{L}) periodic x/y, t1=1, LandauGauge(0.01), Anderson U[-1,1], "
                "M={M} complex-Gaussian kets, dt=0.05")
WORKLOAD = WORKLOAD_FMT.format(L=LX, M=M_KETS)


# ------------------------------------------------------------------------------------------
# synthetic inputs (seeded numpy PCG64)
# ------------------------------------------------------------------------------------------
def make_disorder(N):
    rng = np.random.default_rng(SEED)
    return rng.uniform(-W_DISORDER / 2, W_DISORDER / 2, size=N)


def make_kets(N, M, rank=0, dtype=np.complex128, out=None):
    """Complex Gaussian kets, each normalised; column-major (each ket contiguous)."""
    rng = np.random.default_rng(SEED + 1 + rank)
    X = out if out is not None else np.empty((N, M), dtype=dtype, order="F")
    chunk = 256
    for c0 in range(0, M, chunk):
        c1 = min(M, c0 + chunk)
        re = rng.standard_normal((c1 - c0, N))
        im = rng.standard_normal((c1 - c0, N))
        z = re + 1j * im
        z /= np.linalg.norm(z, axis=1, keepdims=True)
        X[:, c0:c1] = z.T.astype(X.dtype)
    return X


# ------------------------------------------------------------------------------------------
# clocks during the timed region
# ------------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self._t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0])); smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------------
def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


TRAFFIC_RECORD = "cheb_stream_c32_256x256.traffic.json"
TRAFFIC_RECORD_COMP = "cheb_stream_c32_comp_256x256.traffic.json"


def kernel_source_hash(sources):
    """sha256 over the kernel's source files (repo-relative paths), in the listed order."""
    import hashlib
    h = hashlib.sha256()
    for rel in sources:
        h.update((ROOT / rel).read_bytes())
    return h.hexdigest()


def profile_traffic(record: str = TRAFFIC_RECORD):
    """DRAM bytes per launch of the dominant kernel from the committed ncu record, valid only
    while the kernel's sources hash to the value the record was captured with.

    Returns (bytes per captured launch, sites x kets of the captured launch, record) or
    (None, None, reason)."""
    f = ROOT / "profiles" / record
    if not f.exists():
        return None, None, "no ncu record"
    rec = json.loads(f.read_text())
    if kernel_source_hash(rec["sources"]) != rec["source_sha256"]:
        return None, None, "stale ncu record: the kernel's sources changed since the capture"
    return (float(rec["dram_bytes_read"]) + float(rec["dram_bytes_write"]),
            float(rec["sites"]) * float(rec["kets"]), rec)


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_reference(steps, warmup, sample_kets=None, cpu_seconds=None, nthreads=None):
    """Times the oracle's C restatement of KrylovKitExp on a bounded sample of the workload.

    With ``cpu_seconds`` the number of timed steps is chosen so that the sample costs about
    that much CPU time (wall time x threads).  ``nthreads`` None: all host threads."""
    from oracle import krylov, lm_oracle as o
    lat = o.SquareLattice(LX, LY, periodic=(True, True))
    V = make_disorder(lat.N)
    H, _, _, _ = o.tightbinding_hamiltonian_fast(lat, field=o.LandauGauge(B_FIELD), onsite=V)
    csr = krylov.CSR(H)
    threads = nthreads or krylov.max_threads()
    mk = sample_kets or 2 * threads
    X = make_kets(lat.N, mk)
    t_one = None
    for _ in range(max(warmup, 1)):
        t0 = time.perf_counter()
        X = krylov.krylov_expv_block(csr, DT, X, tol=1e-12, kdim=30, nthreads=threads)
        t_one = time.perf_counter() - t0
    if cpu_seconds:
        steps = int(min(200, max(1, math.ceil(cpu_seconds / (t_one * threads)))))
    t0 = time.perf_counter()
    for _ in range(steps):
        X = krylov.krylov_expv_block(csr, DT, X, tol=1e-12, kdim=30, nthreads=threads)
    dt = time.perf_counter() - t0
    return {"value": mk * steps / dt, "unit": "ket-steps/s", "cores": threads, "kind": "port",
            "sample": f"{mk} of the {M_KETS} kets x {steps} steps (Lanczos exponentiate, tol 1e-12, "
                      f"krylovdim 30), {dt:.2f} s wall, {dt * threads:.1f} s CPU"}


def run_reference_arm(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    cb = cpu_reference(args.steps, args.warmup)
    line = {"metric": METRIC, "impl": "reference", "value": cb["value"], "unit": "ket-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * (2 * cb["cores"]) / cb["value"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample_kets_per_step": 2 * cb["cores"],
                       "l2": "CPU run"},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "ket-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------------------------------
BATCH_WORKLOAD = ("{n} independent LxL open lattices, L ~ U{{16..96}}, t1=1, PointFlux(B,(L//2+0.5)^2) with "
                  "B ~ U[0,0.3], disorder U[-W/2,W/2] with W ~ U[0,3], dense P_0 per lattice, dt=0.1")


def _batch_instances(n, prec, panel, p0="random", budget_frac=0.85):
    """The first n lattices of the seeded batching workload, each with its dense P_0, in one
    lmgpu.Batch (not yet updated).  p0 "random": principal submatrices of one seeded random
    Hermitian matrix (the step's cost does not depend on P_0's values); "densitymatrix": the
    FermiDirac ensemble of each lattice at mu = 0, T = 0.1 (densitymatrix on the device)."""
    import ctypes as C
    import torch
    import lmgpu
    from lmgpu import _lib
    ctx = lmgpu.default_context()
    rng = np.random.default_rng(SEED + 7)
    Ls = rng.integers(16, 97, size=n)
    Bs = rng.uniform(0, 0.3, size=n)
    Ws = rng.uniform(0, 3, size=n)
    dtype = np.complex64 if prec == "c32" else np.complex128
    elem = 8 if prec == "c32" else 16
    free = torch.cuda.mem_get_info()[0]
    budget = budget_frac * free
    take, used = [], 0
    for i, L in enumerate(Ls):
        N_i = int(L) ** 2
        need = elem * N_i * N_i + (2 * elem * N_i * min(panel, N_i) if panel else elem * N_i * N_i)
        if used + need > budget:
            break
        take.append(i)
        used += need
    Pbig, Nmax = None, 0
    if p0 == "random":
        Nmax = int(max(Ls[take])) ** 2
        R = (rng.standard_normal((Nmax, Nmax), dtype=np.float32)
             + 1j * rng.standard_normal((Nmax, Nmax), dtype=np.float32)).astype(dtype)
        Pbig = np.asfortranarray((R + R.conj().T) * (0.5 / math.sqrt(Nmax)))
        del R
    batch = lmgpu.Batch("density", prec)
    if panel:
        batch.set_panel(panel)
    states = []
    for i in take:
        L = int(Ls[i])
        lat = lmgpu.SquareLattice(L, L)
        V = np.random.default_rng(SEED + 1000 + i).uniform(-Ws[i] / 2, Ws[i] / 2, size=L * L)
        H = lmgpu.tightbinding_hamiltonian(lat, V, field=lmgpu.PointFlux(float(Bs[i]), (L // 2 + 0.5, L // 2 + 0.5)))
        if p0 == "random":
            st = lmgpu.DensityMatrix.__new__(lmgpu.DensityMatrix)
            lmgpu.DeviceState.__init__(st, lat, None, _lib.LM_DENSITY, prec, None, ctx, shape=(L * L, L * L))
            ctx.check(ctx.lib.lm_state_upload(st.handle, Pbig.ctypes.data_as(C.c_void_p), Nmax))
        else:
            st = lmgpu.densitymatrix(H, mu=0.0, T=0.1, precision=prec)
        batch.add(H, st)
        states.append(st)
    return batch, states, Ls, take, used


def batch_roofline(sum_n2, K, ms_per_step, sm_mhz=None):
    """Roofline fields of a dense-P batch step (c32): two fused passes and a conjugate transpose.

    * frac: the per-order formula 5*K*sum N^2*8 B per pass (the bytes of K unfused order passes);
      the fused passes keep all K orders on chip, so it exceeds 1.
    * dram_frac: the physical bytes, each pass and the transpose reading and writing every
      lattice's block once (3 x 2 x sum N^2 x 8 B), which is the traffic the counters measure for
      the lattice-resident form (profiles/cheb_resident_c32_batch_uneven_lattices.md).
    * fma_frac: the useful FP32 FMAs (20 per site-order with complex hops) of both passes against
      the device's SMs x 128 FMA/clk at the SM clock."""
    import torch
    peak, kind = measured_peak_hbm()
    sec = ms_per_step / 1000.0
    alg = 2 * 5.0 * K * sum_n2 * 8
    phys = 3 * 2.0 * sum_n2 * 8
    mhz = sm_mhz or 2070.0
    sms = torch.cuda.get_device_properties(0).multi_processor_count if torch.cuda.is_available() else 152
    fma = 2 * 20.0 * K * sum_n2 / sec / (sms * 128 * mhz * 1e6)
    return {"bound": "compute (the stencil arithmetic's latency at 12 warps per SM; DRAM traffic is the "
                     "algorithmic minimum)",
            "achieved_formula_gbs": alg / sec / 1e9, "frac": alg / sec / 1e9 / peak,
            "dram_gbs": phys / sec / 1e9, "dram_frac": phys / sec / 1e9 / peak, "fma_frac": fma,
            "peak": peak, "unit": "GB/s", "peak_source": f"{kind} (MEASURED_PEAKS.json hbm_gbs)",
            "note": "frac: the per-order formula 5*K*sum N^2*s per pass; dram_frac: 3 x 2 x sum N^2 x 8 B per "
                    "step (two passes and the transpose); fma_frac: 20 useful FMAs per site-order"}


def batch_subrecord(n, steps, warmup):
    """A small instance of the batching workload for the default line: the first n lattices,
    P_0 from densitymatrix (mu = 0, T = 0.1), tuned, stepped through the captured graphs."""
    import torch
    import lmgpu
    ctx = lmgpu.default_context()
    ext = torch.cuda.ExternalStream(ctx.stream_ptr(), device=torch.device("cuda", 0))
    t0 = time.perf_counter()
    batch, states, Ls, take, used = _batch_instances(n, "c32", 0, p0="densitymatrix", budget_frac=0.5)
    tr0 = np.array([s.trace() for s in states])
    batch.update(0.1)
    tune = batch.tune(steps=1)
    info = batch.info()
    setup = time.perf_counter() - t0
    for _ in range(warmup):
        batch.step()
    ctx.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for _ in range(steps):
        batch.step()
    e1.record(ext)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    tr1 = np.array([s.trace() for s in states])
    ket_steps = sum(2 * int(Ls[i]) ** 2 for i in take)
    return {"value": ket_steps * steps / (ms / 1000.0), "unit": "ket-steps/s", "ms_per_step": ms / steps,
            "steps": steps, "warmup": warmup, "instances": len(take),
            "sum_N2": int(sum(int(Ls[i]) ** 4 for i in take)), "chebyshev_order": info["K"], "tuned": tune,
            "fused_form": ("lattice-resident (csrc/lmgpu_resident.cu): a whole ket on chip for all K orders, one CTA "
                           "up to 4608 sites, a cluster of two CTAs up to 9216; the region form for the rest"),
            "roofline": batch_roofline(sum(int(Ls[i]) ** 4 for i in take), info["K"], ms / steps),
            "p0": "densitymatrix(h, mu=0, T=0.1) per lattice (device Chebyshev Fermi operator)",
            "trace_drift_max": float(np.abs(tr1 - tr0).max() / np.abs(tr0).max()), "setup_s": setup,
            "workload": BATCH_WORKLOAD.format(n=len(take)) + " (the first lattices of the seeded 512)"}


def run_batch_workload(args):
    """The batching workload: uneven dense-P lattices stepped together (one graph per step).

    P_0 of every lattice is a principal submatrix of one seeded random Hermitian matrix (a
    stand-in of the right shape: the step's cost does not depend on P_0's values; parity of
    the batched path with true densitymatrix P_0 is covered by the GPU tests).  Ket-steps: a
    dense-P step U P U^dagger counts 2N per lattice."""
    import torch
    import lmgpu
    ctx = lmgpu.default_context()
    ext = torch.cuda.ExternalStream(ctx.stream_ptr(), device=torch.device("cuda", 0))
    n = args.instances
    prec = args.precision
    # c64 runs the per-order kernels on column panels in place (P + 2 N w scratch per lattice);
    # c32 runs the fused kernel on full buffers (P + one recurrence buffer)
    panel = args.panel if args.panel is not None else (1024 if prec == "c64" else 0)
    ctx.set_resident_form(args.batch_form == "resident")
    t_setup = time.perf_counter()
    batch, states, Ls, take, used = _batch_instances(n, prec, panel)
    batch.update(0.1)
    tune = batch.tune(steps=1)
    info = batch.info()
    t_setup = time.perf_counter() - t_setup
    for _ in range(args.warmup):
        batch.step()
    ctx.synchronize()
    clk = ClockSampler(0)
    clk.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for _ in range(args.steps):
        batch.step()
    e1.record(ext)
    e1.synchronize()
    clocks = clk.stop()
    ms = e0.elapsed_time(e1)
    ket_steps = sum(2 * int(Ls[i]) ** 2 for i in take)
    tr = [s.trace() for s in states[:4]]
    line = {"metric": "ket-steps/s (batched dense-P lattices)", "value": ket_steps * args.steps / (ms / 1000.0),
            "unit": "ket-steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "dtype": prec,
            "data": "synthetic (seeded; P_0 = principal submatrices of one random Hermitian matrix)",
            "config": {"workload": BATCH_WORKLOAD.format(n=n), "instances_run": len(take),
                       "instances_requested": n, "sum_N2": int(sum(int(Ls[i]) ** 4 for i in take)),
                       "chebyshev_order": info["K"], "tuned": tune, "setup_s": t_setup,
                       "device_bytes": used, "panel_columns": panel, "fused_form": args.batch_form},
            "roofline": batch_roofline(sum(int(Ls[i]) ** 4 for i in take), info["K"], ms / args.steps,
                                       clocks.get("sm_mhz")),
            "clocks": clocks, "trace_sample": tr}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------------------------------
ADJOINT_WORKLOAD = ("SquareLattice(64,64) open, M=2048 lowest eigenstates of h(V0), V0 ~ U[-0.1,0.1], "
                    "50 PointFlux amplitudes at (32.5,32.5) (init 0.1, 8 steps each), dt=0.05, 400 steps, "
                    "checkpoint every 20, loss sum_i (rho_i(T) - rho*_i)^2")


def run_adjoint_workload(args):
    """The differentiation workload: one loss_and_grad = the forward pass with checkpoints, the
    recomputation of every segment, the adjoint recurrence and the co-state propagation.
    `value` counts forward ket-steps (M x 400) per second of loss_and_grad."""
    import torch
    import lmgpu
    ctx = lmgpu.default_context()
    ext = torch.cuda.ExternalStream(ctx.stream_ptr(), device=torch.device("cuda", 0))
    L, M, dt, nsteps, spi = 64, 2048, 0.05, 400, 8
    point = (32.5, 32.5)
    rng = np.random.default_rng(SEED + 11)
    V = rng.uniform(-0.1, 0.1, L * L)
    B = np.full(50, 0.1)
    lat = lmgpu.SquareLattice(L, L)
    if args.adjoint_init == "random":  # same cost, no eigensystem
        psi0 = (rng.standard_normal((L * L, M)) + 1j * rng.standard_normal((L * L, M))) / math.sqrt(2 * L * L)
    else:  # the M lowest eigenstates from the library's eigensystem
        eig = lmgpu.diagonalize(lmgpu.tightbinding_hamiltonian(lat, V, field=lmgpu.PointFlux(B[0], point)))
        psi0 = eig.vectors(0, M).to_numpy()
        del eig
    c = rng.uniform(20, 44, size=2)
    r2 = ((lat.coords() - c) ** 2).sum(axis=1)
    target = 0.5 + 0.2 * np.exp(-r2 / (2 * 6.0 ** 2))
    prob = lmgpu.DensityLossAdjoint(lat, psi0, target, dt, nsteps, spi, point, precision=args.precision)
    for _ in range(max(1, args.warmup // 3)):
        prob.loss_and_grad(V, B)
    ctx.synchronize()
    reps = max(1, min(args.steps, 3))
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    clk = ClockSampler(0)
    clk.start()
    e0.record(ext)
    for _ in range(reps):
        loss, gV, gB = prob.loss_and_grad(V, B)
    e1.record(ext)
    e1.synchronize()
    clocks = clk.stop()
    ms = e0.elapsed_time(e1) / reps
    line = {"metric": "forward ket-steps/s of loss_and_grad (forward + checkpointed adjoint)",
            "value": M * nsteps / (ms / 1000.0), "unit": "ket-steps/s", "n_gpus": 1, "steps": reps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "dtype": args.precision,
            "data": ("synthetic (seeded; psi_0 = lowest eigenstates of h(V0) from the library's eigensystem)"
                     if args.adjoint_init == "eigh" else "synthetic (seeded; psi_0 = random complex-Gaussian kets)"),
            "config": {"workload": ADJOINT_WORKLOAD, "N": L * L, "M": M, "tol": prob.tol,
                       "step_unit": "one loss_and_grad"},
            "loss": loss, "grad_norm_V": float(np.linalg.norm(gV)), "grad_norm_B": float(np.linalg.norm(gB)),
            "clocks": clocks}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------------------------------
KPM_WORKLOAD = ("SquareLattice(256,256) periodic x/y, t1=1, LandauGauge(0.01), Anderson U[-1,1], "
                "256 random-phase vectors, 2048 Chebyshev moments")


def run_kpm_workload(args):
    """Chebyshev moments for the KPM density of states: 1024 stencil passes over a 256-vector
    block (doubling relations), FP64.  `value` = vector-moments per second."""
    import torch
    import lmgpu
    ctx = lmgpu.default_context()
    ext = torch.cuda.ExternalStream(ctx.stream_ptr(), device=torch.device("cuda", 0))
    lat = lmgpu.SquareLattice(LX, LY, boundaries={"axis1": True, "axis2": True})
    N, R, nmom = lat.N, 256, 2048
    H = lmgpu.tightbinding_hamiltonian(lat, make_disorder(N), field=lmgpu.LandauGauge(B_FIELD))
    vecs = lmgpu.DeviceState(lat, lmgpu.kpm._phase_vectors(N, R, SEED), 0, "c64")
    bounds = lmgpu.kpm._bounds(H, ctx)
    for _ in range(max(1, args.warmup // 3)):
        lmgpu.kpm.moments(H, 64, vecs, bounds=bounds)
    reps = max(1, min(args.steps, 3))
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    clk = ClockSampler(0)
    clk.start()
    e0.record(ext)
    for _ in range(reps):
        mu, _ = lmgpu.kpm.moments(H, nmom, vecs, bounds=bounds)  # the default: double-float recurrence
    e1.record(ext)
    e1.synchronize()
    clocks = clk.stop()
    ms = e0.elapsed_time(e1) / reps
    # the same call with the FP64 recurrence (LM_OPT_KPM = 0)
    ctx.set_kpm_doublefloat(False)
    try:
        lmgpu.kpm.moments(H, 64, vecs, bounds=bounds)
        e0.record(ext)
        for _ in range(reps):
            mu64, _ = lmgpu.kpm.moments(H, nmom, vecs, bounds=bounds)
        e1.record(ext)
        e1.synchronize()
        ms64 = e0.elapsed_time(e1) / reps
    finally:
        ctx.set_kpm_doublefloat(True)
    passes = (nmom + 1) // 2 + 1
    # per pass, FP64 path: the recurrence reads T_{n+1} and T_n and writes T_{n+2}; the two
    # dot products read T_n (twice) and T_{n+1}: six block passes of N*R*16 bytes.  The
    # double-float path forms both dots in one read of T_n and T_{n+1}: five passes.
    alg = 5.0 * N * R * 16 * passes
    alg64 = 6.0 * N * R * 16 * passes
    peak, peak_kind = measured_peak_hbm()
    line = {"metric": "KPM vector-moments/s (Chebyshev moments, double-float recurrence)",
            "value": R * nmom / (ms / 1000.0),
            "unit": "vector-moments/s", "n_gpus": 1, "steps": reps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "dtype": "df32 pairs (recurrence), f64 (dots, moments)",
            "data": "synthetic (seeded PCG64 random-phase vectors)",
            "config": {"workload": KPM_WORKLOAD, "N": N, "vectors": R, "moments": nmom, "passes": passes,
                       "step_unit": "one lm_kpm_moments call"},
            "roofline": {"bound": "hbm", "achieved": alg / (ms / 1000.0) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": alg / (ms / 1000.0) / 1e9 / peak, "traffic": None,
                         "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                         "alg_bytes_per_call": alg,
                         "note": "whole call (recurrence + dot kernels): 5 block passes per pass (the double-float "
                                 "dots read T_n and T_n+1 once for both moments)"},
            "mu0_over_N": float(mu[0] / (N * R)), "clocks": clocks,
            "fp64": {"value": R * nmom / (ms64 / 1000.0), "ms_per_step": ms64, "speedup_of_default": ms64 / ms,
                     "roofline_frac": alg64 / (ms64 / 1000.0) / 1e9 / peak,
                     "max_moment_diff_over_mu0": float(np.abs(mu64 - mu).max() / abs(mu[0])),
                     "note": "LM_OPT_KPM = 0: the recurrence in FP64 (GB300 runs FP64 at 1/64 of FP32)"}}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------------------------------
DM_WORKLOAD = ("SquareLattice(96,96) open (the largest lattice of the batching workload), t1=1, "
               "PointFlux(0.2, (48.5, 48.5)), disorder U[-1.5,1.5]; densitymatrix(H; mu=0, T=0.1) and "
               "densitymatrix(H; mu=0) at T = 0")


def run_densitymatrix_workload(args):
    """P_0 = densitymatrix(H; mu, T) on the library's kernels, N = 9216:
    * T = 0.1: the Chebyshev series of the occupation applied to the identity (double-float
      recurrence by default, FP64 with LM_OPT_KPM = 0);
    * T = 0: the library's FP64 eigensystem (Householder tridiagonalisation, bisection, inverse
      iteration, back-transformation, weighted projector);
    each against cuSOLVER's dense eigensolver on the same GPU (torch.linalg.eigh, timed here as
    a baseline only).  `value` = matrices per second of the T = 0 route."""
    import torch
    import lmgpu
    ctx = lmgpu.default_context()
    L = 96
    lat = lmgpu.SquareLattice(L, L)
    V = np.random.default_rng(SEED + 3).uniform(-1.5, 1.5, L * L)
    H = lmgpu.tightbinding_hamiltonian(lat, V, field=lmgpu.PointFlux(0.2, (48.5, 48.5)))

    def sync():
        ctx.synchronize()
        torch.cuda.synchronize()

    def timed(fn, warm=True):
        if warm:
            fn()
        sync()
        t0 = time.perf_counter()
        out = fn()
        sync()
        return time.perf_counter() - t0, out

    # cuSOLVER baseline: dense H from the library's CSC, eigh, projector by matmul (FP64)
    colptr, rowval, nz = H.csc()
    cols = np.repeat(np.arange(L * L), np.diff(colptr))
    Hd = torch.sparse_coo_tensor(torch.as_tensor(np.stack([rowval - 1, cols])), torch.as_tensor(nz),
                                 (L * L, L * L)).to_dense().to("cuda")

    def cusolver(T):
        w, U = torch.linalg.eigh(Hd)
        occ = (w <= 0.0).double() if T == 0 else 0.5 * (1.0 - torch.tanh(w / (2 * T)))
        return (U * occ) @ U.conj().T

    t_cheb, Pc = timed(lambda: lmgpu.densitymatrix(H, mu=0.0, T=0.1, method="chebyshev"))
    ctx.set_kpm_doublefloat(False)
    try:
        t_cheb64, Pc64 = timed(lambda: lmgpu.densitymatrix(H, mu=0.0, T=0.1, method="chebyshev"), warm=False)
    finally:
        ctx.set_kpm_doublefloat(True)
    t_zero, Pz = timed(lambda: lmgpu.densitymatrix(H, mu=0.0), warm=False)
    t_cu0, Pcu0 = timed(lambda: cusolver(0.0))
    t_cu1, Pcu1 = timed(lambda: cusolver(0.1), warm=False)
    a = torch.as_tensor(Pc.to_numpy(), device="cuda")
    a64 = torch.as_tensor(Pc64.to_numpy(), device="cuda")
    z = torch.as_tensor(Pz.to_numpy(), device="cuda")
    r = lambda x, y: float(torch.linalg.norm(x - y) / torch.linalg.norm(y))
    line = {"metric": "densitymatrix at T = 0 on the library's eigensystem: matrices/s",
            "value": 1.0 / t_zero, "unit": "matrices/s", "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": t_zero * 1e3, "higher_is_better": True, "dtype": "f64 (c64 matrices)",
            "data": "synthetic (seeded disorder)", "config": {"workload": DM_WORKLOAD, "N": L * L},
            "zero_temperature": {"ms": t_zero * 1e3, "cusolver_ms": t_cu0 * 1e3, "speedup_over_cusolver": t_cu0 / t_zero,
                                 "rel_diff_vs_cusolver": r(z, Pcu0), "trace": float(torch.trace(z).real)},
            "chebyshev_T01": {"ms": t_cheb * 1e3, "fp64_recurrence_ms": t_cheb64 * 1e3,
                              "cusolver_ms": t_cu1 * 1e3, "speedup_over_cusolver": t_cu1 / t_cheb,
                              "rel_diff_vs_cusolver": r(a, Pcu1), "fp64_rel_diff_vs_cusolver": r(a64, Pcu1)},
            "note": "wall clock, host timer around fully synchronised calls; cuSOLVER (torch.linalg.eigh) and "
                    "its projector are a timed baseline, not part of the library's path"}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------------------------------
GENERAL_WORKLOAD = ("HoneycombLattice(180,180) open (N = 64800), t1=1, LandauGauge(0.01), Anderson U[-1,1], "
                    "M=512 complex-Gaussian kets, dt=0.05, through the general sparse (ELL) path")


def honeycomb_csc(a, b, B, V):
    """Nearest-neighbour honeycomb H (open, Landau phases) as a scipy CSC matrix: the workload
    generator of the general-path bench (sites ordered by (j1, j2, basis))."""
    import scipy.sparse as sp
    j1, j2 = np.meshgrid(np.arange(1, a + 1), np.arange(1, b + 1), indexing="ij")
    j1, j2 = j1.ravel(), j2.ravel()
    A = ((j1 - 1) * b + (j2 - 1)) * 2
    xa = j1 + 0.5 * j2
    ya = (math.sqrt(3) / 2) * j2
    rows, cols = [], []
    for dj1, dj2 in ((0, 0), (-1, 0), (0, -1)):
        ok = (j1 + dj1 >= 1) & (j2 + dj2 >= 1)
        rows.append(A[ok])
        cols.append((((j1 + dj1 - 1) * b + (j2 + dj2 - 1)) * 2 + 1)[ok])
    i = np.concatenate(rows)
    j = np.concatenate(cols)
    xi, yi = xa[i // 2], ya[i // 2]
    xj = (j // 2 // b + 1) + 0.5 * (j // 2 % b + 1) + 0.5
    yj = (math.sqrt(3) / 2) * (j // 2 % b + 1) + math.sqrt(3) / 6
    v = np.exp(-2j * math.pi * (xi + xj) * (yj - yi) * B / 2)
    N = 2 * a * b
    H = sp.coo_matrix((np.concatenate([v, v.conj(), V]),
                       (np.concatenate([i, j, np.arange(N)]), np.concatenate([j, i, np.arange(N)]))), shape=(N, N))
    return H.tocsc()


def run_general_workload(args):
    """Ket steps through lm_ell_* (a honeycomb lattice given as a CSC matrix), c32."""
    import torch
    import lmgpu
    ctx = lmgpu.default_context()
    ext = torch.cuda.ExternalStream(ctx.stream_ptr(), device=torch.device("cuda", 0))
    a = b = 180
    N, M = 2 * a * b, 512
    V = np.random.default_rng(SEED + 5).uniform(-1, 1, N)
    H = lmgpu.SparseHamiltonian(lmgpu.Sites(N, name="honeycomb"), honeycomb_csc(a, b, B_FIELD, V))
    st = lmgpu.KetBlock(H.lattice, make_kets(N, M, dtype=np.complex64), precision="c32")
    solver = lmgpu.ChebyshevGPU()
    solver.update_solver(H, DT)
    for _ in range(args.warmup):
        solver.step(st)
    K = solver.order(st)[0]
    ctx.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for _ in range(args.steps):
        solver.step(st)
    e1.record(ext)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    alg = 5.0 * K * N * M * 8  # the per-order formula, per step
    peak, peak_kind = measured_peak_hbm()
    del st
    # the same lattice as lmgpu.HoneycombLattice: H assembled on the device from the bond
    # geometry, and the brick layout steps the kets through the x-streaming kernel
    lat = lmgpu.HoneycombLattice(a, b)
    Hb = lmgpu.tightbinding_hamiltonian(lat, V, field=lmgpu.LandauGauge(B_FIELD))
    sb = lmgpu.KetBlock(lat, make_kets(N, M, dtype=np.complex64), precision="c32")
    solver_b = lmgpu.ChebyshevGPU()
    solver_b.update_solver(Hb, DT)
    n_stream0 = ctx.stream_launches()
    for _ in range(args.warmup):
        solver_b.step(sb)
    brick_streamed = ctx.stream_launches() - n_stream0 == args.warmup
    Kb = solver_b.order(sb)[0]
    ctx.synchronize()
    e0.record(ext)
    for _ in range(args.steps):
        solver_b.step(sb)
    e1.record(ext)
    e1.synchronize()
    ms_b = e0.elapsed_time(e1) / args.steps
    # the reference's own benchmark loop on this lattice (benchmarks/benchmark_evolution_const.jl:
    # Evolution with a constant H, localdensity at every moment): kets from pinned host memory,
    # both inside the timed region
    del sb
    pin = torch.empty((M, N), dtype=torch.complex64, pin_memory=True)
    Xh = pin.numpy().T
    Xh[:] = make_kets(N, M, dtype=np.complex64)
    e2e_state = lmgpu.DeviceState(lat, None, 0, "c32", shape=(N, M))
    ev = lmgpu.Evolution(lmgpu.ChebyshevGPU(), Hb, e2e_state)
    evs = ev.current_states()[0]
    evs.upload_from(Xh)
    lmgpu.timesequences([lmgpu.moment_density], ev([DT * (k + 1) for k in range(args.warmup)]), nslots=8)
    ev.time = 0.0
    ctx.synchronize()
    e0.record(ext)
    evs.upload_from(Xh)
    (ts_rho,) = lmgpu.timesequences([lmgpu.moment_density], ev([DT * (k + 1) for k in range(args.steps)]), nslots=8)
    e1.record(ext)
    e1.synchronize()
    assert len(ts_rho) == args.steps
    ms_e2e = e0.elapsed_time(e1) / args.steps
    brick_e2e = {"value": M / (ms_e2e / 1000.0), "unit": "ket-steps/s", "ms_per_step": ms_e2e,
                 "h2d_bytes_per_step": int(N * M * 8 / args.steps), "d2h_bytes_per_step": int(N * 8),
                 "path": "Evolution(ChebyshevGPU, H, kets) over timesequences([moment_density], ev(times)): "
                         "localdensity every moment (the reference's constant-H benchmark loop)"}
    brick = {"value": M / (ms_b / 1000.0), "unit": "ket-steps/s", "ms_per_step": ms_b, "K": Kb, "e2e": brick_e2e,
             "streamed": brick_streamed,
             "path": "HoneycombLattice(180,180) + tightbinding_hamiltonian (device assembly); lm_ell_set_layout "
                     "honeycomb: cheb_stream_c32_kernel<K, 4> (all K orders per launch)",
             "speedup_over_ell": ms / ms_b}
    line = {"metric": "ket-steps/s (general sparse path)", "value": M / (ms / 1000.0), "unit": "ket-steps/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "dtype": "c32", "data": "synthetic (seeded PCG64)",
            "config": {"workload": GENERAL_WORKLOAD, "N": N, "M": M, "K": K, "nnz": int(len(H.rowval))},
            "roofline": {"bound": "hbm", "achieved": alg / (ms / 1000.0) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": alg / (ms / 1000.0) / 1e9 / peak, "traffic": None,
                         "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                         "kernel": "cheb_order_ell_kernel (one launch per order)"},
            "honeycomb_brick": brick}
    print(json.dumps(line))
    return 0


REFBENCH_WORKLOAD = ("the reference's evolution benchmarks (benchmarks/benchmark_evolution_const.jl, "
                     "benchmark_evolution_dynamic.jl, model benchmarks/models.jl:3-12) on HoneycombLattice(224,224) "
                     "(N = 100,352; a parallelogram patch standing in for the Circle shape), t1 = -2.8, "
                     "pn-junction potential 0.2 inside r/2, SymmetricGauge(3.0 x 1.519e-3) constant or ramped as "
                     "3.0 min(t/5, 1), one ket, t = 0:0.1:10 (101 moments), localdensity at every moment, ComplexF64")


def run_refbench_workload(args):
    """The reference's own evolution benchmark loop: one ket of a ~1e5-site graphene patch evolved
    over t = 0:0.1:10 with localdensity at every moment, for a constant H and for a field ramp;
    timed on the device from the host ket to the last density, and the oracle's Krylov port of
    KrylovKitExp (one host thread: one ket) timed on the constant-H loop.  The reference's
    starting state is the ground state; a seeded random ket stands in (the cost does not depend
    on it)."""
    import torch
    import lmgpu
    from oracle import krylov, lm_oracle as o
    ctx = lmgpu.default_context()
    ext = torch.cuda.ExternalStream(ctx.stream_ptr(), device=torch.device("cuda", 0))
    a = b = 224
    lat = lmgpu.HoneycombLattice(a, b)
    N = lat.N
    xy = lat.coords()
    c = xy.mean(axis=0)
    r = math.sqrt(N * (math.sqrt(3) / 4) / math.pi)  # radius of a disk of N sites (area sqrt(3)/4 per site)
    V = np.where(((xy - c) ** 2).sum(axis=1) < (r / 2) ** 2, 0.2, 0.0)
    B0 = 3.0 * 1.519e-3
    times = [0.1 * k for k in range(101)]
    rng = np.random.default_rng(SEED + 11)
    psi = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    psi /= np.linalg.norm(psi)
    h_const = lmgpu.tightbinding_hamiltonian(lat, V, t1=-2.8, field=lmgpu.SymmetricGauge(B0))
    h_dyn = lambda t: lmgpu.tightbinding_hamiltonian(lat, V, t1=-2.8,
                                                      field=lmgpu.SymmetricGauge(B0 * min(t / 5.0, 1.0)))

    def run(h):
        ev = lmgpu.Evolution(lmgpu.ChebyshevGPU(), h, lmgpu.Ket(lat, psi))
        (ts,) = lmgpu.timesequences([lmgpu.moment_density], ev(times), nslots=8)
        return ts

    for h in (h_const, h_dyn):  # warm-up: builds, tables, rings
        run(h)
    res = {}
    for name, h in (("constant", h_const), ("dynamic", h_dyn)):
        ms = []
        for _ in range(max(args.steps, 1)):
            ctx.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            ts = run(h)
            e1.record(ext)
            e1.synchronize()
            assert len(ts) == len(times)
            ms.append(e0.elapsed_time(e1))
        res[name] = {"ms_per_run": float(np.median(ms)), "runs": len(ms),
                     "moments_per_s": len(times) / (float(np.median(ms)) / 1000.0)}
    # the oracle's Krylov port on the same constant-H loop (its matrix from the oracle's
    # restatement of the lattice and field)
    Ho, _ = o.honeycomb_hamiltonian(a, b, t1=-2.8, field=o.SymmetricGauge(B0), onsite=V)
    csr = krylov.CSR(Ho)
    X = psi.reshape(-1, 1).astype(np.complex128)
    t0 = time.perf_counter()
    for _ in range(len(times) - 1):
        X = krylov.krylov_expv_block(csr, 0.1, X, tol=1e-12, kdim=30, nthreads=1)
        _ = np.abs(X[:, 0]) ** 2
    cpu_ms = (time.perf_counter() - t0) * 1000.0
    line = {"metric": "ms per run of the reference's evolution benchmark loop (101 moments)",
            "value": res["constant"]["ms_per_run"], "unit": "ms", "n_gpus": 1, "steps": args.steps,
            "higher_is_better": False, "dtype": "c64", "data": "synthetic (seeded random ket; the patch stands "
            "in for the Circle shape)", "config": {"workload": REFBENCH_WORKLOAD, "N": N},
            "gpu": res, "cpu_port_constant": {"ms_per_run": cpu_ms, "cores": 1, "kind": "port",
                                             "sample": "the whole 100-step constant-H loop, Lanczos exponentiate "
                                                       "(tol 1e-12, krylovdim 30) and |psi|^2 per step"},
            "gpu_over_cpu_constant": cpu_ms / res["constant"]["ms_per_run"]}
    print(json.dumps(line))
    return 0


def run_readouts_workload(args):
    """The per-moment readouts of the kets workload, c32: localdensity and DensityCurrents on
    every bond, each through the readout ring (kernel + asynchronous download), timed with CUDA
    events over `steps` readouts."""
    import torch
    import lmgpu
    ctx = lmgpu.default_context()
    ext = torch.cuda.ExternalStream(ctx.stream_ptr(), device=torch.device("cuda", 0))
    lat = lmgpu.SquareLattice(LX, LY, boundaries={"axis1": True, "axis2": True})
    N, M = lat.N, args.kets
    V = np.random.default_rng(SEED + 1).uniform(-1, 1, N)
    H = lmgpu.tightbinding_hamiltonian(lat, V, field=lmgpu.LandauGauge(B_FIELD))
    st = lmgpu.KetBlock(lat, make_kets(N, M, dtype=np.complex64), precision="c32")
    peak, peak_kind = measured_peak_hbm()
    out = {}
    for kind in ("density", "currents"):
        length = N if kind == "density" else int(lat.nbonds())
        ring = lmgpu.timesequence.ReadoutRing(length, 8)
        push = (lambda t: ring.push_density(st, t)) if kind == "density" else (lambda t: ring.push_currents(H, st, t))
        for i in range(args.warmup):
            ring.wait(push(float(i)))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        pending = []
        e0.record(ext)
        for i in range(args.steps):
            pending.append(push(float(i)))
            if len(pending) == 8:
                ring.wait(pending.pop(0))
        e1.record(ext)
        e1.synchronize()
        for q in pending:
            ring.wait(q)
        ms = e0.elapsed_time(e1) / args.steps
        alg = N * M * 8  # one read of the ket block
        out[kind] = {"ms_per_readout": ms, "achieved_gbs": alg / (ms / 1000.0) / 1e9,
                     "frac": alg / (ms / 1000.0) / 1e9 / peak}
    line = {"metric": "ms per readout (density, currents), c32", "value": out["density"]["ms_per_readout"],
            "unit": "ms", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": False,
            "dtype": "c32", "data": "synthetic (seeded PCG64)",
            "config": {"workload": WORKLOAD, "N": N, "M": M},
            "readouts": out, "peak": peak, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
            "note": "algorithmic bytes = one read of the ket block; each readout includes its ring download"}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------------------------------
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="lmgpu", choices=["lmgpu", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--kets", type=int, default=M_KETS)
    ap.add_argument("--workload", default="kets",
                    choices=["kets", "batch", "adjoint", "kpm", "densitymatrix", "general", "readouts", "refbench"],
                    help="kets: the 256^2 ket-block workload (default); batch: 512 uneven dense-P lattices; "
                         "adjoint: loss_and_grad of the 64^2 differentiation workload; kpm: DOS moments; "
                         "densitymatrix: P_0 at T > 0, Chebyshev vs eigensolver; general: honeycomb via ELL; "
                         "readouts: localdensity and DensityCurrents of the kets workload; refbench: the "
                         "reference's own evolution benchmark loop (one graphene ket, 101 moments)")
    ap.add_argument("--instances", type=int, default=512)
    ap.add_argument("--batch-instances", type=int, default=64,
                    help="lattices of the batch sub-record of the default line (0: none)")
    ap.add_argument("--batch-form", default="resident", choices=["resident", "region"],
                    help="batch: lattices that fit on chip in the lattice-resident form (default) or all in "
                         "the region form (bit-identical results)")
    ap.add_argument("--panel", type=int, default=None,
                    help="batch: column-panel width of the per-order path (default 1024 for c64, off for c32)")
    ap.add_argument("--precision", default="c32", choices=["c32", "c64"])
    ap.add_argument("--adjoint-init", default="eigh", choices=["eigh", "random"],
                    help="initial kets of the adjoint workload: lowest eigenstates (default) or random")
    ap.add_argument("--L", type=int, default=256,
                    help="kets workload: side of the periodic square lattice (512 with --kets 1024 is config 3)")
    ap.add_argument("--fused-form", default="stream", choices=["stream", "region"],
                    help="form of the fused c32 step: x-streaming (where the lattice allows) or region")
    ap.add_argument("--err-steps", type=int, default=400,
                    help="steps of the untimed pass that measures the chosen form's error against FP64 "
                         "(400: the plain-method configuration's full length)")
    ap.add_argument("--tol32", type=float, default=1e-9,
                    help="series truncation of the FP32 form (1e-9 keeps 200-step runs within 1e-6; "
                         "1e-7 is one order cheaper and enough for short runs)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    global LX, LY, WORKLOAD
    LX = LY = int(args.L)
    WORKLOAD = WORKLOAD_FMT.format(L=LX, M=args.kets)
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.workload == "batch":
        return run_batch_workload(args)
    if args.workload == "adjoint":
        return run_adjoint_workload(args)
    if args.workload == "kpm":
        return run_kpm_workload(args)
    if args.workload == "densitymatrix":
        return run_densitymatrix_workload(args)
    if args.workload == "general":
        return run_general_workload(args)
    if args.workload == "refbench":
        return run_refbench_workload(args)
    if args.workload == "readouts":
        return run_readouts_workload(args)

    rank, world, local = dist_info()
    import torch
    import lmgpu
    from lmgpu import device as D
    D.set_default_device(local)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    ctx = lmgpu.default_context()
    ctx.set_stream_form(args.fused_form == "stream")
    ext = torch.cuda.ExternalStream(ctx.stream_ptr(), device=torch.device("cuda", local))
    lat = lmgpu.SquareLattice(LX, LY, boundaries={"axis1": True, "axis2": True})
    N, M = lat.N, args.kets
    V = make_disorder(N)
    H = lmgpu.tightbinding_hamiltonian(lat, V, field=lmgpu.LandauGauge(B_FIELD))
    X = make_kets(N, M, rank)

    def barrier():
        ctx.synchronize()
        if dist is not None:
            dist.barrier()

    def timed_steps(state, solver, steps, timing=False):
        cache = solver.evolution_cache(state)
        solver.update_solver(H, DT)
        for _ in range(args.warmup):
            solver.step(state, cache)
        barrier()
        ctx.reset_timing()
        ctx.set_timing(timing)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        for _ in range(steps):
            solver.step(state, cache)
        e1.record(ext)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        order_ms, order_launches, launches = ctx.timing()
        ctx.set_timing(False)
        if dist is not None:
            t = torch.tensor([ms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms, order_ms, order_launches, launches

    # ---- FP32 form (c32) ---------------------------------------------------------------
    s32 = lmgpu.KetBlock(lat, X, precision="c32")
    solver32 = lmgpu.ChebyshevGPU(tol=args.tol32, renorm_every=20)
    clk = ClockSampler(local)
    clk.start()
    n_stream0 = ctx.stream_launches()
    ms32, _, _, launches32 = timed_steps(s32, solver32, args.steps)
    streamed = ctx.stream_launches() - n_stream0 > 0
    K32, a32, b32 = solver32.order(s32)
    # dominant kernel timing pass (events around every Chebyshev sweep, resolved lazily)
    _, order_ms, order_launches, _ = timed_steps(s32, solver32, args.steps, timing=True)

    # ---- compensated FP32 form (value + rounding residual per amplitude) --------------
    del s32
    s32c = lmgpu.KetBlock(lat, X, precision="c32", compensated=True)
    solver32c = lmgpu.ChebyshevGPU(tol=args.tol32, renorm_every=20)
    n_stream0 = ctx.stream_launches()
    ms32c, _, _, launches32c = timed_steps(s32c, solver32c, args.steps)
    streamed_c = ctx.stream_launches() - n_stream0 > 0
    _, order_ms_c, order_launches_c, _ = timed_steps(s32c, solver32c, args.steps, timing=True)
    del s32c

    # ---- plain form (c64) --------------------------------------------------------------
    s64 = lmgpu.KetBlock(lat, X, precision="c64")
    solver64 = lmgpu.ChebyshevGPU()
    ms64, _, _, _ = timed_steps(s64, solver64, args.steps)
    clocks = clk.stop()
    clocks["window"] = "sampled every 100 ms over the timed c32, compensated c32 and c64 passes"
    K64, _, _ = solver64.order(s64)

    del s64

    # ---- error of the FP32 forms against FP64 over the configuration's full length ------
    # an untimed pass: all forms from the same kets, err_steps steps of the same H and dt
    def fp32_error(compensated):
        s32e = lmgpu.KetBlock(lat, X, precision="c32", compensated=compensated)
        sol32e = lmgpu.ChebyshevGPU(tol=args.tol32, renorm_every=20)
        c32e = sol32e.evolution_cache(s32e)
        sol32e.update_solver(H, DT)
        for _ in range(args.err_steps):
            sol32e.step(s32e, c32e)
        r32 = lmgpu.localdensity(s32e).values
        J32 = lmgpu.DensityCurrents(H, s32e).bond_values()
        return {"density": float(np.linalg.norm(r32 - r64) / np.linalg.norm(r64)),
                "currents": float(np.linalg.norm(J32 - J64) / np.linalg.norm(J64)),
                "norm_drift": float(np.abs(s32e.norms() - 1.0).max()),
                "norm_drift_fp64": drift64, "steps": args.err_steps, "kets": M}

    s64e = lmgpu.KetBlock(lat, X, precision="c64")
    sol64e = lmgpu.ChebyshevGPU()
    sol64e.update_solver(H, DT)
    for _ in range(args.err_steps):
        sol64e.step(s64e)
    r64 = lmgpu.localdensity(s64e).values
    J64 = lmgpu.DensityCurrents(H, s64e).bond_values()
    drift64 = float(np.abs(s64e.norms() - 1.0).max())
    del s64e
    err_plain32 = fp32_error(False)
    err_comp = fp32_error(True) if streamed_c else None
    # the chosen form: the compensated one where it meets the metric's 1e-6 bar, else plain FP32
    use_comp = err_comp is not None and max(err_comp["density"], err_comp["currents"]) <= 1e-6
    err = err_comp if use_comp else err_plain32

    # ---- end to end through the public API with host buffers ----------------------------
    # The reference README's loop: every moment of ev(times) yields localdensity(P) and
    # DensityCurrents(H, P), and h(t) is a genuinely time-dependent Hamiltonian (the Landau
    # amplitude and the on-site potential both change every step; the potential is written
    # into pinned host memory each step, uploaded and assembled on the device).
    pin_X = torch.empty((M, N), dtype=torch.complex64, pin_memory=True)
    Xh = pin_X.numpy().T  # (N, M) Fortran view of pinned memory
    Xh[:] = X.astype(np.complex64)
    pin_V = [torch.empty(N, dtype=torch.float64, pin_memory=True).numpy() for _ in range(2)]
    nb = int(lat.nbonds())

    def h(t):
        k = int(round(t / DT))
        pv = pin_V[k % 2]
        np.add(V, 0.05 * math.sin(0.5 * t), out=pv)
        return lmgpu.tightbinding_hamiltonian(lat, pv, field=lmgpu.LandauGauge(B_FIELD * (1.0 + 0.1 * math.sin(t))))

    e2e_state = lmgpu.DeviceState(lat, None, 0, "c32", shape=(N, M))
    if use_comp:
        e2e_state.set_compensation(True)
    ev = lmgpu.Evolution(lmgpu.ChebyshevGPU(tol=args.tol32, renorm_every=20), h, e2e_state)
    evs = ev.current_states()[0]
    times = [DT * (k + 1) for k in range(args.steps)]
    readouts = [lmgpu.moment_density, lmgpu.moment_currents]
    evs.upload_from(Xh)  # untimed warm-up of the pinned-buffer upload and of both readout rings
    lmgpu.timesequences(readouts, ev([DT * (k + 1) for k in range(args.warmup)]), nslots=8)
    e0 = torch.cuda.Event(enable_timing=True)
    eu = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    ev.time = 0.0
    barrier()
    e0.record(ext)
    evs.upload_from(Xh)
    eu.record(ext)
    ts_rho, ts_J = lmgpu.timesequences(readouts, ev(times), nslots=8)
    e1.record(ext)
    e1.synchronize()
    assert len(ts_rho) == args.steps and len(ts_J) == args.steps
    ms_e2e = e0.elapsed_time(e1)
    ms_upload = e0.elapsed_time(eu)
    if dist is not None:
        t_ = torch.tensor([ms_e2e], device="cuda")
        dist.all_reduce(t_, op=dist.ReduceOp.MAX)
        ms_e2e = float(t_.item())
    h2d = (N * M * 8 + args.steps * N * 8) / args.steps
    d2h = N * 8 + nb * 8
    del e2e_state, ev, evs

    # ---- a small instance of the batching workload (observed on every default run) ----
    batch_rec = None
    if world == 1 and args.batch_instances > 0:
        batch_rec = batch_subrecord(args.batch_instances, steps=3, warmup=max(args.warmup, 3))

    # ---- report ----------------------------------------------------------------------
    if rank != 0:
        if dist is not None:
            dist.barrier()
            dist.destroy_process_group()
        return 0
    ms32_plain = ms32
    # per-launch time of the step kernel of each FP32 form (its event-timed pass)
    launch_ms_plain = order_ms / max(order_launches // max(K32, 1), 1)
    launch_ms_comp = order_ms_c / max(order_launches_c // max(K32, 1), 1)
    value_plain32 = world * M * args.steps / (ms32 / 1000.0)
    value_comp = world * M * args.steps / (ms32c / 1000.0)
    if use_comp:
        ms32, order_ms, order_launches, launches32, streamed = ms32c, order_ms_c, order_launches_c, launches32c, streamed_c
    value = world * M * args.steps / (ms32 / 1000.0)
    plain = world * M * args.steps / (ms64 / 1000.0)
    # one launch of the temporally blocked kernel applies all K32 orders of a step; its
    # algorithmic bytes are the per-ket-step figure 5*K*N*s times the M kets it advances, plus
    # for the compensated form the residual plane read and written once (2 x 8 B per site-ket)
    s_bytes = 8
    sweeps = max(order_launches // max(K32, 1), 1)
    alg_bytes_launch = 5.0 * K32 * N * M * s_bytes + (2.0 * N * M * s_bytes if use_comp else 0.0)
    avg_launch_ms = order_ms / sweeps
    achieved = alg_bytes_launch / (avg_launch_ms / 1000.0) / 1e9
    peak, peak_kind = measured_peak_hbm()
    traffic, traffic_src = None, None
    if streamed:
        kname = (f"cheb_stream_c32_kernel<{K32}, 3, {'true' if use_comp else 'false'}> (x-streaming form: all K "
                 f"orders of one step per launch{', compensated state' if use_comp else ''})")
        rec_name = TRAFFIC_RECORD_COMP if use_comp else TRAFFIC_RECORD
        t_cap, units_cap, rec = profile_traffic(rec_name)
        if t_cap is not None and rec.get("K") == K32:
            traffic = t_cap * (N * M) / units_cap
            traffic_src = (f"ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch at {rec['sites']} sites x "
                           f"{rec['kets']} kets (profiles/{rec_name}, source sha256 {rec['source_sha256'][:12]} "
                           f"matches), scaled by sites x kets")
        else:
            traffic_src = rec if isinstance(rec, str) else "ncu record is for another order"
    else:
        kname = "cheb_fused_c32_kernel (region form: all K orders of one step per launch)"
        traffic_src = "no ncu record for the region form in this build"
    # FP32 FMA pipe: the useful FMAs of a site-order are the real diagonal (2), the real x-hops
    # of the Landau gauge (2 x 2), the complex y-hops (2 x 4) and the accumulator term (2)
    fma_site_order = 16
    props = torch.cuda.get_device_properties(local)
    sm_mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    fma_peak = props.multi_processor_count * 128 * sm_mhz * 1e6
    fma_rate = fma_site_order * N * M * K32 / (avg_launch_ms / 1000.0)
    line = {
        "metric": METRIC, "value": value, "unit": "ket-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms32 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c32",
        "data": "synthetic (seeded PCG64: complex-Gaussian kets, U[-1,1] disorder)",
        "config": {"workload": WORKLOAD, "N": N, "M_per_gpu": M, "dt": DT,
                   "chebyshev_order_c32": K32, "chebyshev_order_c64": K64,
                   "spectral_half_width": a32, "tol_c32": args.tol32, "tol_c64": 1e-12,
                   "renorm_every": 20,
                   "l2": f"inputs larger than L2 (ket block {N * M * 8 / 1e9:.2f} GB c32 vs 0.129 GB L2)"},
        "plain_fp64": {"value": plain, "unit": "ket-steps/s", "ms_per_step": ms64 / args.steps,
                       "dtype": "c64"},
        "chosen_over_plain": value / plain,
        "chosen_form": ("c32 compensated (FP32 value + its rounding residual as a bfloat16 pair per site, "
                        "error-free TwoProd/TwoSum on FP32 pairs in the x-streaming kernel)" if use_comp else "c32"),
        "rel_err_vs_fp64": err,
        "fp32_forms": {
            "plain_c32": {"value": value_plain32, "ms_per_step": ms32_plain / args.steps,
                          "ms_per_launch": launch_ms_plain, "rel_err_vs_fp64": err_plain32},
            "compensated_c32": {"value": value_comp, "ms_per_step": ms32c / args.steps,
                                "ms_per_launch": launch_ms_comp, "rel_err_vs_fp64": err_comp,
                                "streamed": streamed_c},
        },
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "kernel": kname,
                     "alg_bytes_per_launch": alg_bytes_launch, "avg_launch_ms": avg_launch_ms,
                     "launches_timed": sweeps, "traffic_source": traffic_src,
                     # physical fractions: what the temporally blocked kernel really moves and
                     # computes per launch
                     "dram_gbs": (traffic / (avg_launch_ms / 1000.0) / 1e9) if traffic else None,
                     "dram_frac": (traffic / (avg_launch_ms / 1000.0) / 1e9 / peak) if traffic else None,
                     "fma_frac": fma_rate / fma_peak,
                     "fma_note": (f"{fma_site_order} useful FP32 FMAs per site-order x N x M x K per launch / "
                                  f"({props.multi_processor_count} SMs x 128 FMA/clk x {sm_mhz:.0f} MHz median "
                                  f"SM clock of the run)"),
                     "note": "frac is the per-order formula 5*K*N*M*s: all K orders of a step run on chip, so "
                             "it exceeds 1; dram_frac and fma_frac are the physical fractions"},
        "e2e": {"value": world * M * args.steps / (ms_e2e / 1000.0), "unit": "ket-steps/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ms_per_step": ms_e2e / args.steps,
                "path": "Evolution(ChebyshevGPU, t -> tightbinding_hamiltonian(l, V(t); LandauGauge(B(t)))) "
                        "over timesequences([moment_density, moment_currents], ev(times)): both readouts "
                        "every moment through readout rings, asynchronous downloads",
                "upload_ms": ms_upload},
        "gpu_launches": int(launches32),
        "clocks": clocks,
    }
    if batch_rec is not None:
        line["batch"] = batch_rec
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_reference(1, 1, cpu_seconds=20.0)
        one = cpu_reference(1, 1, sample_kets=2, cpu_seconds=8.0, nthreads=1)
        line["cpu_baseline"]["single_core"] = {k: one[k] for k in ("value", "unit", "cores", "sample")}
    print(json.dumps(line))
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
