"""Numerical design check (CPU) for a double-float KPM recurrence: the Chebyshev moments of an
FP32-pair ("double-float") recurrence against the FP64 recurrence.

The KPM and Fermi-operator recurrences run in FP64, which GB300 executes at 1/64 of its FP32
rate.  A recurrence on pairs of FP32 numbers (hi + lo, about 48 significant bits) would move the
arithmetic to the FP32 pipe.  Its risk is accuracy: the three-term recurrence
T_{n+1} = 2 H~ T_n - T_{n-1} cancels at every pass.  This test emulates that arithmetic exactly
in numpy float32 and measures the moment error after hundreds of passes.  Every float32
operation rounds once; products are split with Dekker's method, so no fused multiply-add is
needed.  Both the accurate and the cheaper ("sloppy") double-word addition are measured.  The
moment tolerance of the KPM parity tests is 1e-11 mu_0.
"""
import numpy as np
import pytest

from oracle import lm_oracle as o

f32 = np.float32


def two_sum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def fast_two_sum(a, b):
    s = a + b
    return s, b - (s - a)


def split(a):
    c = f32(4097.0) * a  # 2^12 + 1 for a 24-bit significand
    hi = c - (c - a)
    return hi, a - hi


def two_prod(a, b):
    p = a * b
    ah, al = split(a)
    bh, bl = split(b)
    return p, ((ah * bh - p) + ah * bl + al * bh) + al * bl


def add_accurate(xh, xl, yh, yl):
    s, e = two_sum(xh, yh)
    t, f = two_sum(xl, yl)
    e = e + t
    s, e = fast_two_sum(s, e)
    e = e + f
    return fast_two_sum(s, e)


def add_sloppy(xh, xl, yh, yl):
    s, e = two_sum(xh, yh)
    e = e + (xl + yl)
    return fast_two_sum(s, e)


def mul(xh, xl, yh, yl):
    p, e = two_prod(xh, yh)
    e = e + (xh * yl + xl * yh)
    return fast_two_sum(p, e)


def to_df(x):
    hi = x.astype(f32)
    return hi, (x - hi.astype(np.float64)).astype(f32)


def from_df(h, lo):
    return h.astype(np.float64) + lo.astype(np.float64)


def moments(L, nv, npass, add, seed=1):
    """(FP64, double-float, plain FP32) moments of nv random-phase vectors on an L x L periodic
    Landau lattice with disorder; the stencil is summed in a fixed order over the row's slots."""
    lat = o.SquareLattice(L, L, periodic=(True, True))
    H = o.tightbinding_hamiltonian(lat, field=o.LandauGauge(0.01), onsite=o.anderson_disorder(lat.N, 2.0, seed))
    Hd = H.toarray()
    w = np.linalg.eigvalsh(Hd)
    emin, emax = w[0] - 0.05, w[-1] + 0.05
    a, b = (emax - emin) / 2, (emax + emin) / 2
    Ht = (Hd - b * np.eye(lat.N)) / a
    N = lat.N
    v = np.exp(2j * np.pi * np.random.default_rng(seed).random((N, nv))) / np.sqrt(N)

    T0, T1 = v.copy(), Ht @ v
    mu64 = [np.real(np.vdot(v, T0)), np.real(np.vdot(v, T1))]
    for _ in range(2, npass):
        T0, T1 = T1, 2 * (Ht @ T1) - T0
        mu64.append(np.real(np.vdot(v, T1)))

    # ELL slots: row r holds its stored entries in column order, zero-padded
    width = max(int(np.count_nonzero(Ht[r])) for r in range(N))
    cols = np.zeros((N, width), dtype=np.int64)
    vals = np.zeros((N, width), dtype=np.complex128)
    for r in range(N):
        nz = np.nonzero(Ht[r])[0]
        cols[r, :len(nz)] = nz
        vals[r, :len(nz)] = Ht[r, nz]
    hr, hrl = to_df(vals.real)
    hi, hil = to_df(vals.imag)

    def matvec(x):
        xr, xrl, xi, xil = x
        yr = np.zeros((N, nv), f32), np.zeros((N, nv), f32)
        yi = np.zeros((N, nv), f32), np.zeros((N, nv), f32)
        for j in range(width):
            c = cols[:, j]
            ar, arl, ai, ail = hr[:, j, None], hrl[:, j, None], hi[:, j, None], hil[:, j, None]
            p = mul(ar, arl, xr[c], xrl[c])
            q = mul(ai, ail, xi[c], xil[c])
            re = add(p[0], p[1], -q[0], -q[1])
            p = mul(ar, arl, xi[c], xil[c])
            q = mul(ai, ail, xr[c], xrl[c])
            im = add(p[0], p[1], q[0], q[1])
            yr = add(yr[0], yr[1], re[0], re[1])
            yi = add(yi[0], yi[1], im[0], im[1])
        return yr[0], yr[1], yi[0], yi[1]

    def mu_of(x):
        return np.real(np.vdot(v, from_df(x[0], x[1]) + 1j * from_df(x[2], x[3])))

    vr, vi = to_df(v.real), to_df(v.imag)
    T0 = (vr[0], vr[1], vi[0], vi[1])
    T1 = matvec(T0)
    mudf = [mu_of(T0), mu_of(T1)]
    two = (f32(2.0), f32(0.0))
    for _ in range(2, npass):
        y = matvec(T1)
        r = mul(two[0], two[1], y[0], y[1])
        r = add(r[0], r[1], -T0[0], -T0[1])
        i = mul(two[0], two[1], y[2], y[3])
        i = add(i[0], i[1], -T0[2], -T0[3])
        T0, T1 = T1, (r[0], r[1], i[0], i[1])
        mudf.append(mu_of(T1))
    # a plain FP32 recurrence (complex64) for contrast
    H32 = Ht.astype(np.complex64)
    v32 = v.astype(np.complex64)
    T0, T1 = v32.copy(), H32 @ v32
    mu32 = [np.real(np.vdot(v, T0.astype(np.complex128))), np.real(np.vdot(v, T1.astype(np.complex128)))]
    for _ in range(2, npass):
        T0, T1 = T1, np.complex64(2) * (H32 @ T1) - T0
        mu32.append(np.real(np.vdot(v, T1.astype(np.complex128))))
    return np.array(mu64), np.array(mudf), np.array(mu32)


@pytest.mark.parametrize("add", [add_accurate, add_sloppy], ids=["accurate", "sloppy"])
def test_doublefloat_moments_track_fp64(add):
    mu64, mudf, mu32 = moments(L=8, nv=4, npass=512, add=add)
    err = np.abs(mudf - mu64) / abs(mu64[0])
    # measured about 7e-15 after 512 passes (1.2e-14 after 1024): three orders of magnitude
    # inside the moment tolerance of the KPM parity tests
    assert err.max() <= 1e-12, err.max()
    # a plain FP32 recurrence, for contrast, is far outside it
    assert (np.abs(mu32 - mu64) / abs(mu64[0])).max() > 1e-8
