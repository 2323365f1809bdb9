// Device building blocks shared by the per-order Chebyshev kernels (single lattice and batch).
#pragma once
#include <cuda_runtime.h>

#include "lmgpu_internal.cuh"

namespace lmgpu {

template <typename T> struct CT;
template <> struct CT<double> {
    typedef double2 V;
    static __device__ __forceinline__ V make(double a, double b) { return make_double2(a, b); }
};
template <> struct CT<float> {
    typedef float2 V;
    static __device__ __forceinline__ V make(float a, float b) { return make_float2(a, b); }
};

// ------------------------------------------------------------------------------------------
// Neighbour routing on the square lattice (src/core/boundaries.jl:251-289 for the periodic
// case: a destination one step outside is wrapped by the axis translation).
// ------------------------------------------------------------------------------------------
struct Nbr {
    int64_t xp, xm, yp, ym;   // neighbour site indices (self when the bond is absent)
    bool hxp, hxm, hyp, hym;  // bond present
};

__device__ __forceinline__ Nbr neighbours(const Geom& g, int64_t s) {
    Nbr n;
    const int64_t xi = s / g.Ly, yi = s - xi * g.Ly;
    // +x
    if (xi + 1 < g.Lx) { n.xp = s + g.Ly; n.hxp = true; }
    else if (g.per_x) { n.xp = yi; n.hxp = true; }
    else { n.xp = s; n.hxp = false; }
    // -x
    if (xi > 0) { n.xm = s - g.Ly; n.hxm = true; }
    else if (g.per_x) { n.xm = (g.Lx - 1) * g.Ly + yi; n.hxm = true; }
    else { n.xm = s; n.hxm = false; }
    // +y
    if (yi + 1 < g.Ly) { n.yp = s + 1; n.hyp = true; }
    else if (g.per_y) { n.yp = s - yi; n.hyp = true; }
    else { n.yp = s; n.hyp = false; }
    // -y
    if (yi > 0) { n.ym = s - 1; n.hym = true; }
    else if (g.per_y) { n.ym = s + g.Ly - 1; n.hym = true; }
    else { n.ym = s; n.hym = false; }
    return n;
}

// ------------------------------------------------------------------------------------------
// One order of the Chebyshev recurrence for exp(-i H dt), H~ = (H - b)/a:
//   FIRST: T1 = H~ T0            -> tq;   y  = c0 T0 + c1 T1
//   MID  : Tk = 2 H~ T(k-1) - T(k-2) -> tq (in place over T(k-2));  y += ck Tk
//   LAST : out = phase * (y + cK TK)   -> tq (in place over T(K-2))
// c_k = s (k even) or -i s (k odd); the tables hold 2H/a and 2(V-b)/a.
// Layout: SITE_FAST -> element (site, ket) at ket*ld + site (column-major ket block);
//         otherwise   -> element (site, ket) at site*ld + ket (row of a column-major matrix).
// CONJ applies conj(H) (used for the right factor U^dagger of a density-matrix step).
// ------------------------------------------------------------------------------------------
template <typename R, int MODE, bool SITE_FAST, bool CONJ, int INNER>
__device__ __forceinline__ void cheb_order_block(
    const Geom& g, const typename CT<R>::V* __restrict__ hop2, const R* __restrict__ diag2,
    const typename CT<R>::V* __restrict__ tp, typename CT<R>::V* tq, typename CT<R>::V* y,
    int64_t ld, int64_t M, R c0, R cs, int odd, R ph_re, R ph_im, int64_t lane, int64_t g_first, int64_t g_stride) {
    typedef typename CT<R>::V V;
    const int64_t nfast = SITE_FAST ? g.N : M;
    const int64_t nslow = SITE_FAST ? M : g.N;
    if (lane >= nfast) return;
    // SITE_FAST: the site is fixed per thread, so its stencil row is loaded once.
    Nbr nb;
    V hxp, hxm, hyp, hym;
    R d = 0;
    auto load_row = [&](int64_t s) {
        nb = neighbours(g, s);
        V z = CT<R>::make(0, 0);
        hxp = nb.hxp ? hop2[s] : z;
        hyp = nb.hyp ? hop2[g.N + s] : z;
        V t = nb.hxm ? hop2[nb.xm] : z;  // H[s, s-x] = conj(H[s-x, s])
        hxm = CT<R>::make(t.x, -t.y);
        t = nb.hym ? hop2[g.N + nb.ym] : z;
        hym = CT<R>::make(t.x, -t.y);
        if (CONJ) {
            hxp.y = -hxp.y; hyp.y = -hyp.y; hxm.y = -hxm.y; hym.y = -hym.y;
        }
        d = diag2[s];
    };
    if (SITE_FAST) load_row(lane);

    for (int64_t g0 = g_first; g0 < nslow; g0 += g_stride) {
#pragma unroll
        for (int j = 0; j < INNER; ++j) {
            const int64_t slow = g0 + j;
            if (slow >= nslow) break;
            int64_t site, ket;
            if (SITE_FAST) { site = lane; ket = slow; }
            else { site = slow; ket = lane; load_row(site); }
            auto at = [&](int64_t s) -> int64_t { return SITE_FAST ? ket * ld + s : s * ld + ket; };
            const V v0 = tp[at(site)];
            const V vxp = tp[at(nb.xp)], vxm = tp[at(nb.xm)];
            const V vyp = tp[at(nb.yp)], vym = tp[at(nb.ym)];
            V acc;
            if (MODE == CHEB_FIRST) {
                acc = CT<R>::make(0, 0);
            } else {
                const V q = tq[at(site)];
                acc = CT<R>::make(-q.x, -q.y);
            }
            acc.x = fma(hxp.x, vxp.x, acc.x); acc.x = fma(-hxp.y, vxp.y, acc.x);
            acc.y = fma(hxp.x, vxp.y, acc.y); acc.y = fma(hxp.y, vxp.x, acc.y);
            acc.x = fma(hxm.x, vxm.x, acc.x); acc.x = fma(-hxm.y, vxm.y, acc.x);
            acc.y = fma(hxm.x, vxm.y, acc.y); acc.y = fma(hxm.y, vxm.x, acc.y);
            acc.x = fma(hyp.x, vyp.x, acc.x); acc.x = fma(-hyp.y, vyp.y, acc.x);
            acc.y = fma(hyp.x, vyp.y, acc.y); acc.y = fma(hyp.y, vyp.x, acc.y);
            acc.x = fma(hym.x, vym.x, acc.x); acc.x = fma(-hym.y, vym.y, acc.x);
            acc.y = fma(hym.x, vym.y, acc.y); acc.y = fma(hym.y, vym.x, acc.y);
            acc.x = fma(d, v0.x, acc.x);
            acc.y = fma(d, v0.y, acc.y);
            if (MODE == CHEB_FIRST) {
                // T1 = (sum)/2 exactly, y = c0 T0 + c1 T1 with c1 = -i s (or +i s when conj)
                const V t1 = CT<R>::make(acc.x * R(0.5), acc.y * R(0.5));
                tq[at(site)] = t1;
                V yy;
                yy.x = fma(cs, t1.y, c0 * v0.x);
                yy.y = fma(-cs, t1.x, c0 * v0.y);
                y[at(site)] = yy;
            } else {
                V yy = y[at(site)];
                if (odd) {
                    yy.x = fma(cs, acc.y, yy.x);
                    yy.y = fma(-cs, acc.x, yy.y);
                } else {
                    yy.x = fma(cs, acc.x, yy.x);
                    yy.y = fma(cs, acc.y, yy.y);
                }
                if (MODE == CHEB_MID) {
                    tq[at(site)] = acc;
                    y[at(site)] = yy;
                } else {
                    V o;
                    o.x = fma(ph_re, yy.x, -ph_im * yy.y);
                    o.y = fma(ph_re, yy.y, ph_im * yy.x);
                    tq[at(site)] = o;
                }
            }
        }
    }
}


}  // namespace lmgpu
