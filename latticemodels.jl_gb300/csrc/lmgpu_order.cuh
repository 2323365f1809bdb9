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
// Sum of products over kets.  Acc<double> is a plain FP64 accumulator.  Acc<float> is a
// double-float accumulator: an unevaluated pair hi + lo.  Each product is split exactly by an
// FMA, and Knuth's TwoSum adds it.  The pair carries ~48 significant bits at FP32 issue rates.
// GB300 runs FP64 at 1/64 of its FP32 rate, so an FP64 accumulator per element would bound the
// readout and gradient kernels of c32 states.
// ------------------------------------------------------------------------------------------
template <typename R> struct Acc;
template <> struct Acc<double> {
    double v = 0.0;
    __device__ __forceinline__ void add_prod(double a, double b) { v = fma(a, b, v); }
    __device__ __forceinline__ double get() const { return v; }
};
template <> struct Acc<float> {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add_prod(float a, float b) {
        const float p = __fmul_rn(a, b);
        const float pe = __fmaf_rn(a, b, -p);  // a*b = p + pe exactly
        const float s = __fadd_rn(hi, p);      // TwoSum(hi, p) = s + e exactly
        const float bp = __fsub_rn(s, hi);
        const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(p, bp));
        hi = s;
        lo = __fadd_rn(lo, __fadd_rn(e, pe));
    }
    __device__ __forceinline__ double get() const { return (double)hi + (double)lo; }
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
//   FIRST: T1 = H~ T0            -> tq;   y  = c0 T0 + c1 T1 (+ g0 T0 + g1 T1 in FP32, see ChebLo)
//   MID  : Tk = 2 H~ T(k-1) - T(k-2) -> tq (in place over T(k-2));  y += ck Tk
//   LAST : out = phase * (y + cK TK)   -> tq (in place over T(K-2))
// c_k = s (k even) or -i s (k odd); the tables hold 2H/a and 2(V-b)/a.
// Layout: SITE_FAST -> element (site, ket) at ket*ld + site (column-major ket block);
//         otherwise   -> element (site, ket) at site*ld + ket (row of a column-major matrix).
// CONJ applies conj(H) (used for the right factor U^dagger of a density-matrix step).
// ------------------------------------------------------------------------------------------
// Order epilogue at one (site, ket) element with index i, given acc = (2H~) T_{k-1} - T_{k-2}
// (FIRST: acc = 2H~ T0 and v0 = T0):
//   FIRST: T1 = acc/2 -> tq;  y = c0 T0 + c1 T1 (+ g0 T0 + g1 T1 in FP32, see ChebLo)
//   MID  : T_k = acc -> tq;   y += c_k T_k
//   LAST : out = phase * (y + c_K T_K) -> tq
template <typename R, int MODE>
__device__ __forceinline__ void cheb_epilogue(typename CT<R>::V acc, typename CT<R>::V v0, typename CT<R>::V* tq,
                                              typename CT<R>::V* y, int64_t i, R c0, R cs, int odd, R ph_re, R ph_im,
                                              const ChebLo& lo) {
    typedef typename CT<R>::V V;
    if (MODE == CHEB_FIRST) {
        // T1 = (sum)/2 exactly, y = c0 T0 + c1 T1 with c1 = -i s (or +i s when conj)
        const V t1 = CT<R>::make(acc.x * R(0.5), acc.y * R(0.5));
        tq[i] = t1;
        V yy;
        if (sizeof(R) == sizeof(float)) {
            // second words g0 T0 + g1 T1 first, the dominant c0 T0 last
            R lx = fma(R(lo.g0_re), v0.x, fma(R(-lo.g0_im), v0.y, fma(R(lo.g1_re), t1.x, R(-lo.g1_im) * t1.y)));
            R ly = fma(R(lo.g0_re), v0.y, fma(R(lo.g0_im), v0.x, fma(R(lo.g1_re), t1.y, R(lo.g1_im) * t1.x)));
            yy.x = fma(c0, v0.x, fma(cs, t1.y, lx));
            yy.y = fma(c0, v0.y, fma(-cs, t1.x, ly));
        } else {
            yy.x = fma(cs, t1.y, c0 * v0.x);
            yy.y = fma(-cs, t1.x, c0 * v0.y);
        }
        y[i] = yy;
    } else {
        V yy = y[i];
        if (odd) {
            yy.x = fma(cs, acc.y, yy.x);
            yy.y = fma(-cs, acc.x, yy.y);
        } else {
            yy.x = fma(cs, acc.x, yy.x);
            yy.y = fma(cs, acc.y, yy.y);
        }
        if (MODE == CHEB_MID) {
            tq[i] = acc;
            y[i] = yy;
        } else {
            V o;
            o.x = fma(ph_re, yy.x, -ph_im * yy.y);
            o.y = fma(ph_re, yy.y, ph_im * yy.x);
            tq[i] = o;
        }
    }
}

// XR: every x-hop is real (the Landau gauge, no twist across x), so the x-neighbour terms take
// 2 FMAs instead of 4; the skipped terms multiply a zero imaginary part.
template <typename R, int MODE, bool SITE_FAST, bool CONJ, int INNER, bool XR = false>
__device__ __forceinline__ void cheb_order_block(
    const Geom& g, const typename CT<R>::V* __restrict__ hop2, const R* __restrict__ diag2,
    const typename CT<R>::V* __restrict__ tp, typename CT<R>::V* tq, typename CT<R>::V* y,
    int64_t ld, int64_t M, R c0, R cs, int odd, R ph_re, R ph_im, ChebLo lo, int64_t lane, int64_t g_first,
    int64_t g_stride) {
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
            if (XR) {
                acc.x = fma(hxp.x, vxp.x, acc.x);
                acc.y = fma(hxp.x, vxp.y, acc.y);
                acc.x = fma(hxm.x, vxm.x, acc.x);
                acc.y = fma(hxm.x, vxm.y, acc.y);
            } else {
                acc.x = fma(hxp.x, vxp.x, acc.x); acc.x = fma(-hxp.y, vxp.y, acc.x);
                acc.y = fma(hxp.x, vxp.y, acc.y); acc.y = fma(hxp.y, vxp.x, acc.y);
                acc.x = fma(hxm.x, vxm.x, acc.x); acc.x = fma(-hxm.y, vxm.y, acc.x);
                acc.y = fma(hxm.x, vxm.y, acc.y); acc.y = fma(hxm.y, vxm.x, acc.y);
            }
            acc.x = fma(hyp.x, vyp.x, acc.x); acc.x = fma(-hyp.y, vyp.y, acc.x);
            acc.y = fma(hyp.x, vyp.y, acc.y); acc.y = fma(hyp.y, vyp.x, acc.y);
            acc.x = fma(hym.x, vym.x, acc.x); acc.x = fma(-hym.y, vym.y, acc.x);
            acc.y = fma(hym.x, vym.y, acc.y); acc.y = fma(hym.y, vym.x, acc.y);
            acc.x = fma(d, v0.x, acc.x);
            acc.y = fma(d, v0.y, acc.y);
            cheb_epilogue<R, MODE>(acc, v0, tq, y, at(site), c0, cs, odd, ph_re, ph_im, lo);
        }
    }
}


// ------------------------------------------------------------------------------------------
// Line integrals of the gauge fields, evaluated exactly as written in the reference
// (src/zoo/magneticfields.jl:15, :31, :72-85, :89-104), without contraction.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ double li_pointflux_axial(double flux, double px, double py, double x1, double y1,
                                     double x2, double y2) {
    x1 = __dsub_rn(x1, px); y1 = __dsub_rn(y1, py);
    x2 = __dsub_rn(x2, px); y2 = __dsub_rn(y2, py);
    const double n1 = sqrt(__dadd_rn(__dmul_rn(x1, x1), __dmul_rn(y1, y1)));
    const double n2 = sqrt(__dadd_rn(__dmul_rn(x2, x2), __dmul_rn(y2, y2)));
    if (n1 < 1e-11 || n2 < 1e-11) return 0.0 * flux;
    const double nnorm = __dmul_rn(n1, n2);
    const double det = __dsub_rn(__dmul_rn(x1, y2), __dmul_rn(x2, y1));
    const double dot = __dadd_rn(__dmul_rn(x1, x2), __dmul_rn(y1, y2));
    const double cosang = __ddiv_rn(__ddiv_rn(dot, nnorm), 1.0 + 1e-11);
    const double sgn = (det > 0.0) ? 1.0 : ((det < 0.0) ? -1.0 : 0.0);
    const double angle = __dmul_rn(acos(cosang), sgn);
    return __ddiv_rn(__dmul_rn(angle, flux), 2.0 * M_PI);
}

__device__ __forceinline__ double li_pointflux_singular(double flux, double px, double py, double x1, double y1,
                                        double x2, double y2) {
    x1 = __dsub_rn(x1, px); y1 = __dsub_rn(y1, py);
    x2 = __dsub_rn(x2, px); y2 = __dsub_rn(y2, py);
    const double sg = __dsub_rn(x2, x1);
    if (fabs(sg) < 1e-11) return 0.0 * flux;
    if (__dmul_rn(x1, x2) > 0.0 || fmax(x1, x2) == 0.0) return 0.0 * flux;
    const double yint = __ddiv_rn(__dadd_rn(__dmul_rn(-y1, x2), __dmul_rn(y2, x1)), __dsub_rn(x1, x2));
    if (yint > 0.0) return 0.0 * flux;
    return __dmul_rn(flux, (sg > 0.0) ? 1.0 : -1.0);
}

__device__ __forceinline__ double field_line_integral(const Geom& g, const FieldSet& f, double x1, double y1,
                                                     double x2, double y2) {
    double li = 0.0;
    for (int c = 0; c < f.n; ++c) {
        const FieldComp fc = f.c[c];
        const double A = f.amp[c];
        double v = 0.0;
        switch (fc.kind) {
            case LM_FIELD_LANDAU:  // (x1+x2)*(y2-y1)*B/2
                v = __ddiv_rn(__dmul_rn(__dmul_rn(__dadd_rn(x1, x2), __dsub_rn(y2, y1)), A), 2.0);
                break;
            case LM_FIELD_SYMMETRIC:  // (x1*y2 - x2*y1)/2*B
                v = __dmul_rn(__ddiv_rn(__dsub_rn(__dmul_rn(x1, y2), __dmul_rn(x2, y1)), 2.0), A);
                break;
            case LM_FIELD_POINTFLUX_AXIAL:
            case LM_FIELD_POINTFLUX_SINGULAR:
                if (fc.replicate) {
                    // adapt_field: images p - sum_i n_i T_i over CartesianIndex(-1..1)^d,
                    // first boundary fastest, singular gauge (magneticfields.jl:237-266)
                    const int nb = (g.per_x ? 1 : 0) + (g.per_y ? 1 : 0);
                    const int nimg = (nb == 2) ? 9 : 3;
                    double acc = 0.0;
                    for (int im = 0; im < nimg; ++im) {
                        int n0 = im % 3 - 1, n1 = im / 3 - 1;
                        double rx = 0.0, ry = 0.0;
                        if (g.per_x && g.per_y) {
                            rx = -(double)n0 * (double)g.Lx;
                            ry = -(double)n1 * (double)g.Ly;
                        } else if (g.per_x) {
                            rx = -(double)n0 * (double)g.Lx;
                        } else {
                            ry = -(double)n0 * (double)g.Ly;
                        }
                        const double t = li_pointflux_singular(A, __dadd_rn(fc.px, rx), __dadd_rn(fc.py, ry),
                                                               x1, y1, x2, y2);
                        acc = (im == 0) ? t : __dadd_rn(acc, t);
                    }
                    v = acc;
                } else if (fc.kind == LM_FIELD_POINTFLUX_AXIAL) {
                    v = li_pointflux_axial(A, fc.px, fc.py, x1, y1, x2, y2);
                } else {
                    v = li_pointflux_singular(A, fc.px, fc.py, x1, y1, x2, y2);
                }
                break;
            default:
                v = 0.0;
        }
        li = (c == 0) ? v : __dadd_rn(li, v);
    }
    return li;
}

}  // namespace lmgpu
