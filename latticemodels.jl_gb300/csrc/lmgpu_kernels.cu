// CUDA kernels of the lmgpu evolution backend (sm_103a).
//
// Hot path: one Chebyshev order of exp(-i H dt) applied to a block of kets, with H the
// nearest-neighbour tight-binding stencil of a square lattice whose hopping phases and
// on-site terms are assembled on the device.  Every kernel launches on the context stream.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>

#include "lmgpu_internal.cuh"
#include "lmgpu_order.cuh"

namespace lmgpu {

// ------------------------------------------------------------------------------------------
// Complex helpers (no fused contraction where the reference's rounding is restated).
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ double2 cmul_rn(double2 a, double2 b) {
    return make_double2(__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)),
                        __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}

// H[s, s+e] = t1 * f * exp(-2 pi i LI(r_s, r_s + e)) for e = x (dir 0) and y (dir 1);
// absent bonds store 0 (src/operators/builder.jl:282-285).
__global__ void assemble_kernel(Geom g, FieldSet f, double t1, double2* __restrict__ hop) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.N) return;
    const int64_t xi = s / g.Ly, yi = s - xi * g.Ly;
    const double x1 = (double)(xi + 1), y1 = (double)(yi + 1);
#pragma unroll
    for (int dir = 0; dir < 2; ++dir) {
        const bool inside = (dir == 0) ? (xi + 1 < g.Lx) : (yi + 1 < g.Ly);
        const bool per = (dir == 0) ? g.per_x : g.per_y;
        double2 val = make_double2(0.0, 0.0);
        if (inside || per) {
            const double x2 = (dir == 0) ? x1 + 1.0 : x1;  // unwrapped destination (old_site)
            const double y2 = (dir == 0) ? y1 : y1 + 1.0;
            double2 fac = make_double2(1.0, 0.0);
            if (!inside) {
                const double th = (dir == 0) ? g.twist_x : g.twist_y;
                if (th != 0.0) {
                    double sn, cs;
                    sincos(th, &sn, &cs);
                    fac = make_double2(cs, sn);
                }
            }
            const double li = (f.n > 0) ? field_line_integral(g, f, x1, y1, x2, y2) : 0.0;
            const double theta = __dmul_rn(-2.0 * M_PI, li);
            double sn, cs;
            sincos(theta, &sn, &cs);
            const double2 tot = cmul_rn(fac, make_double2(cs, sn));
            val = make_double2(__dmul_rn(t1, tot.x), __dmul_rn(t1, tot.y));
        }
        hop[dir * g.N + s] = val;
    }
}

cudaError_t launch_assemble(lm_ctx* ctx, const Geom& g, const FieldSet& f, double t1, double2* hop) {
    const int thr = 128;
    const int64_t blocks = (g.N + thr - 1) / thr;
    assemble_kernel<<<(unsigned)blocks, thr, 0, ctx->stream>>>(g, f, t1, hop);
    ctx->launches++;
    return cudaGetLastError();
}

// 2*H/a hopping and 2*(V-b)/a diagonal tables in FP64 and FP32.
__global__ void normalise_kernel(int64_t N, const double2* __restrict__ hop, const double* __restrict__ onsite,
                                 double a, double b, double2* __restrict__ hop2, double* __restrict__ diag2,
                                 float2* __restrict__ hop2f, float* __restrict__ diag2f) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    const double sc = 2.0 / a;
#pragma unroll
    for (int dir = 0; dir < 2; ++dir) {
        const double2 h = hop[dir * N + s];
        const double2 v = make_double2(h.x * sc, h.y * sc);
        hop2[dir * N + s] = v;
        hop2f[dir * N + s] = make_float2((float)v.x, (float)v.y);
    }
    const double V = onsite ? onsite[s] : 0.0;
    const double d = (V - b) * sc;
    diag2[s] = d;
    diag2f[s] = (float)d;
}

cudaError_t launch_normalise(lm_ctx* ctx, const Geom& g, const double2* hop, const double* onsite, double a,
                             double b, double2* hop2, double* diag2, float2* hop2f, float* diag2f) {
    const int thr = 256;
    const int64_t blocks = (g.N + thr - 1) / thr;
    normalise_kernel<<<(unsigned)blocks, thr, 0, ctx->stream>>>(g.N, hop, onsite, a, b, hop2, diag2, hop2f, diag2f);
    ctx->launches++;
    return cudaGetLastError();
}

// One order of the Chebyshev recurrence for one lattice (see cheb_order_block).
template <typename R, int MODE, bool SITE_FAST, bool CONJ, int INNER, bool XR>
__global__ void __launch_bounds__(256) cheb_order_kernel(
    Geom g, const typename CT<R>::V* __restrict__ hop2, const R* __restrict__ diag2,
    const typename CT<R>::V* __restrict__ tp, typename CT<R>::V* tq, typename CT<R>::V* y,
    int64_t ld, int64_t M, R c0, R cs, int odd, R ph_re, R ph_im, ChebLo lo) {
    const int64_t lane = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // fast dimension
    cheb_order_block<R, MODE, SITE_FAST, CONJ, INNER, XR>(g, hop2, diag2, tp, tq, y, ld, M, c0, cs, odd, ph_re,
                                                          ph_im, lo, lane, (int64_t)blockIdx.y * INNER,
                                                          (int64_t)gridDim.y * INNER);
}

template <typename R, int MODE, bool SF, bool CJ, bool XR>
static void launch_cheb_t(lm_ctx* ctx, const Geom& g, const void* hop2, const void* diag2, const void* tp,
                          void* tq, void* y, int64_t ld, int64_t m, double c0, ChebCoef ck, double ph_re,
                          double ph_im, ChebLo lo) {
    typedef typename CT<R>::V V;
    constexpr int INNER = 4;
    const int thr = SF ? 256 : 128;
    const int64_t nfast = SF ? g.N : m;
    const int64_t nslow = SF ? m : g.N;
    const int64_t gx = (nfast + thr - 1) / thr;
    int64_t gy = (nslow + INNER - 1) / INNER;
    if (gy > 65535) gy = 65535;
    dim3 grid((unsigned)gx, (unsigned)gy);
    cheb_order_kernel<R, MODE, SF, CJ, INNER, XR><<<grid, thr, 0, ctx->stream>>>(
        g, (const V*)hop2, (const R*)diag2, (const V*)tp, (V*)tq, (V*)y, ld, m, (R)c0, (R)ck.s, ck.odd,
        (R)ph_re, (R)ph_im, lo);
}

template <typename R, bool SF, bool CJ, bool XR>
static void dispatch_mode_x(int mode, lm_ctx* ctx, const Geom& g, const void* hop2, const void* diag2,
                            const void* tp, void* tq, void* y, int64_t ld, int64_t m, double c0, ChebCoef ck,
                            double pr, double pi, ChebLo lo) {
    if (mode == CHEB_FIRST) launch_cheb_t<R, CHEB_FIRST, SF, CJ, XR>(ctx, g, hop2, diag2, tp, tq, y, ld, m, c0, ck, pr, pi, lo);
    else if (mode == CHEB_MID) launch_cheb_t<R, CHEB_MID, SF, CJ, XR>(ctx, g, hop2, diag2, tp, tq, y, ld, m, c0, ck, pr, pi, lo);
    else launch_cheb_t<R, CHEB_LAST, SF, CJ, XR>(ctx, g, hop2, diag2, tp, tq, y, ld, m, c0, ck, pr, pi, lo);
}

template <typename R, bool SF, bool CJ>
static void dispatch_mode(int mode, bool xreal, lm_ctx* ctx, const Geom& g, const void* hop2, const void* diag2,
                          const void* tp, void* tq, void* y, int64_t ld, int64_t m, double c0, ChebCoef ck,
                          double pr, double pi, ChebLo lo) {
    if (xreal) dispatch_mode_x<R, SF, CJ, true>(mode, ctx, g, hop2, diag2, tp, tq, y, ld, m, c0, ck, pr, pi, lo);
    else dispatch_mode_x<R, SF, CJ, false>(mode, ctx, g, hop2, diag2, tp, tq, y, ld, m, c0, ck, pr, pi, lo);
}

cudaError_t launch_cheb_order(lm_ctx* ctx, const Geom& g, int precision, int site_fast, int conj, int mode,
                              const void* hop2, const void* diag2, const void* tp, void* tq, void* y,
                              int64_t ld, int64_t m, double c0, ChebCoef ck, double ph_re, double ph_im,
                              ChebLo lo, bool xreal) {
    if (precision == LM_C64) {
        if (site_fast) {
            if (conj) dispatch_mode<double, true, true>(mode, xreal, ctx, g, hop2, diag2, tp, tq, y, ld, m, c0, ck, ph_re, ph_im, lo);
            else dispatch_mode<double, true, false>(mode, xreal, ctx, g, hop2, diag2, tp, tq, y, ld, m, c0, ck, ph_re, ph_im, lo);
        } else {
            if (conj) dispatch_mode<double, false, true>(mode, xreal, ctx, g, hop2, diag2, tp, tq, y, ld, m, c0, ck, ph_re, ph_im, lo);
            else dispatch_mode<double, false, false>(mode, xreal, ctx, g, hop2, diag2, tp, tq, y, ld, m, c0, ck, ph_re, ph_im, lo);
        }
    } else {
        if (site_fast) {
            if (conj) dispatch_mode<float, true, true>(mode, xreal, ctx, g, hop2, diag2, tp, tq, y, ld, m, c0, ck, ph_re, ph_im, lo);
            else dispatch_mode<float, true, false>(mode, xreal, ctx, g, hop2, diag2, tp, tq, y, ld, m, c0, ck, ph_re, ph_im, lo);
        } else {
            if (conj) dispatch_mode<float, false, true>(mode, xreal, ctx, g, hop2, diag2, tp, tq, y, ld, m, c0, ck, ph_re, ph_im, lo);
            else dispatch_mode<float, false, false>(mode, xreal, ctx, g, hop2, diag2, tp, tq, y, ld, m, c0, ck, ph_re, ph_im, lo);
        }
    }
    ctx->launches++;
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------------
// Elementwise helpers
// ------------------------------------------------------------------------------------------
template <typename R>
__global__ void scale_kernel(typename CT<R>::V* x, int64_t n, int64_t m, int64_t ld, R re, R im) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int64_t k = blockIdx.y; k < m; k += gridDim.y) {
        typename CT<R>::V v = x[k * ld + i];
        x[k * ld + i] = CT<R>::make(re * v.x - im * v.y, re * v.y + im * v.x);
    }
}

cudaError_t launch_scale(lm_ctx* ctx, int precision, void* x, int64_t n, int64_t m, int64_t ld, double re,
                         double im) {
    dim3 grid((unsigned)((n + 255) / 256), (unsigned)(m < 65535 ? m : 65535));
    if (precision == LM_C64) scale_kernel<double><<<grid, 256, 0, ctx->stream>>>((double2*)x, n, m, ld, re, im);
    else scale_kernel<float><<<grid, 256, 0, ctx->stream>>>((float2*)x, n, m, ld, (float)re, (float)im);
    ctx->launches++;
    return cudaGetLastError();
}

template <typename RS, typename RD>
__global__ void convert_kernel(const typename CT<RS>::V* src, typename CT<RD>::V* dst, int64_t n, int64_t m,
                               int64_t lds, int64_t ldd) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int64_t k = blockIdx.y; k < m; k += gridDim.y) {
        typename CT<RS>::V v = src[k * lds + i];
        dst[k * ldd + i] = CT<RD>::make((RD)v.x, (RD)v.y);
    }
}

cudaError_t launch_convert(lm_ctx* ctx, int to_precision, const void* src, void* dst, int64_t n, int64_t m,
                           int64_t ld_src, int64_t ld_dst) {
    dim3 grid((unsigned)((n + 255) / 256), (unsigned)(m < 65535 ? m : 65535));
    if (to_precision == LM_C32)
        convert_kernel<double, float><<<grid, 256, 0, ctx->stream>>>((const double2*)src, (float2*)dst, n, m, ld_src, ld_dst);
    else
        convert_kernel<float, double><<<grid, 256, 0, ctx->stream>>>((const float2*)src, (double2*)dst, n, m, ld_src, ld_dst);
    ctx->launches++;
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------------
// Readouts.  Sums over kets use Acc<R> (FP64 for c64 states, double-float FP32 for c32
// states).  Every sum is over a fixed order (no atomics): the readouts are bit-reproducible.
// ------------------------------------------------------------------------------------------
constexpr int kReadWarps = 8;  // warps of a readout block; they split the kets

// localdensity of a ket block: rho_s = sum_k w_k |psi_sk|^2.  A block owns 32*VEC consecutive
// sites (lane -> VEC sites: c32 with VEC = 8 reads four 16-byte words per ket, so a warp reads
// 2 KB of one ket at a time) and the kets of slice blockIdx.y, [y*kslice, (y+1)*kslice); its 8
// warps take kets k = k0 + warp, k0 + warp + 8, ...; the 8 partial sums are added in warp order
// and written to plane y of out (out + y*n).  With more than one slice, slice_sum_kernel adds
// the planes in slice order.
template <typename R, int VEC, bool WEIGHTED>
__global__ void __launch_bounds__(32 * kReadWarps) localdensity_kets_kernel(
    const typename CT<R>::V* __restrict__ x, int64_t n, int64_t m, int64_t ld, const double* __restrict__ w,
    double* __restrict__ out, int64_t kslice) {
    typedef typename CT<R>::V V;
    __shared__ double red[kReadWarps][32 * VEC];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t s0 = (int64_t)blockIdx.x * (32 * VEC) + (int64_t)lane * VEC;
    const int64_t k0 = (int64_t)blockIdx.y * kslice;
    const int64_t k1 = k0 + kslice < m ? k0 + kslice : m;
    out += (int64_t)blockIdx.y * n;
    Acc<R> acc[VEC];
    double accw[VEC];
#pragma unroll
    for (int j = 0; j < VEC; ++j) accw[j] = 0.0;
    if (s0 < n) {
#pragma unroll 4
        for (int64_t k = k0 + warp; k < k1; k += kReadWarps) {
            V v[VEC];
            if (VEC >= 2) {
#pragma unroll
                for (int h = 0; h < VEC / 2; ++h) {
                    const float4 q = __ldg(reinterpret_cast<const float4*>(x + k * ld + s0) + h);
                    v[2 * h] = CT<R>::make(q.x, q.y);
                    v[2 * h + 1] = CT<R>::make(q.z, q.w);
                }
            } else {
                v[0] = x[k * ld + s0];
            }
#pragma unroll
            for (int j = 0; j < VEC; ++j) {
                if (WEIGHTED) {
                    accw[j] = fma(w[k], (double)v[j].x * (double)v[j].x + (double)v[j].y * (double)v[j].y, accw[j]);
                } else {
                    acc[j].add_prod(v[j].x, v[j].x);
                    acc[j].add_prod(v[j].y, v[j].y);
                }
            }
        }
    }
#pragma unroll
    for (int j = 0; j < VEC; ++j) red[warp][lane * VEC + j] = WEIGHTED ? accw[j] : acc[j].get();
    __syncthreads();
    if (threadIdx.x < 32 * VEC) {
        const int64_t s = (int64_t)blockIdx.x * (32 * VEC) + threadIdx.x;
        if (s < n) {
            double t = 0.0;
#pragma unroll
            for (int q = 0; q < kReadWarps; ++q) t += red[q][threadIdx.x];
            out[s] = t;
        }
    }
}

// localdensity of a density matrix: Re P[s,s].
template <typename R>
__global__ void localdensity_dm_kernel(const typename CT<R>::V* __restrict__ x, int64_t n, int64_t ld,
                                       double* __restrict__ out) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) out[s] = (double)x[s * ld + s].x;
}

// out[s] = sum over q = 0..S-1, in that order, of part[q*n + s].
__global__ void slice_sum_kernel(const double* __restrict__ part, int64_t n, int S, double* __restrict__ out) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    double t = part[s];
    for (int q = 1; q < S; ++q) t += part[(int64_t)q * n + s];
    out[s] = t;
}

// Number of ket slices S for a readout grid of `chunks` site chunks, `wave` resident blocks:
// the S <= 8 (at least 64 kets per slice) that minimises waves(chunks S) / S x (1 + 0.06 S).
// The first factor is the work per SM including the last, partly filled wave; the second the
// cost of shorter blocks and of the partial planes.  Measured (c32, ms per readout):
//   density, 256^2 sites x 2048 kets, S = 1 / 2 / 4 / 7 / 19: 0.215 / 0.173 / 0.182 / 0.180 / 0.197
//     (the rule: 2); 512^2 x 1024: 0.338 / 0.364 / 0.347 / 0.357 / 0.401 (the rule: 1);
//   bond currents, 256^2 x 2048, S = 1 / 4 / 8: 0.653 / 0.483 / 0.495 (the rule: 4).
// The model ranks the measured slice counts of each case in the measured order.
static int readout_slices(int64_t chunks, int64_t m, int64_t wave) {
    if (wave <= 0 || chunks <= 0) return 1;
    const int smax = (int)std::max<int64_t>(1, std::min<int64_t>(8, m / 64));
    int best = 1;
    double tbest = 1e300;
    for (int S = 1; S <= smax; ++S) {
        const double waves = (double)((chunks * S + wave - 1) / wave);
        const double t = waves / S * (1.0 + 0.06 * S);
        if (t < tbest * (1.0 - 1e-9)) {
            tbest = t;
            best = S;
        }
    }
    return best;
}

static cudaError_t ensure_readout_part(lm_ctx* ctx, size_t n) {
    if (ctx->ld_part_cap >= n) return cudaSuccess;
    if (ctx->d_ld_part) cudaFree(ctx->d_ld_part);
    ctx->d_ld_part = nullptr;
    ctx->ld_part_cap = 0;
    cudaError_t e = cudaMalloc((void**)&ctx->d_ld_part, n * sizeof(double));
    if (e == cudaSuccess) ctx->ld_part_cap = n;
    return e;
}

template <typename R, int VEC, bool WEIGHTED>
static cudaError_t launch_ld_kets_w(lm_ctx* ctx, const void* x, int64_t n, int64_t m, int64_t ld, const double* w,
                                    double* out) {
    typedef typename CT<R>::V V;
    auto kern = localdensity_kets_kernel<R, VEC, WEIGHTED>;
    const int64_t chunks = (n + 32 * VEC - 1) / (32 * VEC);
    static const int per_sm = [] {  // resident blocks per SM of this instantiation
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, localdensity_kets_kernel<R, VEC, WEIGHTED>,
                                                          32 * kReadWarps, 0) != cudaSuccess) {
            (void)cudaGetLastError();
            b = 0;
        }
        return b;
    }();
    int S = readout_slices(chunks, m, (int64_t)per_sm * ctx->sm_count);
    if (ctx->ld_slices_override > 0) S = ctx->ld_slices_override;
    if (S > 1 && ensure_readout_part(ctx, (size_t)S * (size_t)n) != cudaSuccess) {
        (void)cudaGetLastError();  // clear the failed allocation: the single-slice grid needs no scratch
        S = 1;
    }
    const int64_t kslice = (m + S - 1) / S;
    dim3 grid((unsigned)chunks, (unsigned)S);
    kern<<<grid, 32 * kReadWarps, 0, ctx->stream>>>((const V*)x, n, m, ld, w, S > 1 ? ctx->d_ld_part : out, kslice);
    if (S > 1) {
        slice_sum_kernel<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(ctx->d_ld_part, n, S, out);
        ctx->launches++;
    }
    return cudaSuccess;
}

template <typename R, int VEC>
static cudaError_t launch_ld_kets(lm_ctx* ctx, const void* x, int64_t n, int64_t m, int64_t ld, const double* w,
                                  double* out) {
    return w ? launch_ld_kets_w<R, VEC, true>(ctx, x, n, m, ld, w, out)
             : launch_ld_kets_w<R, VEC, false>(ctx, x, n, m, ld, w, out);
}

cudaError_t launch_localdensity(lm_ctx* ctx, int precision, int kind, const void* x, int64_t n, int64_t m,
                                int64_t ld, const double* w, double* out) {
    if (n <= 0) return cudaSuccess;
    if (kind == LM_DENSITY) {
        const unsigned blocks = (unsigned)((n + 127) / 128);
        if (precision == LM_C64) localdensity_dm_kernel<double><<<blocks, 128, 0, ctx->stream>>>((const double2*)x, n, ld, out);
        else localdensity_dm_kernel<float><<<blocks, 128, 0, ctx->stream>>>((const float2*)x, n, ld, out);
    } else if (precision == LM_C64) {
        // the FP64 pipe bounds c64 (two DFMAs per element): wider lanes measured slower
        launch_ld_kets<double, 1>(ctx, x, n, m, ld, w, out);
    } else if (n % 8 == 0 && ld % 2 == 0 && ((uintptr_t)x & 15) == 0) {
        launch_ld_kets<float, 8>(ctx, x, n, m, ld, w, out);  // 2 KB of a ket per warp load
    } else if (n % 2 == 0 && ld % 2 == 0 && ((uintptr_t)x & 15) == 0) {
        launch_ld_kets<float, 2>(ctx, x, n, m, ld, w, out);  // 16-byte loads of site pairs
    } else {
        launch_ld_kets<float, 1>(ctx, x, n, m, ld, w, out);
    }
    ctx->launches++;
    return cudaGetLastError();
}

// Bond currents J = 2 Im(H[i,j] P[j,i]) for the +x and +y bond of every site, written in the
// reference's bond order (all +x bonds in source order, then all +y bonds).  H[i,j] is the
// accumulated matrix entry: on a 2-site periodic axis the reverse bond adds conj(H[j,i]).
__device__ __forceinline__ void bond_write(const Geom& g, const double2* __restrict__ hop, int64_t s, int dir,
                                           const Nbr& nb, double pr, double pi, double* __restrict__ out) {
    const int64_t j = dir == 0 ? nb.xp : nb.yp;
    const int64_t jm = dir == 0 ? nb.xm : nb.ym;
    double2 h = hop[dir * g.N + s];
    if (j == jm) {  // two-site periodic axis: both bonds join s and j
        const double2 r = hop[dir * g.N + j];
        h.x += r.x;
        h.y -= r.y;
    }
    const double J = 2.0 * (h.x * pi + h.y * pr);  // Im(h * p)
    const int64_t xi = s / g.Ly, yi = s - xi * g.Ly;
    const int64_t nbx = g.per_x ? g.N : (g.Lx - 1) * g.Ly;
    out[dir == 0 ? s : nbx + (g.per_y ? s : xi * (g.Ly - 1) + yi)] = J;
}

// Ket blocks: P[j,s] = sum_k w_k psi_jk conj(psi_sk).  A block owns 32 consecutive sites (one
// per lane); its 8 warps split the kets; partial sums are added in warp order.
template <typename R, bool WEIGHTED>
__global__ void __launch_bounds__(32 * kReadWarps) bond_currents_kets_kernel(
    Geom g, const double2* __restrict__ hop, const typename CT<R>::V* __restrict__ x, int64_t m, int64_t ld,
    const double* __restrict__ w, double* __restrict__ out) {
    typedef typename CT<R>::V V;
    __shared__ double red[kReadWarps][4][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t s = (int64_t)blockIdx.x * 32 + lane;
    Nbr nb;
    Acc<R> a[4];  // (re, im) of the +x bond, then of the +y bond
    double aw[4] = {0.0, 0.0, 0.0, 0.0};
    if (s < g.N) {
        nb = neighbours(g, s);
        // absent bonds read the site itself (always in bounds) and are not written
        const int64_t jx = nb.hxp ? nb.xp : s, jy = nb.hyp ? nb.yp : s;
        // unrolled so that four kets' loads are in flight per thread; the sums keep their order
#pragma unroll 4
        for (int64_t k = warp; k < m; k += kReadWarps) {
            const V b = x[k * ld + s];
            const V cx = x[k * ld + jx], cy = x[k * ld + jy];  // c * conj(b)
            if (WEIGHTED) {
                const double wk = w[k];
                aw[0] += wk * ((double)cx.x * (double)b.x + (double)cx.y * (double)b.y);
                aw[1] += wk * ((double)cx.y * (double)b.x - (double)cx.x * (double)b.y);
                aw[2] += wk * ((double)cy.x * (double)b.x + (double)cy.y * (double)b.y);
                aw[3] += wk * ((double)cy.y * (double)b.x - (double)cy.x * (double)b.y);
            } else {
                a[0].add_prod(cx.x, b.x);
                a[0].add_prod(cx.y, b.y);
                a[1].add_prod(cx.y, b.x);
                a[1].add_prod(-cx.x, b.y);
                a[2].add_prod(cy.x, b.x);
                a[2].add_prod(cy.y, b.y);
                a[3].add_prod(cy.y, b.x);
                a[3].add_prod(-cy.x, b.y);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) red[warp][q][lane] = WEIGHTED ? aw[q] : a[q].get();
    __syncthreads();
    if (warp == 0 && s < g.N) {
        double v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            double t = 0.0;
            for (int r = 0; r < kReadWarps; ++r) t += red[r][q][lane];
            v[q] = t;
        }
        if (nb.hxp) bond_write(g, hop, s, 0, nb, v[0], v[1], out);
        if (nb.hyp) bond_write(g, hop, s, 1, nb, v[2], v[3], out);
    }
}

// Density matrices: P[j,s] read directly.
template <typename R>
__global__ void bond_currents_dm_kernel(Geom g, const double2* __restrict__ hop, const typename CT<R>::V* __restrict__ x,
                                        int64_t ld, double* __restrict__ out) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.N) return;
    const Nbr nb = neighbours(g, s);
#pragma unroll
    for (int dir = 0; dir < 2; ++dir) {
        if (!(dir == 0 ? nb.hxp : nb.hyp)) continue;
        const typename CT<R>::V v = x[s * ld + (dir == 0 ? nb.xp : nb.yp)];
        bond_write(g, hop, s, dir, nb, (double)v.x, (double)v.y, out);
    }
}

// c32 ket blocks with Ly % 4 == 0: a lane owns 4 consecutive sites of one lattice column, so
// a warp reads 1 KB of a ket per load (the 256-byte pieces of the kernel above, from kets
// 512 KB apart, held DRAM to about a quarter of its bandwidth).  The +x neighbours are the
// same 4 rows of the next column (contiguous); the +y neighbours are the lane's own next sites
// and, for the fourth, one extra 8-byte load.  Each site gets the products of the kernel above
// in the same ket order within a slice.  Block y takes the kets of slice y and writes its
// 4 partial sums per site to plane y of `part`; bond_currents_slices_kernel adds the planes in
// slice order and writes the bonds.
template <bool WEIGHTED>
__global__ void __launch_bounds__(32 * kReadWarps) bond_currents_kets4_kernel(
    Geom g, const float2* __restrict__ x, int64_t m, int64_t ld, const double* __restrict__ w, int64_t kslice,
    double* __restrict__ part) {
    __shared__ double red[kReadWarps][4][128];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t s0 = (int64_t)blockIdx.x * 128 + (int64_t)lane * 4;
    const int64_t k0 = (int64_t)blockIdx.y * kslice;
    const int64_t k1 = k0 + kslice < m ? k0 + kslice : m;
    Acc<float> a[4][4];
    double aw[4][4];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) aw[j][q] = 0.0;
    if (s0 < g.N) {
        const int64_t xi = s0 / g.Ly, yi0 = s0 - xi * g.Ly;
        // +x: the same rows of the next column (absent bonds read the sites themselves and are
        // not written); +y of the fourth site: the next row, the column start, or itself
        const int64_t jx = xi + 1 < g.Lx ? s0 + g.Ly : (g.per_x ? yi0 : s0);
        const int64_t jy3 = yi0 + 4 < g.Ly ? s0 + 4 : (g.per_y ? s0 - yi0 : s0 + 3);
#pragma unroll 2
        for (int64_t k = k0 + warp; k < k1; k += kReadWarps) {
            const float4* xb = reinterpret_cast<const float4*>(x + k * ld + s0);
            const float4* xc = reinterpret_cast<const float4*>(x + k * ld + jx);
            const float4 b01 = __ldg(xb), b23 = __ldg(xb + 1), c01 = __ldg(xc), c23 = __ldg(xc + 1);
            const float2 y3 = __ldg(x + k * ld + jy3);
            const float2 b[4] = {make_float2(b01.x, b01.y), make_float2(b01.z, b01.w), make_float2(b23.x, b23.y),
                                 make_float2(b23.z, b23.w)};
            const float2 cxs[4] = {make_float2(c01.x, c01.y), make_float2(c01.z, c01.w), make_float2(c23.x, c23.y),
                                   make_float2(c23.z, c23.w)};
            const float2 cys[4] = {b[1], b[2], b[3], y3};
            const double wk = WEIGHTED ? w[k] : 1.0;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float2 bb = b[j], cx = cxs[j], cy = cys[j];  // c * conj(b)
                if (WEIGHTED) {
                    aw[j][0] += wk * ((double)cx.x * (double)bb.x + (double)cx.y * (double)bb.y);
                    aw[j][1] += wk * ((double)cx.y * (double)bb.x - (double)cx.x * (double)bb.y);
                    aw[j][2] += wk * ((double)cy.x * (double)bb.x + (double)cy.y * (double)bb.y);
                    aw[j][3] += wk * ((double)cy.y * (double)bb.x - (double)cy.x * (double)bb.y);
                } else {
                    a[j][0].add_prod(cx.x, bb.x);
                    a[j][0].add_prod(cx.y, bb.y);
                    a[j][1].add_prod(cx.y, bb.x);
                    a[j][1].add_prod(-cx.x, bb.y);
                    a[j][2].add_prod(cy.x, bb.x);
                    a[j][2].add_prod(cy.y, bb.y);
                    a[j][3].add_prod(cy.y, bb.x);
                    a[j][3].add_prod(-cy.x, bb.y);
                }
            }
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) red[warp][q][lane * 4 + j] = WEIGHTED ? aw[j][q] : a[j][q].get();
    __syncthreads();
    if (threadIdx.x < 128) {
        const int64_t s = (int64_t)blockIdx.x * 128 + threadIdx.x;
        if (s < g.N) {
            double* pl = part + (int64_t)blockIdx.y * 4 * g.N;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                double t = 0.0;
                for (int r = 0; r < kReadWarps; ++r) t += red[r][q][threadIdx.x];
                pl[(int64_t)q * g.N + s] = t;
            }
        }
    }
}

// Adds the S slice planes of bond_currents_kets4_kernel in slice order and writes the bonds.
__global__ void bond_currents_slices_kernel(Geom g, const double2* __restrict__ hop, const double* __restrict__ part,
                                            int S, double* __restrict__ out) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.N) return;
    double v[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        double t = part[(int64_t)q * g.N + s];
        for (int y = 1; y < S; ++y) t += part[((int64_t)y * 4 + q) * g.N + s];
        v[q] = t;
    }
    const Nbr nb = neighbours(g, s);
    if (nb.hxp) bond_write(g, hop, s, 0, nb, v[0], v[1], out);
    if (nb.hyp) bond_write(g, hop, s, 1, nb, v[2], v[3], out);
}

template <bool WEIGHTED>
static cudaError_t launch_bond_currents4(lm_ctx* ctx, const Geom& g, const double2* hop, const float2* x, int64_t m,
                                         int64_t ld, const double* w, double* out) {
    const int64_t chunks = (g.N + 127) / 128;
    static const int per_sm = [] {  // resident blocks per SM of this instantiation
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, bond_currents_kets4_kernel<WEIGHTED>, 32 * kReadWarps,
                                                          0) != cudaSuccess) {
            (void)cudaGetLastError();
            b = 0;
        }
        return b;
    }();
    int S = readout_slices(chunks, m, (int64_t)per_sm * ctx->sm_count);
    if (ctx->ld_slices_override > 0) S = ctx->ld_slices_override;
    cudaError_t e = ensure_readout_part(ctx, (size_t)S * 4 * (size_t)g.N);
    if (e != cudaSuccess) return e;  // the caller falls back to the one-site-per-lane kernel
    const int64_t kslice = (m + S - 1) / S;
    bond_currents_kets4_kernel<WEIGHTED><<<dim3((unsigned)chunks, (unsigned)S), 32 * kReadWarps, 0, ctx->stream>>>(
        g, x, m, ld, w, kslice, ctx->d_ld_part);
    bond_currents_slices_kernel<<<(unsigned)((g.N + 255) / 256), 256, 0, ctx->stream>>>(g, hop, ctx->d_ld_part, S, out);
    ctx->launches++;
    return cudaSuccess;
}

cudaError_t launch_bond_currents(lm_ctx* ctx, const Geom& g, int precision, int kind, const double2* hop,
                                 const void* x, int64_t m, int64_t ld, const double* w, double* out) {
    if (g.N <= 0) return cudaSuccess;
    if (kind == LM_DENSITY) {
        const unsigned blocks = (unsigned)((g.N + 127) / 128);
        if (precision == LM_C64) bond_currents_dm_kernel<double><<<blocks, 128, 0, ctx->stream>>>(g, hop, (const double2*)x, ld, out);
        else bond_currents_dm_kernel<float><<<blocks, 128, 0, ctx->stream>>>(g, hop, (const float2*)x, ld, out);
    } else {
        const unsigned blocks = (unsigned)((g.N + 31) / 32);
        const int thr = 32 * kReadWarps;
        if (precision == LM_C64) {
            if (w) bond_currents_kets_kernel<double, true><<<blocks, thr, 0, ctx->stream>>>(g, hop, (const double2*)x, m, ld, w, out);
            else bond_currents_kets_kernel<double, false><<<blocks, thr, 0, ctx->stream>>>(g, hop, (const double2*)x, m, ld, w, out);
        } else if (g.Ly % 4 == 0 && ld % 2 == 0 && ((uintptr_t)x & 15) == 0 && !ctx->currents_scalar) {
            cudaError_t e = w ? launch_bond_currents4<true>(ctx, g, hop, (const float2*)x, m, ld, w, out)
                              : launch_bond_currents4<false>(ctx, g, hop, (const float2*)x, m, ld, w, out);
            if (e == cudaErrorMemoryAllocation) {  // no scratch for the partial sums
                (void)cudaGetLastError();
                if (w) bond_currents_kets_kernel<float, true><<<blocks, thr, 0, ctx->stream>>>(g, hop, (const float2*)x, m, ld, w, out);
                else bond_currents_kets_kernel<float, false><<<blocks, thr, 0, ctx->stream>>>(g, hop, (const float2*)x, m, ld, w, out);
            } else if (e != cudaSuccess) {
                return e;
            }
        } else {
            if (w) bond_currents_kets_kernel<float, true><<<blocks, thr, 0, ctx->stream>>>(g, hop, (const float2*)x, m, ld, w, out);
            else bond_currents_kets_kernel<float, false><<<blocks, thr, 0, ctx->stream>>>(g, hop, (const float2*)x, m, ld, w, out);
        }
    }
    ctx->launches++;
    return cudaGetLastError();
}

// Per-column norms: one block of 512 threads per column, fixed-order tree reduction.
template <typename R, int VEC>
__global__ void __launch_bounds__(512) column_norms_kernel(const typename CT<R>::V* __restrict__ x, int64_t n,
                                                           int64_t ld, double* __restrict__ out) {
    typedef typename CT<R>::V V;
    __shared__ double red[16];
    const int64_t k = blockIdx.x;
    Acc<R> acc;
    const V* col = x + k * ld;
    for (int64_t i = (int64_t)threadIdx.x * VEC; i < n; i += (int64_t)blockDim.x * VEC) {
        if (VEC == 2) {
            const float4 q = __ldg(reinterpret_cast<const float4*>(col + i));
            acc.add_prod(q.x, q.x);
            acc.add_prod(q.y, q.y);
            acc.add_prod(q.z, q.z);
            acc.add_prod(q.w, q.w);
        } else {
            const V v = col[i];
            acc.add_prod(v.x, v.x);
            acc.add_prod(v.y, v.y);
        }
    }
    double t = acc.get();
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x < 32) {
        t = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) out[k] = sqrt(t);
    }
}

cudaError_t launch_column_norms(lm_ctx* ctx, int precision, const void* x, int64_t n, int64_t m, int64_t ld,
                                double* out) {
    if (m <= 0) return cudaSuccess;
    if (precision == LM_C64)
        column_norms_kernel<double, 1><<<(unsigned)m, 512, 0, ctx->stream>>>((const double2*)x, n, ld, out);
    else if (n % 2 == 0 && ld % 2 == 0 && ((uintptr_t)x & 15) == 0)
        column_norms_kernel<float, 2><<<(unsigned)m, 512, 0, ctx->stream>>>((const float2*)x, n, ld, out);
    else
        column_norms_kernel<float, 1><<<(unsigned)m, 512, 0, ctx->stream>>>((const float2*)x, n, ld, out);
    ctx->launches++;
    return cudaGetLastError();
}

// x[:, k] *= target[k] / norms[k].  A block rescales 256 * 4 * VEC consecutive elements of one
// column (VEC = 2: c32 site pairs as 16-byte words).
template <typename R, int VEC>
__global__ void __launch_bounds__(256) rescale_columns_kernel(typename CT<R>::V* x, int64_t n, int64_t m, int64_t ld,
                                                              const double* __restrict__ norms,
                                                              const double* __restrict__ target) {
    constexpr int PER = 4 * VEC;  // elements per thread
    for (int64_t k = blockIdx.y; k < m; k += gridDim.y) {
        const double nk = norms[k];
        const R f = (R)(nk > 0.0 ? target[k] / nk : 1.0);
        typename CT<R>::V* col = x + k * ld;
        for (int64_t i0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * VEC; i0 < n;
             i0 += (int64_t)gridDim.x * blockDim.x * PER) {
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int64_t i = i0 + (int64_t)u * blockDim.x * VEC;
                if (i >= n) break;
                if (VEC == 2) {
                    float4* p = reinterpret_cast<float4*>(col + i);
                    float4 q = *p;
                    q.x *= f; q.y *= f; q.z *= f; q.w *= f;
                    *p = q;
                } else {
                    typename CT<R>::V v = col[i];
                    v.x *= f;
                    v.y *= f;
                    col[i] = v;
                }
            }
        }
    }
}

cudaError_t launch_rescale_columns(lm_ctx* ctx, int precision, void* x, int64_t n, int64_t m, int64_t ld,
                                   const double* norms, const double* target) {
    if (m <= 0) return cudaSuccess;
    const bool pairs = precision == LM_C32 && n % 2 == 0 && ld % 2 == 0 && ((uintptr_t)x & 15) == 0;
    const int64_t per_block = 256 * 4 * (pairs ? 2 : 1);
    const int64_t bx = std::min<int64_t>((n + per_block - 1) / per_block, 1024);
    const dim3 grid((unsigned)bx, (unsigned)(m < 65535 ? m : 65535));
    if (precision == LM_C64)
        rescale_columns_kernel<double, 1><<<grid, 256, 0, ctx->stream>>>((double2*)x, n, m, ld, norms, target);
    else if (pairs)
        rescale_columns_kernel<float, 2><<<grid, 256, 0, ctx->stream>>>((float2*)x, n, m, ld, norms, target);
    else
        rescale_columns_kernel<float, 1><<<grid, 256, 0, ctx->stream>>>((float2*)x, n, m, ld, norms, target);
    ctx->launches++;
    return cudaGetLastError();
}

// Norms of hi + lo (compensated ComplexF32 columns).  Each thread sums |hi + lo|^2 =
// hi^2 + (the rounding error of hi^2) + 2 hi lo over its elements as an FP32 pair (TwoProd and
// TwoSum), which keeps about 44 bits without an FP64 operation per element (GB300's FP64 and
// FP32<->FP64 conversion rates are a small fraction of its FP32 rate); the threads' pairs are
// then summed in FP64 in a fixed order.
__global__ void __launch_bounds__(512) column_norms_comp_kernel(const float2* __restrict__ hi,
                                                                const uint32_t* __restrict__ lo, int64_t n,
                                                                int64_t ld, double* __restrict__ out) {
    __shared__ double red[16];
    const int64_t k = blockIdx.x;
    float S = 0.0f, C = 0.0f;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const float2 a = hi[k * ld + i];
        const unsigned code = lo[k * ld + i];
        const float lx = res_lo_x(code), ly = res_lo_y(code);
        float px, ex, py, ey, t;
        two_prod(a.x, a.x, px, ex);
        two_prod(a.y, a.y, py, ey);
        const float e = (ex + ey) + 2.0f * fmaf(a.x, lx, a.y * ly);
        two_sum(S, px, S, t);
        C += t;
        two_sum(S, py, S, t);
        C += t + e;
    }
    double t = (double)S + (double)C;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x < 32) {
        t = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) out[k] = sqrt(t);
    }
}

cudaError_t launch_column_norms_comp(lm_ctx* ctx, const float2* hi, const uint32_t* lo, int64_t n, int64_t m,
                                     int64_t ld, double* out) {
    if (m <= 0) return cudaSuccess;
    column_norms_comp_kernel<<<(unsigned)m, 512, 0, ctx->stream>>>(hi, lo, n, ld, out);
    ctx->launches++;
    return cudaGetLastError();
}

// (hi + lo)[:, k] *= f = target[k] / norms[k]: f as an FP32 pair (fh + fl, formed once per block
// and column), the product hi fh exact by TwoProd, the small terms hi fl + lo fh added to its
// error, and the sum split again into hi and its encoded residual.
__global__ void __launch_bounds__(256) rescale_columns_comp_kernel(float2* hi, uint32_t* lo, int64_t n, int64_t m,
                                                                   int64_t ld, const double* __restrict__ norms,
                                                                   const double* __restrict__ target) {
    __shared__ float2 fs;
    for (int64_t k = blockIdx.y; k < m; k += gridDim.y) {
        __syncthreads();  // the previous column's factor has been read
        if (threadIdx.x == 0) {
            const double nk = norms[k];
            const double f = nk > 0.0 ? target[k] / nk : 1.0;
            const float fh = (float)f;
            fs = make_float2(fh, (float)(f - (double)fh));
        }
        __syncthreads();
        const float fh = fs.x, fl = fs.y;
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
            const float2 a = hi[k * ld + i];
            const unsigned code = lo[k * ld + i];
            const float l[2] = {res_lo_x(code), res_lo_y(code)};
            const float h[2] = {a.x, a.y};
            float o[2], r[2];
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                float p, e;
                two_prod(h[c], fh, p, e);
                e = fmaf(h[c], fl, fmaf(l[c], fh, e));
                o[c] = p + e;
                r[c] = e - (o[c] - p);
            }
            hi[k * ld + i] = make_float2(o[0], o[1]);
            lo[k * ld + i] = res_encode(r[0], r[1]);
        }
    }
}

cudaError_t launch_rescale_columns_comp(lm_ctx* ctx, float2* hi, uint32_t* lo, int64_t n, int64_t m, int64_t ld,
                                        const double* norms, const double* target) {
    if (m <= 0) return cudaSuccess;
    const int64_t bx = std::min<int64_t>((n + 255) / 256, 1024);
    const dim3 grid((unsigned)bx, (unsigned)(m < 65535 ? m : 65535));
    rescale_columns_comp_kernel<<<grid, 256, 0, ctx->stream>>>(hi, lo, n, m, ld, norms, target);
    ctx->launches++;
    return cudaGetLastError();
}

// Single-block FP64 sum (deterministic order).
__global__ void sum_kernel(const double* __restrict__ v, int64_t n, double* __restrict__ out) {
    __shared__ double red[32];
    double acc = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) acc += v[i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        acc = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) *out = acc;
    }
}

cudaError_t launch_sum(lm_ctx* ctx, const double* v, int64_t n, double* out1) {
    sum_kernel<<<1, 1024, 0, ctx->stream>>>(v, n, out1);
    ctx->launches++;
    return cudaGetLastError();
}

}  // namespace lmgpu
