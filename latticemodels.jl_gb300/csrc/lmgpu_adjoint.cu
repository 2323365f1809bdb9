// Adjoint of the Chebyshev evolution: gradients of a density loss with respect to the
// on-site potentials and the field amplitudes.
//
// Forward step n:  psi_{n+1} = U_n psi_n,  U_n = e^{-ib dt} sum_k c_k T_k(H~_n),  H~ = (H - b)/a
// with a, b, K fixed (frozen spectral bounds), so U_n is an exact polynomial in H_n and its
// discrete adjoint is exact.  With the co-state lambda_{n+1} = dL/dpsi*_{n+1} (L real):
//
//   lambda_n = U_n^dagger lambda_{n+1}           (the propagator with conjugate coefficients)
//   dL/dtheta += Re e^{-ib dt} sum_{k>=1} < beta_k , s_k >,   s_1 = D~ T_0,  s_k = 2 D~ T_{k-1}
//
// where D~ = (dH/dtheta)/a and beta is the adjoint of the three-term recurrence,
//   beta_k = conj(c_k) lambda + 2 H~ beta_{k+1} - beta_{k+2},  beta_{K+1} = beta_{K+2} = 0.
// For an on-site potential V_i, < beta, D~ T > = conj(beta_i) T_i / a summed over kets; for a
// field amplitude A, dH[s, s+e]/dA = -2 pi i LI_e(A = 1) H[s, s+e] on every bond.
//
// lm_adjoint_step recomputes T_0 .. T_{K-1} from psi_n, then runs the beta recurrence and the
// gradient sums in one fused pass per order (FP64 results; c32 sums in double-float); the caller applies U^dagger to lambda with a solver
// updated for -dt (the same polynomial with conjugate coefficients).
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <new>
#include <vector>

#include "lmgpu_internal.cuh"
#include "lmgpu_order.cuh"

namespace lmgpu {

// out = alpha * (2H~) tp - tpp + w * lam   (tables hold 2H/a and 2(V-b)/a; tpp, lam optional)
// w = conj(c_k): (s, 0) for even k, (0, s) for odd k (conj(-i s) = i s).
// With y non-null, also y += cy * out (the real-coefficient Chebyshev series of lm_cheb_apply).
// XR: every x-hop is real, so the x-neighbour terms take 2 FMAs instead of 4.
template <typename R, bool XR>
__global__ void __launch_bounds__(256) adj_recur_kernel(Geom g, const typename CT<R>::V* __restrict__ hop2,
                                                        const R* __restrict__ diag2,
                                                        const typename CT<R>::V* __restrict__ tp,
                                                        const typename CT<R>::V* __restrict__ tpp,
                                                        const typename CT<R>::V* __restrict__ lam,
                                                        typename CT<R>::V* __restrict__ out, int64_t ld, int64_t M,
                                                        R alpha, R w_re, R w_im, typename CT<R>::V* __restrict__ y,
                                                        R cy) {
    typedef typename CT<R>::V V;
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.N) return;
    const Nbr nb = neighbours(g, s);
    const V z = CT<R>::make(0, 0);
    const V hxp = nb.hxp ? hop2[s] : z, hyp = nb.hyp ? hop2[g.N + s] : z;
    V t = nb.hxm ? hop2[nb.xm] : z;
    const V hxm = CT<R>::make(t.x, -t.y);
    t = nb.hym ? hop2[g.N + nb.ym] : z;
    const V hym = CT<R>::make(t.x, -t.y);
    const R d = diag2[s];
    for (int64_t m = blockIdx.y; m < M; m += gridDim.y) {
        const int64_t o = m * ld;
        V acc = z;
        if (tp) {
            const V v0 = tp[o + s], vxp = tp[o + nb.xp], vxm = tp[o + nb.xm], vyp = tp[o + nb.yp], vym = tp[o + nb.ym];
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
            acc.x *= alpha;
            acc.y *= alpha;
        }
        if (tpp) {
            const V q = tpp[o + s];
            acc.x -= q.x;
            acc.y -= q.y;
        }
        if (lam) {
            const V l = lam[o + s];
            acc.x = fma(w_re, l.x, fma(-w_im, l.y, acc.x));
            acc.y = fma(w_re, l.y, fma(w_im, l.x, acc.y));
        }
        out[o + s] = acc;
        if (y) {
            V t = y[o + s];
            t.x = fma(cy, acc.x, t.x);
            t.y = fma(cy, acc.y, t.y);
            y[o + s] = t;
        }
    }
}

// out = alpha (2H~) tp - tpp + w lam over an n x M block (the three-term Chebyshev recurrence
// and its adjoint; KPM uses it for the moments).  out may alias tpp.
cudaError_t launch_stencil_recur(lm_ctx* ctx, const Geom& g, int precision, const void* hop2, const void* diag2,
                                 const void* tp, const void* tpp, const void* lam, void* out, int64_t ld, int64_t M,
                                 double alpha, double wre, double wim, void* y, double cy, bool xreal) {
    if (M <= 0 || g.N <= 0) return cudaSuccess;
    const dim3 grid((unsigned)((g.N + 255) / 256), (unsigned)(M < 65535 ? M : 65535));
#define LM_RECUR(R, V, XRV)                                                                                   \
    adj_recur_kernel<R, XRV><<<grid, 256, 0, ctx->stream>>>(g, (const V*)hop2, (const R*)diag2, (const V*)tp, \
                                                           (const V*)tpp, (const V*)lam, (V*)out, ld, M,        \
                                                           (R)alpha, (R)wre, (R)wim, (V*)y, (R)cy)
    if (precision == LM_C64) {
        if (xreal) LM_RECUR(double, double2, true);
        else LM_RECUR(double, double2, false);
    } else {
        if (xreal) LM_RECUR(float, float2, true);
        else LM_RECUR(float, float2, false);
    }
#undef LM_RECUR
    ctx->launches++;
    return cudaGetLastError();
}

// One order k of the adjoint, fused: the beta recurrence and the gradient sums in one pass.
//   beta_k = conj(c_k) lambda + (2H~) beta_{k+1} - beta_{k+2}         (written to bk)
//   gV[s] += f Re( ph * sum_m conj(beta_k,sm) T_sm )
//   gA    += f Re( ph * sum_s [ D[s,s+x] S1x + D[s,s+y] S1y + conj(D[s-x,s]) S2x + conj(D[s-y,s]) S2y ] )
//            S1e = sum_m conj(beta_k,sm) T_{s+e,m},  S2e = sum_m conj(beta_k,sm) T_{s-e,m}
// with T = T_{k-1}, ph = e^{-ib dt}, f = 1/a (k = 1) or 2/a (k >= 2), D = dH/dA per bond (owned
// by its source site).  Every bond enters twice -- conj(b_s) D T_j at its source s and
// conj(b_j) conj(D) T_s at its destination j -- so a thread needs only its own beta_k and
// read-only neighbours of T.  A block owns 32 sites and one chunk of the kets (blockIdx.y);
// its 8 warps split the chunk and their partial sums are added in warp order.  gV_part and
// gA_part have one writer per entry per launch and lm_adjoint_gradients adds them in chunk
// and block order, so the gradients are bit-reproducible.  c32 sums are double-float.
template <typename R>
__global__ void __launch_bounds__(256, sizeof(R) == sizeof(float) ? 3 : 2) adj_beta_grad_kernel(
    Geom g, const typename CT<R>::V* __restrict__ hop2, const R* __restrict__ diag2,
    const typename CT<R>::V* __restrict__ b1, const typename CT<R>::V* __restrict__ b2,
    const typename CT<R>::V* __restrict__ lam, typename CT<R>::V* __restrict__ bk, R w_re, R w_im,
    const double2* __restrict__ dhop, const typename CT<R>::V* __restrict__ T, int64_t ld, int64_t M, int64_t mchunk,
    double ph_re, double ph_im, double f, double* __restrict__ gV_part, double* __restrict__ gA_part) {
    typedef typename CT<R>::V V;
    __shared__ double red[8][10][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t s = (int64_t)blockIdx.x * 32 + lane;
    const int64_t m0 = (int64_t)blockIdx.y * mchunk, m1 = min(M, m0 + mchunk);
    Acc<R> a[10];  // conj(b)T_s (re, im); S1x; S1y; S2x; S2y
    Nbr nb;
    if (s < g.N) {
        nb = neighbours(g, s);
        const V z = CT<R>::make(0, 0);
        const V hxp = nb.hxp ? hop2[s] : z, hyp = nb.hyp ? hop2[g.N + s] : z;
        V t = nb.hxm ? hop2[nb.xm] : z;
        const V hxm = CT<R>::make(t.x, -t.y);
        t = nb.hym ? hop2[g.N + nb.ym] : z;
        const V hym = CT<R>::make(t.x, -t.y);
        const R d = diag2[s];
        for (int64_t m = m0 + warp; m < m1; m += 8) {
            const int64_t o = m * ld;
            V acc = z;
            if (b1) {
                const V v0 = b1[o + s], vxp = b1[o + nb.xp], vxm = b1[o + nb.xm], vyp = b1[o + nb.yp], vym = b1[o + nb.ym];
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
            }
            if (b2) {
                const V q = b2[o + s];
                acc.x -= q.x;
                acc.y -= q.y;
            }
            const V l = lam[o + s];
            acc.x = fma(w_re, l.x, fma(-w_im, l.y, acc.x));
            acc.y = fma(w_re, l.y, fma(w_im, l.x, acc.y));
            bk[o + s] = acc;
            const V b = acc, ts = T[o + s];
            a[0].add_prod(b.x, ts.x);
            a[0].add_prod(b.y, ts.y);
            a[1].add_prod(b.x, ts.y);
            a[1].add_prod(-b.y, ts.x);
            if (dhop) {
                const V tn[4] = {T[o + nb.xp], T[o + nb.yp], T[o + nb.xm], T[o + nb.ym]};
#pragma unroll
                for (int q = 0; q < 4; ++q) {  // conj(b) T_n
                    a[2 + 2 * q].add_prod(b.x, tn[q].x);
                    a[2 + 2 * q].add_prod(b.y, tn[q].y);
                    a[3 + 2 * q].add_prod(b.x, tn[q].y);
                    a[3 + 2 * q].add_prod(-b.y, tn[q].x);
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 10; ++q) red[warp][q][lane] = a[q].get();
    __syncthreads();
    if (warp != 0) return;
    double v[10];
#pragma unroll
    for (int q = 0; q < 10; ++q) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += red[w][q][lane];
        v[q] = t;
    }
    double ga = 0.0;
    if (s < g.N) {
        gV_part[(int64_t)blockIdx.y * g.N + s] += f * (ph_re * v[0] - ph_im * v[1]);
        if (dhop) {
            const double2 zz = make_double2(0.0, 0.0);
            const double2 D[4] = {nb.hxp ? dhop[s] : zz, nb.hyp ? dhop[g.N + s] : zz, nb.hxm ? dhop[nb.xm] : zz,
                                  nb.hym ? dhop[g.N + nb.ym] : zz};
            double zr = 0.0, zi = 0.0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const double sr = v[2 + 2 * q], si = v[3 + 2 * q];
                if (q < 2) {  // D S
                    zr += D[q].x * sr - D[q].y * si;
                    zi += D[q].x * si + D[q].y * sr;
                } else {      // conj(D) S
                    zr += D[q].x * sr + D[q].y * si;
                    zi += D[q].x * si - D[q].y * sr;
                }
            }
            ga = f * (ph_re * zr - ph_im * zi);
        }
    }
    if (gA_part) {
        for (int o = 16; o > 0; o >>= 1) ga += __shfl_down_sync(0xffffffffu, ga, o);
        if (lane == 0) gA_part[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] += ga;
    }
}

// rho_s = sum_m |psi_sm|^2; loss = sum_s (rho_s - target_s)^2; lambda = 4 (rho_s - target_s) psi.
// A block owns 32 sites (8 warps split the kets); loss_part[block] receives its partial loss.
template <typename R>
__global__ void __launch_bounds__(256) adj_seed_kernel(int64_t N, const typename CT<R>::V* __restrict__ psi,
                                                       typename CT<R>::V* __restrict__ lam, int64_t ld, int64_t M,
                                                       const double* __restrict__ target,
                                                       double* __restrict__ loss_part) {
    typedef typename CT<R>::V V;
    __shared__ double red[8][32];
    __shared__ double diff_s[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t s = (int64_t)blockIdx.x * 32 + lane;
    Acc<R> acc;
    if (s < N)
        for (int64_t m = warp; m < M; m += 8) {
            const V v = psi[m * ld + s];
            acc.add_prod(v.x, v.x);
            acc.add_prod(v.y, v.y);
        }
    red[warp][lane] = acc.get();
    __syncthreads();
    if (warp == 0) {
        double rho = 0.0;
        for (int w = 0; w < 8; ++w) rho += red[w][lane];
        const double diff = s < N ? rho - target[s] : 0.0;
        diff_s[lane] = diff;
        double l = diff * diff;
        for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
        if (lane == 0) loss_part[blockIdx.x] = l;
    }
    __syncthreads();
    if (s < N) {
        const R fct = (R)(4.0 * diff_s[lane]);
        for (int64_t m = warp; m < M; m += 8) {
            const V v = psi[m * ld + s];
            lam[m * ld + s] = CT<R>::make(fct * v.x, fct * v.y);
        }
    }
}

// dH[s, s+e]/dA_c = -2 pi i LI_c(A_c = 1) H[s, s+e] for field component c.
__global__ void flux_derivative_kernel(Geom g, FieldSet f, int comp, const double2* __restrict__ hop,
                                       double2* __restrict__ dhop) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.N) return;
    FieldSet one = f;
    one.n = 1;
    one.c[0] = f.c[comp];
    one.amp[0] = 1.0;
    const int64_t xi = s / g.Ly, yi = s - xi * g.Ly;
    const double x1 = (double)(xi + 1), y1 = (double)(yi + 1);
#pragma unroll
    for (int dir = 0; dir < 2; ++dir) {
        const double x2 = dir == 0 ? x1 + 1.0 : x1, y2 = dir == 0 ? y1 : y1 + 1.0;
        const double li = field_line_integral(g, one, x1, y1, x2, y2);
        const double2 h = hop[dir * g.N + s];
        const double w = -2.0 * M_PI * li;  // d/dA e^{-2 pi i A li} = -2 pi i li (...)
        dhop[dir * g.N + s] = make_double2(-w * h.y, w * h.x);  // (i w) h
    }
}

}  // namespace lmgpu

using namespace lmgpu;

struct lm_adjoint {
    lm_ctx* ctx = nullptr;
    int64_t n = 0, m = 0;
    int precision = LM_C64;
    size_t elem = 16;
    int K = 0;
    std::vector<void*> T;  // T_0 .. T_{K-1} (T_0 aliases psi during a step)
    void* B[3] = {nullptr, nullptr, nullptr};
    double* d_gV = nullptr;     // per ket chunk, one partial per site (nchunk x n)
    double* d_gA = nullptr;     // per gradient slot, one partial per (chunk, 32-site block)
    int nslots = 0;
    int64_t nblk = 0;           // 32-site blocks of the gradient and seed kernels
    int64_t nchunk = 1, mchunk = 1;  // ket chunks of the gradient kernel (grid y) and their size
    double* d_loss = nullptr;   // one partial per 32-site block (nblk)
    double* d_target = nullptr;
    double2* d_dhop = nullptr;
};

static void adj_free_stack(lm_adjoint* a) {
    for (size_t i = 1; i < a->T.size(); ++i)
        if (a->T[i]) cudaFree(a->T[i]);
    a->T.clear();
    for (auto& b : a->B) {
        if (b) cudaFree(b);
        b = nullptr;
    }
}

static int adj_alloc(lm_ctx* ctx, void** p, size_t bytes) {
    if (cudaMalloc(p, bytes) != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return set_err(ctx, LM_ERR_OOM, "lm_adjoint: device allocation failed");
    }
    return LM_OK;
}

static int adj_ensure_stack(lm_adjoint* a, int K) {
    if (a->K == K && !a->T.empty()) return LM_OK;
    adj_free_stack(a);
    const size_t bytes = a->elem * (size_t)a->n * (size_t)a->m;
    a->T.assign((size_t)K, nullptr);
    for (int k = 1; k < K; ++k) {
        int rc = adj_alloc(a->ctx, &a->T[(size_t)k], bytes);
        if (rc != LM_OK) return rc;
    }
    for (auto& b : a->B) {
        int rc = adj_alloc(a->ctx, &b, bytes);
        if (rc != LM_OK) return rc;
    }
    a->K = K;
    return LM_OK;
}

extern "C" {

int lm_adjoint_create(lm_ctx* ctx, int64_t n, int64_t m, int precision, int nslots, lm_adjoint** out) {
    if (!ctx) return LM_ERR_ARG;
    if (!out) return set_err(ctx, LM_ERR_ARG, "lm_adjoint_create: null output");
    *out = nullptr;
    if (n < 1 || m < 1 || nslots < 0) return set_err(ctx, LM_ERR_ARG, "lm_adjoint_create: bad sizes");
    if (precision != LM_C64 && precision != LM_C32) return set_err(ctx, LM_ERR_ARG, "lm_adjoint_create: unknown precision");
    lm_adjoint* a = new (std::nothrow) lm_adjoint();
    if (!a) return set_err(ctx, LM_ERR_OOM, "host allocation");
    a->ctx = ctx;
    a->n = n;
    a->m = m;
    a->precision = precision;
    a->elem = precision == LM_C64 ? 16 : 8;
    a->nslots = nslots;
    a->nblk = (n + 31) / 32;
    // enough (block, chunk) pairs for ~6 blocks per SM, chunks of at least 64 kets
    const int64_t want = ((int64_t)6 * std::max(ctx->sm_count, 1) + a->nblk - 1) / a->nblk;
    a->nchunk = std::max<int64_t>(1, std::min<int64_t>(want, (m + 63) / 64));
    a->mchunk = (m + a->nchunk - 1) / a->nchunk;
    a->nchunk = (m + a->mchunk - 1) / a->mchunk;
    cudaSetDevice(ctx->device);
    const size_t gA_len = (size_t)(nslots > 0 ? nslots : 1) * (size_t)a->nblk * (size_t)a->nchunk;
    const size_t gV_len = (size_t)n * (size_t)a->nchunk;
    int rc = adj_alloc(ctx, (void**)&a->d_gV, sizeof(double) * gV_len);
    if (rc == LM_OK) rc = adj_alloc(ctx, (void**)&a->d_gA, sizeof(double) * gA_len);
    if (rc == LM_OK) rc = adj_alloc(ctx, (void**)&a->d_loss, sizeof(double) * (size_t)a->nblk);
    if (rc == LM_OK) rc = adj_alloc(ctx, (void**)&a->d_target, sizeof(double) * (size_t)n);
    if (rc == LM_OK) rc = adj_alloc(ctx, (void**)&a->d_dhop, sizeof(double2) * 2 * (size_t)n);
    if (rc != LM_OK) {
        if (a->d_gV) cudaFree(a->d_gV);
        if (a->d_gA) cudaFree(a->d_gA);
        if (a->d_loss) cudaFree(a->d_loss);
        if (a->d_target) cudaFree(a->d_target);
        if (a->d_dhop) cudaFree(a->d_dhop);
        delete a;
        return rc;
    }
    cudaMemsetAsync(a->d_gV, 0, sizeof(double) * gV_len, ctx->stream);
    cudaMemsetAsync(a->d_gA, 0, sizeof(double) * gA_len, ctx->stream);
    *out = a;
    return LM_OK;
}

int lm_adjoint_destroy(lm_adjoint* a) {
    if (!a) return LM_OK;
    cudaSetDevice(a->ctx->device);
    cudaStreamSynchronize(a->ctx->stream);
    adj_free_stack(a);
    cudaFree(a->d_gV);
    cudaFree(a->d_gA);
    cudaFree(a->d_loss);
    cudaFree(a->d_target);
    cudaFree(a->d_dhop);
    delete a;
    return LM_OK;
}

int lm_adjoint_reset(lm_adjoint* a) {
    if (!a) return LM_ERR_ARG;
    lm_ctx* ctx = a->ctx;
    cudaSetDevice(ctx->device);
    CUDA_TRY(ctx, cudaMemsetAsync(a->d_gV, 0, sizeof(double) * (size_t)a->n * (size_t)a->nchunk, ctx->stream), "memset");
    CUDA_TRY(ctx, cudaMemsetAsync(a->d_gA, 0,
                                  sizeof(double) * (size_t)(a->nslots > 0 ? a->nslots : 1) * (size_t)a->nblk *
                                      (size_t)a->nchunk,
                                  ctx->stream),
             "memset");
    return LM_OK;
}

int lm_adjoint_seed(lm_adjoint* a, lm_state* psi, const double* target, lm_state* lam, double* loss) {
    if (!a) return LM_ERR_ARG;
    lm_ctx* ctx = a->ctx;
    if (!psi || !lam || !target || !loss) return set_err(ctx, LM_ERR_ARG, "lm_adjoint_seed: null argument");
    if (psi->n != a->n || psi->m != a->m || lam->n != a->n || lam->m != a->m || psi->precision != a->precision ||
        lam->precision != a->precision || psi->kind != LM_KETS || lam->kind != LM_KETS)
        return set_err(ctx, LM_ERR_ARG, "lm_adjoint_seed: state shapes differ from the adjoint");
    cudaSetDevice(ctx->device);
    CUDA_TRY(ctx, cudaMemcpyAsync(a->d_target, target, sizeof(double) * (size_t)a->n, cudaMemcpyHostToDevice, ctx->stream),
             "upload target");
    const unsigned blocks = (unsigned)a->nblk;
    if (a->precision == LM_C64)
        adj_seed_kernel<double><<<blocks, 256, 0, ctx->stream>>>(a->n, (const double2*)psi->d_data, (double2*)lam->d_data,
                                                                 psi->ld, a->m, a->d_target, a->d_loss);
    else
        adj_seed_kernel<float><<<blocks, 256, 0, ctx->stream>>>(a->n, (const float2*)psi->d_data, (float2*)lam->d_data,
                                                                psi->ld, a->m, a->d_target, a->d_loss);
    ctx->launches++;
    CUDA_TRY(ctx, cudaGetLastError(), "seed kernel");
    std::vector<double> part((size_t)a->nblk);
    CUDA_TRY(ctx, cudaMemcpyAsync(part.data(), a->d_loss, sizeof(double) * part.size(), cudaMemcpyDeviceToHost,
                                  ctx->stream),
             "download loss");
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    double tot = 0.0;
    for (double v : part) tot += v;  // block order
    *loss = tot;
    return LM_OK;
}

int lm_adjoint_step(lm_adjoint* a, lm_solver* s, lm_ham* h, int component, int slot, lm_state* psi, lm_state* lam) {
    if (!a || !s) return LM_ERR_ARG;
    lm_ctx* ctx = a->ctx;
    if (!h || !psi || !lam) return set_err(ctx, LM_ERR_ARG, "lm_adjoint_step: null argument");
    if (!s->valid || s->ham != h) return set_err(ctx, LM_ERR_STATE, "lm_adjoint_step: update the solver with this Hamiltonian first");
    if (psi->n != a->n || psi->m != a->m || lam->n != a->n || lam->m != a->m || psi->precision != a->precision ||
        lam->precision != a->precision)
        return set_err(ctx, LM_ERR_ARG, "lm_adjoint_step: state shapes differ from the adjoint");
    if (component >= h->fields.n || (component >= 0 && (slot < 0 || slot >= a->nslots)))
        return set_err(ctx, LM_ERR_ARG, "lm_adjoint_step: bad field component or gradient slot");
    cudaSetDevice(ctx->device);
    const Geom& g = h->lat->g;
    const int K = s->K;
    int rc = adj_ensure_stack(a, K);
    if (rc != LM_OK) return rc;
    const bool f64 = a->precision == LM_C64;
    const void* hop2 = f64 ? (const void*)s->d_hop2 : (const void*)s->d_hop2f;
    const void* diag2 = f64 ? (const void*)s->d_diag2 : (const void*)s->d_diag2f;
    const int64_t ld = psi->ld, M = a->m;
    auto recur = [&](const void* tp, const void* tpp, const void* lamp, void* out, double alpha, double wre,
                     double wim) -> cudaError_t {
        return launch_stencil_recur(ctx, g, a->precision, hop2, diag2, tp, tpp, lamp, out, ld, M, alpha, wre, wim,
                                    nullptr, 0.0);
    };
    // T_0 = psi_n (aliased), T_1 = H~ T_0, T_k = 2 H~ T_{k-1} - T_{k-2}  (k < K)
    a->T[0] = psi->d_data;
    for (int k = 1; k < K; ++k) {
        CUDA_TRY(ctx, recur(a->T[(size_t)k - 1], k >= 2 ? a->T[(size_t)k - 2] : nullptr, nullptr, a->T[(size_t)k],
                            k == 1 ? 0.5 : 1.0, 0.0, 0.0),
                 "adjoint forward recurrence");
    }
    // field derivative table
    const double2* dhop = nullptr;
    if (component >= 0) {
        flux_derivative_kernel<<<(unsigned)((g.N + 255) / 256), 256, 0, ctx->stream>>>(g, h->fields, component, h->d_hop,
                                                                                       a->d_dhop);
        ctx->launches++;
        CUDA_TRY(ctx, cudaGetLastError(), "flux derivative kernel");
        dhop = a->d_dhop;
    }
    // beta_K .. beta_1 with gradient terms; B[k % 3] rotates
    const dim3 ggrid((unsigned)a->nblk, (unsigned)a->nchunk);
    double* gA = component >= 0 ? a->d_gA + (size_t)slot * (size_t)a->nblk * (size_t)a->nchunk : nullptr;
    for (int k = K; k >= 1; --k) {
        const ChebCoef c = s->coef[(size_t)k];
        const double wre = c.odd ? 0.0 : c.s, wim = c.odd ? c.s : 0.0;  // conj(c_k)
        void* bk = a->B[k % 3];
        const void* b1 = k + 1 <= K ? a->B[(k + 1) % 3] : nullptr;
        const void* b2 = k + 2 <= K ? a->B[(k + 2) % 3] : nullptr;
        const double f = (k == 1 ? 1.0 : 2.0) / s->a;
        if (f64)
            adj_beta_grad_kernel<double><<<ggrid, 256, 0, ctx->stream>>>(
                g, (const double2*)hop2, (const double*)diag2, (const double2*)b1, (const double2*)b2,
                (const double2*)lam->d_data, (double2*)bk, wre, wim, dhop, (const double2*)a->T[(size_t)k - 1], ld, M,
                a->mchunk, s->phase_re, s->phase_im, f, a->d_gV, gA);
        else
            adj_beta_grad_kernel<float><<<ggrid, 256, 0, ctx->stream>>>(
                g, (const float2*)hop2, (const float*)diag2, (const float2*)b1, (const float2*)b2,
                (const float2*)lam->d_data, (float2*)bk, (float)wre, (float)wim, dhop,
                (const float2*)a->T[(size_t)k - 1], ld, M, a->mchunk, s->phase_re, s->phase_im, f, a->d_gV, gA);
        ctx->launches++;
        CUDA_TRY(ctx, cudaGetLastError(), "adjoint beta/gradient kernel");
    }
    return LM_OK;
}

int lm_adjoint_gradients(lm_adjoint* a, double* gV, double* gA) {
    if (!a) return LM_ERR_ARG;
    lm_ctx* ctx = a->ctx;
    cudaSetDevice(ctx->device);
    const size_t nc = (size_t)a->nchunk, nb = (size_t)a->nblk;
    std::vector<double> pv, pa;
    if (gV) {
        pv.resize((size_t)a->n * nc);
        CUDA_TRY(ctx, cudaMemcpyAsync(pv.data(), a->d_gV, sizeof(double) * pv.size(), cudaMemcpyDeviceToHost, ctx->stream),
                 "download gV");
    }
    if (gA && a->nslots > 0) {
        pa.resize((size_t)a->nslots * nb * nc);
        CUDA_TRY(ctx, cudaMemcpyAsync(pa.data(), a->d_gA, sizeof(double) * pa.size(), cudaMemcpyDeviceToHost, ctx->stream),
                 "download gA");
    }
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    if (gV)
        for (int64_t i = 0; i < a->n; ++i) {
            double tot = 0.0;
            for (size_t c = 0; c < nc; ++c) tot += pv[c * (size_t)a->n + (size_t)i];  // chunk order
            gV[i] = tot;
        }
    for (int j = 0; gA && j < a->nslots; ++j) {
        double tot = 0.0;
        const double* p = pa.data() + (size_t)j * nb * nc;
        for (size_t q = 0; q < nb * nc; ++q) tot += p[q];  // chunk-major block order
        gA[j] = tot;
    }
    return LM_OK;
}

int lm_solver_set_bounds(lm_solver* s, double emin, double emax) {
    if (!s) return LM_ERR_ARG;
    if (!(emin == 0.0 && emax == 0.0) && !(isfinite(emin) && isfinite(emax) && emax > emin))
        return set_err(s->ctx, LM_ERR_ARG, "lm_solver_set_bounds: need emin < emax (or 0, 0 for automatic)");
    s->fixed_bounds = !(emin == 0.0 && emax == 0.0);
    s->fix_emin = emin;
    s->fix_emax = emax;
    s->valid = 0;
    return LM_OK;
}

}  // extern "C"
