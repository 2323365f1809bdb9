// Temporally blocked Chebyshev step (ComplexF32 recurrence) for the square-lattice stencil.
//
// One launch applies the whole series  y = e^{-ib dt} sum_{k<=K} c_k T_k(H~) x  to a
// column-major ket block: every ket is read once (a spatial tile plus a halo of K sites)
// and the result written once, instead of five vector passes per Chebyshev order.
//
// Tiling: a CTA of 512 threads owns a region of 32 (x) x 64 (y) sites; thread (tx, ty)
// holds the four consecutive y-sites 4ty..4ty+3 of row tx in registers (T_{k-1}, T_{k-2},
// the accumulator y and its stencil coefficients).  Per order, the rows are exchanged
// through a double-buffered shared-memory copy of T_{k-1} (x neighbours) and warp shuffles
// (y neighbours: a warp holds two complete rows).  The valid part of the region shrinks by
// one site per order, so after K orders the inner (32-2K) x (64-2K) sites are exact and are
// written out.  Positions outside the lattice (open axes) hold zeros and zero coefficients;
// periodic axes wrap the halo.  Work items are (tile, 8 kets); persistent CTAs stride over
// them with consecutive items on neighbouring tiles of the same kets, so halo re-reads hit L2.
#include <cuda_runtime.h>

#include "lmgpu_internal.cuh"

namespace lmgpu {

namespace {
constexpr int RX = 32;        // region extent along x (threads along x)
constexpr int TY = 16;        // threads along y
constexpr int S = 4;          // sites per thread along y
constexpr int RY = TY * S;    // region extent along y
constexpr int NTHR = RX * TY; // 512
constexpr int KETS_PER_ITEM = 8;
}  // namespace

struct FusedCoef {
    float s[kFusedMaxK + 1];
    int odd[kFusedMaxK + 1];
    int K;
    float ph_re, ph_im;   // e^{-ib dt}
    float a0_re, a0_im;   // e^{-ib dt} c_0
};

__device__ __forceinline__ float2 ld_site(const float2* __restrict__ p, int64_t site) {
    return site >= 0 ? __ldg(p + site) : make_float2(0.f, 0.f);
}

// Region coordinate -> lattice site (0-based) or -1 outside an open axis.
__device__ __forceinline__ int64_t wrap_axis(int64_t c, int64_t L, int per) {
    if (c >= 0 && c < L) return c;
    if (!per) return -1;
    c %= L;
    return c < 0 ? c + L : c;
}

__global__ void __launch_bounds__(NTHR, 1)
cheb_fused_c32_kernel(Geom g, const float2* __restrict__ hop2, const float* __restrict__ diag2,
                      const float2* __restrict__ x, float2* __restrict__ out, int64_t ld, int64_t M,
                      int H, int ntx, int nty, int64_t nitems, FusedCoef cf) {
    __shared__ float4 buf[2][RX][RY / 2];  // T_{k-1} double buffer, 2 x 16 KB

    const int t = threadIdx.x;
    const int tx = t / TY;
    const int ty = t % TY;
    const int lane = t & 31;
    const int warp_row0 = (t >> 5) * 2;  // the two rows a warp holds
    const int IX = RX - 2 * H, IY = RY - 2 * H;
    const int64_t ntiles = (int64_t)ntx * nty;
    const int64_t kchunks = (M + KETS_PER_ITEM - 1) / KETS_PER_ITEM;

    for (int64_t item = blockIdx.x; item < nitems; item += gridDim.x) {
        const int64_t tile = item % ntiles;
        const int64_t kc = item / ntiles;
        if (kc >= kchunks) break;
        const int64_t tile_x = tile / nty, tile_y = tile % nty;
        const int64_t gx = tile_x * IX - H + tx;  // lattice x of my row (unwrapped)
        const int64_t xs = wrap_axis(gx, g.Lx, g.per_x);
        const int64_t xsm = wrap_axis(gx - 1, g.Lx, g.per_x);

        int64_t site[S];
        float2 hx[S], hxm[S], hy[S];
        float d[S];
        float2 hym0 = make_float2(0.f, 0.f);
        bool interior[S];
#pragma unroll
        for (int j = 0; j < S; ++j) {
            const int ry = ty * S + j;
            const int64_t gy = tile_y * IY - H + ry;
            const int64_t ys = wrap_axis(gy, g.Ly, g.per_y);
            site[j] = (xs >= 0 && ys >= 0) ? xs * g.Ly + ys : -1;
            hx[j] = ld_site(hop2, site[j]);
            hy[j] = site[j] >= 0 ? __ldg(hop2 + g.N + site[j]) : make_float2(0.f, 0.f);
            d[j] = site[j] >= 0 ? __ldg(diag2 + site[j]) : 0.f;
            const int64_t sm = (xsm >= 0 && ys >= 0) ? xsm * g.Ly + ys : -1;  // site at x-1
            const float2 h = ld_site(hop2, sm);
            hxm[j] = make_float2(h.x, -h.y);
            interior[j] = tx >= H && tx < RX - H && ry >= H && ry < RY - H && gx < g.Lx && gy < g.Ly;
            if (j == 0) {
                const int64_t ysm = wrap_axis(gy - 1, g.Ly, g.per_y);
                const int64_t s2 = (xs >= 0 && ysm >= 0) ? xs * g.Ly + ysm : -1;  // site at y-1
                const float2 hh = s2 >= 0 ? __ldg(hop2 + g.N + s2) : make_float2(0.f, 0.f);
                hym0 = make_float2(hh.x, -hh.y);
            }
        }

        const int64_t k_begin = kc * KETS_PER_ITEM;
        const int64_t k_end = min(M, k_begin + KETS_PER_ITEM);
        float2 nxt[S];
#pragma unroll
        for (int j = 0; j < S; ++j) nxt[j] = site[j] >= 0 ? __ldg(x + k_begin * ld + site[j]) : make_float2(0.f, 0.f);

        for (int64_t ket = k_begin; ket < k_end; ++ket) {
            // yv accumulates the small part sum_{k>=1} c_k T_k; the dominant c_0 T_0 term is
            // added once at the end with a single rounding (x0 keeps T_0).
            float2 t1[S], t0[S], yv[S], x0[S];
#pragma unroll
            for (int j = 0; j < S; ++j) {
                t1[j] = nxt[j];
                x0[j] = nxt[j];
                t0[j] = make_float2(0.f, 0.f);
                yv[j] = make_float2(0.f, 0.f);
            }
            if (ket + 1 < k_end) {  // prefetch the next ket of this item
#pragma unroll
                for (int j = 0; j < S; ++j)
                    nxt[j] = site[j] >= 0 ? __ldg(x + (ket + 1) * ld + site[j]) : make_float2(0.f, 0.f);
            }
            buf[0][tx][ty * 2] = make_float4(t1[0].x, t1[0].y, t1[1].x, t1[1].y);
            buf[0][tx][ty * 2 + 1] = make_float4(t1[2].x, t1[2].y, t1[3].x, t1[3].y);
            __syncthreads();

            for (int k = 1; k <= cf.K; ++k) {
                const int cur = (k - 1) & 1;
                // warps whose two rows both lie outside the valid region skip the order
                const bool active = (warp_row0 + 1 >= k) && (warp_row0 < RX - k);
                if (active) {
                    const int xp = min(tx + 1, RX - 1), xm = max(tx - 1, 0);
                    const float4 p0 = buf[cur][xp][ty * 2], p1 = buf[cur][xp][ty * 2 + 1];
                    const float4 m0 = buf[cur][xm][ty * 2], m1 = buf[cur][xm][ty * 2 + 1];
                    const float2 vxp[S] = {make_float2(p0.x, p0.y), make_float2(p0.z, p0.w),
                                           make_float2(p1.x, p1.y), make_float2(p1.z, p1.w)};
                    const float2 vxm[S] = {make_float2(m0.x, m0.y), make_float2(m0.z, m0.w),
                                           make_float2(m1.x, m1.y), make_float2(m1.z, m1.w)};
                    float2 up, dn;  // y-1 of my first site, y+1 of my last site
                    up.x = __shfl_up_sync(0xffffffffu, t1[S - 1].x, 1);
                    up.y = __shfl_up_sync(0xffffffffu, t1[S - 1].y, 1);
                    dn.x = __shfl_down_sync(0xffffffffu, t1[0].x, 1);
                    dn.y = __shfl_down_sync(0xffffffffu, t1[0].y, 1);
                    (void)lane;
                    float2 tk[S];
#pragma unroll
                    for (int j = 0; j < S; ++j) {
                        const float2 vyp = (j < S - 1) ? t1[j + 1] : dn;
                        const float2 vym = (j > 0) ? t1[j - 1] : up;
                        const float2 hym = (j > 0) ? make_float2(hy[j - 1].x, -hy[j - 1].y) : hym0;
                        float2 acc = (k == 1) ? make_float2(0.f, 0.f) : make_float2(-t0[j].x, -t0[j].y);
                        acc.x = fmaf(hx[j].x, vxp[j].x, acc.x); acc.x = fmaf(-hx[j].y, vxp[j].y, acc.x);
                        acc.y = fmaf(hx[j].x, vxp[j].y, acc.y); acc.y = fmaf(hx[j].y, vxp[j].x, acc.y);
                        acc.x = fmaf(hxm[j].x, vxm[j].x, acc.x); acc.x = fmaf(-hxm[j].y, vxm[j].y, acc.x);
                        acc.y = fmaf(hxm[j].x, vxm[j].y, acc.y); acc.y = fmaf(hxm[j].y, vxm[j].x, acc.y);
                        acc.x = fmaf(hy[j].x, vyp.x, acc.x); acc.x = fmaf(-hy[j].y, vyp.y, acc.x);
                        acc.y = fmaf(hy[j].x, vyp.y, acc.y); acc.y = fmaf(hy[j].y, vyp.x, acc.y);
                        acc.x = fmaf(hym.x, vym.x, acc.x); acc.x = fmaf(-hym.y, vym.y, acc.x);
                        acc.y = fmaf(hym.x, vym.y, acc.y); acc.y = fmaf(hym.y, vym.x, acc.y);
                        acc.x = fmaf(d[j], t1[j].x, acc.x);
                        acc.y = fmaf(d[j], t1[j].y, acc.y);
                        if (k == 1) { acc.x *= 0.5f; acc.y *= 0.5f; }  // tables hold 2H/a
                        tk[j] = acc;
                    }
                    const float sk = cf.s[k];
                    const int odd = cf.odd[k];
#pragma unroll
                    for (int j = 0; j < S; ++j) {
                        if (odd) {
                            yv[j].x = fmaf(sk, tk[j].y, yv[j].x);
                            yv[j].y = fmaf(-sk, tk[j].x, yv[j].y);
                        } else {
                            yv[j].x = fmaf(sk, tk[j].x, yv[j].x);
                            yv[j].y = fmaf(sk, tk[j].y, yv[j].y);
                        }
                        t0[j] = t1[j];
                        t1[j] = tk[j];
                    }
                    if (k < cf.K) {
                        buf[k & 1][tx][ty * 2] = make_float4(t1[0].x, t1[0].y, t1[1].x, t1[1].y);
                        buf[k & 1][tx][ty * 2 + 1] = make_float4(t1[2].x, t1[2].y, t1[3].x, t1[3].y);
                    }
                }
                __syncthreads();
            }
#pragma unroll
            for (int j = 0; j < S; ++j) {
                if (interior[j]) {
                    // out = e^{-ib dt} (c_0 x + y): the small terms first, the large one last
                    float2 r;
                    r.x = fmaf(cf.ph_re, yv[j].x, -cf.ph_im * yv[j].y);
                    r.y = fmaf(cf.ph_re, yv[j].y, cf.ph_im * yv[j].x);
                    r.x = fmaf(-cf.a0_im, x0[j].y, r.x);
                    r.y = fmaf(cf.a0_im, x0[j].x, r.y);
                    float2 o;
                    o.x = fmaf(cf.a0_re, x0[j].x, r.x);
                    o.y = fmaf(cf.a0_re, x0[j].y, r.y);
                    out[ket * ld + site[j]] = o;
                }
            }
        }
    }
}

int fused_supported(int precision, int K) { return precision == LM_C32 && K >= 2 && K <= kFusedMaxK; }

cudaError_t launch_cheb_fused_c32(lm_ctx* ctx, const Geom& g, const float2* hop2, const float* diag2,
                                  const float2* x, float2* out, int64_t ld, int64_t m, int K,
                                  const ChebCoef* coef, double ph_re, double ph_im) {
    FusedCoef cf{};
    cf.K = K;
    for (int k = 0; k <= K; ++k) {
        cf.s[k] = (float)coef[k].s;
        cf.odd[k] = coef[k].odd;
    }
    cf.ph_re = (float)ph_re;
    cf.ph_im = (float)ph_im;
    cf.a0_re = (float)(ph_re * coef[0].s);
    cf.a0_im = (float)(ph_im * coef[0].s);
    const int H = K;
    const int IX = RX - 2 * H, IY = RY - 2 * H;
    const int ntx = (int)((g.Lx + IX - 1) / IX), nty = (int)((g.Ly + IY - 1) / IY);
    const int64_t kchunks = (m + KETS_PER_ITEM - 1) / KETS_PER_ITEM;
    const int64_t nitems = (int64_t)ntx * nty * kchunks;
    int64_t grid = ctx->sm_count > 0 ? ctx->sm_count : 152;
    if (grid > nitems) grid = nitems;
    cheb_fused_c32_kernel<<<(unsigned)grid, NTHR, 0, ctx->stream>>>(g, hop2, diag2, x, out, ld, m, H, ntx, nty,
                                                                      nitems, cf);
    ctx->launches++;
    return cudaGetLastError();
}

}  // namespace lmgpu
