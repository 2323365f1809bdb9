// Temporally blocked Chebyshev step (ComplexF32 recurrence) for the square-lattice stencil,
// for one lattice or for a batch of independent lattices of different sizes.
//
// One launch applies the whole series  y = e^{-ib dt} sum_{k<=K} c_k T_k(H~) x  to
// column-major ket blocks: every ket is read once (a spatial tile plus a halo of K sites) and
// the result written once, instead of five vector passes per Chebyshev order.
//
// Tiling: a CTA of 512 threads owns a region of 32 (x) x 64 (y) sites; thread (tx, ty) holds
// the S = 4 consecutive y-sites S ty .. S ty + S-1 of row tx in registers (T_{k-1}, T_{k-2},
// the accumulator and the stencil coefficients).  Per order, rows are exchanged through a
// double-buffered shared-memory copy of T_{k-1} (x neighbours) and warp shuffles (y
// neighbours: a warp holds whole rows).  Built with LM_FUSED_SITES=2 the CTA has 1024
// threads of 2 sites.  The valid part of the region shrinks by one site per order, so after
// K orders the inner (32-2K) x (64-2K) sites are exact and are written out.  Periodic axes wrap the
// halo.  Along an open axis the first and last regions of a lattice sit on the lattice edge:
// the stencil has no bond across it, so nothing shrinks there and those regions write out up
// to the edge (a lattice no longer than a region is one tile along that axis, with no halo).
// Positions outside the lattice hold zeros and zero coefficients.
//
// Work items are (instance, tile, 16 kets).  A single lattice strides over its items
// statically; a batch pulls items from a global atomic counter (the work queue), so CTAs
// that finish small lattices early take more items.  The next item's first ket is staged
// global -> shared with cp.async while the current ket is computed; order 1 reads its
// neighbours straight from that staging buffer.  Consecutive items are neighbouring tiles of
// the same kets, so halo re-reads hit L2.
#include <cuda_runtime.h>

#include "lmgpu_internal.cuh"

namespace lmgpu {

// Sites per thread along y: 4 (512 threads, a warp holds two rows) or 2 (1024 threads, a warp
// holds one row); the region stays 32 x 64 either way.
#ifndef LM_FUSED_SITES
#define LM_FUSED_SITES 4
#endif
namespace {
constexpr int RX = 32;         // region extent along x (threads along x)
constexpr int S = LM_FUSED_SITES;  // sites per thread along y
static_assert(S == 2 || S == 4, "LM_FUSED_SITES must be 2 or 4");
constexpr int TY = 64 / S;     // threads along y
constexpr int RY = TY * S;     // region extent along y
constexpr int NTHR = RX * TY;  // 512 or 1024
constexpr int HALVES = S / 2;  // float4 words per thread and row (a float4 = two sites)
constexpr int ROWS_PER_WARP = 32 / TY;
constexpr int KB = 1;          // kets a thread advances together
// one buffer = KB kets x RX rows x HALVES x TY float4
constexpr int BUF_F4 = KB * RX * HALVES * TY;
constexpr int SMEM_BYTES = 4 * BUF_F4 * 16;  // T double buffer + staging double buffer
constexpr int DESC_WORDS = (int)(sizeof(FusedInst) + 3) / 4;
}  // namespace

__device__ __forceinline__ int fidx(int kk, int row, int h, int ty) { return ((kk * RX + row) * HALVES + h) * TY + ty; }

// The S sites of thread ty in row `row` of buffer `buf`, and the reverse.
__device__ __forceinline__ void load_sites(const float4* buf, int kk, int row, int ty, float2 v[S]) {
#pragma unroll
    for (int h = 0; h < HALVES; ++h) {
        const float4 q = buf[fidx(kk, row, h, ty)];
        v[2 * h] = make_float2(q.x, q.y);
        v[2 * h + 1] = make_float2(q.z, q.w);
    }
}
__device__ __forceinline__ void store_sites(float4* buf, int kk, int row, int ty, const float2 v[S]) {
#pragma unroll
    for (int h = 0; h < HALVES; ++h) buf[fidx(kk, row, h, ty)] = make_float4(v[2 * h].x, v[2 * h].y, v[2 * h + 1].x, v[2 * h + 1].y);
}

// Region coordinate -> lattice coordinate (0-based) or -1 outside an open axis.
__device__ __forceinline__ int64_t wrap_axis(int64_t c, int64_t L, int per) {
    if (c >= 0 && c < L) return c;
    if (!per) return -1;
    c %= L;
    return c < 0 ? c + L : c;
}

// Tiling of one axis of length L by regions of R sites with a halo of H: region origin and
// written range [w0, w1) of tile t (lattice coordinates; periodic origins may be negative).
struct AxisTile {
    int64_t origin, w0, w1;
};

__host__ __device__ __forceinline__ int64_t axis_ntiles(int64_t L, int per, int R, int H) {
    const int64_t I = R - 2 * H;
    if (per) return (L + I - 1) / I;
    if (L <= R) return 1;
    const int64_t rest = L - 2 * (int64_t)(R - H);
    return 2 + (rest > 0 ? (rest + I - 1) / I : 0);
}

__host__ __device__ __forceinline__ AxisTile axis_tile(int64_t L, int per, int R, int H, int64_t t, int64_t n) {
    const int64_t I = R - 2 * H;
    AxisTile a;
    if (per) {
        a.w0 = t * I;
        a.w1 = a.w0 + I < L ? a.w0 + I : L;
        a.origin = a.w0 - H;
    } else if (n == 1) {
        a.origin = 0;
        a.w0 = 0;
        a.w1 = L;
    } else if (t == 0) {
        a.origin = 0;
        a.w0 = 0;
        a.w1 = R - H;
    } else {
        a.w0 = (R - H) + (t - 1) * I;
        if (t == n - 1) {
            a.origin = L - R;
            a.w1 = L;
        } else {
            a.origin = a.w0 - H;
            a.w1 = a.w0 + I;
        }
    }
    return a;
}

struct TileMap {
    int site[S];  // lattice site of each of my four positions, -1 outside (N < 2^31)
    int gx;       // unwrapped lattice x of my row
    int gy0;      // unwrapped lattice y of my first position
    int wx0, wx1, wy0, wy1;  // written range of the tile
    int hard_lo, hard_hi;    // the region's low / high x edge is an open lattice edge
};

__device__ __forceinline__ TileMap tile_map(const Geom& g, int64_t tile, int nty, int H, int tx, int ty) {
    TileMap m;
    const int64_t ntx_all = axis_ntiles(g.Lx, g.per_x, RX, H);
    const int64_t tile_x = tile / nty, tile_y = tile % nty;
    const AxisTile ax = axis_tile(g.Lx, g.per_x, RX, H, tile_x, ntx_all);
    const AxisTile ay = axis_tile(g.Ly, g.per_y, RY, H, tile_y, nty);
    m.wx0 = (int)ax.w0; m.wx1 = (int)ax.w1;
    m.wy0 = (int)ay.w0; m.wy1 = (int)ay.w1;
    m.hard_lo = !g.per_x && ax.origin == 0;
    m.hard_hi = !g.per_x && ax.origin + RX >= g.Lx;
    m.gx = (int)(ax.origin + tx);
    m.gy0 = (int)(ay.origin + ty * S);
    const int64_t xs = wrap_axis(m.gx, g.Lx, g.per_x);
#pragma unroll
    for (int j = 0; j < S; ++j) {
        const int64_t ys = wrap_axis(m.gy0 + j, g.Ly, g.per_y);
        m.site[j] = (xs >= 0 && ys >= 0) ? (int)(xs * g.Ly + ys) : -1;
    }
    return m;
}

__device__ __forceinline__ void cp_async8(float4* smem_f4, int half, const float2* src, bool valid) {
    const unsigned dst = (unsigned)__cvta_generic_to_shared(smem_f4) + (unsigned)half * 8u;
    const int n = valid ? 8 : 0;  // n = 0 fills the 8 bytes with zeros
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src), "r"(n));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Stages kets k0 .. k0+KB-1 (those below k_end) of my four positions into `stage`.
__device__ __forceinline__ void prefetch_kets(float4* stage, const TileMap& m, const float2* x, int64_t ld,
                                              int64_t k0, int64_t k_end, int tx, int ty) {
#pragma unroll
    for (int kk = 0; kk < KB; ++kk) {
        const int64_t ket = k0 + kk;
#pragma unroll
        for (int j = 0; j < S; ++j) {
            const bool ok = ket < k_end && m.site[j] >= 0;
            const float2* src = ok ? x + ket * ld + m.site[j] : x;
            cp_async8(&stage[fidx(kk, tx, j >> 1, ty)], j & 1, src, ok);
        }
    }
    cp_async_commit();
}


// Instance holding global item `item` (largest i with table[i].item_begin <= item).
__device__ __forceinline__ int find_instance(const FusedInst* __restrict__ table, int ninst, int64_t item) {
    int lo = 0, hi = ninst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&table[mid].item_begin) <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Cooperative copy of an instance descriptor into shared memory (threads < DESC_WORDS).
__device__ __forceinline__ void load_desc(FusedInst* dst, const FusedInst* src, int t) {
    if (t < DESC_WORDS) reinterpret_cast<int*>(dst)[t] = __ldg(reinterpret_cast<const int*>(src) + t);
}

// XR: every x-hop of every instance is real (Landau gauge or no field, no twist across x), so
// the x-neighbour terms take 2 FMAs instead of 4.
template <int K, bool XR>
__global__ void __launch_bounds__(NTHR, 1)
cheb_fused_c32_kernel(FusedInst single, const FusedInst* __restrict__ table, int ninst, int64_t nitems,
                      unsigned long long* queue) {
    constexpr int H = K;  // halo = number of orders
    extern __shared__ float4 smem[];
    __shared__ FusedInst s_desc[2];   // current and next instance
    __shared__ long long s_item[2];   // next work items (alternating slots)
    auto tb = [](int i) { return i * BUF_F4; };
    auto sbuf = [](int i) { return (2 + i) * BUF_F4; };

    const int t = threadIdx.x;
    const int tx = t / TY;
    const int ty = t % TY;
    const int warp_row0 = (t >> 5) * ROWS_PER_WARP;  // the rows a warp holds

    // next item id: the work queue for a batch, a static stride for one lattice
    long long last_static = (long long)blockIdx.x - gridDim.x;
    auto fetch = [&]() -> long long {
        if (queue) return (long long)atomicAdd(queue, 1ull);
        last_static += gridDim.x;
        return last_static;
    };
    auto desc_of = [&](long long it) -> const FusedInst* {
        return table ? &table[find_instance(table, ninst, it)] : nullptr;
    };

    if (t == 0) {
        s_item[0] = fetch();
        s_item[1] = fetch();
    }
    __syncthreads();
    long long item = s_item[0];
    int nslot = 1;  // slot holding the upcoming item
    if (item >= nitems) return;
    int dslot = 0;
    {
        const FusedInst* src = desc_of(item);
        if (src) load_desc(&s_desc[0], src, t);
        else if (t == 0) s_desc[0] = single;
    }
    __syncthreads();

    int64_t lit = item - s_desc[0].item_begin;  // item within the instance
    int64_t ntiles = (int64_t)s_desc[0].ntx * s_desc[0].nty;
    TileMap m = tile_map(s_desc[0].g, lit % ntiles, s_desc[0].nty, H, tx, ty);
    int64_t k_begin = (lit / ntiles) * kFusedKetsPerItem;
    int64_t k_end = min(s_desc[0].M, k_begin + kFusedKetsPerItem);
    prefetch_kets(smem + sbuf(0), m, s_desc[0].x, s_desc[0].ld, k_begin, k_end, tx, ty);
    int sb = 0;

    while (true) {
        const FusedInst& D = s_desc[dslot];
        const Geom g = D.g;
        // stencil coefficients of my positions (shared by every ket of the item)
        float2 hx[S], hxm[S], hy[S];
        float d[S];
        float2 hym0 = make_float2(0.f, 0.f);
        unsigned interior = 0;  // bit j: position j is written out
        {
            const float2* hop2 = D.hop2;
            const float* diag2 = D.diag2;
            const int64_t xsm = wrap_axis(m.gx - 1, g.Lx, g.per_x);
            const int64_t xs = wrap_axis(m.gx, g.Lx, g.per_x);
#pragma unroll
            for (int j = 0; j < S; ++j) {
                const int s = m.site[j];
                const int64_t ys = wrap_axis(m.gy0 + j, g.Ly, g.per_y);
                hx[j] = s >= 0 ? __ldg(hop2 + s) : make_float2(0.f, 0.f);
                hy[j] = s >= 0 ? __ldg(hop2 + g.N + s) : make_float2(0.f, 0.f);
                d[j] = s >= 0 ? __ldg(diag2 + s) : 0.f;
                const int64_t sm = (xsm >= 0 && ys >= 0) ? xsm * g.Ly + ys : -1;  // site at x-1
                const float2 h = sm >= 0 ? __ldg(hop2 + sm) : make_float2(0.f, 0.f);
                hxm[j] = make_float2(h.x, -h.y);
                const int gy = m.gy0 + j;
                if (m.gx >= m.wx0 && m.gx < m.wx1 && gy >= m.wy0 && gy < m.wy1 && s >= 0) interior |= 1u << j;
            }
            const int64_t ysm = wrap_axis(m.gy0 - 1, g.Ly, g.per_y);
            const int64_t s2 = (xs >= 0 && ysm >= 0) ? xs * g.Ly + ysm : -1;  // site at y-1
            const float2 hh = s2 >= 0 ? __ldg(hop2 + g.N + s2) : make_float2(0.f, 0.f);
            hym0 = make_float2(hh.x, -hh.y);
        }
        const int64_t cur_k_end = k_end;
        const TileMap cur = m;
        bool have_next_item = false;

        for (int64_t k0 = k_begin; k0 < cur_k_end; k0 += KB) {
            cp_async_wait_all();
            __syncthreads();  // staged kets visible; the previous kets are done with every buffer
            if (k0 + KB < cur_k_end) {
                prefetch_kets(smem + sbuf(sb ^ 1), cur, D.x, D.ld, k0 + KB, cur_k_end, tx, ty);
            } else {
                // last kets of this item: take the next item and stage its first kets
                const long long nxt = s_item[nslot];
                if (nxt < nitems) {
                    const FusedInst* src = desc_of(nxt);
                    if (src) load_desc(&s_desc[dslot ^ 1], src, t);
                    else if (t == 0) s_desc[dslot ^ 1] = single;
                    if (t == 0) s_item[nslot ^ 1] = fetch();
                    nslot ^= 1;
                    __syncthreads();  // next descriptor visible
                    const FusedInst& Dn = s_desc[dslot ^ 1];
                    item = nxt;
                    lit = item - Dn.item_begin;
                    ntiles = (int64_t)Dn.ntx * Dn.nty;
                    m = tile_map(Dn.g, lit % ntiles, Dn.nty, H, tx, ty);
                    k_begin = (lit / ntiles) * kFusedKetsPerItem;
                    k_end = min(Dn.M, k_begin + kFusedKetsPerItem);
                    prefetch_kets(smem + sbuf(sb ^ 1), m, Dn.x, Dn.ld, k_begin, k_end, tx, ty);
                    have_next_item = true;
                }
            }
            const int stage = sbuf(sb);

            // T_{k-1} and T_{k-2} of my positions live in registers (t1, t2); the shared buffers
            // carry T_{k-1} to the x-neighbours, T_0 comes from the staging buffer.
            float2 t1[KB][S], t2[KB][S], yv[KB][S];
#pragma unroll
            for (int kk = 0; kk < KB; ++kk) {
                load_sites(smem + stage, kk, tx, ty, t1[kk]);
#pragma unroll
                for (int j = 0; j < S; ++j) yv[kk][j] = make_float2(0.f, 0.f);
            }

#pragma unroll
            for (int k = 1; k <= K; ++k) {
                const int src = (k == 1) ? stage : tb((k - 1) & 1);
                const int dst = tb(k & 1);
                // warps whose two rows both lie outside the valid region skip the order (the
                // valid rows shrink by one per order, except at an open lattice edge)
                const bool active =
                    (cur.hard_lo || warp_row0 + ROWS_PER_WARP - 1 >= k) && (cur.hard_hi || warp_row0 < RX - k);
                // T_k of my positions; a skipped warp takes zeros (its rows stay invalid), so the
                // register rotation below is unconditional and compiles to renaming
                float2 tk[KB][S];
                if (active) {
                    const int xp = min(tx + 1, RX - 1), xm = max(tx - 1, 0);
                    const float sk = D.s[k];
#pragma unroll
                    for (int kk = 0; kk < KB; ++kk) {
                        float2 vxp[S], vxm[S];
                        load_sites(smem + src, kk, xp, ty, vxp);
                        load_sites(smem + src, kk, xm, ty, vxm);
                        float2 up, dn;  // y-1 of my first position, y+1 of my last
                        up.x = __shfl_up_sync(0xffffffffu, t1[kk][S - 1].x, 1);
                        up.y = __shfl_up_sync(0xffffffffu, t1[kk][S - 1].y, 1);
                        dn.x = __shfl_down_sync(0xffffffffu, t1[kk][0].x, 1);
                        dn.y = __shfl_down_sync(0xffffffffu, t1[kk][0].y, 1);
#pragma unroll
                        for (int j = 0; j < S; ++j) {
                            const float2 vyp = (j < S - 1) ? t1[kk][j + 1] : dn;
                            const float2 vym = (j > 0) ? t1[kk][j - 1] : up;
                            const float2 hym = (j > 0) ? make_float2(hy[j - 1].x, -hy[j - 1].y) : hym0;
                            float2 acc = (k == 1) ? make_float2(0.f, 0.f) : make_float2(-t2[kk][j].x, -t2[kk][j].y);
                            if (XR) {
                                acc.x = fmaf(hx[j].x, vxp[j].x, acc.x);
                                acc.y = fmaf(hx[j].x, vxp[j].y, acc.y);
                                acc.x = fmaf(hxm[j].x, vxm[j].x, acc.x);
                                acc.y = fmaf(hxm[j].x, vxm[j].y, acc.y);
                            } else {
                                acc.x = fmaf(hx[j].x, vxp[j].x, acc.x); acc.x = fmaf(-hx[j].y, vxp[j].y, acc.x);
                                acc.y = fmaf(hx[j].x, vxp[j].y, acc.y); acc.y = fmaf(hx[j].y, vxp[j].x, acc.y);
                                acc.x = fmaf(hxm[j].x, vxm[j].x, acc.x); acc.x = fmaf(-hxm[j].y, vxm[j].y, acc.x);
                                acc.y = fmaf(hxm[j].x, vxm[j].y, acc.y); acc.y = fmaf(hxm[j].y, vxm[j].x, acc.y);
                            }
                            acc.x = fmaf(hy[j].x, vyp.x, acc.x); acc.x = fmaf(-hy[j].y, vyp.y, acc.x);
                            acc.y = fmaf(hy[j].x, vyp.y, acc.y); acc.y = fmaf(hy[j].y, vyp.x, acc.y);
                            acc.x = fmaf(hym.x, vym.x, acc.x); acc.x = fmaf(-hym.y, vym.y, acc.x);
                            acc.y = fmaf(hym.x, vym.y, acc.y); acc.y = fmaf(hym.y, vym.x, acc.y);
                            acc.x = fmaf(d[j], t1[kk][j].x, acc.x);
                            acc.y = fmaf(d[j], t1[kk][j].y, acc.y);
                            if (k == 1) { acc.x *= 0.5f; acc.y *= 0.5f; }  // tables hold 2H/a
                            tk[kk][j] = acc;
                        }
#pragma unroll
                        for (int j = 0; j < S; ++j) {
                            const float2 t = tk[kk][j];
                            if (k == 1) {  // y = -i s_1 T1 + g0 T0 + g1 T1 (t1 still holds T0)
                                const ChebLo lo = D.lo;
                                const float2 x = t1[kk][j];
                                const float lx = fmaf(lo.g0_re, x.x, fmaf(-lo.g0_im, x.y,
                                                 fmaf(lo.g1_re, t.x, -lo.g1_im * t.y)));
                                const float ly = fmaf(lo.g0_re, x.y, fmaf(lo.g0_im, x.x,
                                                 fmaf(lo.g1_re, t.y, lo.g1_im * t.x)));
                                yv[kk][j].x = fmaf(sk, t.y, lx);
                                yv[kk][j].y = fmaf(-sk, t.x, ly);
                            } else if (k & 1) {  // c_k = -i s_k
                                yv[kk][j].x = fmaf(sk, t.y, yv[kk][j].x);
                                yv[kk][j].y = fmaf(-sk, t.x, yv[kk][j].y);
                            } else {      // c_k = s_k
                                yv[kk][j].x = fmaf(sk, t.x, yv[kk][j].x);
                                yv[kk][j].y = fmaf(sk, t.y, yv[kk][j].y);
                            }
                        }
                        if (k < K) {
                            store_sites(smem + dst, kk, tx, ty, tk[kk]);
                        }
                    }
                } else {
#pragma unroll
                    for (int kk = 0; kk < KB; ++kk)
#pragma unroll
                        for (int j = 0; j < S; ++j) tk[kk][j] = make_float2(0.f, 0.f);
                }
#pragma unroll
                for (int kk = 0; kk < KB; ++kk)
#pragma unroll
                    for (int j = 0; j < S; ++j) {
                        t2[kk][j] = t1[kk][j];
                        t1[kk][j] = tk[kk][j];
                    }
                if (k < K) __syncthreads();
            }

            // out = e^{-ib dt} y + a0 x (a0 = e^{-ib dt} c_0): the small terms first, the dominant one last
            const float ph_re = D.ph_re, ph_im = D.ph_im, a0_re = D.a0_re, a0_im = D.a0_im;
#pragma unroll
            for (int kk = 0; kk < KB; ++kk) {
                const int64_t ket = k0 + kk;
                if (ket >= cur_k_end) break;
                float2* outk = D.out + ket * D.ld;
                float2 x0[S];
                load_sites(smem + stage, kk, tx, ty, x0);
#pragma unroll
                for (int j = 0; j < S; ++j) {
                    if (interior & (1u << j)) {
                        float2 r;
                        r.x = fmaf(ph_re, yv[kk][j].x, -ph_im * yv[kk][j].y);
                        r.y = fmaf(ph_re, yv[kk][j].y, ph_im * yv[kk][j].x);
                        r.x = fmaf(-a0_im, x0[j].y, r.x);
                        r.y = fmaf(a0_im, x0[j].x, r.y);
                        float2 o;
                        o.x = fmaf(a0_re, x0[j].x, r.x);
                        o.y = fmaf(a0_re, x0[j].y, r.y);
                        outk[cur.site[j]] = o;
                    }
                }
            }
            sb ^= 1;
        }
        if (!have_next_item) break;
        dslot ^= 1;
    }
    cp_async_wait_all();
}

int fused_supported(int precision, int K) { return precision == LM_C32 && K >= 2 && K <= kFusedMaxK; }
int fused_supported_geom(const Geom& g) { return g.N < (int64_t)1 << 31 && g.Lx < (1 << 30) && g.Ly < (1 << 30); }

int64_t fused_items(const Geom& g, int K, int64_t m, int* ntx, int* nty) {
    *ntx = (int)axis_ntiles(g.Lx, g.per_x, RX, K);
    *nty = (int)axis_ntiles(g.Ly, g.per_y, RY, K);
    const int64_t kchunks = (m + kFusedKetsPerItem - 1) / kFusedKetsPerItem;
    return (int64_t)(*ntx) * (*nty) * kchunks;
}

void fused_fill_coef(FusedInst& d, int K, const ChebCoef* coef, double ph_re, double ph_im) {
    for (int k = 0; k <= kFusedMaxK; ++k) d.s[k] = k <= K ? (float)coef[k].s : 0.f;
    d.ph_re = (float)ph_re;
    d.ph_im = (float)ph_im;
    d.a0_re = (float)(ph_re * coef[0].s);
    d.a0_im = (float)(ph_im * coef[0].s);
    d.lo = cheb_lo(ph_re, ph_im, coef[0].s, coef[1].s, true);
}

template <bool XR>
static cudaError_t set_fused_attr(int K) {
    switch (K) {
#define LM_ATTR_CASE(KK) \
    case KK:             \
        return cudaFuncSetAttribute(cheb_fused_c32_kernel<KK, XR>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
        LM_ATTR_CASE(2) LM_ATTR_CASE(3) LM_ATTR_CASE(4) LM_ATTR_CASE(5)
        LM_ATTR_CASE(6) LM_ATTR_CASE(7) LM_ATTR_CASE(8)
#undef LM_ATTR_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

cudaError_t ensure_fused_attr(lm_ctx* ctx, int K, bool xreal) {
    const unsigned bit = 1u << (K + (xreal ? 16 : 0));
    if (ctx->fused_attr & bit) return cudaSuccess;
    const cudaError_t e = xreal ? set_fused_attr<true>(K) : set_fused_attr<false>(K);
    if (e == cudaSuccess) ctx->fused_attr |= bit;
    return e;
}

template <bool XR>
static cudaError_t launch_fused_k(lm_ctx* ctx, int K, int grid, const FusedInst& one, const FusedInst* d_table,
                                  int ninst, int64_t nitems, unsigned long long* d_queue) {
    switch (K) {
#define LM_FUSED_CASE(KK)                                                                                   \
    case KK:                                                                                              \
        cheb_fused_c32_kernel<KK, XR><<<(unsigned)grid, NTHR, SMEM_BYTES, ctx->stream>>>(one, d_table, ninst, \
                                                                                         nitems, d_queue);   \
        return cudaGetLastError();
        LM_FUSED_CASE(2) LM_FUSED_CASE(3) LM_FUSED_CASE(4) LM_FUSED_CASE(5)
        LM_FUSED_CASE(6) LM_FUSED_CASE(7) LM_FUSED_CASE(8)
#undef LM_FUSED_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

cudaError_t launch_fused_table(lm_ctx* ctx, int K, bool xreal, const FusedInst* single, const FusedInst* d_table,
                               int ninst, int64_t nitems, unsigned long long* d_queue, int grid) {
    if (nitems <= 0) return cudaSuccess;
    if (grid <= 0) grid = ctx->sm_count > 0 ? ctx->sm_count : 152;
    if (grid > nitems) grid = (int)nitems;
    FusedInst one{};
    if (single) one = *single;
    cudaError_t e = ensure_fused_attr(ctx, K, xreal);
    if (e != cudaSuccess) return e;
    e = xreal ? launch_fused_k<true>(ctx, K, grid, one, d_table, ninst, nitems, d_queue)
              : launch_fused_k<false>(ctx, K, grid, one, d_table, ninst, nitems, d_queue);
    ctx->launches++;
    return e;
}

cudaError_t launch_cheb_fused_c32(lm_ctx* ctx, const Geom& g, const float2* hop2, const float* diag2,
                                  const float2* x, float2* out, int64_t ld, int64_t m, int K, bool xreal,
                                  const ChebCoef* coef, double ph_re, double ph_im, const float4* spack,
                                  int stream_mode, uint32_t* comp) {
    FusedInst d{};
    d.g = g;
    d.hop2 = hop2;
    d.diag2 = diag2;
    d.x = x;
    d.out = out;
    d.ld = ld;
    d.M = m;
    d.item_begin = 0;
    fused_fill_coef(d, K, coef, ph_re, ph_im);
    d.comp = comp;
    if (spack) return launch_cheb_stream_c32(ctx, d, K, stream_mode, spack);
    if (comp) return cudaErrorNotSupported;  // the compensation plane is carried by the streaming form only
    const int64_t nitems = fused_items(g, K, m, &d.ntx, &d.nty);
    return launch_fused_table(ctx, K, xreal, &d, nullptr, 1, nitems, nullptr, 0);
}

}  // namespace lmgpu
