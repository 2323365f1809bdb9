// x-streaming form of the temporally blocked Chebyshev step (ComplexF32 recurrence) for one
// square lattice: y = e^{-ib dt} sum_{k<=K} c_k T_k(H~) x applied to a column-major ket block.
//
// A warp owns one ket and one strip of 64 sites along y (lane l holds the site pair
// 2l, 2l+1) and walks along x.  At step s it loads column s of the ket (order 0) and advances
// every order k = 1..K by one column, order k working on column s - k: T_k(x) needs
// T_{k-1} at x-1, x, x+1 and T_{k-2} at x, and order k-1 produced column x+1 earlier in the
// same step.  So each order keeps the last three columns of its T in registers (a rotation
// of period three), the y-neighbours come from the adjacent lanes by shuffles,
// and the accumulator y(x) = sum_k c_k T_k(x) waits in a per-warp shared-memory ring of
// K+1 columns until order K completes it.  With uniform columns it is updated once per group
// of three orders, from the windows, which still hold T_j(x) of the group's earlier orders.
// Column s + 3 of the ket is staged into a second ring by cp.async while column s is being
// used.  On a periodic y axis with uniform columns the stencil runs on (re, im) float pairs
// (fma.rn.f32x2).
//
// Only the y direction has a halo: after K orders the sites K .. 63-K of a strip are exact
// (at an open lattice edge the strip sits on the edge and writes up to it), while along x a
// range [xa, xb) of columns costs (xb - xa) + 2K steps.  Every warp takes an equal share of
// all the (strip, ket, column) work, so the only redundancy along x is 2K steps per item a
// warp starts or finishes.  The region form (32 x 64 sites
// with a halo on both axes) computes about twice the sites it writes at K = 6; this form
// computes about 1.25 times.  Each site-order uses the same sequence of FMAs as the region
// form, so the two give bit-identical results.
//
// Coefficients come from planes that stream_pack_kernel packs whenever the FP32 stencil
// tables change: columns padded on both sides (periodic ones wrapped, open ones zero), so an
// order's record sits at a linear offset with no wrap or bounds logic.  With uniform columns
// (every hop of a column equal: the Landau gauge without a twist along y, MODE 2/3) a
// column's hops are one record kept in shared memory for the whole lattice, and an order
// reads only the diagonal pair of its sites, staged by cp.async together with the ket column.
//
// Requirements (checked by stream_supported): Ly even, so every lane's pair is a 16-byte
// aligned, unsplit pair of sites; Lx >= 2K + 3, so a column index leaves [0, Lx) by less
// than one lattice length; K <= 6 with real x-hops, K <= 5 otherwise (the register budget of
// the three-column windows).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "lmgpu_internal.cuh"

namespace lmgpu {

// Warps per CTA (one ket each); 16 caps a thread at 128 registers, 12 at 170.
#ifndef LM_STREAM_WARPS
#define LM_STREAM_WARPS 16
#endif
// 1: the periodic uniform-column mode computes on float pairs (fma.rn.f32x2); 0: scalar FMAs.
#ifndef LM_STREAM_PAIRED
#define LM_STREAM_PAIRED 1
#endif
// 1: the three-column windows rotate by register moves at the end of every step; 0: the
// step loop is unrolled three times and the rotation is renaming (more code in flight);
// 2: unrolled in the uniform-column modes (few coefficient registers), rotating otherwise.
#ifndef LM_STREAM_ROTATE
#define LM_STREAM_ROTATE 2
#endif

namespace {
constexpr int SW = LM_STREAM_WARPS;
// The per-site-plane modes need more than 128 registers a thread at their largest orders (the
// brick stencil at K = 6; the compensated output on top of MODE 0/1 at K >= 5): they run 12 warps
// per CTA (up to 170 registers).
#ifndef LM_STREAM_WARPS_BRICK6
#define LM_STREAM_WARPS_BRICK6 12
#endif
__host__ __device__ constexpr int stream_warps(int K, int mode, bool cmp = false) {
    return ((mode == 4 && K >= 6) || (cmp && (mode == 0 || mode == 1 || mode == 4) && K >= 5)) ? LM_STREAM_WARPS_BRICK6
                                                                                               : SW;
}
constexpr int SR = 64;       // strip width along y: 32 lanes x 2 sites
constexpr int SPF = 3;       // columns of the ket staged ahead
constexpr int kStreamMaxK = 6;
// Packed coefficient planes: padded columns x = -kPadL .. Lx + kPadR - 1 (periodic columns
// wrapped, open ones zero), one float4 per (column, site pair) and plane, plus one zero pair
// at the end of every plane for lanes outside the lattice.
constexpr int kPadL = 2 * kStreamMaxK + 2;
constexpr int kPadR = kStreamMaxK;
constexpr int kPlanes = 5;
// plane 0: real parts {hx0, hx1, hxm0, hxm1} (real x-hops); 1: {hx0, hx1}; 2: {hxm0, hxm1};
// 3: {hy0, hy1}; 4: {hym0, d0, d1}.  hx: hop to x+1; hxm: conj of the hop from x-1 to x;
// hy: hop to y+1; hym0: conj of the hop from y-1 to the first site; d: diagonal.

__host__ __device__ constexpr int stream_halo(int K) { return K + (K & 1); }  // even: pairs stay aligned
__host__ __device__ constexpr int stream_ring_f4(int K) { return ((K + 1) + (K + 1 + SPF)) * 32; }
// Uniform-column modes also keep, per warp, a ring of the diagonal pairs of the staged columns
// (same slots as the ket ring) and, per CTA, the column records of the whole lattice.
__host__ __device__ constexpr int stream_dring_f4(int K) { return (K + 1 + SPF) * 16; }
constexpr int kStreamSmemMax = 232448;  // bytes of shared memory a CTA may use
// Column records per lattice column in shared memory: MODE 2 keeps {hx, hxm, hy.re, hy.im};
// MODE 3 keeps the pair forms {hx, hx, hxm, hxm}, {hy.re, hy.re, hy.im, 0} and their negatives.
__host__ __device__ constexpr int stream_crec_f4(int mode) { return mode == 3 ? 4 : 1; }
// Compensated blocks: a per-warp ring of the residual words (two per lane: its two sites) of
// the columns that the next SPF + 1 steps complete, staged with the ket columns.
constexpr int kResRing = SPF + 1;
static_assert(kResRing == 4, "the residual ring is indexed with & 3");
// float4 offset, in a CTA's dynamic shared memory, of what follows the rings and (uniform-column
// modes) the diagonal-pair rings and column records: the residual rings of a compensated block
__host__ __device__ constexpr int stream_base_f4(int K, int mode, int Xp, int nw) {
    return nw * stream_ring_f4(K) + ((mode == 2 || mode == 3) ? nw * stream_dring_f4(K) + Xp * stream_crec_f4(mode) : 0);
}
}  // namespace

// Accumulator coefficients of the paired form (MODE 3): {sigma_k s_k, sigma_k s_k}.
struct StreamPairs {
    float2 s2[kStreamMaxK + 1];
};

namespace {

__device__ __forceinline__ void cp_async16(float4* dst_smem, const void* src, bool valid) {
    const unsigned dst = (unsigned)__cvta_generic_to_shared(dst_smem);
    const int n = valid ? 16 : 0;  // n = 0 fills the 16 bytes with zeros
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(n));
}
__device__ __forceinline__ void cp_async8s(float2* dst_smem, const void* src, bool valid) {
    const unsigned dst = (unsigned)__cvta_generic_to_shared(dst_smem);
    const int n = valid ? 8 : 0;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src), "r"(n));
}
__device__ __forceinline__ void cp_async_commit_s() { asm volatile("cp.async.commit_group;\n" ::); }
// d = a * b + c on both halves of a float pair in one instruction (two round-to-nearest FMAs:
// the same results as two fmaf calls).
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) {
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
        "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}
template <int N>
__device__ __forceinline__ void cp_async_wait_s() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Packed FP32 pairs: one instruction each for both halves, the same rounding as the scalar
// operation on each half.
#define LM_F32X2_BINOP(NAME, OP)                                                                     \
    __device__ __forceinline__ float2 NAME(float2 a, float2 b) {                                     \
        float2 d;                                                                                    \
        asm("{\n\t.reg .b64 ra, rb, rd;\n\t"                                                          \
            "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t" OP                                   \
            " rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"                                               \
            : "=f"(d.x), "=f"(d.y)                                                                   \
            : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));                                               \
        return d;                                                                                    \
    }
LM_F32X2_BINOP(fadd2, "add.rn.f32x2")
LM_F32X2_BINOP(fsub2, "sub.rn.f32x2")
LM_F32X2_BINOP(fmul2, "mul.rn.f32x2")
#undef LM_F32X2_BINOP

// (hi + lo) = a1 x1 + a2 x2 + r + a1 l on both components of a compensated output at once:
// a1 x1 (the dominant term for the workloads' small spectral centres: a1 + i a2 = e^{-ib dt} c_0)
// exact by TwoProd (a1n = -a1 gives its error negated), its sum with q = a2 x2 + r by TwoSum,
// the decoded residual l and both errors in FP32, and the final FastTwoSum split.
__device__ __forceinline__ void comp_sum2(float2 a1, float2 a1n, float2 x1, float2 a2, float2 x2, float2 r, float2 l,
                                          float2& hi, float2& lo) {
    const float2 p = fmul2(a1, x1);
    const float2 en = ffma2(a1n, x1, p);  // -(a1 x1 - p)
    const float2 q = ffma2(a2, x2, r);
    const float2 s = fadd2(p, q);
    const float2 bb = fsub2(s, p);
    const float2 f = fadd2(fsub2(p, fsub2(s, bb)), fsub2(q, bb));
    const float2 t = ffma2(a1, l, fsub2(f, en));
    hi = fadd2(s, t);
    lo = fsub2(t, fsub2(hi, s));
}

__device__ __forceinline__ int wrap_axis_i(int64_t c, int64_t L, int per) {
    if (c >= 0 && c < L) return (int)c;
    if (!per) return -1;
    c %= L;
    return (int)(c < 0 ? c + L : c);
}

// Tiling of the y axis into strips of SR sites with halo H (the same rule as the region form).
__host__ __device__ __forceinline__ int64_t strip_count(int64_t L, int per, int H) {
    const int64_t I = SR - 2 * H;
    if (per) return (L + I - 1) / I;
    if (L <= SR) return 1;
    const int64_t rest = L - 2 * (int64_t)(SR - H);
    return 2 + (rest > 0 ? (rest + I - 1) / I : 0);
}
__device__ __forceinline__ void strip_range(int64_t L, int per, int H, int64_t t, int64_t n, int64_t* origin,
                                            int64_t* w0, int64_t* w1) {
    const int64_t I = SR - 2 * H;
    if (per) {
        *w0 = t * I;
        *w1 = *w0 + I < L ? *w0 + I : L;
        *origin = *w0 - H;
    } else if (n == 1) {
        *origin = 0; *w0 = 0; *w1 = L;
    } else if (t == 0) {
        *origin = 0; *w0 = 0; *w1 = SR - H;
    } else {
        *w0 = (SR - H) + (t - 1) * I;
        if (t == n - 1) {
            *origin = L - SR;
            *w1 = L;
        } else {
            *origin = *w0 - H;
            *w1 = *w0 + I;
        }
    }
}
}  // namespace

__device__ __forceinline__ int wrap_mod(int64_t c, int64_t L) {
    c %= L;
    return (int)(c < 0 ? c + L : c);
}

__global__ void stream_pack_kernel(const Geom g, const float2* __restrict__ hop2, const float* __restrict__ diag2,
                                   float4* __restrict__ pk, float2* __restrict__ pd, float4* __restrict__ pc, int npair,
                                   int Xp, long long plane) {
    const long long n = (long long)Xp * npair + 1;
    const float2 z = make_float2(0.f, 0.f);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float2 hx[2] = {z, z}, hxm[2] = {z, z}, hy[2] = {z, z}, hym0 = z;
        float d[2] = {0.f, 0.f};
        if (i < n - 1) {
            const int xp = (int)(i / npair), yp = (int)(i % npair);
            const int64_t x = (int64_t)xp - kPadL;
            const int xs = g.per_x ? wrap_mod(x, g.Lx) : ((x >= 0 && x < g.Lx) ? (int)x : -1);
            if (xs >= 0) {
                const int y0 = 2 * yp;
                const int xsm = g.per_x ? wrap_mod((int64_t)xs - 1, g.Lx) : xs - 1;
                const int ysm = g.per_y ? wrap_mod((int64_t)y0 - 1, g.Ly) : y0 - 1;
                const float2* hopy = hop2 + g.N;
                for (int j = 0; j < 2; ++j) {
                    const int64_t site = (int64_t)xs * g.Ly + y0 + j;
                    hx[j] = hop2[site];
                    hy[j] = hopy[site];
                    d[j] = diag2[site];
                    if (xsm >= 0) {
                        const float2 h = hop2[(int64_t)xsm * g.Ly + y0 + j];
                        hxm[j] = make_float2(h.x, -h.y);
                    }
                }
                if (ysm >= 0) {
                    const float2 h = hopy[(int64_t)xs * g.Ly + ysm];
                    hym0 = make_float2(h.x, -h.y);
                }
            }
        }
        pd[i] = make_float2(d[0], d[1]);
        if (i < n - 1 && i % npair == 0) {  // column record: the hops of row 0 (pair 0)
            pc[i / npair] = make_float4(hx[0].x, hxm[0].x, hy[0].x, hy[0].y);
        }
        pk[i] = make_float4(hx[0].x, hx[1].x, hxm[0].x, hxm[1].x);
        pk[plane + i] = make_float4(hx[0].x, hx[0].y, hx[1].x, hx[1].y);
        pk[2 * plane + i] = make_float4(hxm[0].x, hxm[0].y, hxm[1].x, hxm[1].y);
        pk[3 * plane + i] = make_float4(hy[0].x, hy[0].y, hy[1].x, hy[1].y);
        pk[4 * plane + i] = make_float4(hym0.x, hym0.y, d[0], d[1]);
    }
}

// MODE 4: the honeycomb in the reference's site order, (j1, j2, s) -> (j1 - 1) 2b + 2(j2 - 1) + s - 1,
// read as an a x 2b "brick" lattice: a lane's pair is one unit cell (A, B); A's neighbours are
// B of its cell, B of the cell below (lane - 1) and B of column x - 1, B's are A of its cell, A
// of the cell above (lane + 1) and A of column x + 1 (planes 0-2 of ensure_brick_pack).
// MODE 0: complex x-hops (planes 1-4); 1: real x-hops (planes 0, 3, 4); 2: uniform columns --
// real x-hops and every hop of a column equal (the Landau gauge without a twist along y), so an
// order reads the diagonal pair of its sites and one column record shared by the warp; 3: the
// same on a periodic y axis (no edge rows).
// CMP: the ket block carries a residual plane D.comp (a bfloat16 pair per site, res_encode),
// staged with the ket columns: the output a0 (x + x_lo) + e^{-ib dt} y is formed with
// error-free products and sums (comp_sum2) and written as hi (the block) and its encoded
// residual (the plane, in place), so the state's own FP32 rounding does not accumulate from
// step to step.
template <int K, int MODE, bool CMP>
__global__ void __launch_bounds__(stream_warps(K, MODE, CMP) * 32, 1)
cheb_stream_c32_kernel(const FusedInst D, const StreamPairs SP, const float4* __restrict__ pk,
                       const float2* __restrict__ pd, const float4* __restrict__ pc, int npair, long long plane,
                       int nty, long long ncols, long long nwarps) {
    constexpr bool BRICK = MODE == 4;
    constexpr bool XR = MODE >= 1 && !BRICK;
    constexpr bool UC = MODE == 2 || MODE == 3;
    constexpr bool YEDGE = MODE == 2;
    // MODE 3 runs the stencil on float pairs (ffma2).  It keeps S_k = sigma_k T_k with sigma_k = +1
    // for k mod 4 in {0, 1} and -1 otherwise, so that the T_{k-2} term enters every chain with a
    // plus sign (sigma_k = -sigma_{k-2}); the hops of order k then carry the sign
    // sigma_k sigma_{k-1} = (-1)^(k+1), taken from the negated column records for even k.  Round
    // to nearest is symmetric under negation, so S_k is exactly sigma_k T_k of the other modes.
    constexpr bool PAIRED = LM_STREAM_PAIRED && MODE == 3;
    // orders per accumulator update: 3 with uniform columns; 1 (an update per order) in the
    // per-site coefficient modes, whose windows leave no registers to hold T_j longer
    constexpr int AG = UC ? 3 : 1;
    constexpr int H = stream_halo(K);
    constexpr int YR = K + 1;          // accumulator ring: columns x .. x+K in flight
    constexpr int XS = K + 1 + SPF;    // ket ring: column s+SPF staged, column s-K still read
    constexpr bool ROT = LM_STREAM_ROTATE == 1 || (LM_STREAM_ROTATE == 2 && !UC);
    constexpr int NP = ROT ? 1 : 3;    // steps per unrolled loop body
    extern __shared__ float4 smem[];
    // the warp index through a shuffle, so that the compiler sees it (and the item, column and
    // ring-slot arithmetic derived from it) as warp-uniform and can keep that on the uniform pipe
    const int warp = __shfl_sync(0xffffffffu, (int)(threadIdx.x >> 5), 0), lane = threadIdx.x & 31;
    float4* yring = smem + warp * stream_ring_f4(K);
    float4* xring = yring + YR * 32;
    const Geom g = D.g;
    const int Lx = (int)g.Lx, Ly = (int)g.Ly;
    const int per_x = g.per_x;
    const float4* __restrict__ P0 = pk;
    const float4* __restrict__ P1 = pk + plane;
    const float4* __restrict__ P2 = pk + 2 * plane;
    const float4* __restrict__ P3 = pk + 3 * plane;
    const float4* __restrict__ P4 = pk + 4 * plane;
    // uniform columns: diagonal-pair ring per warp, column records per CTA
    constexpr int NW = stream_warps(K, MODE, CMP);
    float2* dring = reinterpret_cast<float2*>(smem + NW * stream_ring_f4(K)) + warp * XS * 32;
    float4* ctab = smem + NW * (stream_ring_f4(K) + stream_dring_f4(K));
    uint2* rring = reinterpret_cast<uint2*>(smem + stream_base_f4(K, MODE, (int)D.g.Lx + kPadL + kPadR, NW)) +
                   warp * kResRing * 32;
    if (UC) {
        const int Xp = Lx + kPadL + kPadR;
        for (int i = threadIdx.x; i < Xp; i += NW * 32) {
            const float4 q = __ldg(pc + i);  // {hx, hxm, hy.re, hy.im}
            if (PAIRED) {
                ctab[4 * i + 0] = make_float4(q.x, q.x, q.y, q.y);
                ctab[4 * i + 1] = make_float4(q.z, q.z, q.w, 0.f);
                ctab[4 * i + 2] = make_float4(-q.x, -q.x, -q.y, -q.y);
                ctab[4 * i + 3] = make_float4(-q.z, -q.z, -q.w, 0.f);
            } else {
                ctab[i] = q;
            }
        }
        __syncthreads();
    }

    // Work: the columns of every (strip, ket) item, items in the order strip-major, ket-minor;
    // warp w takes the contiguous share [w ncols / nwarps, (w+1) ncols / nwarps) of them, i.e.
    // column ranges [xa, xb) of one or more consecutive items.
    const long long w = (long long)blockIdx.x * NW + warp;
    if (w >= nwarps) return;
    const long long c_end = (w + 1) * ncols / nwarps;  // ncols * nwarps < 2^63
    for (long long c = w * ncols / nwarps; c < c_end;) {
        const long long item = c / Lx;
        const int xa = (int)(c - item * Lx);
        const long long rest = c_end - c;
        const int xb = rest < (long long)(Lx - xa) ? xa + (int)rest : Lx;
        c += xb - xa;
        const long long ket = item % D.M;
        const long long tile = item / D.M;
        const int strip = (int)tile;
        int64_t origin, w0, w1;
        strip_range(g.Ly, g.per_y, H, strip, nty, &origin, &w0, &w1);
        const int gy = (int)origin + 2 * lane;
        const int ys = wrap_axis_i(gy, g.Ly, g.per_y);       // my pair (ys, ys+1), or -1 outside
        const bool wr = ys >= 0 && gy >= w0 && gy < w1;
        // my coefficient records: column x at offset loff + (x + kPadL) * lstep of every plane;
        // the zero pair outside the lattice
        const int loff = ys >= 0 ? ys / 2 : (int)(plane - 1);
        const int lstep = ys >= 0 ? npair : 0;
        // uniform columns along an open y axis: no bond above the last row or below the first
        const bool y_last = YEDGE && !g.per_y && ys + 1 == Ly - 1;
        const bool y_first = YEDGE && !g.per_y && ys == 0;
        const int n0 = xb - xa + 2 * K;
        const int nsteps = n0 + (NP - n0 % NP) % NP;
        const int s0 = xb + K - nsteps;  // xa - K, moved back so that nsteps is a multiple of NP
        const float2* xk = D.x + ket * D.ld;
        float2* outk = D.out + ket * D.ld;

        // residual words of my site pair in the ket's columns (output columns lie in [xa, xb))
        uint32_t* const rbase = CMP ? D.comp + ket * D.ld + (ys >= 0 ? ys : 0) : nullptr;
        int stage_slot = 0;  // ring slot of the next staged column
        // the next column to stage (stage() runs for idx = 0, 1, 2, ... in turn): its lattice
        // column (wrapped once at most on a periodic axis: -K-2 <= s0 < Lx; outside [0, Lx) on an
        // open one), the offset of my pair in it and its diagonal-pair record, advanced per call
        int sxc = (per_x && s0 < 0) ? s0 + Lx : s0;
        long long soff = (long long)sxc * Ly + ys;
        long long doff = loff + (long long)(s0 + kPadL) * lstep;
        long long roff = (long long)(s0 - K) * Ly;  // compensated blocks: residual offset of column s0 - K
        auto stage = [&](int idx) {
            const bool v = idx < nsteps && sxc >= 0 && sxc < Lx && ys >= 0;
            cp_async16(&xring[stage_slot * 32 + lane], v ? xk + soff : xk, v);
            if (UC) {  // the diagonal pair of the same column (padded records: always in range)
                const bool vd = idx < nsteps;
                cp_async8s(&dring[stage_slot * 32 + lane], vd ? pd + doff : pd, vd);
            }
            ++sxc;
            soff += Ly;
            doff += lstep;
            if (per_x && sxc == Lx) {
                sxc = 0;
                soff -= (long long)Lx * Ly;
            }
            if (CMP) {  // the residual words of the column that step idx completes (xo < xb: idx < nsteps)
                const int xo = s0 + idx - K;
                const bool vr = wr && xo >= xa && xo < xb;
                cp_async8s(reinterpret_cast<float2*>(&rring[(idx & 3) * 32 + lane]), vr ? rbase + roff : D.comp, vr);
                roff += Ly;  // the next call stages column xo + 1 (its offset unwrapped: only [xa, xb) is read)
            }
            cp_async_commit_s();
            stage_slot = stage_slot + 1 == XS ? 0 : stage_slot + 1;
        };
#pragma unroll
        for (int i = 0; i < SPF; ++i) stage(i);

        // T_j of my sites, three columns per order 1 <= j < K (slot = producing step mod 3);
        // T_0 is read from the ket ring instead (W[0] stays unused)
        float2 W[K][3][2];
#pragma unroll
        for (int j = 1; j < K; ++j)
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) W[j][cc][0] = W[j][cc][1] = make_float2(0.f, 0.f);

        int xslot = 0;  // base mod XS: the ket-ring slot of column s0 + base
        long long xoff = (long long)(s0 - K) * Ly;  // column offset of this step's output column s - K
        int yslot = 0;  // idx mod YR
        for (int base = 0; base < nsteps; base += NP) {
            // ket-ring slots of the columns s0 + base - K .. s0 + base + NP - 1 (xslot holds
            // column s0 + base): column s - k of step p sits in xsl[p - k + K], so no order
            // wraps a slot index of its own
            int xsl[K + NP];
            {
                int v = xslot - K;
                if (v < 0) v += XS;  // K < XS
#pragma unroll
                for (int j = 0; j < K + NP; ++j) {
                    xsl[j] = v;
                    v = v + 1 == XS ? 0 : v + 1;
                }
            }
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                // window slots of the columns produced at this step, one and two steps ago
                const int c0 = ROT ? 0 : p, c1 = ROT ? 1 : (p + 2) % 3, c2 = ROT ? 2 : (p + 1) % 3;
                const int idx = base + p;
                const int s = s0 + idx;
                // the column records of column s (column s - k sits k records before)
                const float4* const cs = ctab + (s + kPadL) * stream_crec_f4(MODE);
                stage(idx + SPF);
                cp_async_wait_s<SPF>();  // the group of column idx has landed
                // ket ring slots of columns s-1 and s-2 (T_0 of order 1's x and x-1)
                const int xs1 = xsl[p - 1 + K];
                const int xs2 = xsl[p - 2 + K];
                const int ro = loff + (s + kPadL) * lstep;  // records of column s
#pragma unroll
                for (int k = 1; k <= K; ++k) {
                    const int x = s - k;
                    const int o = ro - k * lstep;
                    float2 hx[2], hxm[2], hy[2], hym[2];
                    float d[2];
                    if (UC) {
                        const float2 qd = dring[xsl[p - k + K] * 32 + lane];
                        d[0] = qd.x;
                        d[1] = qd.y;
                        // MODE 3 reads its paired records in the stencil below
                        const float4 qc = PAIRED ? make_float4(0.f, 0.f, 0.f, 0.f) : cs[-k];
                        hx[0] = hx[1] = make_float2(qc.x, 0.f);
                        hxm[0] = hxm[1] = make_float2(qc.y, 0.f);
                        hy[0] = make_float2(qc.z, qc.w);
                        hy[1] = (YEDGE && y_last) ? make_float2(0.f, 0.f) : hy[0];
                        hym[0] = (YEDGE && y_first) ? make_float2(0.f, 0.f) : make_float2(qc.z, -qc.w);
                        hym[1] = make_float2(qc.z, -qc.w);
                    } else if (BRICK && o >= 0) {
                        // brick planes: {h_AB, h_A,B(lane-1)}, {h_A,B(x-1), h_B,A(x+1)}, {h_B,A(lane+1), dA, dB}
                        const float4 q0 = __ldg(P0 + o), q1 = __ldg(P1 + o), q2 = __ldg(P2 + o);
                        hy[0] = make_float2(q0.x, q0.y);   // A -> B of the same cell (y + 1)
                        hym[1] = make_float2(q0.x, -q0.y); // B -> A of the same cell (y - 1)
                        hym[0] = make_float2(q0.z, q0.w);  // A -> B of the cell below (lane - 1)
                        hxm[0] = make_float2(q1.x, q1.y);  // A -> B of column x - 1
                        hx[1] = make_float2(q1.z, q1.w);   // B -> A of column x + 1
                        hy[1] = make_float2(q2.x, q2.y);   // B -> A of the cell above (lane + 1)
                        hx[0] = hxm[1] = make_float2(0.f, 0.f);
                        d[0] = q2.z;
                        d[1] = q2.w;
                    } else if (o >= 0) {
                        const float4 qy = __ldg(P3 + o), qd = __ldg(P4 + o);
                        hy[0] = make_float2(qy.x, qy.y);
                        hy[1] = make_float2(qy.z, qy.w);
                        hym[0] = make_float2(qd.x, qd.y);
                        hym[1] = make_float2(hy[0].x, -hy[0].y);
                        d[0] = qd.z;
                        d[1] = qd.w;
                        if (XR) {
                            const float4 q = __ldg(P0 + o);
                            hx[0] = make_float2(q.x, 0.f);
                            hx[1] = make_float2(q.y, 0.f);
                            hxm[0] = make_float2(q.z, 0.f);
                            hxm[1] = make_float2(q.w, 0.f);
                        } else {
                            const float4 q = __ldg(P1 + o), r = __ldg(P2 + o);
                            hx[0] = make_float2(q.x, q.y);
                            hx[1] = make_float2(q.z, q.w);
                            hxm[0] = make_float2(r.x, r.y);
                            hxm[1] = make_float2(r.z, r.w);
                        }
                    } else {
                        hx[0] = hx[1] = hxm[0] = hxm[1] = hy[0] = hy[1] = hym[0] = hym[1] = make_float2(0.f, 0.f);
                        d[0] = d[1] = 0.f;
                    }

                    // T_{k-1} at x+1 (this step), x and x-1
                    float2 tp[2], tc[2], tm[2];
                    if (k == 1) {
                        const float4 a = xring[xsl[p + K] * 32 + lane], b = xring[xs1 * 32 + lane], c = xring[xs2 * 32 + lane];
                        tp[0] = make_float2(a.x, a.y); tp[1] = make_float2(a.z, a.w);
                        tc[0] = make_float2(b.x, b.y); tc[1] = make_float2(b.z, b.w);
                        tm[0] = make_float2(c.x, c.y); tm[1] = make_float2(c.z, c.w);
                    } else {
                        tp[0] = W[k - 1][c0][0]; tp[1] = W[k - 1][c0][1];
                        tc[0] = W[k - 1][c1][0]; tc[1] = W[k - 1][c1][1];
                        tm[0] = W[k - 1][c2][0]; tm[1] = W[k - 1][c2][1];
                    }
                    float2 up, dn;  // y-1 of my first site, y+1 of my second
                    up.x = __shfl_up_sync(0xffffffffu, tc[1].x, 1);
                    up.y = __shfl_up_sync(0xffffffffu, tc[1].y, 1);
                    dn.x = __shfl_down_sync(0xffffffffu, tc[0].x, 1);
                    dn.y = __shfl_down_sync(0xffffffffu, tc[0].y, 1);
                    const float2 vyp[2] = {tc[1], dn};
                    const float2 vym[2] = {up, tc[0]};

                    float2 tk[2];
                    if (PAIRED) {
                        // signed records of column x: {h hx, h hx, h hxm, h hxm}, {h hy.re, h hy.re, h hy.im, 0}
                        const float4* cr = cs - 4 * k + ((k & 1) ? 0 : 2);
                        const float4 r0 = cr[0], r1 = cr[1];
                        const float2 px = make_float2(r0.x, r0.y), pxm = make_float2(r0.z, r0.w);
                        const float2 py = make_float2(r1.x, r1.y);
                        const float hyi = r1.z;
                        const float dd[2] = {(k & 1) ? d[0] : -d[0], (k & 1) ? d[1] : -d[1]};
#pragma unroll
                        for (int j = 0; j < 2; ++j) {
                            float2 acc = make_float2(0.f, 0.f);
                            if (k == 2) {  // S_0 = T_0(x): column s-2 of the ket ring
                                const float4 q = xring[xs2 * 32 + lane];
                                acc = j == 0 ? make_float2(q.x, q.y) : make_float2(q.z, q.w);
                            } else if (k > 2) {
                                acc = W[k - 2][c2][j];  // S_{k-2}(x)
                            }
                            acc = ffma2(px, tp[j], acc);
                            acc = ffma2(pxm, tm[j], acc);
                            acc = ffma2(py, vyp[j], acc);
                            acc.x = fmaf(-hyi, vyp[j].y, acc.x);
                            acc.y = fmaf(hyi, vyp[j].x, acc.y);
                            acc = ffma2(py, vym[j], acc);  // the conjugate hop: same real part
                            acc.x = fmaf(hyi, vym[j].y, acc.x);
                            acc.y = fmaf(-hyi, vym[j].x, acc.y);
                            acc.x = fmaf(dd[j], tc[j].x, acc.x);
                            acc.y = fmaf(dd[j], tc[j].y, acc.y);
                            if (k == 1) { acc.x *= 0.5f; acc.y *= 0.5f; }
                            tk[j] = acc;
                        }
                    } else
#pragma unroll
                    for (int j = 0; j < 2; ++j) {
                        float2 acc = make_float2(0.f, 0.f);
                        if (k == 2) {  // T_0(x) = column s-2 of the ket ring
                            const float4 q = xring[xs2 * 32 + lane];
                            const float2 t2 = j == 0 ? make_float2(q.x, q.y) : make_float2(q.z, q.w);
                            acc = make_float2(-t2.x, -t2.y);
                        } else if (k > 2) {
                            const float2 t2 = W[k - 2][c2][j];  // T_{k-2}(x)
                            acc = make_float2(-t2.x, -t2.y);
                        }
                        const float2 vxp = tp[j], vxm = tm[j];
                        if (BRICK) {  // A's x-neighbour is B of column x-1, B's is A of column x+1
                            const float2 hb = j == 0 ? hxm[0] : hx[1];
                            const float2 vb = j == 0 ? tm[1] : tp[0];
                            acc.x = fmaf(hb.x, vb.x, acc.x); acc.x = fmaf(-hb.y, vb.y, acc.x);
                            acc.y = fmaf(hb.x, vb.y, acc.y); acc.y = fmaf(hb.y, vb.x, acc.y);
                        } else if (XR) {
                            acc.x = fmaf(hx[j].x, vxp.x, acc.x);
                            acc.y = fmaf(hx[j].x, vxp.y, acc.y);
                            acc.x = fmaf(hxm[j].x, vxm.x, acc.x);
                            acc.y = fmaf(hxm[j].x, vxm.y, acc.y);
                        } else {
                            acc.x = fmaf(hx[j].x, vxp.x, acc.x); acc.x = fmaf(-hx[j].y, vxp.y, acc.x);
                            acc.y = fmaf(hx[j].x, vxp.y, acc.y); acc.y = fmaf(hx[j].y, vxp.x, acc.y);
                            acc.x = fmaf(hxm[j].x, vxm.x, acc.x); acc.x = fmaf(-hxm[j].y, vxm.y, acc.x);
                            acc.y = fmaf(hxm[j].x, vxm.y, acc.y); acc.y = fmaf(hxm[j].y, vxm.x, acc.y);
                        }
                        acc.x = fmaf(hy[j].x, vyp[j].x, acc.x); acc.x = fmaf(-hy[j].y, vyp[j].y, acc.x);
                        acc.y = fmaf(hy[j].x, vyp[j].y, acc.y); acc.y = fmaf(hy[j].y, vyp[j].x, acc.y);
                        acc.x = fmaf(hym[j].x, vym[j].x, acc.x); acc.x = fmaf(-hym[j].y, vym[j].y, acc.x);
                        acc.y = fmaf(hym[j].x, vym[j].y, acc.y); acc.y = fmaf(hym[j].y, vym[j].x, acc.y);
                        acc.x = fmaf(d[j], tc[j].x, acc.x);
                        acc.y = fmaf(d[j], tc[j].y, acc.y);
                        if (k == 1) { acc.x *= 0.5f; acc.y *= 0.5f; }  // tables hold 2H/a
                        tk[j] = acc;
                    }
                    if (k < K) {
                        W[k][c0][0] = tk[0];
                        W[k][c0][1] = tk[1];
                    }

                    // Accumulator y(x) = sum_k c_k T_k(x), added up in groups of AG orders when
                    // the last order e of a group has produced column x = s - e: T_j(x) of every
                    // order j <= e of the group is then still in its window (age e - j < AG <= 3).
                    // Each column gets the same FMAs in the same order as one update per order
                    // gives; the shared ring carries y(x) from one group to the next.
                    if (k % AG != 0 && k != K) continue;
                    const int gb = ((k - 1) / AG) * AG + 1;  // first order of the group
                    int ys_k = yslot - k;
                    if (ys_k < 0) ys_k += YR;
                    float4* yr = &yring[ys_k * 32 + lane];
                    // T_jj(x) (S_jj in the paired mode) for gb <= jj <= k
                    auto tval = [&](int jj, int j) -> float2 {
                        return jj == k ? tk[j] : (jj == k - 1 ? W[jj][c1][j] : W[jj][c2][j]);
                    };
                    float2 yv[2];
                    if (gb == 1) {  // y = -i s_1 T1 + g0 T0 + g1 T1
                        float2 t0[2] = {tc[0], tc[1]};  // T_0(s - 1): order 1's centre column
                        if (k > 1) {
                            const float4 q0 = xring[xsl[p - k + K] * 32 + lane];
                            t0[0] = make_float2(q0.x, q0.y);
                            t0[1] = make_float2(q0.z, q0.w);
                        }
                        const ChebLo lo = D.lo;
                        const float s1 = D.s[1];
#pragma unroll
                        for (int j = 0; j < 2; ++j) {
                            const float2 x0 = t0[j], t = tval(1, j);
                            const float lx = fmaf(lo.g0_re, x0.x, fmaf(-lo.g0_im, x0.y, fmaf(lo.g1_re, t.x, -lo.g1_im * t.y)));
                            const float ly = fmaf(lo.g0_re, x0.y, fmaf(lo.g0_im, x0.x, fmaf(lo.g1_re, t.y, lo.g1_im * t.x)));
                            yv[j].x = fmaf(s1, t.y, lx);
                            yv[j].y = fmaf(-s1, t.x, ly);
                        }
                    } else {
                        const float4 q = *yr;
                        yv[0] = make_float2(q.x, q.y);
                        yv[1] = make_float2(q.z, q.w);
                    }
#pragma unroll
                    for (int jj = (gb == 1 ? 2 : gb); jj <= k; ++jj) {
                        const float sk = D.s[jj];
#pragma unroll
                        for (int j = 0; j < 2; ++j) {
                            const float2 t = tval(jj, j);
                            if (PAIRED) {  // t = S_jj = sigma_jj T_jj
                                const float sks = (jj & 2) ? -sk : sk;
                                if (jj & 1) {
                                    yv[j].x = fmaf(sks, t.y, yv[j].x);
                                    yv[j].y = fmaf(-sks, t.x, yv[j].y);
                                } else {
                                    yv[j] = ffma2(SP.s2[jj], t, yv[j]);
                                }
                            } else if (jj & 1) {  // c_jj = -i s_jj
                                yv[j].x = fmaf(sk, t.y, yv[j].x);
                                yv[j].y = fmaf(-sk, t.x, yv[j].y);
                            } else {      // c_jj = s_jj
                                yv[j].x = fmaf(sk, t.x, yv[j].x);
                                yv[j].y = fmaf(sk, t.y, yv[j].y);
                            }
                        }
                    }
                    if (k < K) {
                        *yr = make_float4(yv[0].x, yv[0].y, yv[1].x, yv[1].y);
                    } else if (wr && x >= xa && x < xb) {
                        // x lies in [xa, xb), inside the lattice: its offset is xoff, unwrapped
                        // out = e^{-ib dt} y + a0 x (a0 = e^{-ib dt} c_0): the small terms first
                        const float4 q = xring[xsl[p] * 32 + lane];
                        const float2 x0[2] = {make_float2(q.x, q.y), make_float2(q.z, q.w)};
                        const float ph_re = D.ph_re, ph_im = D.ph_im, a0_re = D.a0_re, a0_im = D.a0_im;
                        float2 o[2];
                        if (CMP) {
                            // the two sites' residuals, staged with the ket columns
                            uint2* lp = reinterpret_cast<uint2*>(rbase + xoff);
                            const uint2 lq = rring[(idx & 3) * 32 + lane];
                            const float2 a1 = make_float2(a0_re, a0_re), a1n = make_float2(-a0_re, -a0_re);
                            const float2 a2 = make_float2(-a0_im, a0_im);
                            unsigned enc[2];
#pragma unroll
                            for (int j = 0; j < 2; ++j) {
                                const unsigned lw = j == 0 ? lq.x : lq.y;
                                const float lx = res_lo_x(lw), ly = res_lo_y(lw);
                                // the series and a0 l's cross term go with the small terms
                                const float rx = fmaf(-a0_im, ly, fmaf(ph_re, yv[j].x, -ph_im * yv[j].y));
                                const float ry = fmaf(a0_im, lx, fmaf(ph_re, yv[j].y, ph_im * yv[j].x));
                                float2 ol;
                                comp_sum2(a1, a1n, x0[j], a2, make_float2(x0[j].y, x0[j].x), make_float2(rx, ry),
                                          make_float2(lx, ly), o[j], ol);
                                enc[j] = res_encode(ol.x, ol.y);
                            }
                            *lp = make_uint2(enc[0], enc[1]);
                        } else {
#pragma unroll
                            for (int j = 0; j < 2; ++j) {
                                float2 r;
                                r.x = fmaf(ph_re, yv[j].x, -ph_im * yv[j].y);
                                r.y = fmaf(ph_re, yv[j].y, ph_im * yv[j].x);
                                r.x = fmaf(-a0_im, x0[j].y, r.x);
                                r.y = fmaf(a0_im, x0[j].x, r.y);
                                o[j].x = fmaf(a0_re, x0[j].x, r.x);
                                o[j].y = fmaf(a0_re, x0[j].y, r.y);
                            }
                        }
                        *reinterpret_cast<float4*>(outk + xoff + ys) = make_float4(o[0].x, o[0].y, o[1].x, o[1].y);
                    }
                }
                yslot = yslot + 1 == YR ? 0 : yslot + 1;
                xoff += Ly;
                if (ROT) {
#pragma unroll
                    for (int j = 1; j < K; ++j) {
                        W[j][2][0] = W[j][1][0]; W[j][2][1] = W[j][1][1];
                        W[j][1][0] = W[j][0][0]; W[j][1][1] = W[j][0][1];
                    }
                }
            }
            xslot += NP;  // NP < XS
            if (xslot >= XS) xslot -= XS;
        }
        cp_async_wait_s<0>();
        __syncwarp();  // the next item reuses this warp's rings
    }
}

bool stream_supported(const Geom& g, int K, int mode, const void* x, const void* out, int64_t ld) {
    // complex x-hops (MODE 0) leave registers for K <= 5; the brick stencil (MODE 4) has three
    // neighbours per site and fits K = 6
    return K >= 2 && K <= (mode >= 1 ? kStreamMaxK : kStreamMaxK - 1) && g.Ly % 2 == 0 && g.Lx >= 2 * K + 3 && g.N < ((int64_t)1 << 31) &&
           ld % 2 == 0 && ((uintptr_t)x & 15) == 0 && ((uintptr_t)out & 15) == 0;
}

static void pack_dims(const Geom& g, int* npair, int* Xp, long long* plane) {
    *npair = (int)(g.Ly / 2);
    *Xp = (int)g.Lx + kPadL + kPadR;
    *plane = (long long)(*Xp) * (*npair) + 1;
}

// Layout of the packed buffer (float4 units): kPlanes planes, the diagonal pairs (float2, one
// per record), the column records.
struct PackPtrs {
    float4* pk;
    float2* pd;
    float4* pc;
};
static size_t pack_f4(const Geom& g) {
    int npair, Xp;
    long long plane;
    pack_dims(g, &npair, &Xp, &plane);
    return (size_t)kPlanes * plane + (size_t)(plane + 1) / 2 + (size_t)Xp;
}
static PackPtrs pack_ptrs(float4* base, const Geom& g) {
    int npair, Xp;
    long long plane;
    pack_dims(g, &npair, &Xp, &plane);
    PackPtrs p;
    p.pk = base;
    p.pd = reinterpret_cast<float2*>(base + (size_t)kPlanes * plane);
    p.pc = base + (size_t)kPlanes * plane + (size_t)(plane + 1) / 2;
    return p;
}

int ensure_stream_pack(lm_solver* s, const Geom& g) {
    lm_ctx* ctx = s->ctx;
    int npair, Xp;
    long long plane;
    pack_dims(g, &npair, &Xp, &plane);
    const size_t need = pack_f4(g);
    if (s->spack_f4 != need) {
        if (s->d_spack) cudaFree(s->d_spack);
        s->d_spack = nullptr;
        s->spack_f4 = 0;
        s->spack_version = ~0ull;
        const cudaError_t e = cudaMalloc((void**)&s->d_spack, sizeof(float4) * need);
        if (e != cudaSuccess) {
            s->d_spack = nullptr;
            cudaGetLastError();
            return set_err(ctx, LM_ERR_OOM, "x-streaming coefficient planes: out of device memory");
        }
        s->spack_f4 = need;
    }
    if (s->spack_version == s->tab_version) return LM_OK;
    const long long n = plane;
    const unsigned grid = (unsigned)std::min<long long>((n + 255) / 256, 4096);
    const PackPtrs pp = pack_ptrs(s->d_spack, g);
    stream_pack_kernel<<<grid, 256, 0, ctx->stream>>>(g, s->d_hop2f, s->d_diag2f, pp.pk, pp.pd, pp.pc, npair, Xp,
                                                      plane);
    ctx->launches++;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return check_cuda(ctx, e, "x-streaming coefficient planes");
    s->spack_version = s->tab_version;
    return LM_OK;
}

// Honeycomb brick planes from the normalised ELL values: record (padded column xp, pair l) of
// plane q holds the values that `bmap` (5 ELL value indices per unit cell, -1 = no bond)
// names, periodic columns wrapped and open ones zero, plus the zero record at the end.
__global__ void brick_pack_kernel(int64_t Lx, int per_x, const int* __restrict__ bmap, const float2* __restrict__ v2f,
                                  const float* __restrict__ d2f, float4* __restrict__ pk, int npair, int Xp,
                                  long long plane) {
    const long long n = (long long)Xp * npair + 1;
    const float2 z = make_float2(0.f, 0.f);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float2 h[5] = {z, z, z, z, z};
        float dA = 0.f, dB = 0.f;
        if (i < n - 1) {
            const int xp = (int)(i / npair), l = (int)(i % npair);
            const int64_t x = (int64_t)xp - kPadL;
            const int xs = per_x ? wrap_mod(x, Lx) : ((x >= 0 && x < Lx) ? (int)x : -1);
            if (xs >= 0) {
                const long long cell = (long long)xs * npair + l;
#pragma unroll
                for (int q = 0; q < 5; ++q) {
                    const int e = bmap[cell * 5 + q];
                    if (e >= 0) h[q] = v2f[e];
                }
                dA = d2f[2 * cell];
                dB = d2f[2 * cell + 1];
            }
        }
        pk[i] = make_float4(h[0].x, h[0].y, h[1].x, h[1].y);
        pk[plane + i] = make_float4(h[2].x, h[2].y, h[3].x, h[3].y);
        pk[2 * plane + i] = make_float4(h[4].x, h[4].y, dA, dB);
    }
}

int ensure_brick_pack(lm_solver* s, const Geom& g, const int* d_bmap) {
    lm_ctx* ctx = s->ctx;
    int npair, Xp;
    long long plane;
    pack_dims(g, &npair, &Xp, &plane);
    const size_t need = pack_f4(g);
    if (s->spack_f4 != need) {
        if (s->d_spack) cudaFree(s->d_spack);
        s->d_spack = nullptr;
        s->spack_f4 = 0;
        const cudaError_t e = cudaMalloc((void**)&s->d_spack, sizeof(float4) * need);
        if (e != cudaSuccess) {
            s->d_spack = nullptr;
            cudaGetLastError();
            return set_err(ctx, LM_ERR_OOM, "brick coefficient planes: out of device memory");
        }
        s->spack_f4 = need;
        s->bpack_valid = 0;
    }
    s->spack_version = ~0ull;  // the square-lattice planes are no longer in the buffer
    if (s->bpack_valid) return LM_OK;
    const unsigned grid = (unsigned)std::min<long long>((plane + 255) / 256, 4096);
    brick_pack_kernel<<<grid, 256, 0, ctx->stream>>>(g.Lx, g.per_x, d_bmap, s->d_ev2f, s->d_ed2f, s->d_spack, npair, Xp,
                                                     plane);
    ctx->launches++;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return check_cuda(ctx, e, "brick coefficient planes");
    s->bpack_valid = 1;
    return LM_OK;
}

static int stream_smem_bytes(int K, int mode, int Xp, bool cmp = false) {
    const bool uc = mode == 2 || mode == 3;
    const int nw = stream_warps(K, mode, cmp);
    return nw * stream_ring_f4(K) * 16 + (uc ? nw * stream_dring_f4(K) * 16 + Xp * 16 * stream_crec_f4(mode) : 0) +
           (cmp ? nw * kResRing * 32 * 8 : 0);
}

bool stream_comp_supported(const Geom& g, int K, int mode) {
    int m = (mode == 2 && g.per_y) ? 3 : mode;
    if ((m == 2 || m == 3) && stream_smem_bytes(K, m, (int)g.Lx + kPadL + kPadR) > kStreamSmemMax) m = 1;  // as launched
    return stream_smem_bytes(K, m, (int)g.Lx + kPadL + kPadR, true) <= kStreamSmemMax;
}

template <int MODE, bool CMP>
static cudaError_t launch_stream_k(lm_ctx* ctx, int K, int grid, const FusedInst& d, const StreamPairs& sp,
                                   const float4* spack, int nty, long long ncols, long long nwarps) {
    int npair, Xp;
    long long plane;
    pack_dims(d.g, &npair, &Xp, &plane);
    const PackPtrs pp = pack_ptrs(const_cast<float4*>(spack), d.g);
    const unsigned long long bit = 1ull << (K + 8 * MODE);
    unsigned long long& attr = CMP ? ctx->stream_attr_comp : ctx->stream_attr;
    switch (K) {
#define LM_STREAM_CASE(KK)                                                                                       \
    case KK: {                                                                                                   \
        const int smem = stream_smem_bytes(KK, MODE, Xp, CMP);                                                   \
        if (!(attr & bit)) {                                                                                     \
            cudaError_t e = cudaFuncSetAttribute(cheb_stream_c32_kernel<KK, MODE, CMP>,                          \
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, kStreamSmemMax);   \
            if (e != cudaSuccess) return e;                                                                      \
            attr |= bit;                                                                                         \
        }                                                                                                        \
        cheb_stream_c32_kernel<KK, MODE, CMP><<<(unsigned)grid, stream_warps(KK, MODE, CMP) * 32, smem, ctx->stream>>>( \
            d, sp, pp.pk, pp.pd, pp.pc, npair, plane, nty, ncols, nwarps);                                           \
        return cudaGetLastError();                                                                               \
    }
        LM_STREAM_CASE(2) LM_STREAM_CASE(3) LM_STREAM_CASE(4) LM_STREAM_CASE(5) LM_STREAM_CASE(6)
#undef LM_STREAM_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

cudaError_t launch_cheb_stream_c32(lm_ctx* ctx, const FusedInst& d, int K, int mode, const float4* spack) {
    const int H = stream_halo(K);
    const int64_t nty = strip_count(d.g.Ly, d.g.per_y, H);
    const long long ncols = (long long)nty * d.M * d.g.Lx;
    if (ncols <= 0) return cudaSuccess;
    // one warp per SM slot, but at least 8K columns per warp (a share costs 2K extra steps
    // for every item it touches)
    int m = (mode == 2 && d.g.per_y) ? 3 : mode;
    if ((m == 2 || m == 3) && stream_smem_bytes(K, m, (int)d.g.Lx + kPadL + kPadR) > kStreamSmemMax) m = 1;  // very long x
    const int nw = stream_warps(K, m, d.comp != nullptr);
    const long long slots = (long long)(ctx->sm_count > 0 ? ctx->sm_count : 152) * nw;
    const long long nwarps = std::max<long long>(1, std::min<long long>(slots, ncols / (8 * K)));
    const int grid = (int)((nwarps + nw - 1) / nw);
    StreamPairs sp;
    for (int k = 0; k <= kStreamMaxK; ++k) {
        const float v = k <= K ? ((k & 2) ? -d.s[k] : d.s[k]) : 0.f;  // sigma_k s_k
        sp.s2[k] = make_float2(v, v);
    }
    cudaError_t e;
    if (d.comp) {  // compensated block (stream_comp_supported checked by the caller)
        e = m == 4   ? launch_stream_k<4, true>(ctx, K, grid, d, sp, spack, (int)nty, ncols, nwarps)
            : m == 3 ? launch_stream_k<3, true>(ctx, K, grid, d, sp, spack, (int)nty, ncols, nwarps)
            : m == 2 ? launch_stream_k<2, true>(ctx, K, grid, d, sp, spack, (int)nty, ncols, nwarps)
            : m == 1 ? launch_stream_k<1, true>(ctx, K, grid, d, sp, spack, (int)nty, ncols, nwarps)
                     : launch_stream_k<0, true>(ctx, K, grid, d, sp, spack, (int)nty, ncols, nwarps);
    } else {
        e = m == 4   ? launch_stream_k<4, false>(ctx, K, grid, d, sp, spack, (int)nty, ncols, nwarps)
            : m == 3 ? launch_stream_k<3, false>(ctx, K, grid, d, sp, spack, (int)nty, ncols, nwarps)
            : m == 2 ? launch_stream_k<2, false>(ctx, K, grid, d, sp, spack, (int)nty, ncols, nwarps)
            : m == 1 ? launch_stream_k<1, false>(ctx, K, grid, d, sp, spack, (int)nty, ncols, nwarps)
                     : launch_stream_k<0, false>(ctx, K, grid, d, sp, spack, (int)nty, ncols, nwarps);
    }
    ctx->launches++;
    ctx->stream_launches++;
    return e;
}

}  // namespace lmgpu
