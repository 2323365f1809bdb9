// Lattice-resident Chebyshev step (ComplexF32 recurrence) for a batch of small lattices.
//
// One launch applies  y = e^{-ib dt} sum_{k<=K} c_k T_k(H~) x  to every ket of every instance of
// a descriptor table.  The whole lattice of a ket stays on chip for the K orders: a thread
// holds a block of kResC columns x kResR consecutive rows in registers (T_{k-1}, T_{k-2}, the
// accumulator and the hops of its sites) and exchanges its block once per
// order through a double-buffered shared-memory copy of T_{k-1}.  Nothing is recomputed: the
// region form (lmgpu_fused.cu) recomputes a halo of K sites on every side of its 32 x 64 tiles,
// which on lattices of 16..96 sites per side is most of its work.
//
// A lattice of up to kResThreads blocks fits one CTA, and smaller ones share a CTA, G kets at a
// time (G thread groups of nbx * nby threads).  A lattice of up to 2 kResThreads blocks is split
// along x over a cluster of two CTAs: each holds a half of the block columns, and the threads
// of an edge column also write it into the halo column of the other CTA's exchange buffer
// (distributed shared memory) with st.async, which completes a transaction on that CTA's
// mbarrier for the buffer.  Per order a CTA barrier orders the exchange within a CTA, and only
// the threads that read a halo column wait on the mbarrier: no cluster-wide barrier and no
// memory fence per order.  Two buffers suffice: a thread writes the peer's halo of order k + 2
// only after it received the peer's edge of order k + 1, which the peer sends after reading
// that halo.  A cluster barrier per item orders the items.
//
// Exchange buffer, per parity and thread group: (nby + 2) rows of entries -- the block rows and
// a zero row on each side -- of (ncl + 2) entries -- the CTA's columns and a halo column on each
// side.  An entry (32 bytes) holds the kResR = 4 rows of a block row in one lattice column, two
// float4.  A row of entries is padded by 16 bytes to an odd number of 16-byte units, so that the
// 128-bit accesses of consecutive block rows (consecutive lanes) fall into distinct banks.  With
// this layout every column, row and neighbour offset of a thread's accesses is an immediate from
// three per-thread offsets.  Zero rows and the halo columns of an open axis are never written;
// periodic axes read wrapped entries (Lx a multiple of kResC, Ly of kResR).
//
// Per site the arithmetic is the region form's, operation for operation (the FMA order over
// the x+, x-, y+, y- neighbours and the diagonal, the first order, the accumulator and the
// output), so the two forms give bit-identical results.
//
// Work items are (instance, G kets), pulled from a global atomic counter.  A CTA keeps its
// instance's coefficients in registers across consecutive items of that instance, and stages
// the next item's kets global -> shared with cp.async while it computes the current one.
// Every barrier is reached by all threads of the CTA or cluster in the same sequence (the item
// sequence is fetched by one thread and broadcast, K is the launch's); a wait on an mbarrier
// phase gives up after a bounded number of polls, sets *err and carries on, so the kernel
// always ends and the host reports the error.
#include <cuda_runtime.h>

#include "lmgpu_internal.cuh"
#include "lmgpu_resident.cuh"

namespace lmgpu {

namespace {
constexpr int R = kResR;
constexpr int C = kResC;
constexpr int NT = kResThreads;
static_assert(R == 4, "an exchange entry holds the four rows of a block column as two float4");
constexpr int DESC_WORDS = (int)(sizeof(ResidentInst) / 4);
static_assert(sizeof(ResidentInst) % 4 == 0 && DESC_WORDS <= NT, "descriptor copy");
constexpr int CW = 7;                       // float4 words per thread of the coefficient table
constexpr int CTAB_BYTES = CW * NT * 16;
constexpr int STAGE_F2 = 12 * NT;           // float2 words per staging buffer: G * slab <= 12 G nbx nby
constexpr int STAGE_BYTES = 2 * STAGE_F2 * 8;
constexpr int SMEM_LIMIT = 227 * 1024;
constexpr int STATIC_RESERVE = 1024;        // the kernel's static shared memory (descriptors, items)
constexpr int EXCH_MAX = SMEM_LIMIT - STATIC_RESERVE - CTAB_BYTES - STAGE_BYTES;
}  // namespace

__device__ __forceinline__ unsigned res_cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// Barrier over every thread of the cluster; writes before it (own or the peer's shared memory)
// are visible after it.
__device__ __forceinline__ void res_cluster_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ unsigned res_map_peer(const void* p, unsigned peer) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(peer));
    return r;
}
__device__ __forceinline__ void res_st_peer_s64(unsigned a, long long v) {
    asm volatile("st.shared::cluster.s64 [%0], %1;" ::"r"(a), "l"(v) : "memory");
}
__device__ __forceinline__ void res_st_async_f4(unsigned a, float4 v, unsigned mbar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, [%5];"
                 ::"r"(a), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w), "r"(mbar) : "memory");
}
__device__ __forceinline__ void res_mbar_init(unsigned a) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(a) : "memory");
}
// The CTA's one arrival of a phase, announcing the bytes the peer's st.async will complete.
__device__ __forceinline__ void res_mbar_expect(unsigned a, unsigned bytes) {
    unsigned long long state;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;" : "=l"(state) : "r"(a), "r"(bytes) : "memory");
}
constexpr int kWaitPolls = 1 << 22;
__device__ __forceinline__ void res_mbar_wait(unsigned a, unsigned parity, unsigned long long* err) {
    for (int i = 0; i < kWaitPolls; ++i) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done) : "r"(a), "r"(parity) : "memory");
        if (done) return;
    }
    atomicOr(err, 1ull);
}
template <int CL>
__device__ __forceinline__ void res_sync() {
    if (CL == 2) res_cluster_sync();
    else __syncthreads();
}
// The item barrier in two halves: the arrival (release) right after an item's last order, so
// that it does not wait for the item's output stores, and the wait (acquire) before the next
// item; the CTA barrier after it publishes the staged kets within the CTA.
template <int CL>
__device__ __forceinline__ void res_arrive() {
    if (CL == 2) asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
template <int CL>
__device__ __forceinline__ void res_wait() {
    if (CL == 2) asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
    __syncthreads();
}
__device__ __forceinline__ void res_cp8(float2* dst, const float2* src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 8 : 0));
}
__device__ __forceinline__ void res_cp16(float2* dst, const float2* src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 16 : 0));
}
__device__ __forceinline__ void res_cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void res_cp_wait() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Shared-memory accesses by 32-bit shared-window address (ordered like memory operations).
__device__ __forceinline__ float4 res_lds4(unsigned a) {
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(a)
                 : "memory");
    return v;
}
__device__ __forceinline__ float2 res_lds2(unsigned a) {
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a) : "memory");
    return v;
}
__device__ __forceinline__ void res_sts4(unsigned a, float4 v) {
    asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(a), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}

__device__ __forceinline__ int res_find(const ResidentInst* __restrict__ table, int ninst, long long item) {
    int lo = 0, hi = ninst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&table[mid].item_begin) <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Columns of the lattice this CTA holds: [xs0, xs0 + ncols).
template <int CL>
__device__ __forceinline__ void res_columns(const ResidentInst& D, unsigned rank, int* xs0, int* ncols) {
    if (CL == 1 || rank == 0) {
        *xs0 = 0;
        *ncols = CL == 1 ? D.Lx : D.nbx0 * C;
    } else {
        *xs0 = D.nbx0 * C;
        *ncols = D.Lx - D.nbx0 * C;
    }
}

// A thread's block and its exchange-buffer offsets (bytes within one parity buffer).
struct ResMap {
    int on;           // the thread holds a block of the lattice
    int g;            // its thread group (ket of the item)
    int x0, y0;       // lattice coordinates of the block's first column and row
    unsigned eo;      // the block's entry in column c = 0 (the neighbour columns at -32 and +32 C)
    unsigned eb, et;  // the entry below (block row by - 1) / above (by + 1), column c = 0
    int wa, wb;       // halo entries that column 0 / column C-1 is also written to (-1: none); on a
                      // cluster they lie in the other CTA
    int hw;           // on a cluster: bit 0 / bit 1, the left / right halo column comes from the other CTA
};

template <int CL>
__device__ __forceinline__ void res_map(const ResidentInst& D, unsigned rank, int t, ResMap& m) {
    int u, bx_first, nb_r;
    if (CL == 1) {
        const int tpk = D.nbx * D.nby;
        m.g = t / tpk;
        u = t - m.g * tpk;
        bx_first = 0;
        nb_r = D.nbx;
        m.on = m.g < D.G;
    } else {
        m.g = 0;
        bx_first = rank ? D.nbx0 : 0;
        nb_r = rank ? D.nbx - D.nbx0 : D.nbx0;
        u = t;
        m.on = t < nb_r * D.nby;
    }
    if (!m.on) {
        m.g = 0;
        u = 0;
    }
    const int bxl = u / D.nby;
    const int by = u - bxl * D.nby;
    m.x0 = (bx_first + bxl) * C;
    m.y0 = by * R;
    const int gbase = m.g * D.gs;
    const int col = (bxl * C + 1) * 32;  // padded column of c = 0
    m.eo = (unsigned)(gbase + (by + 1) * D.rs + col);
    int byb = by - 1, byt = by + 1;
    if (D.per_y) {
        if (byb < 0) byb = D.nby - 1;
        if (byt >= D.nby) byt = 0;
    }
    m.eb = (unsigned)(gbase + (byb + 1) * D.rs + col);
    m.et = (unsigned)(gbase + (byt + 1) * D.rs + col);
    m.wa = -1;
    m.wb = -1;
    m.hw = 0;
    if (!m.on) return;
    const int row = gbase + (by + 1) * D.rs;
    if (CL == 1) {
        if (D.per_x) {
            if (m.x0 == 0) m.wa = row + (nb_r * C + 1) * 32;  // column 0 -> right halo
            if (m.x0 + C == D.Lx) m.wb = row;                 // column Lx-1 -> left halo
        }
    } else {
        const int ncl_peer = (rank ? D.nbx0 : D.nbx - D.nbx0) * C;
        if (rank == 0) {
            if (bxl == nb_r - 1) m.wb = row;                                 // last column -> peer's left halo
            if (D.per_x && bxl == 0) m.wa = row + (ncl_peer + 1) * 32;       // column 0 -> peer's right halo
            m.hw = (bxl == nb_r - 1 ? 2 : 0) | (D.per_x && bxl == 0 ? 1 : 0);
        } else {
            if (bxl == 0) m.wa = row + (ncl_peer + 1) * 32;                  // first column -> peer's right halo
            if (D.per_x && m.x0 + C == D.Lx) m.wb = row;                     // column Lx-1 -> peer's left halo
            m.hw = (bxl == 0 ? 1 : 0) | (D.per_x && bxl == nb_r - 1 ? 2 : 0);
        }
    }
}

// Instance set-up: zeroes the exchange buffers, maps the thread, loads the hops of its sites
// (registers), and its diagonal and the hops across its block's lower x and y edges (the
// per-thread table ct: words 0-1 the x-hops from column x0 - 1, 2-3 the y-hops from row
// y0 - 1, 4-6 the diagonal of columns 0-2).
template <int CL>
__device__ __forceinline__ void res_setup(const ResidentInst& D, unsigned rank, int t, float4* E, float4* ct,
                                          ResMap& m, float2 (&hx)[C][R], float2 (&hy)[C][R]) {
    const int n4 = 2 * D.G * D.gs / 16;
    for (int i = t; i < n4; i += NT) E[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    res_map<CL>(D, rank, t, m);
    const int Lx = D.Lx, Ly = D.Ly;
    const int64_t N = (int64_t)Lx * Ly;
#pragma unroll
    for (int c = 0; c < C; ++c)
#pragma unroll
        for (int j = 0; j < R; ++j) {
            const int x = m.x0 + c, y = m.y0 + j;
            const bool ok = m.on && x < Lx && y < Ly;
            const int64_t s = (int64_t)x * Ly + y;
            hx[c][j] = ok ? __ldg(D.hop2 + s) : make_float2(0.f, 0.f);
            hy[c][j] = ok ? __ldg(D.hop2 + N + s) : make_float2(0.f, 0.f);
        }
#pragma unroll
    for (int c = 0; c < C; ++c) {
        float dv[R];
#pragma unroll
        for (int j = 0; j < R; ++j) {
            const int x = m.x0 + c, y = m.y0 + j;
            dv[j] = (m.on && x < Lx && y < Ly) ? __ldg(D.diag2 + (int64_t)x * Ly + y) : 0.f;
        }
        ct[(4 + c) * NT] = make_float4(dv[0], dv[1], dv[2], dv[3]);
    }
    // conj of the x-hop from (x0 - 1, y0 + j) and of the y-hop from (x0 + c, y0 - 1)
    int xm = m.x0 - 1, ym = m.y0 - 1;
    if (xm < 0) xm = D.per_x ? Lx - 1 : -1;
    if (ym < 0) ym = D.per_y ? Ly - 1 : -1;
    float2 hxm[R], hym[C];
#pragma unroll
    for (int j = 0; j < R; ++j) {
        const int y = m.y0 + j;
        const bool ok = m.on && xm >= 0 && y < Ly;
        const float2 h = ok ? __ldg(D.hop2 + (int64_t)xm * Ly + y) : make_float2(0.f, 0.f);
        hxm[j] = make_float2(h.x, -h.y);
    }
#pragma unroll
    for (int c = 0; c < C; ++c) {
        const int x = m.x0 + c;
        const bool ok = m.on && ym >= 0 && x < Lx;
        const float2 h = ok ? __ldg(D.hop2 + N + (int64_t)x * Ly + ym) : make_float2(0.f, 0.f);
        hym[c] = make_float2(h.x, -h.y);
    }
    ct[0] = make_float4(hxm[0].x, hxm[0].y, hxm[1].x, hxm[1].y);
    ct[NT] = make_float4(hxm[2].x, hxm[2].y, hxm[3].x, hxm[3].y);
    ct[2 * NT] = make_float4(hym[0].x, hym[0].y, hym[1].x, hym[1].y);
    ct[3 * NT] = make_float4(hym[2].x, hym[2].y, 0.f, 0.f);
}

// Stages ket k0 + g (g < G, zeros past the last ket) of this CTA's columns into buf + g * slab.
template <int CL>
__device__ __forceinline__ void res_stage(float2* buf, const ResidentInst& D, unsigned rank, int64_t k0, int t) {
    int xs0, ncols;
    res_columns<CL>(D, rank, &xs0, &ncols);
    const int n = ncols * D.Ly;
    for (int g = 0; g < D.G; ++g) {
        const int64_t ket = k0 + g;
        const bool ok = ket < D.M;
        const float2* src = D.x + (ok ? ket * D.ld + (int64_t)xs0 * D.Ly : 0);
        float2* dst = buf + g * D.slab;
        if (D.vec) {  // site pairs: 16-byte aligned on both sides (even Ly, ld and slab)
            for (int s = 2 * t; s < n; s += 2 * NT) res_cp16(dst + s, ok ? src + s : D.x, ok);
        } else {
            for (int s = t; s < n; s += NT) res_cp8(dst + s, ok ? src + s : D.x, ok);
        }
    }
    res_cp_commit();
}

// Writes column c of the block (T_k) into the exchange buffer at shared address Ew, and into a
// halo entry when the column is an edge column (on a cluster: the peer CTA's buffer at cluster
// address peerEw, completing its bytes on the peer's mbarrier peerMb of that buffer).
template <int CL>
__device__ __forceinline__ void res_put(const float2 (&B)[C][R], int c, unsigned Ew, unsigned peerEw, unsigned peerMb,
                                        const ResMap& m) {
    const float4 v0 = make_float4(B[c][0].x, B[c][0].y, B[c][1].x, B[c][1].y);
    const float4 v1 = make_float4(B[c][2].x, B[c][2].y, B[c][3].x, B[c][3].y);
    res_sts4(Ew + m.eo + 32u * c, v0);
    res_sts4(Ew + m.eo + 32u * c + 16u, v1);
    const int w = c == 0 ? m.wa : (c == C - 1 ? m.wb : -1);
    if (w >= 0) {
        if (CL == 2) {
            res_st_async_f4(peerEw + (unsigned)w, v0, peerMb);
            res_st_async_f4(peerEw + (unsigned)w + 16u, v1, peerMb);
        } else {
            res_sts4(Ew + (unsigned)w, v0);
            res_sts4(Ew + (unsigned)w + 16u, v1);
        }
    }
}

// One order: B <- T_k = 2H~ T_{k-1} - T_{k-2} (A = T_{k-1}, B = T_{k-2} on entry; FIRST: A = T_0
// and T_1 = H~ T_0), Y += c_k T_k, and T_k into the exchange buffer when WR.  The operation
// order per site is the region form's.  On a cluster a thread that reads a halo column first
// waits for the phase `parity` of mbarrier mb (the buffer Er).
template <bool XR, bool FIRST, bool ODD, bool WR, int CL>
__device__ __forceinline__ void res_order(const float2 (&A)[C][R], float2 (&B)[C][R], float2 (&Y)[C][R],
                                          const float2 (&hx)[C][R], const float2 (&hy)[C][R], unsigned Er, unsigned Ew,
                                          unsigned peerEw, unsigned peerMb, unsigned ct, const ResMap& m,
                                          float sk, const ChebLo& lo, unsigned mb, unsigned parity,
                                          unsigned long long* err) {
    const unsigned ro = Er + m.eo, rb = Er + m.eb, rt = Er + m.et;
    // per column: the diagonal, the neighbours across the block's lower and upper y edges and
    // the y-hop from below; column c + 1's are loaded before column c is computed, so that
    // their latency overlaps the arithmetic (the exchange stores of column c come after)
    auto load_col = [&](int c, float4& dq, float2& bot, float2& top, float2& hym0) {
        dq = res_lds4(ct + (4u + c) * NT * 16u);
        bot = res_lds2(rb + 32u * c + 24u);  // row 3 of the block row below
        top = res_lds2(rt + 32u * c);        // row 0 of the block row above
        hym0 = res_lds2(ct + (c < 2 ? 2u : 3u) * NT * 16u + 8u * (c & 1));
    };
    float4 dqn;
    float2 botn, topn, hymn;
    if (CL == 2 && (m.hw & 1)) res_mbar_wait(mb, parity, err);
    load_col(0, dqn, botn, topn, hymn);
    float2 lft[R], hxm0[R], rgt[R];
    {
        const float4 l0 = res_lds4(ro - 32u), l1 = res_lds4(ro - 16u);
        lft[0] = make_float2(l0.x, l0.y);
        lft[1] = make_float2(l0.z, l0.w);
        lft[2] = make_float2(l1.x, l1.y);
        lft[3] = make_float2(l1.z, l1.w);
        const float4 e0 = res_lds4(ct), e1 = res_lds4(ct + NT * 16u);
        hxm0[0] = make_float2(e0.x, e0.y);
        hxm0[1] = make_float2(e0.z, e0.w);
        hxm0[2] = make_float2(e1.x, e1.y);
        hxm0[3] = make_float2(e1.z, e1.w);
    }
#pragma unroll
    for (int c = 0; c < C; ++c) {
        const float4 dq = dqn;
        const float2 bot = botn, top = topn, hym0 = hymn;
        const float d[R] = {dq.x, dq.y, dq.z, dq.w};
        if (c + 1 < C) {
            if (c + 1 == C - 1) {
                if (CL == 2 && m.hw == 2) res_mbar_wait(mb, parity, err);
                const float4 r0 = res_lds4(ro + 32u * C), r1 = res_lds4(ro + 32u * C + 16u);
                rgt[0] = make_float2(r0.x, r0.y);
                rgt[1] = make_float2(r0.z, r0.w);
                rgt[2] = make_float2(r1.x, r1.y);
                rgt[3] = make_float2(r1.z, r1.w);
            }
            load_col(c + 1, dqn, botn, topn, hymn);
        }
        // the stencil term by term over the column's R sites (R independent accumulation chains
        // side by side); per site the operation order is the region form's
        float2 acc[R];
#pragma unroll
        for (int j = 0; j < R; ++j) acc[j] = FIRST ? make_float2(0.f, 0.f) : make_float2(-B[c][j].x, -B[c][j].y);
#pragma unroll
        for (int j = 0; j < R; ++j) {  // x + 1
            const float2 vxp = c < C - 1 ? A[c + 1][j] : rgt[j];
            const float2 h = hx[c][j];
            if (XR) {
                acc[j].x = fmaf(h.x, vxp.x, acc[j].x);
                acc[j].y = fmaf(h.x, vxp.y, acc[j].y);
            } else {
                acc[j].x = fmaf(h.x, vxp.x, acc[j].x); acc[j].x = fmaf(-h.y, vxp.y, acc[j].x);
                acc[j].y = fmaf(h.x, vxp.y, acc[j].y); acc[j].y = fmaf(h.y, vxp.x, acc[j].y);
            }
        }
#pragma unroll
        for (int j = 0; j < R; ++j) {  // x - 1
            const float2 vxm = c > 0 ? A[c - 1][j] : lft[j];
            const float2 hxm = c > 0 ? make_float2(hx[c - 1][j].x, -hx[c - 1][j].y) : hxm0[j];
            if (XR) {
                acc[j].x = fmaf(hxm.x, vxm.x, acc[j].x);
                acc[j].y = fmaf(hxm.x, vxm.y, acc[j].y);
            } else {
                acc[j].x = fmaf(hxm.x, vxm.x, acc[j].x); acc[j].x = fmaf(-hxm.y, vxm.y, acc[j].x);
                acc[j].y = fmaf(hxm.x, vxm.y, acc[j].y); acc[j].y = fmaf(hxm.y, vxm.x, acc[j].y);
            }
        }
#pragma unroll
        for (int j = 0; j < R; ++j) {  // y + 1
            const float2 vyp = j < R - 1 ? A[c][j + 1] : top;
            const float2 v = hy[c][j];
            acc[j].x = fmaf(v.x, vyp.x, acc[j].x); acc[j].x = fmaf(-v.y, vyp.y, acc[j].x);
            acc[j].y = fmaf(v.x, vyp.y, acc[j].y); acc[j].y = fmaf(v.y, vyp.x, acc[j].y);
        }
#pragma unroll
        for (int j = 0; j < R; ++j) {  // y - 1
            const float2 vym = j > 0 ? A[c][j - 1] : bot;
            const float2 hym = j > 0 ? make_float2(hy[c][j - 1].x, -hy[c][j - 1].y) : hym0;
            acc[j].x = fmaf(hym.x, vym.x, acc[j].x); acc[j].x = fmaf(-hym.y, vym.y, acc[j].x);
            acc[j].y = fmaf(hym.x, vym.y, acc[j].y); acc[j].y = fmaf(hym.y, vym.x, acc[j].y);
        }
#pragma unroll
        for (int j = 0; j < R; ++j) {  // diagonal, the first order's 1/2, the accumulator
            acc[j].x = fmaf(d[j], A[c][j].x, acc[j].x);
            acc[j].y = fmaf(d[j], A[c][j].y, acc[j].y);
            if (FIRST) {  // the tables hold 2H/a
                acc[j].x *= 0.5f;
                acc[j].y *= 0.5f;
            }
            const float2 x = A[c][j];  // T_0 when FIRST
            const float2 a = acc[j];
            B[c][j] = a;
            if (FIRST) {  // y = -i s_1 T1 + g0 T0 + g1 T1
                const float lx = fmaf(lo.g0_re, x.x, fmaf(-lo.g0_im, x.y, fmaf(lo.g1_re, a.x, -lo.g1_im * a.y)));
                const float ly = fmaf(lo.g0_re, x.y, fmaf(lo.g0_im, x.x, fmaf(lo.g1_re, a.y, lo.g1_im * a.x)));
                Y[c][j].x = fmaf(sk, a.y, lx);
                Y[c][j].y = fmaf(-sk, a.x, ly);
            } else if (ODD) {  // c_k = -i s_k
                Y[c][j].x = fmaf(sk, a.y, Y[c][j].x);
                Y[c][j].y = fmaf(-sk, a.x, Y[c][j].y);
            } else {  // c_k = s_k
                Y[c][j].x = fmaf(sk, a.x, Y[c][j].x);
                Y[c][j].y = fmaf(sk, a.y, Y[c][j].y);
            }
        }
        if (WR) res_put<CL>(B, c, Ew, peerEw, peerMb, m);
    }
}

template <bool XR, int CL>
__global__ void __launch_bounds__(NT, 1)
cheb_resident_c32_kernel(const ResidentInst* __restrict__ table, int ninst, long long nitems,
                         unsigned long long* queue, unsigned long long* err, int K) {
    extern __shared__ float4 smem[];
    __shared__ ResidentInst s_desc[2];
    __shared__ long long s_item[2];
    __shared__ __align__(8) unsigned long long s_mbar[2];  // cluster: per exchange buffer
    const int t = threadIdx.x;
    const unsigned rank = CL == 2 ? res_cluster_rank() : 0u;
    const unsigned peer = rank ^ 1u;
    float4* const ct = smem + t;  // this thread's edge coefficients (CW words, stride NT)
    float2* const stage = reinterpret_cast<float2*>(smem + CW * NT);
    float4* const E = smem + CW * NT + STAGE_F2;  // two staging buffers of STAGE_F2 float2
    const unsigned Es = (unsigned)__cvta_generic_to_shared(E);
    const unsigned cts = (unsigned)__cvta_generic_to_shared(ct);
    const unsigned peerE = CL == 2 ? res_map_peer(E, peer) : 0u;
    unsigned mb_loc[2] = {0u, 0u}, mb_peer[2] = {0u, 0u};
    if (CL == 2) {
        for (int b = 0; b < 2; ++b) {
            mb_loc[b] = (unsigned)__cvta_generic_to_shared(&s_mbar[b]);
            mb_peer[b] = res_map_peer(&s_mbar[b], peer);
        }
        if (t == 0) {
            res_mbar_init(mb_loc[0]);
            res_mbar_init(mb_loc[1]);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
    }
    unsigned ph = 0;  // bit b: parity of the next phase of mbarrier b

    // next item id: one thread of the cluster takes it from the queue and broadcasts it
    auto fetch = [&](int slot) {
        const long long v = (long long)atomicAdd(queue, 1ull);
        s_item[slot] = v;
        if (CL == 2) res_st_peer_s64(res_map_peer(&s_item[slot], peer), v);
    };
    auto load_desc = [&](int slot, long long it) {
        const ResidentInst* src = &table[res_find(table, ninst, it)];
        if (t < DESC_WORDS) reinterpret_cast<int*>(&s_desc[slot])[t] = __ldg(reinterpret_cast<const int*>(src) + t);
    };

    if (t == 0 && rank == 0) {
        fetch(0);
        fetch(1);
    }
    res_sync<CL>();
    long long item = s_item[0];
    if (item >= nitems) return;  // the same for every CTA of the cluster
    int nslot = 1, dslot = 0;
    load_desc(0, item);
    __syncthreads();

    ResMap m;
    float2 hx[C][R], hy[C][R];
    res_setup<CL>(s_desc[0], rank, t, E, ct, m, hx, hy);
    res_stage<CL>(stage, s_desc[0], rank, (item - s_desc[0].item_begin) * s_desc[0].G, t);
    res_arrive<CL>();  // the buffers are zeroed before the other CTA writes into them
    int sb = 0;

    while (true) {
        const ResidentInst& D = s_desc[dslot];
        const unsigned par = (unsigned)(D.G * D.gs);  // bytes per parity buffer
        const int64_t k0 = (item - D.item_begin) * D.G;
        int xs0, ncols;
        res_columns<CL>(D, rank, &xs0, &ncols);
        res_cp_wait();
        res_wait<CL>();  // staged kets visible; every thread of the cluster is done with the previous item

        const bool live = m.on && k0 + m.g < D.M;
        const float2* st = stage + sb * STAGE_F2 + m.g * D.slab;
        float2 A[C][R], B[C][R], Y[C][R];
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const int x = m.x0 + c;
            if (D.vec) {  // even Ly: a site pair lies in the lattice or outside it as a whole
#pragma unroll
                for (int h = 0; h < R / 2; ++h) {
                    const int y = m.y0 + 2 * h;
                    float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (m.on && x < D.Lx && y < D.Ly) q = *reinterpret_cast<const float4*>(st + (x - xs0) * D.Ly + y);
                    A[c][2 * h] = make_float2(q.x, q.y);
                    A[c][2 * h + 1] = make_float2(q.z, q.w);
                }
            } else {
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    const int y = m.y0 + j;
                    A[c][j] = (m.on && x < D.Lx && y < D.Ly) ? st[(x - xs0) * D.Ly + y] : make_float2(0.f, 0.f);
                }
            }
            if (live) res_put<CL>(A, c, Es, peerE, mb_peer[0], m);
        }

        // the next item: its descriptor (another instance) and its kets into the other buffer
        const long long nxt = s_item[nslot];
        const bool have_next = nxt < nitems;
        const bool same = have_next && nxt < D.item_end;
        if (have_next) {
            if (!same) load_desc(dslot ^ 1, nxt);
            if (t == 0 && rank == 0) fetch(nslot ^ 1);
            nslot ^= 1;
            if (!same) __syncthreads();  // the next descriptor is visible in this CTA
            const ResidentInst& Dn = same ? D : s_desc[dslot ^ 1];
            res_stage<CL>(stage + (sb ^ 1) * STAGE_F2, Dn, rank, (nxt - Dn.item_begin) * Dn.G, t);
        }
        // per order: the CTA barrier orders the exchange within the CTA; on a cluster one thread
        // arrives on the mbarrier of the written buffer with the bytes the peer sends into it
        const unsigned xbytes = CL == 2 ? (D.per_x ? 2u : 1u) * (unsigned)D.nby * 32u : 0u;
        auto xdone = [&](int b) {
            __syncthreads();
            if (CL == 2 && t == 0) res_mbar_expect(mb_loc[b], xbytes);
        };
        const unsigned E1 = Es + par, pE1 = peerE + par;
#define LM_RES_ORDER(FI, OD, WR, AA, BB, ER, EW, PEW, PMB, SK, MB, PAR) \
    if (live) res_order<XR, FI, OD, WR, CL>(AA, BB, Y, hx, hy, ER, EW, PEW, PMB, cts, m, SK, D.lo, MB, PAR, err)
        // orders k (even): T_{k-1} in B and buffer 1 -> T_k in A and buffer 0; k (odd, k > 1): T_{k-1}
        // in A and buffer 0 -> T_k in B and buffer 1; the last order writes no buffer
        xdone(0);  // T_0 in buffer 0
        LM_RES_ORDER(true, true, true, A, B, Es, E1, pE1, mb_peer[1], D.s[1], mb_loc[0], ph & 1u);
        ph ^= 1u;
        xdone(1);
        int k = 2;
        for (; k + 1 < K; k += 2) {
            LM_RES_ORDER(false, false, true, B, A, E1, Es, peerE, mb_peer[0], D.s[k], mb_loc[1], (ph >> 1) & 1u);
            ph ^= 2u;
            xdone(0);
            LM_RES_ORDER(false, true, true, A, B, Es, E1, pE1, mb_peer[1], D.s[k + 1], mb_loc[0], ph & 1u);
            ph ^= 1u;
            xdone(1);
        }
        if (k == K) {  // K even
            LM_RES_ORDER(false, false, false, B, A, E1, Es, peerE, mb_peer[0], D.s[k], mb_loc[1], (ph >> 1) & 1u);
            ph ^= 2u;
        } else {  // K odd: orders K - 1 and K
            LM_RES_ORDER(false, false, true, B, A, E1, Es, peerE, mb_peer[0], D.s[k], mb_loc[1], (ph >> 1) & 1u);
            ph ^= 2u;
            xdone(0);
            LM_RES_ORDER(false, true, false, A, B, Es, E1, pE1, mb_peer[1], D.s[k + 1], mb_loc[0], ph & 1u);
            ph ^= 1u;
        }
#undef LM_RES_ORDER
        res_arrive<CL>();  // this item's reads of the exchange buffers are done

        // out = e^{-ib dt} y + a0 x (a0 = e^{-ib dt} c_0): the small terms first, the dominant one last
        if (live) {
            const float ph_re = D.ph_re, ph_im = D.ph_im, a0_re = D.a0_re, a0_im = D.a0_im;
            float2* outk = D.out + (k0 + m.g) * D.ld;
            auto out_site = [&](float2 yv, float2 x0) {
                float2 r;
                r.x = fmaf(ph_re, yv.x, -ph_im * yv.y);
                r.y = fmaf(ph_re, yv.y, ph_im * yv.x);
                r.x = fmaf(-a0_im, x0.y, r.x);
                r.y = fmaf(a0_im, x0.x, r.y);
                float2 o;
                o.x = fmaf(a0_re, x0.x, r.x);
                o.y = fmaf(a0_re, x0.y, r.y);
                return o;
            };
#pragma unroll
            for (int c = 0; c < C; ++c) {
                const int x = m.x0 + c;
                if (x >= D.Lx) continue;
                if (D.vec) {
#pragma unroll
                    for (int h = 0; h < R / 2; ++h) {
                        const int y = m.y0 + 2 * h;
                        if (y < D.Ly) {
                            const float4 q = *reinterpret_cast<const float4*>(st + (x - xs0) * D.Ly + y);
                            const float2 o0 = out_site(Y[c][2 * h], make_float2(q.x, q.y));
                            const float2 o1 = out_site(Y[c][2 * h + 1], make_float2(q.z, q.w));
                            *reinterpret_cast<float4*>(outk + (int64_t)x * D.Ly + y) = make_float4(o0.x, o0.y, o1.x, o1.y);
                        }
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < R; ++j) {
                        const int y = m.y0 + j;
                        if (y < D.Ly) outk[(int64_t)x * D.Ly + y] = out_site(Y[c][j], st[(x - xs0) * D.Ly + y]);
                    }
                }
            }
        }
        if (!have_next) break;
        if (!same) {
            res_wait<CL>();  // every thread of the cluster is done with this instance's exchange buffers
            dslot ^= 1;
            res_setup<CL>(s_desc[dslot], rank, t, E, ct, m, hx, hy);
            res_arrive<CL>();
        }
        item = nxt;
        sb ^= 1;
    }
    res_cp_wait();
    res_wait<CL>();  // the pending arrival: no CTA of the cluster exits while the other may still write into it
}

bool resident_plan(const Geom& g, int64_t m, ResidentInst& d, int* cl) {
    if (g.N >= ((int64_t)1 << 31) || g.Lx < 1 || g.Ly < 1 || m < 1) return false;
    if ((g.per_x && g.Lx % C) || (g.per_y && g.Ly % R)) return false;
    const int64_t nbx = (g.Lx + C - 1) / C, nby = (g.Ly + R - 1) / R;
    if (nby > NT) return false;
    d.Lx = (int)g.Lx;
    d.Ly = (int)g.Ly;
    d.per_x = g.per_x;
    d.per_y = g.per_y;
    d.nbx = (int)nbx;
    d.nby = (int)nby;
    // exchange buffer: 2 parities x G groups x (nby + 2) rows of (ncl + 2) 32-byte entries + 16
    auto row_bytes = [&](int64_t ncl) { return (ncl + 2) * 32 + 16; };
    auto exch_bytes = [&](int64_t G, int64_t ncl) { return 2 * G * (nby + 2) * row_bytes(ncl); };
    if (nbx * nby <= NT) {
        *cl = 1;
        d.nbx0 = (int)nbx;
        d.ncl = (int)(nbx * C);
        int64_t G = std::min<int64_t>(NT / (nbx * nby), m);
        while (G > 1 && exch_bytes(G, d.ncl) > EXCH_MAX) --G;
        if (exch_bytes(G, d.ncl) > EXCH_MAX) return false;
        d.G = (int)G;
    } else {
        const int64_t nbx0 = (nbx + 1) / 2;
        if (nbx0 * nby > NT) return false;
        *cl = 2;
        d.nbx0 = (int)nbx0;
        d.ncl = (int)(nbx0 * C);
        d.G = 1;
        if (exch_bytes(1, d.ncl) > EXCH_MAX) return false;
    }
    d.rs = (int)row_bytes(d.ncl);
    d.gs = (int)((nby + 2) * d.rs);
    d.slab = d.ncl * d.Ly;
    if ((int64_t)d.G * d.slab > STAGE_F2) return false;  // cannot happen: G slab <= 12 G nbx nby <= 12 NT
    d.smem = CTAB_BYTES + STAGE_BYTES + (int)exch_bytes(d.G, d.ncl);
    return true;
}

void resident_fill_coef(ResidentInst& d, int K, const ChebCoef* coef, double ph_re, double ph_im) {
    for (int k = 0; k <= kResMaxK; ++k) d.s[k] = k <= K ? (float)coef[k].s : 0.f;
    d.ph_re = (float)ph_re;
    d.ph_im = (float)ph_im;
    d.a0_re = (float)(ph_re * coef[0].s);
    d.a0_im = (float)(ph_im * coef[0].s);
    d.lo = cheb_lo(ph_re, ph_im, coef[0].s, coef[1].s, true);
}

template <bool XR, int CL>
static cudaError_t set_res_attr(lm_ctx* ctx) {
    const unsigned bit = 1u << (25 + (XR ? 1 : 0) + 2 * (CL - 1));
    if (ctx->fused_attr & bit) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(cheb_resident_c32_kernel<XR, CL>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_LIMIT - STATIC_RESERVE);
    if (e == cudaSuccess) ctx->fused_attr |= bit;
    return e;
}

cudaError_t ensure_resident_attr(lm_ctx* ctx, bool xreal, int cl) {
    if (cl == 1) return xreal ? set_res_attr<true, 1>(ctx) : set_res_attr<false, 1>(ctx);
    return xreal ? set_res_attr<true, 2>(ctx) : set_res_attr<false, 2>(ctx);
}

template <bool XR, int CL>
static cudaError_t launch_res(lm_ctx* ctx, const ResidentInst* d_table, int ninst, int64_t nitems,
                              unsigned long long* d_queue, unsigned long long* d_err, int K, int smem) {
    auto kern = cheb_resident_c32_kernel<XR, CL>;
    cudaError_t ea = set_res_attr<XR, CL>(ctx);
    if (ea != cudaSuccess) return ea;
    const int sms = ctx->sm_count > 0 ? ctx->sm_count : 152;
    int64_t grid = CL == 2 ? (sms / 2) * 2 : sms;
    const int64_t need = nitems * CL;
    if (grid > need) grid = need;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid, 1, 1);
    cfg.blockDim = dim3(NT, 1, 1);
    cfg.dynamicSmemBytes = (size_t)smem;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute attr[1];
    if (CL == 2) {
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = 2;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    }
    return cudaLaunchKernelEx(&cfg, kern, d_table, ninst, (long long)nitems, d_queue, d_err, K);
}

cudaError_t launch_resident_table(lm_ctx* ctx, int K, bool xreal, int cl, const ResidentInst* d_table, int ninst,
                                  int64_t nitems, unsigned long long* d_queue, unsigned long long* d_err, int smem) {
    if (nitems <= 0) return cudaSuccess;
    if (K < 2 || K > kResMaxK || smem > SMEM_LIMIT - STATIC_RESERVE || (cl != 1 && cl != 2)) return cudaErrorInvalidValue;
    cudaError_t e;
    if (cl == 1) e = xreal ? launch_res<true, 1>(ctx, d_table, ninst, nitems, d_queue, d_err, K, smem)
                           : launch_res<false, 1>(ctx, d_table, ninst, nitems, d_queue, d_err, K, smem);
    else e = xreal ? launch_res<true, 2>(ctx, d_table, ninst, nitems, d_queue, d_err, K, smem)
                   : launch_res<false, 2>(ctx, d_table, ninst, nitems, d_queue, d_err, K, smem);
    ctx->launches++;
    return e;
}

}  // namespace lmgpu
