// Batched evolution of many independent lattices of different sizes in the same launches.
//
// A batch holds (Hamiltonian, state) pairs: open or periodic square lattices of any size,
// each with its own field, on-site term and Chebyshev coefficients (its own spectral bounds),
// evolved with one common order K = max_i K_i (instances with smaller K_i simply keep their
// true higher coefficients).  One step is a fixed sequence of launches over flattened work
// items of all instances:
//
//   kets         : one pass  x -> U x
//   density P    : U P (columns), conjugate transpose, U (P U^dagger)   (= U P U^dagger)
//
// where a pass is either the temporally blocked launches (ComplexF32; items pulled from an
// atomic work queue per launch: lattices that fit on chip in the lattice-resident form, on one
// CTA or a cluster of two, for any K <= 40, the rest in the region form for K <= 8) or K
// launches of the per-order kernel over (instance, site block, ket group) items.  The step is captured once per buffer parity into a CUDA graph and
// replayed.  `lm_batch_tune` times the candidate pass shapes (orders per pass: all K in one
// launch or one per launch; kets per thread 2/4/8) on scratch copies and keeps the fastest.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "lmgpu_internal.cuh"
#include "lmgpu_resident.cuh"
#include "lmgpu_order.cuh"

namespace lmgpu {

constexpr int kBatchMaxK = 40;
// side of the out-of-place conjugate-transpose tiles: 64 for ComplexF32 (33 KB of shared memory),
// 32 for ComplexF64 (a 64-tile would exceed the static shared-memory limit)
constexpr int trans_tile(int precision) { return precision == LM_C64 ? 32 : 64; }

struct OrderInst {
    Geom g;
    const void* hop2;
    const void* diag2;
    void* S;  // T0 on entry; T_k for even k
    void* A;  // T_k for odd k
    void* Y;  // accumulator
    int64_t ld, M;
    int64_t item_begin;
    int64_t lane_blocks;  // ceil(N / 256)
    double s[kBatchMaxK + 1];
    double ph_re, ph_im;
    ChebLo lo;  // per-order-form second words (FP32)
};

struct TransInst {
    const void* in;
    void* out;
    int64_t n, ld;
    int64_t item_begin;
    int64_t tiles;  // tiles per dimension (trans_tile x trans_tile)
};

// Panelled batches: dst = src over n x m columns (an odd-K result moved back into place).
struct CopyInst {
    const void* src;
    void* dst;
    int64_t n, m, ld;
    int64_t item_begin;
    int64_t lane_blocks;  // ceil(n / 256)
};

// Panelled batches: P <- P^dagger in place, over the 32 x 32 tile pairs (ti <= tj).
struct IPTransInst {
    void* data;
    int64_t n, ld;
    int64_t item_begin;
    int64_t tiles;  // tiles per dimension
};

template <typename T>
__device__ __forceinline__ int find_item_owner(const T* __restrict__ table, int ninst, int64_t item) {
    int lo = 0, hi = ninst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&table[mid].item_begin) <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// One Chebyshev order k for every instance of the table (items: instance x 256-site block x
// INNER-ket group).
template <typename R, int INNER>
__global__ void __launch_bounds__(256) cheb_order_batch_kernel(const OrderInst* __restrict__ table, int ninst,
                                                               int64_t nitems, int k, int K) {
    typedef typename CT<R>::V V;
    for (int64_t item = blockIdx.x; item < nitems; item += gridDim.x) {
        const OrderInst& D = table[find_item_owner(table, ninst, item)];
        const int64_t local = item - D.item_begin;
        const int64_t lb = local % D.lane_blocks, grp = local / D.lane_blocks;
        const int64_t lane = lb * blockDim.x + threadIdx.x;
        const Geom g = D.g;
        const V* hop2 = (const V*)D.hop2;
        const R* diag2 = (const R*)D.diag2;
        V* S = (V*)D.S;
        V* A = (V*)D.A;
        V* Y = (V*)D.Y;
        const R c0 = (R)D.s[0], cs = (R)D.s[k], pr = (R)D.ph_re, pi = (R)D.ph_im;
        const int64_t g0 = grp * INNER, gs = (int64_t)1 << 62;  // one group per item
        if (k == 1)
            cheb_order_block<R, CHEB_FIRST, true, false, INNER>(g, hop2, diag2, S, A, Y, D.ld, D.M, c0, cs, 1, pr, pi, D.lo,
                                                                lane, g0, gs);
        else if (k < K)
            cheb_order_block<R, CHEB_MID, true, false, INNER>(g, hop2, diag2, (k & 1) ? S : A, (k & 1) ? A : S, Y,
                                                              D.ld, D.M, c0, cs, k & 1, pr, pi, D.lo, lane, g0, gs);
        else
            cheb_order_block<R, CHEB_LAST, true, false, INNER>(g, hop2, diag2, (k & 1) ? S : A, (k & 1) ? A : S, Y,
                                                               D.ld, D.M, c0, cs, k & 1, pr, pi, D.lo, lane, g0, gs);
    }
}

// out = in^dagger for every instance (32 x 32 tiles through shared memory).
// out = in^dagger per instance over TS x TS tiles (TS = 64: each warp access is a contiguous
// 512-byte run of a column on both sides).  A CTA's items increase, so the owning instance is
// found by a forward scan; the next tile's elements are loaded into registers before the current
// tile is written out, so that loads stay in flight while the CTA stores.
template <typename R, int TS>
__global__ void __launch_bounds__(256) transpose_conj_batch_kernel(const TransInst* __restrict__ table, int ninst,
                                                                   int64_t nitems) {
    typedef typename CT<R>::V V;
    constexpr int NJ = TS / 8;  // columns per thread (8 warps), TS / 32 elements per column
    constexpr int NI = TS / 32;
    __shared__ V tile[TS][TS + 1];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
    struct Tile {
        const V* in;
        V* out;
        int64_t n, ld, tr, tc;
    };
    int inst = 0;
    auto tile_of = [&](int64_t item) {
        while (inst + 1 < ninst && __ldg(&table[inst + 1].item_begin) <= item) ++inst;
        const TransInst& D = table[inst];
        const int64_t local = item - D.item_begin;
        Tile T;
        T.in = (const V*)D.in;
        T.out = (V*)D.out;
        T.n = D.n;
        T.ld = D.ld;
        T.tr = local / D.tiles;
        T.tc = local % D.tiles;
        return T;
    };
    auto load = [&](const Tile& T, V (&v)[NJ][NI]) {
#pragma unroll
        for (int j = 0; j < NJ; ++j)
#pragma unroll
            for (int i = 0; i < NI; ++i) {
                const int64_t r = T.tr * TS + tx + 32 * i, c = T.tc * TS + ty + 8 * j;
                if (r < T.n && c < T.n) v[j][i] = T.in[r + c * T.ld];
            }
    };
    int64_t item = blockIdx.x;
    if (item >= nitems) return;
    Tile cur = tile_of(item);
    V v[NJ][NI];
    load(cur, v);
    while (true) {
#pragma unroll
        for (int j = 0; j < NJ; ++j)
#pragma unroll
            for (int i = 0; i < NI; ++i) tile[ty + 8 * j][tx + 32 * i] = v[j][i];
        __syncthreads();
        const int64_t next = item + gridDim.x;
        const bool more = next < nitems;
        Tile nt;
        if (more) {
            nt = tile_of(next);
            load(nt, v);
        }
#pragma unroll
        for (int j = 0; j < NJ; ++j)
#pragma unroll
            for (int i = 0; i < NI; ++i) {
                const int64_t r2 = cur.tc * TS + tx + 32 * i, c2 = cur.tr * TS + ty + 8 * j;
                if (r2 < cur.n && c2 < cur.n) {
                    const V w = tile[tx + 32 * i][ty + 8 * j];
                    cur.out[r2 + c2 * cur.ld] = CT<R>::make(w.x, -w.y);
                }
            }
        __syncthreads();
        if (!more) break;
        cur = nt;
        item = next;
    }
}

template <typename R>
__global__ void __launch_bounds__(256) copy_batch_kernel(const CopyInst* __restrict__ table, int ninst,
                                                         int64_t nitems) {
    typedef typename CT<R>::V V;
    for (int64_t item = blockIdx.x; item < nitems; item += gridDim.x) {
        const CopyInst& D = table[find_item_owner(table, ninst, item)];
        const int64_t local = item - D.item_begin;
        const int64_t col = local / D.lane_blocks, row = (local % D.lane_blocks) * 256 + threadIdx.x;
        if (row < D.n) ((V*)D.dst)[col * D.ld + row] = ((const V*)D.src)[col * D.ld + row];
    }
}

// In place P <- P^dagger for every instance: an item swaps the tiles (ti, tj) and (tj, ti)
// (ti <= tj) through shared memory, conjugating both; a diagonal tile is transposed in place.
template <typename R>
__global__ void __launch_bounds__(256) transpose_conj_inplace_batch_kernel(const IPTransInst* __restrict__ table,
                                                                           int ninst, int64_t nitems) {
    typedef typename CT<R>::V V;
    __shared__ V ta[32][33], tb[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
    for (int64_t item = blockIdx.x; item < nitems; item += gridDim.x) {
        const IPTransInst& D = table[find_item_owner(table, ninst, item)];
        int64_t local = item - D.item_begin;
        int64_t ti = 0;
        while (local >= D.tiles - ti) {  // row ti holds the pairs (ti, ti .. tiles-1)
            local -= D.tiles - ti;
            ++ti;
        }
        const int64_t tj = ti + local;
        V* P = (V*)D.data;
        const int64_t n = D.n, ld = D.ld;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t c = ty + 8 * j;
            const int64_t ra = ti * 32 + tx, ca = tj * 32 + c;  // tile (ti, tj)
            if (ra < n && ca < n) ta[c][tx] = P[ra + ca * ld];
            const int64_t rb = tj * 32 + tx, cb = ti * 32 + c;  // tile (tj, ti)
            if (ti != tj && rb < n && cb < n) tb[c][tx] = P[rb + cb * ld];
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int64_t c = ty + 8 * j;
            // (P^dagger)[tj*32 + tx, ti*32 + c] = conj(P[ti*32 + c, tj*32 + tx]) = conj(ta[tx][c])
            const int64_t r1 = tj * 32 + tx, c1 = ti * 32 + c;
            if (r1 < n && c1 < n) {
                const V v = ta[tx][c];
                P[r1 + c1 * ld] = CT<R>::make(v.x, -v.y);
            }
            const int64_t r2 = ti * 32 + tx, c2 = tj * 32 + c;
            if (ti != tj && r2 < n && c2 < n) {
                const V v = tb[tx][c];
                P[r2 + c2 * ld] = CT<R>::make(v.x, -v.y);
            }
        }
        __syncthreads();
    }
}

}  // namespace lmgpu

using namespace lmgpu;

struct lm_batch {
    lm_ctx* ctx = nullptr;
    int kind = LM_KETS, precision = LM_C32;
    double tol = 1e-7;
    std::vector<lm_ham*> hams;
    std::vector<lm_state*> states;
    std::vector<lm_solver*> solvers;
    int valid = 0;
    double dt = 0.0;
    int K = 0;
    int cfg = -1;         // -1 auto; 0 fused; 1, 2, 3: per-order with 2, 4, 8 kets per thread
    int use_graph = 1;
    // host copies of the per-parity tables (parity p: S/A of every state swapped when p = 1)
    std::vector<FusedInst> hf[2];
    std::vector<OrderInst> ho1[2], ho2[2];
    std::vector<TransInst> ht[2];
    int64_t f_items = 0, o_items = 0, t_items = 0;  // f_items: the region form's (fused pass)
    // lattice-resident part of the fused pass, per parity and cluster size (index cl - 1)
    std::vector<ResidentInst> hr[2][2];
    ResidentInst* dr[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    size_t cap_r[2][2] = {{0, 0}, {0, 0}};
    int64_t r_items[2] = {0, 0};
    int r_smem[2] = {0, 0};
    int r_xreal = 0, f_xreal = 0;  // every instance of the resident / region part has real x-hops
    // device tables
    FusedInst* df[2] = {nullptr, nullptr};
    OrderInst* do1[2] = {nullptr, nullptr};
    OrderInst* do2[2] = {nullptr, nullptr};
    TransInst* dt_[2] = {nullptr, nullptr};
    size_t cap_f[2] = {0, 0}, cap_o1[2] = {0, 0}, cap_o2[2] = {0, 0}, cap_t[2] = {0, 0};
    unsigned long long* dqueue = nullptr;  // work-queue counters: 3 per pass (resident 1, 2, region);
                                           // dqueue[6]: error bits of the resident kernel
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int parity = 0;                         // 1: every state's data currently in its A buffer
    std::vector<void*> base_S, base_A;      // pointers at update time (parity 0)
    // panelled per-order path (lm_batch_set_panel): the recurrence runs on column panels of
    // width panel_w with per-instance panel scratch, in place on the states' data
    int64_t panel_w = 0;
    std::vector<void*> pa, py;              // per-instance panel scratch (A, Y)
    std::vector<size_t> pbytes;             // their sizes
    std::vector<OrderInst*> dpo;            // per panel: order table (device)
    std::vector<CopyInst*> dpc;             // per panel: copy-back table (device, odd K)
    std::vector<int> pn;                    // per panel: instances in the table
    std::vector<int64_t> po_items, pc_items;
    IPTransInst* dip = nullptr;
    int64_t ip_items = 0;
};

static void free_graphs(lm_batch* b) {
    for (int p = 0; p < 2; ++p)
        if (b->graph[p]) {
            cudaGraphExecDestroy(b->graph[p]);
            b->graph[p] = nullptr;
        }
}

static void free_tables(lm_batch* b) {
    for (int p = 0; p < 2; ++p) {
        if (b->df[p]) cudaFree(b->df[p]);
        if (b->do1[p]) cudaFree(b->do1[p]);
        if (b->do2[p]) cudaFree(b->do2[p]);
        if (b->dt_[p]) cudaFree(b->dt_[p]);
        for (int c = 0; c < 2; ++c) {
            if (b->dr[p][c]) cudaFree(b->dr[p][c]);
            b->dr[p][c] = nullptr;
            b->cap_r[p][c] = 0;
        }
        b->df[p] = nullptr;
        b->do1[p] = b->do2[p] = nullptr;
        b->dt_[p] = nullptr;
    }
    for (int p = 0; p < 2; ++p) b->cap_f[p] = b->cap_o1[p] = b->cap_o2[p] = b->cap_t[p] = 0;
}

static void free_panel(lm_batch* b) {
    for (void* q : b->pa) cudaFree(q);
    for (void* q : b->py) cudaFree(q);
    for (auto* t : b->dpo) cudaFree(t);
    for (auto* t : b->dpc) cudaFree(t);
    if (b->dip) cudaFree(b->dip);
    b->pa.clear();
    b->py.clear();
    b->pbytes.clear();
    b->dpo.clear();
    b->dpc.clear();
    b->pn.clear();
    b->po_items.clear();
    b->pc_items.clear();
    b->dip = nullptr;
    b->ip_items = 0;
}

static int inner_of(int cfg) { return cfg == 1 ? 2 : (cfg == 3 ? 8 : 4); }

// Whether instance i runs in the lattice-resident form (its cluster size in *cl).
static bool batch_resident(const lm_batch* b, size_t i, ResidentInst* d, int* cl) {
    if (!b->ctx->resident || b->precision != LM_C32 || b->K < 2 || b->K > kResMaxK) return false;
    ResidentInst tmp{};
    return resident_plan(b->hams[i]->lat->g, b->states[i]->m, d ? *d : tmp, cl);
}

static int batch_fused_ok(const lm_batch* b) {
    if (!b->ctx->fused || b->precision != LM_C32) return 0;
    for (size_t i = 0; i < b->hams.size(); ++i) {
        int cl = 0;
        if (batch_resident(b, i, nullptr, &cl)) continue;
        if (!fused_supported(b->precision, b->K) || !fused_supported_geom(b->hams[i]->lat->g)) return 0;
    }
    return 1;
}

template <typename T>
static int upload_table(lm_ctx* ctx, T** dptr, size_t* cap, const std::vector<T>& host) {
    const size_t need = std::max<size_t>(host.size(), 1) * sizeof(T);
    if (*cap < need) {
        if (*dptr) cudaFree(*dptr);
        *dptr = nullptr;
        *cap = 0;
        cudaError_t e = cudaMalloc((void**)dptr, need);
        if (e != cudaSuccess) {
            *dptr = nullptr;
            cudaGetLastError();
            return set_err(ctx, LM_ERR_OOM, "lm_batch: table allocation failed");
        }
        *cap = need;
    }
    if (!host.empty())
        return check_cuda(ctx, cudaMemcpyAsync(*dptr, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice,
                                               ctx->stream),
                          "lm_batch: table upload");
    return LM_OK;
}

// Builds every per-parity table for the current coefficients, pass shape and pointers.
static int build_tables(lm_batch* b) {
    lm_ctx* ctx = b->ctx;
    const size_t n = b->states.size();
    const int K = b->K;
    const int inner = inner_of(b->cfg);
    std::vector<std::vector<ChebCoef>> coefs(n);
    std::vector<double> J;
    for (size_t i = 0; i < n; ++i) {
        lm_solver* s = b->solvers[i];
        bessel_j_all(s->a * fabs(b->dt), K, J);
        make_coefs(J, K, b->dt >= 0 ? 1.0 : -1.0, coefs[i]);
    }
    for (int p = 0; p < 2; ++p) {
        b->hf[p].clear();
        b->hr[p][0].clear();
        b->hr[p][1].clear();
        b->ho1[p].assign(n, OrderInst{});
        b->ho2[p].assign(n, OrderInst{});
        b->ht[p].assign(n, TransInst{});
        int64_t fi = 0, oi = 0, ti = 0, ri[2] = {0, 0};
        int rsmem[2] = {0, 0};
        bool rxr = true, fxr = true;
        for (size_t i = 0; i < n; ++i) {
            lm_state* st = b->states[i];
            lm_solver* s = b->solvers[i];
            const Geom& g = b->hams[i]->lat->g;
            void* S = p ? b->base_A[i] : b->base_S[i];
            void* A = p ? b->base_S[i] : b->base_A[i];
            const bool f32 = b->precision == LM_C32;
            const void* hop2 = f32 ? (const void*)s->d_hop2f : (const void*)s->d_hop2;
            const void* diag2 = f32 ? (const void*)s->d_diag2f : (const void*)s->d_diag2;
            // fused tables (x = S -> out = A): the lattice-resident form where the lattice fits,
            // the region form otherwise
            ResidentInst rd{};
            int cl = 0;
            if (batch_resident(b, i, &rd, &cl)) {
                rd.hop2 = (const float2*)s->d_hop2f;
                rd.diag2 = s->d_diag2f;
                rd.x = (const float2*)S;
                rd.out = (float2*)A;
                rd.ld = st->ld;
                rd.M = st->m;
                rd.vec = g.Ly % 2 == 0 && st->ld % 2 == 0 && ((uintptr_t)S & 15) == 0 && ((uintptr_t)A & 15) == 0;
                rd.item_begin = ri[cl - 1];
                ri[cl - 1] += (st->m + rd.G - 1) / rd.G;
                rd.item_end = ri[cl - 1];
                resident_fill_coef(rd, K, coefs[i].data(), s->phase_re, s->phase_im);
                rsmem[cl - 1] = std::max(rsmem[cl - 1], rd.smem);
                rxr = rxr && ham_x_real(b->hams[i]);
                b->hr[p][cl - 1].push_back(rd);
            } else {
                FusedInst f{};
                f.g = g;
                f.hop2 = (const float2*)s->d_hop2f;
                f.diag2 = s->d_diag2f;
                f.x = (const float2*)S;
                f.out = (float2*)A;
                f.ld = st->ld;
                f.M = st->m;
                f.item_begin = fi;
                if (K <= kFusedMaxK) {
                    fi += fused_items(g, K, st->m, &f.ntx, &f.nty);
                    fused_fill_coef(f, K, coefs[i].data(), s->phase_re, s->phase_im);
                }
                fxr = fxr && ham_x_real(b->hams[i]);
                b->hf[p].push_back(f);
            }
            // per-order tables
            auto fill_order = [&](OrderInst& o, void* So, void* Ao) {
                o.g = g;
                o.hop2 = hop2;
                o.diag2 = diag2;
                o.S = So;
                o.A = Ao;
                o.Y = st->d_y;
                o.ld = st->ld;
                o.M = st->m;
                o.lane_blocks = (g.N + 255) / 256;
                for (int k = 0; k <= kBatchMaxK; ++k) o.s[k] = k <= K ? coefs[i][(size_t)k].s : 0.0;
                o.ph_re = s->phase_re;
                o.ph_im = s->phase_im;
                o.lo = cheb_lo(o.ph_re, o.ph_im, o.s[0], o.s[1], false);
            };
            OrderInst& o1 = b->ho1[p][i];
            fill_order(o1, S, A);
            o1.item_begin = oi;
            // second density pass: on the transposed block (K even: it sits in A; odd: in S)
            OrderInst& o2 = b->ho2[p][i];
            if (K % 2 == 0) fill_order(o2, A, S);
            else fill_order(o2, S, A);
            o2.item_begin = oi;
            oi += o1.lane_blocks * ((st->m + inner - 1) / inner);
            // transpose table: fused and odd K transpose A -> S, even K (per-order) S -> A
            TransInst& tr = b->ht[p][i];
            const bool fused_path = b->cfg == 0;
            const bool from_S = !fused_path && K % 2 == 0;
            tr.in = from_S ? S : A;
            tr.out = from_S ? A : S;
            tr.n = st->n;
            tr.ld = st->ld;
            tr.tiles = (st->n + trans_tile(b->precision) - 1) / trans_tile(b->precision);
            tr.item_begin = ti;
            ti += tr.tiles * tr.tiles;
        }
        b->f_items = fi;
        b->o_items = oi;
        b->t_items = ti;
        b->r_items[0] = ri[0];
        b->r_items[1] = ri[1];
        b->r_smem[0] = rsmem[0];
        b->r_smem[1] = rsmem[1];
        b->r_xreal = rxr;
        b->f_xreal = fxr;
        int rc = upload_table(ctx, &b->df[p], &b->cap_f[p], b->hf[p]);
        for (int c = 0; c < 2 && rc == LM_OK; ++c) rc = upload_table(ctx, &b->dr[p][c], &b->cap_r[p][c], b->hr[p][c]);
        if (rc == LM_OK) rc = upload_table(ctx, &b->do1[p], &b->cap_o1[p], b->ho1[p]);
        if (rc == LM_OK) rc = upload_table(ctx, &b->do2[p], &b->cap_o2[p], b->ho2[p]);
        if (rc == LM_OK) rc = upload_table(ctx, &b->dt_[p], &b->cap_t[p], b->ht[p]);
        if (rc != LM_OK) return rc;
    }
    return LM_OK;
}

template <typename T>
static int upload_new(lm_ctx* ctx, T** dptr, const std::vector<T>& host) {
    *dptr = nullptr;
    cudaError_t e = cudaMalloc((void**)dptr, std::max<size_t>(host.size(), 1) * sizeof(T));
    if (e == cudaSuccess && !host.empty())
        e = cudaMemcpy(*dptr, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(ctx, LM_ERR_OOM, "lm_batch: panel table allocation failed");
    }
    return LM_OK;
}

// Panelled per-order path: per-instance panel scratch (A, Y: n x min(w, m) each) and, per
// column panel q, an order table over the instances that still have columns there (S = the
// panel's columns of the state, in place), the copy-back table for odd K and the in-place
// transpose table.
static int build_panel_tables(lm_batch* b) {
    lm_ctx* ctx = b->ctx;
    const size_t n = b->states.size();
    const int K = b->K;
    const int inner = inner_of(b->cfg);
    const int64_t w = b->panel_w;
    std::vector<std::vector<ChebCoef>> coefs(n);
    std::vector<double> J;
    for (size_t i = 0; i < n; ++i) {
        bessel_j_all(b->solvers[i]->a * fabs(b->dt), K, J);
        make_coefs(J, K, b->dt >= 0 ? 1.0 : -1.0, coefs[i]);
    }
    // scratch: reuse when the sizes are unchanged
    std::vector<size_t> need(n);
    int64_t npanels = 0;
    for (size_t i = 0; i < n; ++i) {
        const lm_state* st = b->states[i];
        need[i] = st->elem * (size_t)st->ld * (size_t)std::min<int64_t>(w, st->m);
        npanels = std::max<int64_t>(npanels, (st->m + w - 1) / w);
    }
    if (b->pbytes != need) {
        free_panel(b);
        b->pa.assign(n, nullptr);
        b->py.assign(n, nullptr);
        for (size_t i = 0; i < n; ++i) {
            cudaError_t e = cudaMalloc(&b->pa[i], need[i]);
            if (e == cudaSuccess) e = cudaMalloc(&b->py[i], need[i]);
            if (e != cudaSuccess) {
                cudaGetLastError();
                free_panel(b);
                return set_err(ctx, LM_ERR_OOM, "lm_batch: panel scratch allocation failed");
            }
        }
        b->pbytes = need;
    } else {
        for (auto* t : b->dpo) cudaFree(t);
        for (auto* t : b->dpc) cudaFree(t);
        if (b->dip) cudaFree(b->dip);
        b->dpo.clear();
        b->dpc.clear();
        b->dip = nullptr;
    }
    b->pn.clear();
    b->po_items.clear();
    b->pc_items.clear();
    const bool f32 = b->precision == LM_C32;
    for (int64_t q = 0; q < npanels; ++q) {
        std::vector<OrderInst> ot;
        std::vector<CopyInst> ct;
        int64_t oi = 0, ci = 0;
        for (size_t i = 0; i < n; ++i) {
            lm_state* st = b->states[i];
            if (st->m <= q * w) continue;
            const int64_t cols = std::min<int64_t>(w, st->m - q * w);
            lm_solver* sv = b->solvers[i];
            const Geom& g = b->hams[i]->lat->g;
            void* S = (unsigned char*)st->d_data + st->elem * (size_t)st->ld * (size_t)(q * w);
            OrderInst o{};
            o.g = g;
            o.hop2 = f32 ? (const void*)sv->d_hop2f : (const void*)sv->d_hop2;
            o.diag2 = f32 ? (const void*)sv->d_diag2f : (const void*)sv->d_diag2;
            o.S = S;
            o.A = b->pa[i];
            o.Y = b->py[i];
            o.ld = st->ld;
            o.M = cols;
            o.lane_blocks = (g.N + 255) / 256;
            for (int k = 0; k <= kBatchMaxK; ++k) o.s[k] = k <= K ? coefs[i][(size_t)k].s : 0.0;
            o.ph_re = sv->phase_re;
            o.ph_im = sv->phase_im;
            o.lo = cheb_lo(o.ph_re, o.ph_im, o.s[0], o.s[1], false);
            o.item_begin = oi;
            oi += o.lane_blocks * ((cols + inner - 1) / inner);
            ot.push_back(o);
            CopyInst c{};
            c.src = b->pa[i];
            c.dst = S;
            c.n = st->n;
            c.m = cols;
            c.ld = st->ld;
            c.lane_blocks = (st->n + 255) / 256;
            c.item_begin = ci;
            ci += c.lane_blocks * cols;
            ct.push_back(c);
        }
        OrderInst* d1 = nullptr;
        CopyInst* d2 = nullptr;
        int rc = upload_new(ctx, &d1, ot);
        if (rc == LM_OK) rc = upload_new(ctx, &d2, ct);
        b->dpo.push_back(d1);
        b->dpc.push_back(d2);
        if (rc != LM_OK) return rc;
        b->pn.push_back((int)ot.size());
        b->po_items.push_back(oi);
        b->pc_items.push_back(ci);
    }
    std::vector<IPTransInst> it(n);
    int64_t ti = 0;
    for (size_t i = 0; i < n; ++i) {
        const lm_state* st = b->states[i];
        it[i].data = st->d_data;
        it[i].n = st->n;
        it[i].ld = st->ld;
        it[i].tiles = (st->n + 31) / 32;
        it[i].item_begin = ti;
        ti += it[i].tiles * (it[i].tiles + 1) / 2;
    }
    b->ip_items = b->kind == LM_DENSITY ? ti : 0;
    return upload_new(ctx, &b->dip, it);
}

static int grid_for(lm_ctx* ctx, int64_t items, int per_sm) {
    int64_t g = (int64_t)(ctx->sm_count > 0 ? ctx->sm_count : 152) * per_sm;
    if (g > items) g = items;
    if (g < 1) g = 1;
    return (int)g;
}

static cudaError_t launch_order_pass(lm_batch* b, const OrderInst* table, int n, int64_t items) {
    lm_ctx* ctx = b->ctx;
    if (items <= 0) return cudaSuccess;
    const int grid = grid_for(ctx, items, 8);
    const int inner = inner_of(b->cfg);
    for (int k = 1; k <= b->K; ++k) {
        if (b->precision == LM_C64) {
            if (inner == 2) cheb_order_batch_kernel<double, 2><<<grid, 256, 0, ctx->stream>>>(table, n, items, k, b->K);
            else if (inner == 8) cheb_order_batch_kernel<double, 8><<<grid, 256, 0, ctx->stream>>>(table, n, items, k, b->K);
            else cheb_order_batch_kernel<double, 4><<<grid, 256, 0, ctx->stream>>>(table, n, items, k, b->K);
        } else {
            if (inner == 2) cheb_order_batch_kernel<float, 2><<<grid, 256, 0, ctx->stream>>>(table, n, items, k, b->K);
            else if (inner == 8) cheb_order_batch_kernel<float, 8><<<grid, 256, 0, ctx->stream>>>(table, n, items, k, b->K);
            else cheb_order_batch_kernel<float, 4><<<grid, 256, 0, ctx->stream>>>(table, n, items, k, b->K);
        }
        ctx->launches++;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

static cudaError_t launch_transpose(lm_batch* b, const TransInst* table) {
    lm_ctx* ctx = b->ctx;
    const int n = (int)b->states.size();
    const int grid = grid_for(ctx, b->t_items, 8);
    if (b->precision == LM_C64)
        transpose_conj_batch_kernel<double, trans_tile(LM_C64)><<<grid, 256, 0, ctx->stream>>>(table, n, b->t_items);
    else
        transpose_conj_batch_kernel<float, trans_tile(LM_C32)><<<grid, 256, 0, ctx->stream>>>(table, n, b->t_items);
    ctx->launches++;
    return cudaGetLastError();
}

static cudaError_t launch_fused_pass(lm_batch* b, int p, int q) {
    lm_ctx* ctx = b->ctx;
    unsigned long long* qc = b->dqueue + 3 * q;
    cudaError_t e = cudaMemsetAsync(qc, 0, 3 * sizeof(unsigned long long), ctx->stream);
    for (int c = 0; c < 2 && e == cudaSuccess; ++c)
        if (b->r_items[c] > 0)
            e = launch_resident_table(ctx, b->K, b->r_xreal, c + 1, b->dr[p][c], (int)b->hr[p][c].size(),
                                      b->r_items[c], qc + c, b->dqueue + 6, b->r_smem[c]);
    if (e == cudaSuccess && b->f_items > 0)
        e = launch_fused_table(ctx, b->K, b->f_xreal, nullptr, b->df[p], (int)b->hf[p].size(), b->f_items, qc + 2,
                               0);
    return e;
}

// Panelled step: per pass, every column panel runs the K orders in place (an odd-K result is
// copied back from the panel scratch); a density matrix takes an in-place X <- X^dagger
// between its two passes (U P U^dagger = U (U P)^dagger for Hermitian P), as the full-buffer
// path does.
static cudaError_t enqueue_step_panel(lm_batch* b) {
    lm_ctx* ctx = b->ctx;
    const int passes = b->kind == LM_DENSITY ? 2 : 1;
    for (int pass = 0; pass < passes; ++pass) {
        for (size_t q = 0; q < b->dpo.size(); ++q) {
            cudaError_t e = launch_order_pass(b, b->dpo[q], b->pn[q], b->po_items[q]);
            if (e != cudaSuccess) return e;
            if (b->K % 2 == 1 && b->pc_items[q] > 0) {
                const int grid = grid_for(ctx, b->pc_items[q], 8);
                if (b->precision == LM_C64)
                    copy_batch_kernel<double><<<grid, 256, 0, ctx->stream>>>(b->dpc[q], b->pn[q], b->pc_items[q]);
                else
                    copy_batch_kernel<float><<<grid, 256, 0, ctx->stream>>>(b->dpc[q], b->pn[q], b->pc_items[q]);
                ctx->launches++;
                e = cudaGetLastError();
                if (e != cudaSuccess) return e;
            }
        }
        if (b->kind == LM_DENSITY && pass == 0) {
            const int grid = grid_for(ctx, b->ip_items, 8);
            const int n = (int)b->states.size();
            if (b->precision == LM_C64)
                transpose_conj_inplace_batch_kernel<double><<<grid, 256, 0, ctx->stream>>>(b->dip, n, b->ip_items);
            else
                transpose_conj_inplace_batch_kernel<float><<<grid, 256, 0, ctx->stream>>>(b->dip, n, b->ip_items);
            ctx->launches++;
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return e;
        }
    }
    return cudaSuccess;
}

// Enqueues one step for parity p; returns whether the data moves to the other buffer.
static cudaError_t enqueue_step(lm_batch* b, int p, int* moved) {
    cudaError_t e = cudaSuccess;
    if (b->panel_w > 0) {
        *moved = 0;
        return enqueue_step_panel(b);
    }
    if (b->cfg == 0) {
        e = launch_fused_pass(b, p, 0);
        if (e == cudaSuccess && b->kind == LM_DENSITY) {
            e = launch_transpose(b, b->dt_[p]);
            if (e == cudaSuccess) e = launch_fused_pass(b, p, 1);
        }
        *moved = 1;
    } else {
        const int n = (int)b->states.size();
        e = launch_order_pass(b, b->do1[p], n, b->o_items);
        if (b->kind == LM_DENSITY) {
            if (e == cudaSuccess) e = launch_transpose(b, b->dt_[p]);
            if (e == cudaSuccess) e = launch_order_pass(b, b->do2[p], n, b->o_items);
            *moved = 1;
        } else {
            *moved = b->K % 2;  // odd K ends in A
        }
    }
    return e;
}

extern "C" {

int lm_batch_create(lm_ctx* ctx, int kind, int precision, double tol, lm_batch** out) {
    if (!ctx) return LM_ERR_ARG;
    if (!out) return set_err(ctx, LM_ERR_ARG, "lm_batch_create: null output");
    *out = nullptr;
    if (kind != LM_KETS && kind != LM_DENSITY) return set_err(ctx, LM_ERR_ARG, "lm_batch_create: unknown kind");
    if (precision != LM_C64 && precision != LM_C32) return set_err(ctx, LM_ERR_ARG, "lm_batch_create: unknown precision");
    if (!(tol > 0.0 && tol < 1.0)) return set_err(ctx, LM_ERR_ARG, "lm_batch_create: tol must lie in (0, 1)");
    lm_batch* b = new (std::nothrow) lm_batch();
    if (!b) return set_err(ctx, LM_ERR_OOM, "host allocation");
    b->ctx = ctx;
    b->kind = kind;
    b->precision = precision;
    b->tol = tol;
    cudaSetDevice(ctx->device);
    if (cudaMalloc((void**)&b->dqueue, 7 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMemset(b->dqueue, 0, 7 * sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        if (b->dqueue) cudaFree(b->dqueue);
        delete b;
        return set_err(ctx, LM_ERR_OOM, "lm_batch_create: queue allocation failed");
    }
    *out = b;
    return LM_OK;
}

int lm_batch_destroy(lm_batch* b) {
    if (!b) return LM_OK;
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    free_graphs(b);
    free_tables(b);
    free_panel(b);
    if (b->dqueue) cudaFree(b->dqueue);
    for (auto* s : b->solvers) lm_solver_destroy(s);
    delete b;
    return LM_OK;
}

int lm_batch_add(lm_batch* b, lm_ham* ham, lm_state* st, int* index) {
    if (!b) return LM_ERR_ARG;
    lm_ctx* ctx = b->ctx;
    if (!ham || !st) return set_err(ctx, LM_ERR_ARG, "lm_batch_add: null argument");
    if (ham->ctx != ctx || st->ctx != ctx) return set_err(ctx, LM_ERR_ARG, "lm_batch_add: objects from another context");
    if (st->kind != b->kind || st->precision != b->precision)
        return set_err(ctx, LM_ERR_ARG, "lm_batch_add: state kind/precision differ from the batch");
    if (st->n != ham->lat->g.N) return set_err(ctx, LM_ERR_ARG, "lm_batch_add: state size does not match the lattice");
    if (st->d_lo) return set_err(ctx, LM_ERR_NOTSUP, "lm_batch_add: compensated states are stepped one by one");
    for (auto* s : b->states)
        if (s == st) return set_err(ctx, LM_ERR_ARG, "lm_batch_add: state already in the batch");
    lm_solver* s = nullptr;
    int rc = lm_solver_create(ctx, b->tol, &s);
    if (rc != LM_OK) return rc;
    b->hams.push_back(ham);
    b->states.push_back(st);
    b->solvers.push_back(s);
    b->valid = 0;
    free_graphs(b);
    if (index) *index = (int)b->states.size() - 1;
    return LM_OK;
}

int lm_batch_update(lm_batch* b, double dt) {
    if (!b) return LM_ERR_ARG;
    lm_ctx* ctx = b->ctx;
    if (b->states.empty()) return set_err(ctx, LM_ERR_STATE, "lm_batch_update: empty batch");
    if (!isfinite(dt)) return set_err(ctx, LM_ERR_ARG, "lm_batch_update: non-finite dt");
    cudaSetDevice(ctx->device);
    int K = 0;
    for (size_t i = 0; i < b->states.size(); ++i) {
        int rc = lm_solver_update(b->solvers[i], b->hams[i], dt, 0);
        if (rc != LM_OK) return rc;
        K = std::max(K, b->solvers[i]->K);
    }
    if (K > kBatchMaxK) return set_err(ctx, LM_ERR_NOTSUP, "lm_batch_update: Chebyshev order above 40; use smaller dt");
    const int oldK = b->K, oldcfg = b->cfg;
    b->K = K;
    b->dt = dt;
    if (b->cfg < 0 || (b->cfg == 0 && !batch_fused_ok(b))) b->cfg = batch_fused_ok(b) ? 0 : 2;
    if (b->panel_w > 0 && b->cfg == 0) b->cfg = 2;  // panels run the per-order kernels
    // pointers at parity 0 follow the states as they are now
    b->base_S.resize(b->states.size());
    b->base_A.resize(b->states.size());
    for (size_t i = 0; i < b->states.size(); ++i) {
        if (b->panel_w == 0) {
            int rc0 = ensure_scratch(b->states[i]);
            if (rc0 != LM_OK) return rc0;
        }
        b->base_S[i] = b->states[i]->d_data;
        b->base_A[i] = b->states[i]->d_a;
    }
    b->parity = 0;
    if (b->panel_w > 0) {
        free_graphs(b);
        int rc = build_panel_tables(b);
        if (rc != LM_OK) return rc;
        b->valid = 1;
        return LM_OK;
    }
    if (b->cfg != 0)
        for (auto* st : b->states) {
            int rc0 = ensure_accumulator(st);
            if (rc0 != LM_OK) return rc0;
        }
    if (K != oldK || b->cfg != oldcfg) free_graphs(b);
    free_graphs(b);  // tables move when the pointers at parity 0 change
    int rc = build_tables(b);
    if (rc != LM_OK) return rc;
    b->valid = 1;
    return LM_OK;
}

int lm_batch_step(lm_batch* b) {
    if (!b) return LM_ERR_ARG;
    lm_ctx* ctx = b->ctx;
    if (!b->valid) return set_err(ctx, LM_ERR_STATE, "lm_batch_step: lm_batch_update must run first");
    cudaSetDevice(ctx->device);
    // every state must still sit where the tables expect it
    for (size_t i = 0; i < b->states.size(); ++i) {
        void* S = b->parity ? b->base_A[i] : b->base_S[i];
        if (b->states[i]->d_data != S)
            return set_err(ctx, LM_ERR_STATE, "lm_batch_step: a state was stepped outside the batch; call lm_batch_update");
    }
    const int p = b->parity;
    int moved = 0;
    if (b->cfg == 0) {  // kernel attributes are set outside any stream capture
        int rc = LM_OK;
        if (b->f_items > 0)
            rc = check_cuda(ctx, ensure_fused_attr(ctx, b->K, b->f_xreal), "lm_batch_step: kernel attribute");
        for (int c = 0; c < 2 && rc == LM_OK; ++c)
            if (b->r_items[c] > 0)
                rc = check_cuda(ctx, ensure_resident_attr(ctx, b->r_xreal, c + 1), "lm_batch_step: kernel attribute");
        if (rc != LM_OK) return rc;
    }
    if (b->use_graph) {
        if (!b->graph[p]) {
            cudaGraph_t gr = nullptr;
            int rc = check_cuda(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal),
                                "lm_batch_step: begin capture");
            if (rc != LM_OK) return rc;
            cudaError_t e = enqueue_step(b, p, &moved);
            cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &gr);
            if (e != cudaSuccess || e2 != cudaSuccess) {
                if (gr) cudaGraphDestroy(gr);
                return check_cuda(ctx, e != cudaSuccess ? e : e2, "lm_batch_step: capture");
            }
            e = cudaGraphInstantiate(&b->graph[p], gr, 0);
            cudaGraphDestroy(gr);
            if (e != cudaSuccess) {
                b->graph[p] = nullptr;
                return check_cuda(ctx, e, "lm_batch_step: graph instantiate");
            }
        } else {
            moved = b->panel_w > 0 ? 0 : ((b->cfg == 0 || b->kind == LM_DENSITY) ? 1 : b->K % 2);
        }
        int rc = check_cuda(ctx, cudaGraphLaunch(b->graph[p], ctx->stream), "lm_batch_step: graph launch");
        if (rc != LM_OK) return rc;
    } else {
        int rc = check_cuda(ctx, enqueue_step(b, p, &moved), "lm_batch_step");
        if (rc != LM_OK) return rc;
    }
    if (moved) {
        for (auto* st : b->states) std::swap(st->d_data, st->d_a);
        b->parity ^= 1;
    }
    return LM_OK;
}

int lm_batch_set_panel(lm_batch* b, int64_t width) {
    if (!b) return LM_ERR_ARG;
    if (width < 0) return set_err(b->ctx, LM_ERR_ARG, "lm_batch_set_panel: width must be >= 0");
    if (width != b->panel_w) {
        cudaSetDevice(b->ctx->device);
        cudaStreamSynchronize(b->ctx->stream);
        free_graphs(b);
        free_panel(b);
        b->panel_w = width;
        b->valid = 0;
    }
    return LM_OK;
}

int lm_batch_set_graph(lm_batch* b, int enable) {
    if (!b) return LM_ERR_ARG;
    b->use_graph = enable ? 1 : 0;
    return LM_OK;
}

int lm_batch_set_config(lm_batch* b, int cfg) {
    if (!b) return LM_ERR_ARG;
    if (cfg < -1 || cfg > 3) return set_err(b->ctx, LM_ERR_ARG, "lm_batch_set_config: config must be -1..3");
    if (cfg == 0 && b->valid && !batch_fused_ok(b))
        return set_err(b->ctx, LM_ERR_NOTSUP,
                       "lm_batch_set_config: the fused pass needs ComplexF32, and K <= 8 for lattices that do not fit on chip");
    b->cfg = cfg;
    free_graphs(b);
    if (b->valid) {
        // rebuild for the current pointers (parity 0 = where the data is now)
        return lm_batch_update(b, b->dt);
    }
    return LM_OK;
}

int lm_batch_info(lm_batch* b, int* K, int* cfg, int64_t* items, int* ninst) {
    if (!b) return LM_ERR_ARG;
    {  // a halo exchange of the lattice-resident kernel that timed out (its results are not valid)
        unsigned long long errbits = 0;
        cudaSetDevice(b->ctx->device);
        int rc = check_cuda(b->ctx, cudaMemcpy(&errbits, b->dqueue + 6, sizeof(errbits), cudaMemcpyDeviceToHost),
                            "lm_batch_info: error word");
        if (rc != LM_OK) return rc;
        if (errbits) return set_err(b->ctx, LM_ERR_TIMEOUT, "lm_batch: a halo exchange between the CTAs of a cluster timed out");
    }
    if (K) *K = b->K;
    if (cfg) *cfg = b->cfg;
    if (items) {
        int64_t pitems = 0;
        for (int64_t v : b->po_items) pitems += v;
        *items = b->panel_w > 0 ? pitems : (b->cfg == 0 ? b->f_items + b->r_items[0] + b->r_items[1] : b->o_items);
    }
    if (ninst) *ninst = (int)b->states.size();
    return LM_OK;
}

// Times every eligible pass shape on scratch copies of the batch's states (forward steps; a
// leading sample of the instances when all copies would not fit), keeps the fastest; the
// batch's own states are not touched.  ms_out[c] receives the time
// of one step with config c (negative when not eligible).
int lm_batch_tune(lm_batch* b, int steps, double* ms_out, int* best) {
    if (!b) return LM_ERR_ARG;
    lm_ctx* ctx = b->ctx;
    if (!b->valid) return set_err(ctx, LM_ERR_STATE, "lm_batch_tune: lm_batch_update must run first");
    if (steps < 1) steps = 2;
    cudaSetDevice(ctx->device);
    // scratch batch over copies of the states
    lm_batch* t = nullptr;
    int rc = lm_batch_create(ctx, b->kind, b->precision, b->tol, &t);
    if (rc != LM_OK) return rc;
    std::vector<lm_state*> copies;
    // a sample of the instances (in order) whose copies fit in a quarter of the free memory,
    // at most 8 GiB
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const size_t cap = std::min<size_t>(free_b / 4, (size_t)8 << 30);
    size_t used = 0;
    for (size_t i = 0; i < b->states.size() && rc == LM_OK; ++i) {
        const size_t need = 3 * b->states[i]->elem * (size_t)b->states[i]->ld * (size_t)b->states[i]->m;
        if (i > 0 && used + need > cap) break;
        used += need;
        lm_state* c = nullptr;
        rc = lm_state_create(ctx, b->states[i]->n, b->states[i]->m, b->kind, b->precision, &c);
        if (rc == LM_OK) {
            copies.push_back(c);
            rc = lm_state_copy(c, b->states[i]);
        }
        if (rc == LM_OK) rc = lm_batch_add(t, b->hams[i], c, nullptr);
    }
    double best_ms = 1e300;
    int best_cfg = b->cfg;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (rc == LM_OK) rc = check_cuda(ctx, cudaEventCreate(&e0), "cudaEventCreate");
    if (rc == LM_OK) rc = check_cuda(ctx, cudaEventCreate(&e1), "cudaEventCreate");
    for (int c = 0; c <= 3 && rc == LM_OK; ++c) {
        if (ms_out) ms_out[c] = -1.0;
        t->cfg = c;
        t->valid = 0;
        if (c == 0 && (!batch_fused_ok(b) || b->panel_w > 0)) continue;
        rc = lm_batch_update(t, b->dt);
        if (rc != LM_OK) break;
        if (t->cfg != c) continue;
        rc = lm_batch_step(t);  // warm-up (and graph capture)
        if (rc != LM_OK) break;
        cudaEventRecord(e0, ctx->stream);
        for (int s = 0; s < steps && rc == LM_OK; ++s) rc = lm_batch_step(t);
        cudaEventRecord(e1, ctx->stream);
        if (rc != LM_OK) break;
        rc = check_cuda(ctx, cudaEventSynchronize(e1), "cudaEventSynchronize");
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double per = ms / steps;
        if (ms_out) ms_out[c] = per;
        if (per < best_ms) {
            best_ms = per;
            best_cfg = c;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    lm_batch_destroy(t);
    for (auto* c : copies) lm_state_destroy(c);
    if (rc != LM_OK) return rc;
    if (best) *best = best_cfg;
    return lm_batch_set_config(b, best_cfg);
}

}  // extern "C"
