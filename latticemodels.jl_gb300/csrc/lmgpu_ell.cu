// General sparse Hamiltonians: any Hermitian operator that the reference's construct_operator
// builds (src/operators/constructoperator.jl:4-47) -- other lattices (HoneycombLattice,
// KagomeLattice, src/zoo/lattices.jl:145-211), internal degrees of freedom (qwz,
// src/zoo/models.jl:129-137), longer-range hopping -- given as its SparseMatrixCSC.  On the
// device it is an ELL table (row i: up to w off-diagonal (column, value) pairs, column-major
// over the rows so that consecutive threads read consecutive entries) plus the real diagonal.
// The Chebyshev propagator is the same as for the square lattice; only the stencil differs.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <new>
#include <unordered_map>
#include <vector>

#include "lmgpu_internal.cuh"
#include "lmgpu_order.cuh"

namespace lmgpu {

// 2H/a off the diagonal and 2(H_ii - b)/a on it, in FP64 and FP32.
__global__ void ell_normalise_kernel(int64_t n, int w, const double2* __restrict__ vals,
                                     const double* __restrict__ diag, double a, double b, double2* __restrict__ v2,
                                     double* __restrict__ d2, float2* __restrict__ v2f, float* __restrict__ d2f) {
    const double sc = 2.0 / a;
    const int64_t tot = n * (int64_t)w;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < tot + n; i += (int64_t)gridDim.x * blockDim.x) {
        if (i < tot) {
            const double2 v = make_double2(vals[i].x * sc, vals[i].y * sc);
            v2[i] = v;
            v2f[i] = make_float2((float)v.x, (float)v.y);
        } else {
            const int64_t r = i - tot;
            const double d = (diag[r] - b) * sc;
            d2[r] = d;
            d2f[r] = (float)d;
        }
    }
}

// One Chebyshev order over an n x M block with the ELL stencil (see cheb_epilogue for the
// modes).  SITE_FAST: element (site, ket) at ket*ld + site, threads over sites; otherwise at
// site*ld + ket (rows of a density matrix), threads over kets.  CONJ applies conj(H).
template <typename R, int MODE, bool SITE_FAST, bool CONJ>
__global__ void __launch_bounds__(256) cheb_order_ell_kernel(
    int64_t n, int w, const int* __restrict__ cols, const typename CT<R>::V* __restrict__ v2,
    const R* __restrict__ d2, const typename CT<R>::V* __restrict__ tp, typename CT<R>::V* tq,
    typename CT<R>::V* y, int64_t ld, int64_t M, R c0, R cs, int odd, R ph_re, R ph_im, ChebLo lo) {
    typedef typename CT<R>::V V;
    const int64_t lane = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nfast = SITE_FAST ? n : M;
    const int64_t nslow = SITE_FAST ? M : n;
    if (lane >= nfast) return;
    for (int64_t slow = blockIdx.y; slow < nslow; slow += gridDim.y) {
        const int64_t site = SITE_FAST ? lane : slow;
        const int64_t ket = SITE_FAST ? slow : lane;
        auto at = [&](int64_t s) -> int64_t { return SITE_FAST ? ket * ld + s : s * ld + ket; };
        const V v0 = tp[at(site)];
        V acc;
        if (MODE == CHEB_FIRST) {
            acc = CT<R>::make(0, 0);
        } else {
            const V q = tq[at(site)];
            acc = CT<R>::make(-q.x, -q.y);
        }
        for (int k = 0; k < w; ++k) {
            const int64_t e = (int64_t)k * n + site;
            const int c = __ldg(cols + e);
            V h = v2[e];
            if (CONJ) h.y = -h.y;
            const V v = tp[at(c)];
            acc.x = fma(h.x, v.x, acc.x); acc.x = fma(-h.y, v.y, acc.x);
            acc.y = fma(h.x, v.y, acc.y); acc.y = fma(h.y, v.x, acc.y);
        }
        const R d = d2[site];
        acc.x = fma(d, v0.x, acc.x);
        acc.y = fma(d, v0.y, acc.y);
        cheb_epilogue<R, MODE>(acc, v0, tq, y, at(site), c0, cs, odd, ph_re, ph_im, lo);
    }
}

// Site-fast form with the row in registers: a thread owns one site, loads its (at most WMAX)
// stored entries once and applies them to INNER kets (the generic kernel reloads the row for
// every ket).  Same FMA sequence per site-ket as cheb_order_ell_kernel.
template <typename R, int MODE, bool CONJ, int WMAX, int INNER>
__global__ void __launch_bounds__(256) cheb_order_ell_rows_kernel(
    int64_t n, int w, const int* __restrict__ cols, const typename CT<R>::V* __restrict__ v2,
    const R* __restrict__ d2, const typename CT<R>::V* __restrict__ tp, typename CT<R>::V* tq,
    typename CT<R>::V* y, int64_t ld, int64_t M, R c0, R cs, int odd, R ph_re, R ph_im, ChebLo lo) {
    typedef typename CT<R>::V V;
    const int64_t site = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (site >= n) return;
    int c[WMAX];
    V hv[WMAX];
#pragma unroll
    for (int k = 0; k < WMAX; ++k) {
        if (k < w) {
            const int64_t e = (int64_t)k * n + site;
            c[k] = __ldg(cols + e);
            hv[k] = v2[e];
            if (CONJ) hv[k].y = -hv[k].y;
        } else {
            c[k] = (int)site;
            hv[k] = CT<R>::make(0, 0);
        }
    }
    const R d = d2[site];
    for (int64_t k0 = (int64_t)blockIdx.y * INNER; k0 < M; k0 += (int64_t)gridDim.y * INNER) {
#pragma unroll
        for (int j = 0; j < INNER; ++j) {
            const int64_t ket = k0 + j;
            if (ket >= M) break;
            const int64_t base = ket * ld;
            const V v0 = tp[base + site];
            V acc;
            if (MODE == CHEB_FIRST) {
                acc = CT<R>::make(0, 0);
            } else {
                const V q = tq[base + site];
                acc = CT<R>::make(-q.x, -q.y);
            }
#pragma unroll
            for (int k = 0; k < WMAX; ++k) {
                if (k < w) {
                    const V h = hv[k];
                    const V v = tp[base + c[k]];
                    acc.x = fma(h.x, v.x, acc.x); acc.x = fma(-h.y, v.y, acc.x);
                    acc.y = fma(h.x, v.y, acc.y); acc.y = fma(h.y, v.x, acc.y);
                }
            }
            acc.x = fma(d, v0.x, acc.x);
            acc.y = fma(d, v0.y, acc.y);
            cheb_epilogue<R, MODE>(acc, v0, tq, y, base + site, c0, cs, odd, ph_re, ph_im, lo);
        }
    }
}

template <typename R, int MODE, bool SF, bool CJ>
static cudaError_t launch_ell_t(lm_ctx* ctx, const lm_ell* h, const void* v2, const void* d2, const void* tp, void* tq,
                                void* y, int64_t ld, int64_t m, double c0, ChebCoef ck, double pr, double pi,
                                ChebLo lo) {
    typedef typename CT<R>::V V;
    if (SF && h->w <= 8) {
        constexpr int INNER = 4;
        const dim3 grid((unsigned)((h->n + 255) / 256), (unsigned)std::min<int64_t>((m + INNER - 1) / INNER, 65535));
        if (h->w <= 4)
            cheb_order_ell_rows_kernel<R, MODE, CJ, 4, INNER><<<grid, 256, 0, ctx->stream>>>(
                h->n, h->w, h->d_cols, (const V*)v2, (const R*)d2, (const V*)tp, (V*)tq, (V*)y, ld, m, (R)c0,
                (R)ck.s, ck.odd, (R)pr, (R)pi, lo);
        else
            cheb_order_ell_rows_kernel<R, MODE, CJ, 8, INNER><<<grid, 256, 0, ctx->stream>>>(
                h->n, h->w, h->d_cols, (const V*)v2, (const R*)d2, (const V*)tp, (V*)tq, (V*)y, ld, m, (R)c0,
                (R)ck.s, ck.odd, (R)pr, (R)pi, lo);
        ctx->launches++;
        return cudaGetLastError();
    }
    const int thr = 256;
    const int64_t nfast = SF ? h->n : m;
    const int64_t nslow = SF ? m : h->n;
    dim3 grid((unsigned)((nfast + thr - 1) / thr), (unsigned)std::min<int64_t>(nslow, 65535));
    cheb_order_ell_kernel<R, MODE, SF, CJ><<<grid, thr, 0, ctx->stream>>>(
        h->n, h->w, h->d_cols, (const V*)v2, (const R*)d2, (const V*)tp, (V*)tq, (V*)y, ld, m, (R)c0, (R)ck.s, ck.odd,
        (R)pr, (R)pi, lo);
    ctx->launches++;
    return cudaGetLastError();
}

template <typename R, bool SF, bool CJ>
static cudaError_t launch_ell_mode(int mode, lm_ctx* ctx, const lm_ell* h, const void* v2, const void* d2,
                                   const void* tp, void* tq, void* y, int64_t ld, int64_t m, double c0, ChebCoef ck,
                                   double pr, double pi, ChebLo lo) {
    if (mode == CHEB_FIRST) return launch_ell_t<R, CHEB_FIRST, SF, CJ>(ctx, h, v2, d2, tp, tq, y, ld, m, c0, ck, pr, pi, lo);
    if (mode == CHEB_MID) return launch_ell_t<R, CHEB_MID, SF, CJ>(ctx, h, v2, d2, tp, tq, y, ld, m, c0, ck, pr, pi, lo);
    return launch_ell_t<R, CHEB_LAST, SF, CJ>(ctx, h, v2, d2, tp, tq, y, ld, m, c0, ck, pr, pi, lo);
}

static cudaError_t launch_ell_order(lm_ctx* ctx, const lm_ell* h, int precision, int site_fast, int conj, int mode,
                                    const void* v2, const void* d2, const void* tp, void* tq, void* y, int64_t ld,
                                    int64_t m, double c0, ChebCoef ck, double pr, double pi, ChebLo lo) {
    if (precision == LM_C64) {
        if (site_fast) {
            return conj ? launch_ell_mode<double, true, true>(mode, ctx, h, v2, d2, tp, tq, y, ld, m, c0, ck, pr, pi, lo)
                        : launch_ell_mode<double, true, false>(mode, ctx, h, v2, d2, tp, tq, y, ld, m, c0, ck, pr, pi, lo);
        }
        return conj ? launch_ell_mode<double, false, true>(mode, ctx, h, v2, d2, tp, tq, y, ld, m, c0, ck, pr, pi, lo)
                    : launch_ell_mode<double, false, false>(mode, ctx, h, v2, d2, tp, tq, y, ld, m, c0, ck, pr, pi, lo);
    }
    if (site_fast) {
        return conj ? launch_ell_mode<float, true, true>(mode, ctx, h, v2, d2, tp, tq, y, ld, m, c0, ck, pr, pi, lo)
                    : launch_ell_mode<float, true, false>(mode, ctx, h, v2, d2, tp, tq, y, ld, m, c0, ck, pr, pi, lo);
    }
    return conj ? launch_ell_mode<float, false, true>(mode, ctx, h, v2, d2, tp, tq, y, ld, m, c0, ck, pr, pi, lo)
                : launch_ell_mode<float, false, false>(mode, ctx, h, v2, d2, tp, tq, y, ld, m, c0, ck, pr, pi, lo);
}

// One application of the series to (site_fast, ld, m)-laid-out columns S (T0 on entry); the
// result lands in S (K even) or A (K odd): *where = 0 / 1.
static int ell_apply(lm_solver* s, int precision, int site_fast, int conj, void* S, void* A, void* Y, int64_t ld,
                     int64_t m, int* where) {
    lm_ctx* ctx = s->ctx;
    const lm_ell* h = s->ell;
    const void* v2 = precision == LM_C64 ? (const void*)s->d_ev2 : (const void*)s->d_ev2f;
    const void* d2 = precision == LM_C64 ? (const void*)s->d_ed2 : (const void*)s->d_ed2f;
    const int K = s->K;
    const double c0 = s->coef[0].s;
    const double pr = s->phase_re, pi = conj ? -s->phase_im : s->phase_im;
    auto coef = [&](int k) {
        ChebCoef c = s->coef[(size_t)k];
        if (conj && c.odd) c.s = -c.s;
        return c;
    };
    const ChebLo lo = cheb_lo(pr, pi, c0, coef(1).s, false);
    CUDA_TRY(ctx, launch_ell_order(ctx, h, precision, site_fast, conj, CHEB_FIRST, v2, d2, S, A, Y, ld, m, c0, coef(1), pr,
                                   pi, lo),
             "ell chebyshev order 1");
    for (int k = 2; k <= K; ++k) {
        const void* tp = (k % 2 == 0) ? A : S;
        void* tq = (k % 2 == 0) ? S : A;
        const int mode = (k == K) ? CHEB_LAST : CHEB_MID;
        CUDA_TRY(ctx, launch_ell_order(ctx, h, precision, site_fast, conj, mode, v2, d2, tp, tq, Y, ld, m, c0, coef(k), pr,
                                       pi, lo),
                 "ell chebyshev order");
    }
    *where = (K % 2 == 0) ? 0 : 1;
    return LM_OK;
}

int ell_solver_step(lm_solver* s, lm_state* st) {
    lm_ctx* ctx = s->ctx;
    CHECK_ARG(ctx, st->n == s->ell->n, "lm_solver_step: state size does not match the Hamiltonian");
    cudaSetDevice(ctx->device);
    {
        int rc0 = ensure_scratch(st);
        if (rc0 != LM_OK) return rc0;
    }
    if (!st->d_y) {
        const size_t bytes = st->elem * (size_t)st->ld * (size_t)st->m;
        if (cudaMalloc(&st->d_y, bytes) != cudaSuccess) {
            st->d_y = nullptr;
            cudaGetLastError();
            return set_err(ctx, LM_ERR_OOM, "lm_solver_step: accumulator allocation");
        }
    }
    int where = 0;
    const lm_ell* h = s->ell;
    if (h->brick && st->precision == LM_C32 && st->kind == LM_KETS && ctx->fused && ctx->fused_form == 1) {
        // the honeycomb as an a x 2b brick lattice: the x-streaming kernel, all K orders per launch
        Geom g{};
        g.Lx = h->brick_a;
        g.Ly = 2 * h->brick_b;
        g.N = h->n;
        g.per_x = h->brick_px;
        g.per_y = h->brick_py;
        if (stream_supported(g, s->K, 4, st->d_data, st->d_a, st->ld) &&
            (!st->d_lo || stream_comp_supported(g, s->K, 4))) {
            int rc0 = ensure_brick_pack(s, g, h->d_bmap);
            if (rc0 != LM_OK) return rc0;
            cudaEvent_t t0 = nullptr, t1 = nullptr;
            if (ctx->timing) {
                rc0 = timing_event_pair(ctx, &t0, &t1);
                if (rc0 != LM_OK) return rc0;
                CUDA_TRY(ctx, cudaEventRecord(t0, ctx->stream), "cudaEventRecord");
            }
            CUDA_TRY(ctx, launch_cheb_fused_c32(ctx, g, nullptr, nullptr, (const float2*)st->d_data, (float2*)st->d_a,
                                                st->ld, st->m, s->K, false, s->coef.data(), s->phase_re, s->phase_im,
                                                s->d_spack, 4, st->d_lo),
                     "honeycomb x-streaming step");
            if (ctx->timing) {
                CUDA_TRY(ctx, cudaEventRecord(t1, ctx->stream), "cudaEventRecord");
                ctx->ev_launches[ctx->ev_used] = s->K;
                ctx->ev_used++;
            }
            std::swap(st->d_data, st->d_a);
            return LM_OK;
        }
    }
    if (st->d_lo)
        return set_err(ctx, LM_ERR_NOTSUP,
                       "lm_solver_step: a compensated state on a general Hamiltonian needs the honeycomb brick layout "
                       "and the x-streaming form");
    int rc = ell_apply(s, st->precision, 1, 0, st->d_data, st->d_a, st->d_y, st->ld, st->m, &where);
    if (rc != LM_OK) return rc;
    if (where == 1) std::swap(st->d_data, st->d_a);
    if (st->kind == LM_DENSITY) {  // P <- X U^dagger: conj(U) on every row of X
        rc = ell_apply(s, st->precision, 0, 1, st->d_data, st->d_a, st->d_y, st->ld, st->m, &where);
        if (rc != LM_OK) return rc;
        if (where == 1) std::swap(st->d_data, st->d_a);
    }
    return LM_OK;
}

void ell_free_tables(lm_solver* s) {
    cudaFree(s->d_ev2);
    cudaFree(s->d_ed2);
    cudaFree(s->d_ev2f);
    cudaFree(s->d_ed2f);
    s->d_ev2 = nullptr;
    s->d_ed2 = nullptr;
    s->d_ev2f = nullptr;
    s->d_ed2f = nullptr;
    s->ell_tab = 0;
}

// J for every CSC entry: 2 Im(H[i,j] P[j,i]); ket blocks sum over the kets (one thread per
// entry, FP64), density matrices read P[j,i].
template <typename R>
__global__ void ell_currents_kernel(int64_t nnz, const int* __restrict__ row, const int* __restrict__ col,
                                    const double2* __restrict__ hv, int kind, const typename CT<R>::V* __restrict__ x,
                                    int64_t m, int64_t ld, const double* __restrict__ wts, double* __restrict__ out) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x) {
        const int i = row[p], j = col[p];
        if (i == j) {
            out[p] = 0.0;
            continue;
        }
        double pr = 0.0, pim = 0.0;  // P[j, i]
        if (kind == LM_DENSITY) {
            const typename CT<R>::V v = x[(int64_t)i * ld + j];
            pr = v.x;
            pim = v.y;
        } else {
            for (int64_t k = 0; k < m; ++k) {
                const typename CT<R>::V a = x[k * ld + j], b = x[k * ld + i];  // a conj(b)
                const double ww = wts ? wts[k] : 1.0;
                pr += ww * ((double)a.x * b.x + (double)a.y * b.y);
                pim += ww * ((double)a.y * b.x - (double)a.x * b.y);
            }
        }
        const double2 h = hv[p];
        out[p] = 2.0 * (h.x * pim + h.y * pr);
    }
}

// LocalOperatorCurrents per stored entry (r, c) = ((i, k), (j, beta)):
// 2 Im(H[r,c] Q), Q = sum_alpha op[alpha,k] P[c, (i, alpha)]; ket blocks build
// P[c, q] = sum_m w_m x[c,m] conj(x[q,m]) with the operator applied to the conjugated side.
template <typename R>
__global__ void ell_op_currents_kernel(int64_t nnz, const int* __restrict__ row, const int* __restrict__ col,
                                       const double2* __restrict__ hv, int kind,
                                       const typename CT<R>::V* __restrict__ x, int64_t m, int64_t ld,
                                       const double* __restrict__ wts, int ndof, LocalOp op,
                                       double* __restrict__ out) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x) {
        const int r = row[p], c = col[p];
        const int si = r / ndof, kr = r - si * ndof;
        if (si == c / ndof) {
            out[p] = 0.0;
            continue;
        }
        const int64_t q0 = (int64_t)si * ndof;
        double qr = 0.0, qi = 0.0;
        if (kind == LM_DENSITY) {
            for (int a = 0; a < ndof; ++a) {
                const double2 o = op.o[a + kr * ndof];
                const typename CT<R>::V v = x[(q0 + a) * ld + c];  // P[c, q0 + a]
                qr += o.x * v.x - o.y * v.y;
                qi += o.x * v.y + o.y * v.x;
            }
        } else {
            for (int64_t k = 0; k < m; ++k) {
                double sr = 0.0, sim = 0.0;  // sum_alpha op[alpha,kr] conj(x[q0+alpha, k])
                for (int a = 0; a < ndof; ++a) {
                    const double2 o = op.o[a + kr * ndof];
                    const typename CT<R>::V b = x[k * ld + q0 + a];
                    sr += o.x * b.x + o.y * b.y;
                    sim += o.y * b.x - o.x * b.y;
                }
                const typename CT<R>::V v = x[k * ld + c];
                const double ww = wts ? wts[k] : 1.0;
                qr += ww * (v.x * sr - v.y * sim);
                qi += ww * (v.x * sim + v.y * sr);
            }
        }
        const double2 h = hv[p];
        out[p] = 2.0 * (h.x * qi + h.y * qr);
    }
}

int make_local_op(lm_ctx* ctx, const lm_ell* h, int ndof, const double* op, LocalOp* lop, const char* who) {
    if (!(ndof >= 1 && ndof <= 8 && h->n % ndof == 0))
        return set_err(ctx, LM_ERR_ARG, std::string(who) + ": ndof must be in 1..8 and divide the matrix size");
    *lop = LocalOp{};
    for (int a = 0; a < ndof; ++a)
        for (int b = 0; b < ndof; ++b) {
            const int idx = a + b * ndof;
            if (op) {
                if (!std::isfinite(op[2 * idx]) || !std::isfinite(op[2 * idx + 1]))
                    return set_err(ctx, LM_ERR_ARG, std::string(who) + ": non-finite operator entry");
                lop->o[idx] = make_double2(op[2 * idx], op[2 * idx + 1]);
            } else {
                lop->o[idx] = make_double2(a == b ? 1.0 : 0.0, 0.0);
            }
        }
    return LM_OK;
}

cudaError_t launch_ell_op_currents(lm_ctx* ctx, const lm_ell* h, const lm_state* st, int ndof, const LocalOp& lop,
                                   double* d_out) {
    if (h->nnz == 0) return cudaSuccess;
    const unsigned grid = (unsigned)std::min<int64_t>((h->nnz + 255) / 256, 65535);
    if (st->precision == LM_C64)
        ell_op_currents_kernel<double><<<grid, 256, 0, ctx->stream>>>(
            h->nnz, h->d_crow, h->d_ccol, h->d_cval, st->kind, (const double2*)st->d_data, st->m, st->ld, st->d_w,
            ndof, lop, d_out);
    else
        ell_op_currents_kernel<float><<<grid, 256, 0, ctx->stream>>>(
            h->nnz, h->d_crow, h->d_ccol, h->d_cval, st->kind, (const float2*)st->d_data, st->m, st->ld, st->d_w,
            ndof, lop, d_out);
    ctx->launches++;
    return cudaGetLastError();
}

// Values of a Hamiltonian built from a bond list (lm_ell_create_bonds), thread per CSC entry:
// the sum, in bond order, of base * exp(-2 pi i LI(field; r_src -> r_dst)) over the bonds that
// land on the entry (conjugated for the reverse entry H[dst, src]), the phase formed as the
// square-lattice assembly forms it; the diagonal entry adds the on-site term.  The field
// components of such Hamiltonians have no boundary images, so the geometry is not used.
__global__ void ell_assemble_kernel(int64_t nnz, FieldSet f, const double* __restrict__ bxy,
                                    const double2* __restrict__ bbase, const int64_t* __restrict__ eptr,
                                    const int64_t* __restrict__ eterm, const int64_t* __restrict__ emap,
                                    const double* __restrict__ onsite, double2* __restrict__ cval,
                                    double2* __restrict__ vals, double* __restrict__ diag) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nnz) return;
    const Geom g0{};
    double2 v = make_double2(0.0, 0.0);
    for (int64_t q = eptr[p]; q < eptr[p + 1]; ++q) {
        const int64_t t = eterm[q], b = t >> 1;
        const double* r = bxy + 4 * b;
        const double li = f.n > 0 ? field_line_integral(g0, f, r[0], r[1], r[2], r[3]) : 0.0;
        const double theta = __dmul_rn(-2.0 * M_PI, li);
        double sn, cs;
        sincos(theta, &sn, &cs);
        const double2 base = bbase[b];
        const double wx = __dsub_rn(__dmul_rn(base.x, cs), __dmul_rn(base.y, sn));
        double wy = __dadd_rn(__dmul_rn(base.x, sn), __dmul_rn(base.y, cs));
        if (t & 1) wy = -wy;
        v.x = __dadd_rn(v.x, wx);
        v.y = __dadd_rn(v.y, wy);
    }
    const int64_t slot = emap[p];
    if (slot < 0) {
        const int64_t i = -slot - 1;
        const double d = __dadd_rn(onsite ? onsite[i] : 0.0, v.x);
        cval[p] = make_double2(d, 0.0);
        diag[i] = d;
    } else {
        cval[p] = v;
        vals[slot] = v;
    }
}

}  // namespace lmgpu

using namespace lmgpu;

// Fills the ELL host staging from CSC values (pattern fixed at creation).
static void ell_stage(lm_ell* h, const double* nzval) {
    std::fill(h->h_vals.begin(), h->h_vals.end(), make_double2(0.0, 0.0));
    std::fill(h->h_diag.begin(), h->h_diag.end(), 0.0);
    for (int64_t p = 0; p < h->nnz; ++p) {
        const int64_t slot = h->map[(size_t)p];
        if (slot < 0) h->h_diag[(size_t)(-slot - 1)] += nzval[2 * p];
        else h->h_vals[(size_t)slot] = make_double2(nzval[2 * p], nzval[2 * p + 1]);
    }
}

static int ell_check_and_bounds(lm_ell* h, const double* nzval) {
    lm_ctx* ctx = h->ctx;
    double vmax = 0.0;
    for (int64_t p = 0; p < h->nnz; ++p) {
        if (!isfinite(nzval[2 * p]) || !isfinite(nzval[2 * p + 1]))
            return set_err(ctx, LM_ERR_NONFINITE, "lm_ell: non-finite matrix entry");
        vmax = std::max(vmax, hypot(nzval[2 * p], nzval[2 * p + 1]));
    }
    // Hermitian: H[i,j] = conj(H[j,i]) (the transpose entry must be stored too)
    std::unordered_map<int64_t, int64_t> where;
    where.reserve((size_t)h->nnz * 2);
    for (int64_t p = 0; p < h->nnz; ++p) where[h->csc_row[(size_t)p] * h->n + h->csc_col[(size_t)p]] = p;
    const double tol = 1e-12 * std::max(vmax, 1e-300);
    std::vector<double> rad((size_t)h->n, 0.0), dia((size_t)h->n, 0.0);
    for (int64_t p = 0; p < h->nnz; ++p) {
        const int64_t i = h->csc_row[(size_t)p], j = h->csc_col[(size_t)p];
        const double re = nzval[2 * p], im = nzval[2 * p + 1];
        if (i == j) {
            if (fabs(im) > tol) return set_err(ctx, LM_ERR_ARG, "lm_ell: diagonal entry with an imaginary part");
            dia[(size_t)i] += re;
            continue;
        }
        auto it = where.find(j * h->n + i);
        const double tre = it == where.end() ? 0.0 : nzval[2 * it->second];
        const double tim = it == where.end() ? 0.0 : nzval[2 * it->second + 1];
        if (fabs(re - tre) > tol || fabs(im + tim) > tol) return set_err(ctx, LM_ERR_ARG, "lm_ell: matrix is not Hermitian");
        rad[(size_t)i] += hypot(re, im);
    }
    h->emin = dia[0] - rad[0];
    h->emax = dia[0] + rad[0];
    for (int64_t i = 1; i < h->n; ++i) {
        h->emin = std::min(h->emin, dia[(size_t)i] - rad[(size_t)i]);
        h->emax = std::max(h->emax, dia[(size_t)i] + rad[(size_t)i]);
    }
    return LM_OK;
}

static int ell_upload(lm_ell* h, const double* nzval) {
    lm_ctx* ctx = h->ctx;
    ell_stage(h, nzval);
    std::vector<double2> cval((size_t)h->nnz);
    for (int64_t p = 0; p < h->nnz; ++p) cval[(size_t)p] = make_double2(nzval[2 * p], nzval[2 * p + 1]);
    CUDA_TRY(ctx, cudaMemcpyAsync(h->d_vals, h->h_vals.data(), sizeof(double2) * h->h_vals.size(), cudaMemcpyHostToDevice,
                                  ctx->stream), "upload ell values");
    CUDA_TRY(ctx, cudaMemcpyAsync(h->d_diag, h->h_diag.data(), sizeof(double) * h->h_diag.size(), cudaMemcpyHostToDevice,
                                  ctx->stream), "upload ell diagonal");
    CUDA_TRY(ctx, cudaMemcpyAsync(h->d_cval, cval.data(), sizeof(double2) * cval.size(), cudaMemcpyHostToDevice,
                                  ctx->stream), "upload csc values");
    // the staging vectors are reused by the next call: wait for the copies
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    h->version++;
    return LM_OK;
}

extern "C" {

int lm_ell_create_csc(lm_ctx* ctx, int64_t n, const int64_t* colptr, const int64_t* rowval, const double* nzval,
                      lm_ell** out) {
    if (!ctx) return LM_ERR_ARG;
    CHECK_ARG(ctx, out && colptr && rowval && nzval, "lm_ell_create_csc: null argument");
    *out = nullptr;
    CHECK_ARG(ctx, n >= 1 && n < ((int64_t)1 << 31), "lm_ell_create_csc: bad size");
    CHECK_ARG(ctx, colptr[0] == 1, "lm_ell_create_csc: colptr must start at 1");
    const int64_t nnz = colptr[n] - 1;
    CHECK_ARG(ctx, nnz >= 0, "lm_ell_create_csc: bad colptr");
    for (int64_t j = 0; j < n; ++j) CHECK_ARG(ctx, colptr[j + 1] >= colptr[j], "lm_ell_create_csc: colptr not monotone");
    for (int64_t p = 0; p < nnz; ++p)
        CHECK_ARG(ctx, rowval[p] >= 1 && rowval[p] <= n, "lm_ell_create_csc: row index out of range");
    lm_ell* h = new (std::nothrow) lm_ell();
    if (!h) return set_err(ctx, LM_ERR_OOM, "host allocation");
    h->ctx = ctx;
    h->n = n;
    h->nnz = nnz;
    h->csc_row.resize((size_t)nnz);
    h->csc_col.resize((size_t)nnz);
    std::vector<int> count((size_t)n, 0);
    for (int64_t j = 0; j < n; ++j)
        for (int64_t p = colptr[j] - 1; p < colptr[j + 1] - 1; ++p) {
            h->csc_row[(size_t)p] = rowval[p] - 1;
            h->csc_col[(size_t)p] = j;
            if (rowval[p] - 1 != j) count[(size_t)(rowval[p] - 1)]++;
        }
    int rc = ell_check_and_bounds(h, nzval);
    if (rc != LM_OK) {
        delete h;
        return rc;
    }
    h->w = std::max(1, *std::max_element(count.begin(), count.end()));
    // slots: row i's off-diagonal entries in CSC (column) order; unused slots point at i
    std::vector<int> cols((size_t)n * h->w);
    for (int k = 0; k < h->w; ++k)
        for (int64_t i = 0; i < n; ++i) cols[(size_t)k * n + i] = (int)i;
    std::vector<int> fill((size_t)n, 0);
    h->map.resize((size_t)nnz);
    for (int64_t p = 0; p < nnz; ++p) {
        const int64_t i = h->csc_row[(size_t)p], j = h->csc_col[(size_t)p];
        if (i == j) {
            h->map[(size_t)p] = -(i + 1);
        } else {
            const int k = fill[(size_t)i]++;
            cols[(size_t)k * n + i] = (int)j;
            h->map[(size_t)p] = (int64_t)k * n + i;
        }
    }
    h->h_vals.resize((size_t)n * h->w);
    h->h_diag.resize((size_t)n);
    std::vector<int> crow((size_t)nnz), ccol((size_t)nnz);
    for (int64_t p = 0; p < nnz; ++p) {
        crow[(size_t)p] = (int)h->csc_row[(size_t)p];
        ccol[(size_t)p] = (int)h->csc_col[(size_t)p];
    }
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaMalloc((void**)&h->d_cols, sizeof(int) * cols.size());
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d_vals, sizeof(double2) * h->h_vals.size());
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d_diag, sizeof(double) * (size_t)n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d_crow, sizeof(int) * (size_t)std::max<int64_t>(nnz, 1));
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d_ccol, sizeof(int) * (size_t)std::max<int64_t>(nnz, 1));
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d_cval, sizeof(double2) * (size_t)std::max<int64_t>(nnz, 1));
    if (e == cudaSuccess)
        e = cudaMemcpy(h->d_cols, cols.data(), sizeof(int) * cols.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nnz > 0) e = cudaMemcpy(h->d_crow, crow.data(), sizeof(int) * crow.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nnz > 0) e = cudaMemcpy(h->d_ccol, ccol.data(), sizeof(int) * ccol.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaGetLastError();
        rc = check_cuda(ctx, e, "lm_ell_create_csc: device tables");
        lm_ell_destroy(h);
        return rc;
    }
    rc = ell_upload(h, nzval);
    if (rc != LM_OK) {
        lm_ell_destroy(h);
        return rc;
    }
    *out = h;
    return LM_OK;
}

int lm_ell_destroy(lm_ell* h) {
    if (!h) return LM_OK;
    cudaSetDevice(h->ctx->device);
    cudaStreamSynchronize(h->ctx->stream);
    cudaFree(h->d_cols);
    cudaFree(h->d_vals);
    cudaFree(h->d_diag);
    cudaFree(h->d_crow);
    cudaFree(h->d_ccol);
    cudaFree(h->d_cval);
    cudaFree(h->d_bxy);
    cudaFree(h->d_bbase);
    cudaFree(h->d_eptr);
    cudaFree(h->d_eterm);
    cudaFree(h->d_emap);
    cudaFree(h->d_onsite);
    cudaFree(h->d_bmap);
    delete h;
    return LM_OK;
}

int lm_ell_set_layout(lm_ell* h, int layout, int64_t a, int64_t b, int periodic_a, int periodic_b) {
    if (!h) return LM_ERR_ARG;
    lm_ctx* ctx = h->ctx;
    if (layout == LM_LAYOUT_NONE) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(h->d_bmap);
        h->d_bmap = nullptr;
        h->brick = 0;
        return LM_OK;
    }
    CHECK_ARG(ctx, layout == LM_LAYOUT_HONEYCOMB, "lm_ell_set_layout: unknown layout");
    CHECK_ARG(ctx, a >= 1 && b >= 1 && 2 * a * b == h->n, "lm_ell_set_layout: a x b unit cells of 2 sites must be the n sites");
    // a periodic axis of one or two cells would merge distinct bonds into one stored entry
    CHECK_ARG(ctx, (!periodic_a || a >= 3) && (!periodic_b || b >= 3),
              "lm_ell_set_layout: periodic axes need at least 3 unit cells");
    const int64_t Ly = 2 * b;
    std::vector<int> bm((size_t)(a * b) * 5, -1);
    for (size_t p = 0; p < h->map.size(); ++p) {
        const int64_t e = h->map[p];
        if (e < 0) continue;  // diagonal
        const int64_t r = h->csc_row[p], c = h->csc_col[p];
        const int64_t xr = r / Ly, yr = r % Ly, xc = c / Ly, yc = c % Ly;
        const int sr = (int)(yr & 1), sc = (int)(yc & 1);
        const int64_t lr = yr >> 1, lc = yc >> 1;
        int slot = -1;
        if (sr == 0 && sc == 1) {  // A -> B
            if (xc == xr && lc == lr) slot = 0;
            else if (xc == xr && (lc == lr - 1 || (periodic_b && lr == 0 && lc == b - 1))) slot = 1;
            else if (lc == lr && (xc == xr - 1 || (periodic_a && xr == 0 && xc == a - 1))) slot = 2;
        } else if (sr == 1 && sc == 0) {  // B -> A
            if (xc == xr && lc == lr) continue;  // conj of the A -> B entry of the same cell
            if (lc == lr && (xc == xr + 1 || (periodic_a && xr == a - 1 && xc == 0))) slot = 3;
            else if (xc == xr && (lc == lr + 1 || (periodic_b && lr == b - 1 && lc == 0))) slot = 4;
        }
        if (slot < 0) return set_err(ctx, LM_ERR_ARG, "lm_ell_set_layout: an entry is not a honeycomb nearest-neighbour bond");
        const int64_t cell = xr * b + lr;
        int& dst = bm[(size_t)cell * 5 + slot];
        if (dst >= 0) return set_err(ctx, LM_ERR_ARG, "lm_ell_set_layout: two entries for one honeycomb bond");
        CHECK_ARG(ctx, e < (int64_t)1 << 31, "lm_ell_set_layout: ELL table too large");
        dst = (int)e;
    }
    cudaSetDevice(ctx->device);
    int* d = nullptr;
    if (cudaMalloc((void**)&d, sizeof(int) * bm.size()) != cudaSuccess) {
        cudaGetLastError();
        return set_err(ctx, LM_ERR_OOM, "lm_ell_set_layout: bond map");
    }
    const cudaError_t ce = cudaMemcpy(d, bm.data(), sizeof(int) * bm.size(), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) {
        cudaFree(d);
        return check_cuda(ctx, ce, "lm_ell_set_layout: bond map upload");
    }
    cudaStreamSynchronize(ctx->stream);
    cudaFree(h->d_bmap);
    h->d_bmap = d;
    h->brick = 1;
    h->brick_a = a;
    h->brick_b = b;
    h->brick_px = periodic_a ? 1 : 0;
    h->brick_py = periodic_b ? 1 : 0;
    h->version++;  // solvers rebuild their tables (and the brick planes)
    return LM_OK;
}

int lm_ell_set_values(lm_ell* h, const double* nzval) {
    if (!h) return LM_ERR_ARG;
    CHECK_ARG(h->ctx, nzval != nullptr, "lm_ell_set_values: null values");
    int rc = ell_check_and_bounds(h, nzval);
    if (rc != LM_OK) return rc;
    cudaSetDevice(h->ctx->device);
    return ell_upload(h, nzval);
}

int lm_ell_bounds(const lm_ell* h, double* emin, double* emax) {
    if (!h) return LM_ERR_ARG;
    CHECK_ARG(h->ctx, emin && emax, "lm_ell_bounds: null output");
    *emin = h->emin;
    *emax = h->emax;
    return LM_OK;
}

static void ell_bond_bounds(lm_ell* h) {
    h->emin = h->emax = 0.0;
    for (int64_t i = 0; i < h->n; ++i) {
        const double d = h->h_onsite.empty() ? 0.0 : h->h_onsite[(size_t)i];
        const double lo = d - h->rad[(size_t)i], hi = d + h->rad[(size_t)i];
        if (i == 0 || lo < h->emin) h->emin = lo;
        if (i == 0 || hi > h->emax) h->emax = hi;
    }
}

int lm_ell_create_bonds(lm_ctx* ctx, int64_t n, int64_t nbonds, const int64_t* src, const int64_t* dst,
                        const double* xy, const double* base, lm_ell** out) {
    if (!ctx) return LM_ERR_ARG;
    CHECK_ARG(ctx, out != nullptr, "lm_ell_create_bonds: null output");
    *out = nullptr;
    CHECK_ARG(ctx, n >= 1 && n < ((int64_t)1 << 31), "lm_ell_create_bonds: bad size");
    CHECK_ARG(ctx, nbonds >= 0, "lm_ell_create_bonds: negative bond count");
    CHECK_ARG(ctx, nbonds == 0 || (src && dst && xy && base), "lm_ell_create_bonds: null bond arrays");
    for (int64_t b = 0; b < nbonds; ++b) {
        CHECK_ARG(ctx, src[b] >= 1 && src[b] <= n && dst[b] >= 1 && dst[b] <= n, "lm_ell_create_bonds: site out of range");
        for (int k = 0; k < 4; ++k) CHECK_ARG(ctx, isfinite(xy[4 * b + k]), "lm_ell_create_bonds: non-finite coordinate");
        CHECK_ARG(ctx, isfinite(base[2 * b]) && isfinite(base[2 * b + 1]), "lm_ell_create_bonds: non-finite hop");
    }
    // the pattern: every diagonal entry and both entries of every bond, in CSC order
    std::vector<std::pair<int64_t, int64_t>> keys;  // (column, row), 0-based
    keys.reserve((size_t)(n + 2 * nbonds));
    for (int64_t i = 0; i < n; ++i) keys.push_back({i, i});
    for (int64_t b = 0; b < nbonds; ++b) {
        keys.push_back({dst[b] - 1, src[b] - 1});
        keys.push_back({src[b] - 1, dst[b] - 1});
    }
    std::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    const int64_t nnz = (int64_t)keys.size();
    std::vector<int64_t> colptr((size_t)n + 1, 0), rowval((size_t)nnz);
    for (int64_t p = 0; p < nnz; ++p) {
        colptr[(size_t)keys[(size_t)p].first + 1]++;
        rowval[(size_t)p] = keys[(size_t)p].second + 1;
    }
    colptr[0] = 1;
    for (int64_t j = 0; j < n; ++j) colptr[(size_t)j + 1] += colptr[(size_t)j];
    std::vector<double> zeros((size_t)(2 * nnz), 0.0);
    lm_ell* h = nullptr;
    int rc = lm_ell_create_csc(ctx, n, colptr.data(), rowval.data(), zeros.data(), &h);
    if (rc != LM_OK) return rc;
    // contributions of every entry, in bond order (forward entry, then reverse)
    auto entry = [&](int64_t row, int64_t col) {
        return (int64_t)(std::lower_bound(keys.begin(), keys.end(), std::make_pair(col, row)) - keys.begin());
    };
    std::vector<int64_t> cnt((size_t)nnz + 1, 0);
    std::vector<int64_t> pf((size_t)nbonds), pr((size_t)nbonds);
    for (int64_t b = 0; b < nbonds; ++b) {
        pf[(size_t)b] = entry(src[b] - 1, dst[b] - 1);
        pr[(size_t)b] = entry(dst[b] - 1, src[b] - 1);
        cnt[(size_t)pf[(size_t)b] + 1]++;
        cnt[(size_t)pr[(size_t)b] + 1]++;
    }
    for (int64_t p = 0; p < nnz; ++p) cnt[(size_t)p + 1] += cnt[(size_t)p];
    std::vector<int64_t> term((size_t)(2 * nbonds)), fillp(cnt.begin(), cnt.end() - 1);
    h->rad.assign((size_t)n, 0.0);
    for (int64_t b = 0; b < nbonds; ++b) {
        term[(size_t)fillp[(size_t)pf[(size_t)b]]++] = b << 1;
        term[(size_t)fillp[(size_t)pr[(size_t)b]]++] = (b << 1) | 1;
        const double a = hypot(base[2 * b], base[2 * b + 1]);
        h->rad[(size_t)(src[b] - 1)] += a;
        h->rad[(size_t)(dst[b] - 1)] += a;
    }
    h->nbonds = nbonds;
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaMalloc((void**)&h->d_bxy, sizeof(double) * (size_t)std::max<int64_t>(4 * nbonds, 1));
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d_bbase, sizeof(double2) * (size_t)std::max<int64_t>(nbonds, 1));
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d_eptr, sizeof(int64_t) * (size_t)(nnz + 1));
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d_eterm, sizeof(int64_t) * (size_t)std::max<int64_t>(2 * nbonds, 1));
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->d_emap, sizeof(int64_t) * (size_t)nnz);
    if (e == cudaSuccess && nbonds > 0) {
        e = cudaMemcpy(h->d_bxy, xy, sizeof(double) * (size_t)(4 * nbonds), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(h->d_bbase, base, sizeof(double2) * (size_t)nbonds, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(h->d_eterm, term.data(), sizeof(int64_t) * term.size(), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMemcpy(h->d_eptr, cnt.data(), sizeof(int64_t) * cnt.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_emap, h->map.data(), sizeof(int64_t) * (size_t)nnz, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaGetLastError();
        rc = check_cuda(ctx, e, "lm_ell_create_bonds: device tables");
        lm_ell_destroy(h);
        return rc;
    }
    ell_bond_bounds(h);
    *out = h;
    return LM_OK;
}

int lm_ell_add_field(lm_ell* h, int kind, double px, double py, int* component) {
    if (!h) return LM_ERR_ARG;
    lm_ctx* ctx = h->ctx;
    CHECK_ARG(ctx, h->d_eptr != nullptr, "lm_ell_add_field: the Hamiltonian was not built from bonds");
    CHECK_ARG(ctx, kind >= LM_FIELD_LANDAU && kind <= LM_FIELD_POINTFLUX_SINGULAR, "lm_ell_add_field: unknown field kind");
    CHECK_ARG(ctx, isfinite(px) && isfinite(py), "lm_ell_add_field: non-finite point");
    if (h->fields.n >= kMaxFields) return set_err(ctx, LM_ERR_NOTSUP, "lm_ell_add_field: too many field components");
    FieldComp fc{};
    fc.kind = kind;
    fc.px = px;
    fc.py = py;
    fc.replicate = 0;
    const int idx = h->fields.n;
    h->fields.c[idx] = fc;
    h->fields.amp[idx] = 0.0;
    h->fields.n++;
    h->assembled = 0;
    if (component) *component = idx;
    return LM_OK;
}

int lm_ell_set_onsite(lm_ell* h, const double* v) {
    if (!h) return LM_ERR_ARG;
    lm_ctx* ctx = h->ctx;
    CHECK_ARG(ctx, h->d_eptr != nullptr, "lm_ell_set_onsite: the Hamiltonian was not built from bonds");
    cudaSetDevice(ctx->device);
    if (!v) {
        h->h_onsite.clear();
    } else {
        for (int64_t i = 0; i < h->n; ++i) CHECK_ARG(ctx, isfinite(v[i]), "lm_ell_set_onsite: non-finite value");
        if (!h->d_onsite) {
            cudaError_t e = cudaMalloc((void**)&h->d_onsite, sizeof(double) * (size_t)h->n);
            if (e != cudaSuccess) {
                cudaGetLastError();
                h->d_onsite = nullptr;
                return check_cuda(ctx, e, "lm_ell_set_onsite: allocation");
            }
        }
        h->h_onsite.assign(v, v + h->n);
        // synchronous copy: the caller's array is free when the call returns
        CUDA_TRY(ctx, cudaMemcpyAsync(h->d_onsite, h->h_onsite.data(), sizeof(double) * (size_t)h->n,
                                      cudaMemcpyHostToDevice, ctx->stream), "lm_ell_set_onsite: upload");
        CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "lm_ell_set_onsite: synchronize");
    }
    ell_bond_bounds(h);
    h->assembled = 0;
    return LM_OK;
}

int lm_ell_assemble(lm_ell* h, const double* amplitudes, int namp) {
    if (!h) return LM_ERR_ARG;
    lm_ctx* ctx = h->ctx;
    CHECK_ARG(ctx, h->d_eptr != nullptr, "lm_ell_assemble: the Hamiltonian was not built from bonds");
    CHECK_ARG(ctx, namp == h->fields.n, "lm_ell_assemble: one amplitude per field component");
    for (int c = 0; c < namp; ++c) {
        CHECK_ARG(ctx, amplitudes && isfinite(amplitudes[c]), "lm_ell_assemble: non-finite amplitude");
        h->fields.amp[c] = amplitudes[c];
    }
    cudaSetDevice(ctx->device);
    ell_assemble_kernel<<<(unsigned)((h->nnz + 255) / 256), 256, 0, ctx->stream>>>(
        h->nnz, h->fields, h->d_bxy, h->d_bbase, h->d_eptr, h->d_eterm, h->d_emap,
        h->h_onsite.empty() ? nullptr : h->d_onsite, h->d_cval, h->d_vals, h->d_diag);
    ctx->launches++;
    CUDA_TRY(ctx, cudaGetLastError(), "lm_ell_assemble");
    h->version++;
    h->assembled = 1;
    return LM_OK;
}

int lm_ell_solver_update(lm_solver* s, lm_ell* h, double dt, int force) {
    if (!s) return LM_ERR_ARG;
    lm_ctx* ctx = s->ctx;
    CHECK_ARG(ctx, h != nullptr && h->ctx == ctx, "lm_ell_solver_update: bad Hamiltonian");
    CHECK_ARG(ctx, isfinite(dt), "lm_ell_solver_update: non-finite dt");
    // cache hit: same H and same factor -i*dt (src/evolution.jl:86-88)
    if (!force && s->valid && s->ell == h && s->ell_version == h->version &&
        fabs(dt - s->dt) <= 1.4901161193847656e-08 * std::max(fabs(dt), fabs(s->dt)))
        return LM_OK;
    cudaSetDevice(ctx->device);
    const int64_t tab = h->n * (int64_t)h->w;
    if (s->ell_tab != tab + h->n) {
        ell_free_tables(s);
        cudaError_t e = cudaMalloc((void**)&s->d_ev2, sizeof(double2) * (size_t)tab);
        if (e == cudaSuccess) e = cudaMalloc((void**)&s->d_ed2, sizeof(double) * (size_t)h->n);
        if (e == cudaSuccess) e = cudaMalloc((void**)&s->d_ev2f, sizeof(float2) * (size_t)tab);
        if (e == cudaSuccess) e = cudaMalloc((void**)&s->d_ed2f, sizeof(float) * (size_t)h->n);
        if (e != cudaSuccess) {
            cudaGetLastError();
            ell_free_tables(s);
            s->valid = 0;
            return check_cuda(ctx, e, "lm_ell_solver_update: tables");
        }
        s->ell_tab = tab + h->n;
    }
    plan_propagator(s, h->emin, h->emax, dt);
    const unsigned grid = (unsigned)std::min<int64_t>((tab + h->n + 255) / 256, 4096);
    ell_normalise_kernel<<<grid, 256, 0, ctx->stream>>>(h->n, h->w, h->d_vals, h->d_diag, s->a, s->b, s->d_ev2, s->d_ed2,
                                                        s->d_ev2f, s->d_ed2f);
    s->bpack_valid = 0;
    ctx->launches++;
    CUDA_TRY(ctx, cudaGetLastError(), "ell normalise kernel");
    s->ell = h;
    s->ell_version = h->version;
    s->ham = nullptr;
    s->dt = dt;
    s->valid = 1;
    return LM_OK;
}

int lm_ell_currents(lm_ell* h, lm_state* st, double* out) {
    if (!h) return LM_ERR_ARG;
    lm_ctx* ctx = h->ctx;
    CHECK_ARG(ctx, st != nullptr && st->ctx == ctx && st->n == h->n, "lm_ell_currents: state does not match");
    CHECK_ARG(ctx, out != nullptr, "lm_ell_currents: null output");
    if (h->nnz == 0) return LM_OK;
    cudaSetDevice(ctx->device);
    double* d_out = nullptr;
    CUDA_TRY(ctx, cudaMalloc((void**)&d_out, sizeof(double) * (size_t)h->nnz), "lm_ell_currents: allocation");
    const unsigned grid = (unsigned)std::min<int64_t>((h->nnz + 255) / 256, 65535);
    if (st->precision == LM_C64)
        ell_currents_kernel<double><<<grid, 256, 0, ctx->stream>>>(h->nnz, h->d_crow, h->d_ccol, h->d_cval, st->kind,
                                                                   (const double2*)st->d_data, st->m, st->ld, st->d_w, d_out);
    else
        ell_currents_kernel<float><<<grid, 256, 0, ctx->stream>>>(h->nnz, h->d_crow, h->d_ccol, h->d_cval, st->kind,
                                                                  (const float2*)st->d_data, st->m, st->ld, st->d_w, d_out);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, sizeof(double) * (size_t)h->nnz, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(d_out);
    return check_cuda(ctx, e, "lm_ell_currents");
}

int lm_ell_op_currents(lm_ell* h, lm_state* st, int ndof, const double* op, double* out) {
    if (!h) return LM_ERR_ARG;
    lm_ctx* ctx = h->ctx;
    CHECK_ARG(ctx, st != nullptr && st->ctx == ctx && st->n == h->n, "lm_ell_op_currents: state does not match");
    CHECK_ARG(ctx, out != nullptr, "lm_ell_op_currents: null output");
    LocalOp lop;
    const int rc = make_local_op(ctx, h, ndof, op, &lop, "lm_ell_op_currents");
    if (rc != LM_OK) return rc;
    if (h->nnz == 0) return LM_OK;
    cudaSetDevice(ctx->device);
    double* d_out = nullptr;
    CUDA_TRY(ctx, cudaMalloc((void**)&d_out, sizeof(double) * (size_t)h->nnz), "lm_ell_op_currents: allocation");
    cudaError_t e = launch_ell_op_currents(ctx, h, st, ndof, lop, d_out);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, sizeof(double) * (size_t)h->nnz, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(d_out);
    return check_cuda(ctx, e, "lm_ell_op_currents");
}

}  // extern "C"
