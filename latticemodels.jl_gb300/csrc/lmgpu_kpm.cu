// Kernel polynomial method: Chebyshev moments of the tight-binding Hamiltonian on the device,
// for the density of states and the local density of states without a full eigensystem (the
// reference computes dos / ldos from an Eigensystem or a GreenFunction, src/greenfunction.jl:
// 306-339).  The moments of a block of starting vectors v are
//   mu_n = sum_v <v| T_n(H~) |v>,   H~ = (H - b)/a,
// from the recurrence T_{n+1} = 2 H~ T_n - T_{n-1} on the block and the doubling relations
//   mu_2n = 2 <T_n v|T_n v> - mu_0,   mu_2n+1 = 2 <T_n+1 v|T_n v> - mu_1,
// so nmom moments take about nmom / 2 stencil passes.  With the N unit vectors as the block
// the sum is the exact trace and column j gives the local moments of site j.
//
// lm_cheb_apply evaluates a real Chebyshev series sum_n c_n T_n(H~) on a block (the identity
// gives the matrix function f(H) itself): the Fermi operator of densitymatrix at T > 0
// (src/spectrum.jl:226-257) without an eigensystem.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>

#include <new>
#include <utility>
#include <vector>

#include "lmgpu_internal.cuh"
#include "lmgpu_order.cuh"

namespace lmgpu {

// A = identity (n x n, leading dimension ld).
__global__ void set_identity_kernel(double2* __restrict__ a, int64_t n, int64_t ld) {
    for (int64_t col = blockIdx.y; col < n; col += gridDim.y)
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
            a[col * ld + i] = make_double2(i == col ? 1.0 : 0.0, 0.0);
}

// out[col] = Re sum_i conj(A[i, col]) B[i, col], one block per column (fixed-order reduction).
__global__ void __launch_bounds__(256) column_dots_kernel(const double2* __restrict__ A, const double2* __restrict__ B,
                                                          int64_t n, int64_t ld, int64_t M, double* __restrict__ out) {
    __shared__ double red[8];
    for (int64_t col = blockIdx.x; col < M; col += gridDim.x) {
        const double2* a = A + col * ld;
        const double2* b = B + col * ld;
        double acc = 0.0;
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
            const double2 x = a[i], y = b[i];
            acc = fma(x.x, y.x, fma(x.y, y.y, acc));
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w = 0; w < 8; ++w) t += red[w];
            out[col] = t;
        }
        __syncthreads();
    }
}

// y = y + c x (real c), n complex entries
__global__ void axpy_kernel(double2* __restrict__ y, const double2* __restrict__ x, double c, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double2 v = y[i];
        const double2 u = x[i];
        v.x = fma(c, u.x, v.x);
        v.y = fma(c, u.y, v.y);
        y[i] = v;
    }
}

// y = c x (real c)
__global__ void scaled_copy_kernel(double2* __restrict__ y, const double2* __restrict__ x, double c, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = make_double2(c * x[i].x, c * x[i].y);
}

// Lanczos start vector: entries of modulus 1/sqrt(n) with pseudo-random phases (splitmix64 of
// (seed, i)), so every eigenvector has a component in it almost surely.
__global__ void start_vector_kernel(double2* __restrict__ v, int64_t n, unsigned long long seed) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(i + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        const double phi = 6.283185307179586 * (double)(z >> 11) * (1.0 / 9007199254740992.0);
        double sn, cs;
        sincos(phi, &sn, &cs);
        const double r = rsqrt((double)n);
        v[i] = make_double2(r * cs, r * sn);
    }
}


// ------------------------------------------------------------------------------------------
// Double-float ("df") form of the moment recurrence (LM_OPT_KPM = 1, the default).  A real number is an
// unevaluated sum hi + lo of two FP32 values (about 48 significant bits), so the recurrence
// runs on the FP32 pipe instead of GB300's 1/64-rate FP64 pipe.  A complex df value is a float4
// {re.hi, re.lo, im.hi, im.lo}, the size of a double2, so the FP64 buffers are reused in place.
// Products take the exact FMA error term (p + e = a*b exactly); sums use the double-word
// addition of Dekker and of Knuth's TwoSum.  Every step is an explicit round-to-nearest
// intrinsic, which nvcc never contracts into an FMA or reorders, so the error-free
// transformations stay exact.  An exact emulation of this arithmetic keeps the moments within
// about 1e-14 of FP64 after 1024 passes.
// ------------------------------------------------------------------------------------------
struct DF {
    float h, l;
};
__device__ __forceinline__ DF df_fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_add(DF x, DF y) {
    const float s = __fadd_rn(x.h, y.h);
    const float bb = __fsub_rn(s, x.h);
    float e = __fadd_rn(__fsub_rn(x.h, __fsub_rn(s, bb)), __fsub_rn(y.h, bb));
    e = __fadd_rn(e, __fadd_rn(x.l, y.l));
    return df_fast_two_sum(s, e);
}
__device__ __forceinline__ DF df_mul(DF x, DF y) {
    const float p = __fmul_rn(x.h, y.h);
    float e = __fmaf_rn(x.h, y.h, -p);
    e = __fmaf_rn(x.h, y.l, e);
    e = __fmaf_rn(x.l, y.h, e);
    return df_fast_two_sum(p, e);
}
__device__ __forceinline__ DF df_neg(DF x) { return DF{-x.h, -x.l}; }
__device__ __forceinline__ DF df_re(float4 v) { return DF{v.x, v.y}; }
__device__ __forceinline__ DF df_im(float4 v) { return DF{v.z, v.w}; }
__device__ __forceinline__ DF df_from(double x) {
    const float h = (float)x;
    return DF{h, (float)(x - (double)h)};
}
__device__ __forceinline__ double df_value(DF x) { return (double)x.h + (double)x.l; }

// acc += h v on complex df values (h real when RE).
template <bool RE>
__device__ __forceinline__ void df_cfma(DF& ar, DF& ai, float4 h, float4 v) {
    ar = df_add(ar, df_mul(df_re(h), df_re(v)));
    if (!RE) ar = df_add(ar, df_neg(df_mul(df_im(h), df_im(v))));
    ai = df_add(ai, df_mul(df_re(h), df_im(v)));
    if (!RE) ai = df_add(ai, df_mul(df_im(h), df_re(v)));
}

// In place: n double2 values -> n float4 df values (same bytes per element).
__global__ void to_df_kernel(double2* __restrict__ a, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 v = a[i];
        const DF r = df_from(v.x), m = df_from(v.y);
        reinterpret_cast<float4*>(a)[i] = make_float4(r.h, r.l, m.h, m.l);
    }
}

// The stencil tables in df form: hop (2N double2) -> 2N float4, diag (N double) -> N float2.
__global__ void df_tables_kernel(const double2* __restrict__ hop2, const double* __restrict__ diag2, int64_t N,
                                 float4* __restrict__ hopd, float2* __restrict__ diagd) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < 2 * N; i += (int64_t)gridDim.x * blockDim.x) {
        const DF r = df_from(hop2[i].x), m = df_from(hop2[i].y);
        hopd[i] = make_float4(r.h, r.l, m.h, m.l);
        if (i < N) {
            const DF d = df_from(diag2[i]);
            diagd[i] = make_float2(d.h, d.l);
        }
    }
}

// In place: n float4 df values -> n double2 values.
__global__ void from_df_kernel(double2* __restrict__ a, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 v = reinterpret_cast<const float4*>(a)[i];
        a[i] = make_double2(df_value(DF{v.x, v.y}), df_value(DF{v.z, v.w}));
    }
}

// out = (2H~) tp - tpp on df blocks (the tables hold 2H/a and 2(V-b)/a); out may alias tpp.
// XR: every x-hop is real.  With y non-null also y += c out (c = c_hi + c_lo, the real
// coefficient of a Chebyshev series, lm_cheb_apply).
template <bool XR>
__global__ void __launch_bounds__(256) df_recur_kernel(Geom g, const float4* __restrict__ hopd,
                                                       const float2* __restrict__ diagd, const float4* tp,
                                                       const float4* tpp, float4* out, int64_t ld, int64_t M,
                                                       float4* __restrict__ y, float c_hi, float c_lo) {
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= g.N) return;
    const Nbr nb = neighbours(g, s);
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 hxp = nb.hxp ? hopd[s] : z, hyp = nb.hyp ? hopd[g.N + s] : z;
    float4 t = nb.hxm ? hopd[nb.xm] : z;
    const float4 hxm = make_float4(t.x, t.y, -t.z, -t.w);  // conj of the hop from x-1
    t = nb.hym ? hopd[g.N + nb.ym] : z;
    const float4 hym = make_float4(t.x, t.y, -t.z, -t.w);
    const float2 dd = diagd[s];
    const float4 d = make_float4(dd.x, dd.y, 0.f, 0.f);
    for (int64_t m = blockIdx.y; m < M; m += gridDim.y) {
        const int64_t o = m * ld;
        const float4 q = tpp[o + s];
        DF ar = DF{-q.x, -q.y}, ai = DF{-q.z, -q.w};
        df_cfma<XR>(ar, ai, hxp, tp[o + nb.xp]);
        df_cfma<XR>(ar, ai, hxm, tp[o + nb.xm]);
        df_cfma<false>(ar, ai, hyp, tp[o + nb.yp]);
        df_cfma<false>(ar, ai, hym, tp[o + nb.ym]);
        df_cfma<true>(ar, ai, d, tp[o + s]);
        out[o + s] = make_float4(ar.h, ar.l, ai.h, ai.l);
        if (y) {
            const float4 u = y[o + s];
            const DF c = DF{c_hi, c_lo};
            const DF yr = df_add(DF{u.x, u.y}, df_mul(c, ar)), yi = df_add(DF{u.z, u.w}, df_mul(c, ai));
            y[o + s] = make_float4(yr.h, yr.l, yi.h, yi.l);
        }
    }
}

// out[col] = Re <A, A>, out[M + col] = Re <B, A> per column, in df per thread and then the
// fixed-order FP64 block reduction of column_dots_kernel.
__global__ void __launch_bounds__(256) column_dots2_df_kernel(const float4* __restrict__ A,
                                                              const float4* __restrict__ B, int64_t n, int64_t ld,
                                                              int64_t M, double* __restrict__ out) {
    __shared__ double red[2][8];
    for (int64_t col = blockIdx.x; col < M; col += gridDim.x) {
        const float4* a = A + col * ld;
        const float4* b = B + col * ld;
        DF aa = DF{0.f, 0.f}, ba = DF{0.f, 0.f};
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
            const float4 x = a[i], y = b[i];
            aa = df_add(aa, df_mul(df_re(x), df_re(x)));
            aa = df_add(aa, df_mul(df_im(x), df_im(x)));
            ba = df_add(ba, df_mul(df_re(y), df_re(x)));
            ba = df_add(ba, df_mul(df_im(y), df_im(x)));
        }
        double v[2] = {df_value(aa), df_value(ba)};
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
            if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = v[q];
        }
        __syncthreads();
        if (threadIdx.x < 2) {
            double t = 0.0;
            for (int w = 0; w < 8; ++w) t += red[threadIdx.x][w];
            out[threadIdx.x * M + col] = t;
        }
        __syncthreads();
    }
}

}  // namespace lmgpu

using namespace lmgpu;

// Number of eigenvalues of the symmetric tridiagonal (a, b) below x (Sturm sequence count).
static int sturm_count(const std::vector<double>& a, const std::vector<double>& b, double x) {
    int cnt = 0;
    double q = 1.0;
    for (size_t i = 0; i < a.size(); ++i) {
        const double bb = i ? b[i - 1] * b[i - 1] : 0.0;
        q = (a[i] - x) - (i ? bb / q : 0.0);
        if (q == 0.0) q = -1e-300;
        if (q < 0.0) ++cnt;
    }
    return cnt;
}

// Last component of the unit eigenvector of the tridiagonal (a, b) for eigenvalue theta, by
// inverse iteration with a slightly shifted theta and Gaussian elimination with partial
// pivoting (the factor of a tridiagonal gains one extra superdiagonal).
static double tridiag_last_component(const std::vector<double>& a, const std::vector<double>& b, double theta) {
    const size_t m = a.size();
    if (m == 1) return 1.0;
    const double shift = theta + 1e-10 * (fabs(theta) + 1.0);
    std::vector<double> x(m, 1.0);
    for (int it = 0; it < 3; ++it) {
        // rows: lower l[i] (below diag), diag d[i], upper u1[i], u2[i] (second superdiagonal)
        std::vector<double> d(m), u1(m, 0.0), u2(m, 0.0), rhs(x);
        std::vector<double> l(m, 0.0);
        for (size_t i = 0; i < m; ++i) {
            d[i] = a[i] - shift;
            if (i + 1 < m) u1[i] = b[i];
            if (i > 0) l[i] = b[i - 1];
        }
        for (size_t i = 0; i + 1 < m; ++i) {
            // eliminate l[i+1] (row i+1, column i) with the larger of rows i, i+1 as pivot
            if (fabs(l[i + 1]) > fabs(d[i])) {
                std::swap(d[i], l[i + 1]);
                std::swap(u1[i], d[i + 1]);
                std::swap(u2[i], u1[i + 1]);
                std::swap(rhs[i], rhs[i + 1]);
            }
            const double piv = d[i] != 0.0 ? d[i] : 1e-300;
            const double f = l[i + 1] / piv;
            d[i + 1] -= f * u1[i];
            u1[i + 1] -= f * u2[i];
            rhs[i + 1] -= f * rhs[i];
            l[i + 1] = 0.0;
        }
        for (size_t ii = m; ii-- > 0;) {
            double v = rhs[ii];
            if (ii + 1 < m) v -= u1[ii] * x[ii + 1];
            if (ii + 2 < m) v -= u2[ii] * x[ii + 2];
            x[ii] = v / (d[ii] != 0.0 ? d[ii] : 1e-300);
        }
        double nrm = 0.0;
        for (double v : x) nrm += v * v;
        nrm = sqrt(nrm);
        if (!(nrm > 0.0) || !isfinite(nrm)) return 1.0;  // fall back to the crude bound
        for (double& v : x) v /= nrm;
    }
    return x[m - 1];
}

// The k-th smallest eigenvalue (k = 0 .. m-1) of the tridiagonal by bisection.
static double tridiag_eig(const std::vector<double>& a, const std::vector<double>& b, int k, double lo, double hi) {
    for (int it = 0; it < 200 && hi - lo > 1e-14 * (fabs(lo) + fabs(hi) + 1e-300); ++it) {
        const double mid = 0.5 * (lo + hi);
        if (sturm_count(a, b, mid) > k) hi = mid;
        else lo = mid;
    }
    return 0.5 * (lo + hi);
}

extern "C" {

int lm_kpm_moments(lm_ham* h, double emin, double emax, int nmom, const lm_state* vecs, int per_column,
                   double* out) {
    if (!h) return LM_ERR_ARG;
    lm_ctx* ctx = h->ctx;
    CHECK_ARG(ctx, out != nullptr, "lm_kpm_moments: null output");
    CHECK_ARG(ctx, nmom >= 1, "lm_kpm_moments: need at least one moment");
    CHECK_ARG(ctx, isfinite(emin) && isfinite(emax) && emax > emin, "lm_kpm_moments: need emin < emax");
    if (!h->assembled) return set_err(ctx, LM_ERR_STATE, "lm_kpm_moments: Hamiltonian not assembled");
    const Geom& g = h->lat->g;
    const int64_t N = g.N;
    if (vecs) {
        CHECK_ARG(ctx, vecs->ctx == ctx && vecs->n == N, "lm_kpm_moments: vectors do not match the lattice");
        CHECK_ARG(ctx, vecs->kind == LM_KETS && vecs->precision == LM_C64,
                  "lm_kpm_moments: vectors must be a ComplexF64 ket block");
    }
    const int64_t M = vecs ? vecs->m : N;
    const int64_t ld = vecs ? vecs->ld : N;
    const double a = 0.5 * (emax - emin), b = 0.5 * (emax + emin);
    const int64_t nsteps = (nmom + 1) / 2;  // recurrence passes: T_0 .. T_nsteps
    cudaSetDevice(ctx->device);

    double2* hop2 = nullptr;
    double* diag2 = nullptr;
    float2* hop2f = nullptr;
    float* diag2f = nullptr;
    double2* TA = nullptr;
    double2* TB = nullptr;
    double* dots = nullptr;
    float4* hopd = nullptr;  // double-float tables (LM_OPT_KPM, default on)
    float2* diagd = nullptr;
    const bool use_df = ctx->kpm_df != 0;
    const size_t blk = sizeof(double2) * (size_t)ld * (size_t)M;
    const size_t ndots = (size_t)(nsteps + 1) * 2 * (size_t)M;
    auto release = [&]() {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(hop2); cudaFree(diag2); cudaFree(hop2f); cudaFree(diag2f);
        cudaFree(TA); cudaFree(TB); cudaFree(dots); cudaFree(hopd); cudaFree(diagd);
    };
    cudaError_t e = cudaMalloc((void**)&hop2, sizeof(double2) * 2 * (size_t)N);
    if (e == cudaSuccess) e = cudaMalloc((void**)&diag2, sizeof(double) * (size_t)N);
    if (e == cudaSuccess) e = cudaMalloc((void**)&hop2f, sizeof(float2) * 2 * (size_t)N);
    if (e == cudaSuccess) e = cudaMalloc((void**)&diag2f, sizeof(float) * (size_t)N);
    if (e == cudaSuccess) e = cudaMalloc((void**)&TA, blk);
    if (e == cudaSuccess) e = cudaMalloc((void**)&TB, blk);
    if (e == cudaSuccess) e = cudaMalloc((void**)&dots, sizeof(double) * ndots);
    if (e == cudaSuccess && use_df) e = cudaMalloc((void**)&hopd, sizeof(float4) * 2 * (size_t)N);
    if (e == cudaSuccess && use_df) e = cudaMalloc((void**)&diagd, sizeof(float2) * (size_t)N);
    if (e != cudaSuccess) {
        cudaGetLastError();
        release();
        return check_cuda(ctx, e, "lm_kpm_moments: allocation");
    }
    auto fail = [&](cudaError_t err, const char* what) {
        const int rc = check_cuda(ctx, err, what);
        release();
        return rc;
    };
    e = launch_normalise(ctx, g, h->d_hop, h->d_onsite, a, b, hop2, diag2, hop2f, diag2f);
    if (e != cudaSuccess) return fail(e, "lm_kpm_moments: tables");
    if (vecs) {
        e = cudaMemcpy2DAsync(TA, sizeof(double2) * (size_t)ld, vecs->d_data, sizeof(double2) * (size_t)vecs->ld,
                              sizeof(double2) * (size_t)N, (size_t)M, cudaMemcpyDeviceToDevice, ctx->stream);
    } else {
        const dim3 grid((unsigned)((N + 255) / 256), (unsigned)(N < 65535 ? N : 65535));
        set_identity_kernel<<<grid, 256, 0, ctx->stream>>>(TA, N, ld);
        ctx->launches++;
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return fail(e, "lm_kpm_moments: starting block");
    const unsigned dgrid = (unsigned)(M < 65535 ? M : 65535);
    // T_1 = H~ T_0
    const bool xr = ham_x_real(h);
    e = launch_stencil_recur(ctx, g, LM_C64, hop2, diag2, TA, nullptr, nullptr, TB, ld, M, 0.5, 0.0, 0.0, nullptr, 0.0,
                             xr);
    if (e != cudaSuccess) return fail(e, "lm_kpm_moments: recurrence");
    if (use_df) {  // T_0 and T_1 (FP64) become double-float in place; so do the tables
        const unsigned cgrid = (unsigned)std::min<int64_t>((ld * M + 255) / 256, 65535);
        df_tables_kernel<<<(unsigned)std::min<int64_t>((2 * N + 255) / 256, 65535), 256, 0, ctx->stream>>>(
            hop2, diag2, N, hopd, diagd);
        to_df_kernel<<<cgrid, 256, 0, ctx->stream>>>(TA, ld * M);
        to_df_kernel<<<cgrid, 256, 0, ctx->stream>>>(TB, ld * M);
        ctx->launches += 3;
        e = cudaGetLastError();
        if (e != cudaSuccess) return fail(e, "lm_kpm_moments: double-float conversion");
    }
    const dim3 rgrid((unsigned)((N + 255) / 256), (unsigned)(M < 65535 ? M : 65535));
    double2* Tn = TA;   // T_n
    double2* Tn1 = TB;  // T_{n+1}
    for (int64_t n = 0; n <= nsteps; ++n) {
        double* d = dots + (size_t)n * 2 * (size_t)M;
        if (use_df) {
            column_dots2_df_kernel<<<dgrid, 256, 0, ctx->stream>>>((const float4*)Tn, (const float4*)Tn1, N, ld, M, d);
            ctx->launches += 1;
        } else {
            column_dots_kernel<<<dgrid, 256, 0, ctx->stream>>>(Tn, Tn, N, ld, M, d);
            column_dots_kernel<<<dgrid, 256, 0, ctx->stream>>>(Tn1, Tn, N, ld, M, d + M);
            ctx->launches += 2;
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) return fail(e, "lm_kpm_moments: dots");
        if (n == nsteps) break;
        // T_{n+2} = 2 H~ T_{n+1} - T_n, written over T_n
        if (use_df) {
            if (xr) df_recur_kernel<true><<<rgrid, 256, 0, ctx->stream>>>(g, hopd, diagd, (const float4*)Tn1,
                                                                          (const float4*)Tn, (float4*)Tn, ld, M,
                                                                          nullptr, 0.f, 0.f);
            else df_recur_kernel<false><<<rgrid, 256, 0, ctx->stream>>>(g, hopd, diagd, (const float4*)Tn1,
                                                                        (const float4*)Tn, (float4*)Tn, ld, M,
                                                                        nullptr, 0.f, 0.f);
            ctx->launches++;
            e = cudaGetLastError();
        } else {
            e = launch_stencil_recur(ctx, g, LM_C64, hop2, diag2, Tn1, Tn, nullptr, Tn, ld, M, 1.0, 0.0, 0.0, nullptr,
                                     0.0, xr);
        }
        if (e != cudaSuccess) return fail(e, "lm_kpm_moments: recurrence");
        std::swap(Tn, Tn1);
    }
    std::vector<double> hd(ndots);
    e = cudaMemcpyAsync(hd.data(), dots, sizeof(double) * ndots, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return fail(e, "lm_kpm_moments: download");
    release();
    // assemble the moments column by column (sums over columns in column order)
    const double* d0 = hd.data();
    for (int64_t col = 0; col < (per_column ? M : 1); ++col) {
        for (int k = 0; k < nmom; ++k) {
            const int64_t n = k / 2;
            double v = 0.0;
            for (int64_t c = per_column ? col : 0; c < (per_column ? col + 1 : M); ++c) {
                const double mu0 = d0[c], mu1 = d0[M + c];
                const double nn = d0[(size_t)n * 2 * M + c], n1n = d0[(size_t)n * 2 * M + M + c];
                v += (k == 0) ? mu0 : (k == 1) ? mu1 : (k % 2 == 0 ? 2.0 * nn - mu0 : 2.0 * n1n - mu1);
            }
            out[(size_t)col * (size_t)nmom + (size_t)k] = v;
        }
    }
    // |T_n(x)| <= 1 on [-1, 1]: larger moments mean that [emin, emax] misses part of the spectrum
    for (int64_t col = 0; col < (per_column ? M : 1); ++col) {
        const double* mu = out + (size_t)col * (size_t)nmom;
        for (int k = 1; k < nmom; ++k)
            if (!(fabs(mu[k]) <= fabs(mu[0]) * (1.0 + 1e-6) + 1e-12))
                return set_err(ctx, LM_ERR_NONFINITE,
                               "lm_kpm_moments: moments grow: [emin, emax] does not enclose the spectrum");
    }
    return LM_OK;
}

int lm_cheb_apply(lm_ham* h, double emin, double emax, const double* coef, int ncoef, const lm_state* in,
                  lm_state* out) {
    if (!h) return LM_ERR_ARG;
    lm_ctx* ctx = h->ctx;
    CHECK_ARG(ctx, coef != nullptr && ncoef >= 1, "lm_cheb_apply: need at least one coefficient");
    CHECK_ARG(ctx, out != nullptr && out->ctx == ctx, "lm_cheb_apply: bad output state");
    CHECK_ARG(ctx, isfinite(emin) && isfinite(emax) && emax > emin, "lm_cheb_apply: need emin < emax");
    for (int k = 0; k < ncoef; ++k) CHECK_ARG(ctx, isfinite(coef[k]), "lm_cheb_apply: non-finite coefficient");
    if (!h->assembled) return set_err(ctx, LM_ERR_STATE, "lm_cheb_apply: Hamiltonian not assembled");
    const Geom& g = h->lat->g;
    const int64_t N = g.N;
    if (in) CHECK_ARG(ctx, in->ctx == ctx && in->n == N, "lm_cheb_apply: input does not match the lattice");
    const int64_t M = in ? in->m : N;
    CHECK_ARG(ctx, out->n == N && out->m == M, "lm_cheb_apply: output shape differs from the input");
    const double a = 0.5 * (emax - emin), b = 0.5 * (emax + emin);
    cudaSetDevice(ctx->device);
    double2* hop2 = nullptr;
    double* diag2 = nullptr;
    float2* hop2f = nullptr;
    float* diag2f = nullptr;
    double2* TA = nullptr;
    double2* TB = nullptr;
    double2* Y = nullptr;
    float4* hopd = nullptr;  // double-float tables (LM_OPT_KPM, default on)
    float2* diagd = nullptr;
    const bool use_df = ctx->kpm_df != 0 && ncoef > 2;
    const int64_t ld = N;
    const size_t blk = sizeof(double2) * (size_t)ld * (size_t)M;
    auto release = [&]() {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(hop2); cudaFree(diag2); cudaFree(hop2f); cudaFree(diag2f);
        cudaFree(TA); cudaFree(TB); cudaFree(Y); cudaFree(hopd); cudaFree(diagd);
    };
    cudaError_t e = cudaMalloc((void**)&hop2, sizeof(double2) * 2 * (size_t)N);
    if (e == cudaSuccess) e = cudaMalloc((void**)&diag2, sizeof(double) * (size_t)N);
    if (e == cudaSuccess) e = cudaMalloc((void**)&hop2f, sizeof(float2) * 2 * (size_t)N);
    if (e == cudaSuccess) e = cudaMalloc((void**)&diag2f, sizeof(float) * (size_t)N);
    if (e == cudaSuccess) e = cudaMalloc((void**)&TA, blk);
    if (e == cudaSuccess && ncoef > 1) e = cudaMalloc((void**)&TB, blk);
    if (e == cudaSuccess) e = cudaMalloc((void**)&Y, blk);
    if (e == cudaSuccess && use_df) e = cudaMalloc((void**)&hopd, sizeof(float4) * 2 * (size_t)N);
    if (e == cudaSuccess && use_df) e = cudaMalloc((void**)&diagd, sizeof(float2) * (size_t)N);
    if (e != cudaSuccess) {
        cudaGetLastError();
        release();
        return check_cuda(ctx, e, "lm_cheb_apply: allocation");
    }
    auto fail = [&](cudaError_t err, const char* what) {
        const int rc = check_cuda(ctx, err, what);
        release();
        return rc;
    };
    e = launch_normalise(ctx, g, h->d_hop, h->d_onsite, a, b, hop2, diag2, hop2f, diag2f);
    if (e != cudaSuccess) return fail(e, "lm_cheb_apply: tables");
    // T_0
    if (!in) {
        const dim3 grid((unsigned)((N + 255) / 256), (unsigned)(N < 65535 ? N : 65535));
        set_identity_kernel<<<grid, 256, 0, ctx->stream>>>(TA, N, ld);
        ctx->launches++;
        e = cudaGetLastError();
    } else if (in->precision == LM_C64) {
        e = cudaMemcpy2DAsync(TA, sizeof(double2) * (size_t)ld, in->d_data, sizeof(double2) * (size_t)in->ld,
                              sizeof(double2) * (size_t)N, (size_t)M, cudaMemcpyDeviceToDevice, ctx->stream);
    } else {
        e = launch_convert(ctx, LM_C64, in->d_data, TA, N, M, in->ld, ld);
    }
    if (e != cudaSuccess) return fail(e, "lm_cheb_apply: input block");
    // Y = c_0 T_0
    e = cudaMemcpyAsync(Y, TA, blk, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e == cudaSuccess) e = launch_scale(ctx, LM_C64, Y, N, M, ld, coef[0], 0.0);
    if (e != cudaSuccess) return fail(e, "lm_cheb_apply: first term");
    if (ncoef > 1) {
        // T_1 = H~ T_0, Y += c_1 T_1; then T_{n+1} = 2 H~ T_n - T_{n-1} over T_{n-1}, Y += c_{n+1} T_{n+1}
        const bool xr = ham_x_real(h);
        e = launch_stencil_recur(ctx, g, LM_C64, hop2, diag2, TA, nullptr, nullptr, TB, ld, M, 0.5, 0.0, 0.0, Y,
                                 coef[1], xr);
        if (e != cudaSuccess) return fail(e, "lm_cheb_apply: recurrence");
        double2* Tprev = TA;
        double2* Tn = TB;
        const unsigned cgrid = (unsigned)std::min<int64_t>((ld * M + 255) / 256, 65535);
        if (use_df) {  // T_0, T_1 and Y (FP64 so far) become double-float in place; so do the tables
            df_tables_kernel<<<(unsigned)std::min<int64_t>((2 * N + 255) / 256, 65535), 256, 0, ctx->stream>>>(
                hop2, diag2, N, hopd, diagd);
            to_df_kernel<<<cgrid, 256, 0, ctx->stream>>>(TA, ld * M);
            to_df_kernel<<<cgrid, 256, 0, ctx->stream>>>(TB, ld * M);
            to_df_kernel<<<cgrid, 256, 0, ctx->stream>>>(Y, ld * M);
            ctx->launches += 4;
            e = cudaGetLastError();
            if (e != cudaSuccess) return fail(e, "lm_cheb_apply: double-float conversion");
        }
        const dim3 rgrid((unsigned)((N + 255) / 256), (unsigned)(M < 65535 ? M : 65535));
        for (int k = 2; k < ncoef; ++k) {
            if (use_df) {
                const float c_hi = (float)coef[k], c_lo = (float)(coef[k] - (double)c_hi);
                if (xr) df_recur_kernel<true><<<rgrid, 256, 0, ctx->stream>>>(g, hopd, diagd, (const float4*)Tn,
                                                                              (const float4*)Tprev, (float4*)Tprev,
                                                                              ld, M, (float4*)Y, c_hi, c_lo);
                else df_recur_kernel<false><<<rgrid, 256, 0, ctx->stream>>>(g, hopd, diagd, (const float4*)Tn,
                                                                            (const float4*)Tprev, (float4*)Tprev,
                                                                            ld, M, (float4*)Y, c_hi, c_lo);
                ctx->launches++;
                e = cudaGetLastError();
            } else {
                e = launch_stencil_recur(ctx, g, LM_C64, hop2, diag2, Tn, Tprev, nullptr, Tprev, ld, M, 1.0, 0.0, 0.0,
                                         Y, coef[k], xr);
            }
            if (e != cudaSuccess) return fail(e, "lm_cheb_apply: recurrence");
            std::swap(Tprev, Tn);
        }
        if (use_df) {
            from_df_kernel<<<cgrid, 256, 0, ctx->stream>>>(Y, ld * M);
            ctx->launches++;
            e = cudaGetLastError();
            if (e != cudaSuccess) return fail(e, "lm_cheb_apply: double-float conversion");
        }
    }
    if (out->precision == LM_C64)
        e = cudaMemcpy2DAsync(out->d_data, sizeof(double2) * (size_t)out->ld, Y, sizeof(double2) * (size_t)ld,
                              sizeof(double2) * (size_t)N, (size_t)M, cudaMemcpyDeviceToDevice, ctx->stream);
    else
        e = launch_convert(ctx, LM_C32, Y, out->d_data, N, M, ld, out->ld);
    if (e != cudaSuccess) return fail(e, "lm_cheb_apply: output");
    release();
    return LM_OK;
}

int lm_ham_lanczos_bounds(lm_ham* h, int iters, unsigned long long seed, double* emin, double* emax) {
    if (!h) return LM_ERR_ARG;
    lm_ctx* ctx = h->ctx;
    CHECK_ARG(ctx, emin && emax, "lm_ham_lanczos_bounds: null output");
    CHECK_ARG(ctx, iters >= 2 && iters <= 10000, "lm_ham_lanczos_bounds: iters must be in 2..10000");
    if (!h->assembled) return set_err(ctx, LM_ERR_STATE, "lm_ham_lanczos_bounds: Hamiltonian not assembled");
    const Geom& g = h->lat->g;
    const int64_t N = g.N;
    double glo = 0.0, ghi = 0.0;
    lm_ham_bounds(h, &glo, &ghi);
    const int m = (int)std::min<int64_t>(iters, N);
    cudaSetDevice(ctx->device);
    double2* hop2 = nullptr;
    double* diag2 = nullptr;
    float2* hop2f = nullptr;
    float* diag2f = nullptr;
    double2* buf = nullptr;  // three vectors
    double* dot = nullptr;
    auto release = [&]() {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(hop2); cudaFree(diag2); cudaFree(hop2f); cudaFree(diag2f); cudaFree(buf); cudaFree(dot);
    };
    cudaError_t e = cudaMalloc((void**)&hop2, sizeof(double2) * 2 * (size_t)N);
    if (e == cudaSuccess) e = cudaMalloc((void**)&diag2, sizeof(double) * (size_t)N);
    if (e == cudaSuccess) e = cudaMalloc((void**)&hop2f, sizeof(float2) * 2 * (size_t)N);
    if (e == cudaSuccess) e = cudaMalloc((void**)&diag2f, sizeof(float) * (size_t)N);
    if (e == cudaSuccess) e = cudaMalloc((void**)&buf, sizeof(double2) * 3 * (size_t)N);
    if (e == cudaSuccess) e = cudaMalloc((void**)&dot, sizeof(double));
    if (e != cudaSuccess) {
        cudaGetLastError();
        release();
        return check_cuda(ctx, e, "lm_ham_lanczos_bounds: allocation");
    }
    auto fail = [&](cudaError_t err, const char* what) {
        const int rc = check_cuda(ctx, err, what);
        release();
        return rc;
    };
    // tables for a = 2, b = 0 hold H itself: the recurrence kernel then computes H v - u
    e = launch_normalise(ctx, g, h->d_hop, h->d_onsite, 2.0, 0.0, hop2, diag2, hop2f, diag2f);
    if (e != cudaSuccess) return fail(e, "lm_ham_lanczos_bounds: tables");
    double2* A = buf;          // v_j
    double2* B = buf + N;      // beta_{j-1} v_{j-1}
    double2* Cw = buf + 2 * N; // w
    const unsigned grid = (unsigned)std::min<int64_t>((N + 255) / 256, 4096);
    start_vector_kernel<<<grid, 256, 0, ctx->stream>>>(A, N, seed);
    e = cudaMemsetAsync(B, 0, sizeof(double2) * (size_t)N, ctx->stream);
    if (e != cudaSuccess) return fail(e, "lm_ham_lanczos_bounds: start");
    std::vector<double> al, be;
    auto read_dot = [&](const double2* x, const double2* y, double* v) -> cudaError_t {
        column_dots_kernel<<<1, 256, 0, ctx->stream>>>(x, y, N, N, 1, dot);
        cudaError_t err = cudaGetLastError();
        if (err == cudaSuccess) err = cudaMemcpyAsync(v, dot, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
        if (err == cudaSuccess) err = cudaStreamSynchronize(ctx->stream);
        return err;
    };
    for (int j = 0; j < m; ++j) {
        // w = H v_j - beta_{j-1} v_{j-1}
        e = launch_stencil_recur(ctx, g, LM_C64, hop2, diag2, A, B, nullptr, Cw, N, 1, 1.0, 0.0, 0.0, nullptr, 0.0,
                                 ham_x_real(h));
        double alpha = 0.0, bsq = 0.0;
        if (e == cudaSuccess) e = read_dot(A, Cw, &alpha);
        if (e == cudaSuccess) {
            axpy_kernel<<<grid, 256, 0, ctx->stream>>>(Cw, A, -alpha, N);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = read_dot(Cw, Cw, &bsq);
        if (e != cudaSuccess) return fail(e, "lm_ham_lanczos_bounds: iteration");
        al.push_back(alpha);
        const double beta = sqrt(std::max(bsq, 0.0));
        if (j == m - 1 || beta <= 1e-12 * (fabs(ghi) + fabs(glo))) {
            be.push_back(beta);
            break;  // invariant subspace (or the last step): the tridiagonal is complete
        }
        be.push_back(beta);
        // B = beta v_j, v_{j+1} = w / beta, rotate the buffers
        scaled_copy_kernel<<<grid, 256, 0, ctx->stream>>>(B, A, beta, N);
        scaled_copy_kernel<<<grid, 256, 0, ctx->stream>>>(Cw, Cw, 1.0 / beta, N);
        e = cudaGetLastError();
        if (e != cudaSuccess) return fail(e, "lm_ham_lanczos_bounds: iteration");
        std::swap(A, Cw);
    }
    release();
    const int k = (int)al.size();
    std::vector<double> offd(be.begin(), be.begin() + (k - 1));
    const double lo = tridiag_eig(al, offd, 0, glo - 1.0, ghi + 1.0);
    const double hi = tridiag_eig(al, offd, k - 1, glo - 1.0, ghi + 1.0);
    // Ritz values lie inside the spectrum; pad each extreme by its residual beta_m |s_m| (an
    // eigenvalue lies within it) plus 1 % of the width, and never leave the Gershgorin interval
    const double rlo = be.back() * fabs(tridiag_last_component(al, offd, lo));
    const double rhi = be.back() * fabs(tridiag_last_component(al, offd, hi));
    const double w = 0.01 * (hi - lo);
    *emin = std::max(glo, lo - rlo - w);
    *emax = std::min(ghi, hi + rhi + w);
    return LM_OK;
}

}  // extern "C"
