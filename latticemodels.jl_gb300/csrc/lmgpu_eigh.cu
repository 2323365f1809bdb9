// Hermitian eigensystem on the device (FP64): the eigensolver behind diagonalize and
// densitymatrix (src/spectrum.jl:48-55, :226-257, :317-333), with no vendor library.
//
//   1. The assembled H is written as a dense N x N matrix (column-major).
//   2. Householder reduction to a real symmetric tridiagonal T = Q^H H Q, on the lower
//      triangle: per column one reflector (house_kernel), the symmetric product p = A v over
//      64 x 64 tiles with fixed-order partial sums (hemv_tiles_kernel, hemv_reduce_kernel),
//      and the rank-2 update A -= v w^H + w v^H of the lower tiles (her2_tiles_kernel).  The
//      reflectors stay in the strictly lower part of the matrix, as LAPACK's zhetrd keeps them
//      (Q = H_0 H_1 ... H_{n-2}, H_j = I - tau_j v_j v_j^H, v_j[0] = 1 at row j + 1).
//   3. T splits where an off-diagonal is below 2^-50 |T|; every eigenvalue of every block
//      comes from Sturm-count bisection to machine precision (one thread per eigenvalue).
//   4. Eigenvectors of T by inverse iteration with a pivoted tridiagonal LU, three solves from
//      a pseudo-random start; eigenvalues of a block closer than 1e-5 |T| form a cluster that
//      one thread computes in order, orthogonalising each iterate against the cluster's earlier
//      vectors (exactly degenerate levels of H sit in different blocks).
//   5. Back-transformation X = Q Z, one reflector per launch, and the weighted projector
//      P = sum_k w_k x_k x_k^H over 64 x 64 lower tiles, accumulated over vector chunks.
//
// GB300 runs FP64 at about two FMAs per clock per SM, so every stage is bound by its FP64
// FMAs: the kernels spend none on anything else (complex products are four DFMAs).
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <numeric>
#include <vector>

#include "lmgpu_internal.cuh"
#include "lmgpu_order.cuh"

namespace {

using namespace lmgpu;

constexpr int kTile = 64;             // tile side of the tridiagonalisation and projector kernels
constexpr int kChunk = 1024;          // eigenvectors per back-transformation chunk
constexpr double kSplitRel = 8.881784197001252e-16;  // 2^-50: off-diagonals below kSplitRel |T| split T
constexpr double kClusterRel = 1e-5;  // eigenvalues closer than kClusterRel |T| form a cluster

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 c) {  // a*b + c
    return make_double2(fma(a.x, b.x, fma(-a.y, b.y, c.x)), fma(a.x, b.y, fma(a.y, b.x, c.y)));
}
__device__ __forceinline__ double2 cfma_conj(double2 a, double2 b, double2 c) {  // conj(a)*b + c
    return make_double2(fma(a.x, b.x, fma(a.y, b.y, c.x)), fma(a.x, b.y, fma(-a.y, b.x, c.y)));
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 conjd(double2 a) { return make_double2(a.x, -a.y); }

// ------------------------------------------------------------------------------------------
// 1. Dense assembly.  Square lattice: thread per column c accumulates every entry of column c
// in a fixed order (on-site, then the four bonds), so parallel bonds of a 2-site ring add up
// as the reference's builder adds them (src/operators/builder.jl:296-309).
// ------------------------------------------------------------------------------------------
__global__ void dense_square_kernel(Geom g, const double2* __restrict__ hop, const double* __restrict__ onsite,
                                    double2* __restrict__ A, int64_t lda) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.N) return;
    double2* col = A + c * lda;
    const Nbr nb = neighbours(g, c);
    col[c] = cadd(col[c], make_double2(onsite ? onsite[c] : 0.0, 0.0));
    if (nb.hxp) col[nb.xp] = cadd(col[nb.xp], conjd(hop[c]));            // H[xp, c] = conj(H[c, xp])
    if (nb.hxm) col[nb.xm] = cadd(col[nb.xm], hop[nb.xm]);               // H[xm, c] (the +x bond of xm)
    if (nb.hyp) col[nb.yp] = cadd(col[nb.yp], conjd(hop[g.N + c]));
    if (nb.hym) col[nb.ym] = cadd(col[nb.ym], hop[g.N + nb.ym]);
}

// General sparse H in ELL form: thread per row i adds its stored entries in slot order.
__global__ void dense_ell_kernel(int64_t n, int w, const int* __restrict__ cols, const double2* __restrict__ vals,
                                 const double* __restrict__ diag, double2* __restrict__ A, int64_t lda) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    A[i + i * lda] = cadd(A[i + i * lda], make_double2(diag[i], 0.0));
    for (int k = 0; k < w; ++k) {
        const int64_t c = cols[(int64_t)k * n + i];
        A[i + c * lda] = cadd(A[i + c * lda], vals[(int64_t)k * n + i]);
    }
}

// ------------------------------------------------------------------------------------------
// 2. Householder tridiagonalisation.
// ------------------------------------------------------------------------------------------
// Block-wide sum in a fixed order (deterministic): every thread passes its partial.
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sh) {
    const int t = threadIdx.x;
    sh[t] = v;
    __syncthreads();
#pragma unroll
    for (int s = NT / 2; s > 0; s >>= 1) {
        if (t < s) sh[t] += sh[t + s];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

// Reflector of column j: x = A[j+1:n, j], alpha = x[0].  H = I - tau v v^H with v = (1,
// x[1:]/(alpha - beta)) maps x to (beta, 0, ...), beta real (the zlarfg convention).  Writes
// d[j], e[j], tau[j], the scaled x back into A and v into vbuf; tau = 0 when x is already
// (real, 0, ...).
__global__ void __launch_bounds__(1024) house_kernel(double2* __restrict__ A, int64_t lda, int64_t n, int64_t j,
                                                     double* __restrict__ d, double* __restrict__ e,
                                                     double2* __restrict__ tau, double2* __restrict__ vbuf) {
    __shared__ double sh[1024];
    const int64_t m = n - 1 - j;  // length of x
    double2* x = A + (j + 1) + j * lda;
    // alpha is read before the reduction's barriers: thread 0 overwrites x[0] at the end
    const double2 alpha = x[0];
    double part = 0.0;
    for (int64_t i = 1 + threadIdx.x; i < m; i += blockDim.x) part = fma(x[i].x, x[i].x, fma(x[i].y, x[i].y, part));
    const double xn2 = block_sum<1024>(part, sh);
    double beta;
    double2 tv;
    double2 scal = make_double2(1.0, 0.0);
    if (xn2 == 0.0 && alpha.y == 0.0) {
        beta = alpha.x;
        tv = make_double2(0.0, 0.0);
    } else {
        const double nrm = sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xn2);
        beta = alpha.x >= 0.0 ? -nrm : nrm;
        tv = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
        const double2 den = make_double2(alpha.x - beta, alpha.y);  // 1 / (alpha - beta)
        const double dd = den.x * den.x + den.y * den.y;
        scal = make_double2(den.x / dd, -den.y / dd);
    }
    for (int64_t i = 1 + threadIdx.x; i < m; i += blockDim.x) {
        const double2 v = (tv.x != 0.0 || tv.y != 0.0) ? cmul(x[i], scal) : x[i];
        x[i] = v;
        vbuf[i] = v;
    }
    if (threadIdx.x == 0) {
        vbuf[0] = make_double2(1.0, 0.0);
        x[0] = make_double2(beta, 0.0);
        d[j] = A[j + j * lda].x;
        e[j] = beta;
        tau[j] = tv;
    }
}

// p = A22 v over the lower tiles of the trailing matrix A22 = A[o:n, o:n] (o = j + 1).  Tile
// (I, J), I >= J: part1[J][r] = sum over tile columns of A[r, c] v[c] for r in tile I, and for
// I > J part2[I][c] = sum over tile rows of conj(A[r, c]) v[r] for c in tile J.  The diagonal
// tile takes its upper half from the conjugate of the lower half.
__global__ void __launch_bounds__(256) hemv_tiles_kernel(const double2* __restrict__ A, int64_t lda, int64_t o,
                                                         int64_t m, int nt, const double2* __restrict__ v,
                                                         const double2* __restrict__ tau_j,
                                                         double2* __restrict__ part1, double2* __restrict__ part2) {
    if (tau_j->x == 0.0 && tau_j->y == 0.0) return;
    extern __shared__ double2 S[];  // kTile x (kTile + 1)
    __shared__ double2 red[4][kTile];
    // tile (I, J) from the linear lower-triangle index
    const int64_t q = blockIdx.x;
    int I = (int)((sqrt(8.0 * (double)q + 1.0) - 1.0) * 0.5);
    while ((int64_t)(I + 1) * (I + 2) / 2 <= q) ++I;
    while ((int64_t)I * (I + 1) / 2 > q) --I;
    const int J = (int)(q - (int64_t)I * (I + 1) / 2);
    const int64_t r0 = (int64_t)I * kTile, c0 = (int64_t)J * kTile;
    const int t = threadIdx.x;
    const int ld = kTile + 1;
    for (int k = t; k < kTile * kTile; k += 256) {
        const int rr = k % kTile, cc = k / kTile;
        const int64_t r = r0 + rr, c = c0 + cc;
        double2 a = make_double2(0.0, 0.0);
        if (r < m && c < m) {
            if (I != J || rr >= cc) a = A[(o + r) + (o + c) * lda];
            else a = conjd(A[(o + c) + (o + r) * lda]);
        }
        S[rr + cc * ld] = a;
    }
    __syncthreads();
    // row sums: thread (rr, group of 16 columns)
    {
        const int rr = t % kTile, g = t / kTile;
        double2 acc = make_double2(0.0, 0.0);
#pragma unroll 4
        for (int cc = g * 16; cc < g * 16 + 16; ++cc) {
            const int64_t c = c0 + cc;
            if (c < m) acc = cfma(S[rr + cc * ld], v[c], acc);
        }
        red[g][rr] = acc;
    }
    __syncthreads();
    if (t < kTile) {
        const int64_t r = r0 + t;
        if (r < m) part1[(int64_t)J * m + r] = cadd(cadd(red[0][t], red[1][t]), cadd(red[2][t], red[3][t]));
    }
    if (I == J) return;
    __syncthreads();
    // column sums: thread (cc, group of 16 rows)
    {
        const int cc = t % kTile, g = t / kTile;
        double2 acc = make_double2(0.0, 0.0);
#pragma unroll 4
        for (int rr = g * 16; rr < g * 16 + 16; ++rr) {
            const int64_t r = r0 + rr;
            if (r < m) acc = cfma_conj(S[rr + cc * ld], v[r], acc);
        }
        red[g][cc] = acc;
    }
    __syncthreads();
    if (t < kTile) {
        const int64_t c = c0 + t;
        if (c < m) part2[(int64_t)I * m + c] = cadd(cadd(red[0][t], red[1][t]), cadd(red[2][t], red[3][t]));
    }
}

// p[r] = tau (sum_{J <= I} part1[J][r] + sum_{I' > I} part2[I'][r]), I = r / kTile, in a fixed
// order; pdot[block] = sum over the block's rows of conj(p[r]) v[r].
__global__ void __launch_bounds__(256) hemv_reduce_kernel(int64_t m, int nt, const double2* __restrict__ part1,
                                                          const double2* __restrict__ part2,
                                                          const double2* __restrict__ v, const double2* __restrict__ tau_j,
                                                          double2* __restrict__ p, double2* __restrict__ pdot) {
    __shared__ double sh[256];
    const double2 tv = *tau_j;
    const int64_t r = (int64_t)blockIdx.x * 256 + threadIdx.x;
    double2 dp = make_double2(0.0, 0.0);
    if (r < m && (tv.x != 0.0 || tv.y != 0.0)) {
        const int I = (int)(r / kTile);
        double2 acc = make_double2(0.0, 0.0);
        for (int J = 0; J <= I; ++J) acc = cadd(acc, part1[(int64_t)J * m + r]);
        for (int I2 = I + 1; I2 < nt; ++I2) acc = cadd(acc, part2[(int64_t)I2 * m + r]);
        const double2 pr = cmul(tv, acc);
        p[r] = pr;
        dp = cfma_conj(pr, v[r], dp);
    }
    const double sx = block_sum<256>(dp.x, sh);
    const double sy = block_sum<256>(dp.y, sh);
    if (threadIdx.x == 0) pdot[blockIdx.x] = make_double2(sx, sy);
}

// A22 -= v w^H + w v^H on the lower tiles, w = p - (tau / 2) (p^H v) v; the diagonal stays
// real.  Every block sums the nb partial dots itself (fixed order).
__global__ void __launch_bounds__(256) her2_tiles_kernel(double2* __restrict__ A, int64_t lda, int64_t o, int64_t m,
                                                         const double2* __restrict__ v, const double2* __restrict__ p,
                                                         const double2* __restrict__ pdot, int nb,
                                                         const double2* __restrict__ tau_j) {
    const double2 tv = *tau_j;
    if (tv.x == 0.0 && tv.y == 0.0) return;
    __shared__ double2 wsh[2][kTile];
    __shared__ double2 vsh[2][kTile];
    const int64_t q = blockIdx.x;
    int I = (int)((sqrt(8.0 * (double)q + 1.0) - 1.0) * 0.5);
    while ((int64_t)(I + 1) * (I + 2) / 2 <= q) ++I;
    while ((int64_t)I * (I + 1) / 2 > q) --I;
    const int J = (int)(q - (int64_t)I * (I + 1) / 2);
    const int64_t r0 = (int64_t)I * kTile, c0 = (int64_t)J * kTile;
    double2 dot = make_double2(0.0, 0.0);
    for (int b = 0; b < nb; ++b) dot = cadd(dot, pdot[b]);
    const double2 al = cmul(make_double2(-0.5 * tv.x, -0.5 * tv.y), dot);  // -(tau/2) p^H v
    const int t = threadIdx.x;
    if (t < 2 * kTile) {
        const int side = t / kTile, k = t % kTile;
        const int64_t idx = (side == 0 ? r0 : c0) + k;
        double2 vv = make_double2(0.0, 0.0), ww = make_double2(0.0, 0.0);
        if (idx < m) {
            vv = v[idx];
            ww = cfma(al, vv, p[idx]);
        }
        vsh[side][k] = vv;
        wsh[side][k] = ww;
    }
    __syncthreads();
    for (int k = t; k < kTile * kTile; k += 256) {
        const int rr = k % kTile, cc = k / kTile;
        const int64_t r = r0 + rr, c = c0 + cc;
        if (r >= m || c >= m || (I == J && rr < cc)) continue;
        double2* a = A + (o + r) + (o + c) * lda;
        double2 x = *a;
        // x -= v_r conj(w_c) + w_r conj(v_c)
        const double2 vr = vsh[0][rr], wr = wsh[0][rr], vc = vsh[1][cc], wc = wsh[1][cc];
        x.x -= fma(vr.x, wc.x, fma(vr.y, wc.y, fma(wr.x, vc.x, wr.y * vc.y)));
        x.y -= fma(vr.y, wc.x, fma(-vr.x, wc.y, fma(wr.y, vc.x, -wr.x * vc.y)));
        if (r == c) x.y = 0.0;
        *a = x;
    }
}

// ------------------------------------------------------------------------------------------
// 3. Bisection: thread per (block, local index k): the k-th smallest eigenvalue of the block
// T[s:s+len, s:s+len] by Sturm counts (number of eigenvalues below x from the signs of the
// LDL^T pivots, tiny pivots replaced by -pivmin).
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ int sturm_count(const double* __restrict__ d, const double* __restrict__ e2, int64_t s,
                                           int64_t len, double x, double pivmin) {
    double q = d[s] - x;
    if (fabs(q) < pivmin) q = -pivmin;
    int cnt = q < 0.0;
    for (int64_t i = 1; i < len; ++i) {
        q = d[s + i] - x - e2[s + i - 1] / q;
        if (fabs(q) < pivmin) q = -pivmin;
        cnt += q < 0.0;
    }
    return cnt;
}

__global__ void bisect_kernel(const double* __restrict__ d, const double* __restrict__ e2, const int64_t* __restrict__ job_s,
                              const int64_t* __restrict__ job_len, const int64_t* __restrict__ job_k,
                              const double* __restrict__ job_lo, const double* __restrict__ job_hi, int64_t njobs,
                              double pivmin, double* __restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= njobs) return;
    const int64_t s = job_s[t], len = job_len[t], k = job_k[t];
    double lo = job_lo[t], hi = job_hi[t];
    for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;  // the interval holds no more doubles
        if (hi - lo <= 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)) + pivmin) break;
        if (sturm_count(d, e2, s, len, mid, pivmin) > k) hi = mid;
        else lo = mid;
    }
    out[t] = 0.5 * (lo + hi);
}

// ------------------------------------------------------------------------------------------
// 4. Inverse iteration, thread per cluster.  Members of cluster q are mem[q0 .. q0+cnt) with
// eigenvalue lam[], block (s, len) and a vector slot out[] in vec (len used rows, stride ldv).
// Scratch per thread: dl, dd, du, du2 (len each) and the pivot flags.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ double hash_unit(uint64_t a, uint64_t b) {  // deterministic value in [-1, 1)
    uint64_t x = a * 0x9E3779B97F4A7C15ull ^ (b + 0x632BE59BD9B4E019ull);
    x ^= x >> 31; x *= 0xBF58476D1CE4E5B9ull; x ^= x >> 29; x *= 0x94D049BB133111EBull; x ^= x >> 32;
    return (double)(x >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

__global__ void stein_kernel(const double* __restrict__ d, const double* __restrict__ e, int64_t nclusters,
                             const int64_t* __restrict__ cl_first, const int64_t* __restrict__ cl_count,
                             const int64_t* __restrict__ mem_s, const int64_t* __restrict__ mem_len,
                             const double* __restrict__ mem_lam, const int64_t* __restrict__ mem_seed,
                             double* __restrict__ vec, int64_t ldv, double* __restrict__ scratch, int64_t lds,
                             double pert) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nclusters) return;
    const int64_t f = cl_first[q], cnt = cl_count[q];
    const int64_t s = mem_s[f], len = mem_len[f];
    double* dl = scratch + q * 5 * lds;
    double* dd = dl + lds;
    double* du = dd + lds;
    double* du2 = du + lds;
    double* piv = du2 + lds;  // 1.0 where rows i and i+1 were interchanged
    for (int64_t u = 0; u < cnt; ++u) {
        const int64_t mi = f + u;
        const double lam = mem_lam[mi];
        double* x = vec + mi * ldv;
        if (len == 1) {
            x[0] = 1.0;
            continue;
        }
        // LU of T_b - lam I with partial pivoting
        for (int64_t i = 0; i < len; ++i) {
            dd[i] = d[s + i] - lam;
            if (i + 1 < len) { dl[i] = e[s + i]; du[i] = e[s + i]; }
            du2[i] = 0.0;
            piv[i] = 0.0;
        }
        for (int64_t i = 0; i + 1 < len; ++i) {
            if (fabs(dd[i]) >= fabs(dl[i])) {
                if (dd[i] != 0.0) {
                    const double fct = dl[i] / dd[i];
                    dl[i] = fct;
                    dd[i + 1] -= fct * du[i];
                } else {
                    dl[i] = 0.0;
                }
            } else {
                const double fct = dd[i] / dl[i];
                dd[i] = dl[i];
                dl[i] = fct;
                const double tmp = du[i];
                du[i] = dd[i + 1];
                dd[i + 1] = tmp - fct * dd[i + 1];
                if (i + 2 < len) {
                    du2[i] = du[i + 1];
                    du[i + 1] = -fct * du[i + 1];
                }
                piv[i] = 1.0;
            }
        }
        for (int64_t i = 0; i < len; ++i)
            if (fabs(dd[i]) < pert) dd[i] = dd[i] < 0.0 ? -pert : pert;
        // start vector
        for (int64_t i = 0; i < len; ++i) x[i] = hash_unit((uint64_t)mem_seed[mi], (uint64_t)i);
        for (int it = 0; it < 4; ++it) {
            // orthogonalise against the cluster's earlier vectors
            for (int64_t p = f; p < mi; ++p) {
                const double* z = vec + p * ldv;
                double dot = 0.0;
                for (int64_t i = 0; i < len; ++i) dot = fma(z[i], x[i], dot);
                for (int64_t i = 0; i < len; ++i) x[i] = fma(-dot, z[i], x[i]);
            }
            if (it == 3) break;
            // solve L U y = x in place
            for (int64_t i = 0; i + 1 < len; ++i) {
                if (piv[i] == 0.0) {
                    x[i + 1] -= dl[i] * x[i];
                } else {
                    const double tmp = x[i];
                    x[i] = x[i + 1];
                    x[i + 1] = tmp - dl[i] * x[i + 1];
                }
            }
            x[len - 1] /= dd[len - 1];
            x[len - 2] = (x[len - 2] - du[len - 2] * x[len - 1]) / dd[len - 2];
            for (int64_t i = len - 3; i >= 0; --i) x[i] = (x[i] - du[i] * x[i + 1] - du2[i] * x[i + 2]) / dd[i];
            // normalise (largest entry first, then the 2-norm)
            double mx = 0.0;
            for (int64_t i = 0; i < len; ++i) mx = fmax(mx, fabs(x[i]));
            const double sm = mx > 0.0 ? 1.0 / mx : 1.0;
            double nrm = 0.0;
            for (int64_t i = 0; i < len; ++i) { x[i] *= sm; nrm = fma(x[i], x[i], nrm); }
            const double inv = 1.0 / sqrt(nrm);
            for (int64_t i = 0; i < len; ++i) x[i] *= inv;
        }
        // final normalisation and sign: the entry of largest magnitude is positive
        double nrm = 0.0, mx = 0.0;
        int64_t imx = 0;
        for (int64_t i = 0; i < len; ++i) {
            nrm = fma(x[i], x[i], nrm);
            if (fabs(x[i]) > mx) { mx = fabs(x[i]); imx = i; }
        }
        const double inv = (x[imx] < 0.0 ? -1.0 : 1.0) / sqrt(nrm);
        for (int64_t i = 0; i < len; ++i) x[i] *= inv;
    }
}

// X[:, k] = Z[:, k] as complex (column k's block rows from the member vector, zero elsewhere)
__global__ void scatter_vectors_kernel(int64_t n, int64_t nv, const int64_t* __restrict__ col_mem,
                                       const int64_t* __restrict__ mem_s, const int64_t* __restrict__ mem_len,
                                       const double* __restrict__ vec, int64_t ldv, double2* __restrict__ X,
                                       int64_t ldx) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t k = blockIdx.y;
    if (r >= n || k >= nv) return;
    const int64_t mi = col_mem[k];
    const int64_t s = mem_s[mi], len = mem_len[mi];
    X[r + k * ldx] = make_double2((r >= s && r < s + len) ? vec[mi * ldv + (r - s)] : 0.0, 0.0);
}

// ------------------------------------------------------------------------------------------
// 5. Back-transformation: X <- H_j X = X - tau_j v_j (v_j^H X) on rows j+1.., one block per
// column (the dot, then the update; the second read of the column comes from L2).
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) apply_reflector_kernel(const double2* __restrict__ A, int64_t lda, int64_t n,
                                                              int64_t j, const double2* __restrict__ tau,
                                                              double2* __restrict__ X, int64_t ldx, int64_t nv) {
    __shared__ double sh[256];
    const double2 tv = tau[j];
    if (tv.x == 0.0 && tv.y == 0.0) return;
    const int64_t k = blockIdx.x;
    if (k >= nv) return;
    const int64_t o = j + 1, m = n - o;
    const double2* v = A + o + j * lda;  // v[0] = 1 (stored as beta), v[i] = A[o+i, j]
    double2* x = X + o + k * ldx;
    double2 dp = make_double2(0.0, 0.0);
    for (int64_t i = threadIdx.x; i < m; i += 256) {
        const double2 vi = i == 0 ? make_double2(1.0, 0.0) : v[i];
        dp = cfma_conj(vi, x[i], dp);
    }
    const double sx = block_sum<256>(dp.x, sh);
    const double sy = block_sum<256>(dp.y, sh);
    const double2 g = cmul(tv, make_double2(-sx, -sy));  // -tau (v^H x)
    for (int64_t i = threadIdx.x; i < m; i += 256) {
        const double2 vi = i == 0 ? make_double2(1.0, 0.0) : v[i];
        x[i] = cfma(vi, g, x[i]);
    }
}

// P[r, c] += sum_k w_k X[r, k] conj(X[c, k]) on the lower 64 x 64 tiles of P (I >= J); the
// weights are staged per chunk of 16 vectors.
__global__ void __launch_bounds__(256) projector_tiles_kernel(const double2* __restrict__ X, int64_t ldx, int64_t n,
                                                              int64_t nv, const double* __restrict__ w,
                                                              double2* __restrict__ P, int64_t ldp) {
    __shared__ double2 xr[16][kTile];
    __shared__ double2 xc[16][kTile];
    const int64_t q = blockIdx.x;
    int I = (int)((sqrt(8.0 * (double)q + 1.0) - 1.0) * 0.5);
    while ((int64_t)(I + 1) * (I + 2) / 2 <= q) ++I;
    while ((int64_t)I * (I + 1) / 2 > q) --I;
    const int J = (int)(q - (int64_t)I * (I + 1) / 2);
    const int64_t r0 = (int64_t)I * kTile, c0 = (int64_t)J * kTile;
    const int t = threadIdx.x;
    const int tr = t % 16, tc = t / 16;  // thread owns rows tr + 16 a, columns tc + 16 b (a, b < 4)
    double2 acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = make_double2(0.0, 0.0);
    for (int64_t k0 = 0; k0 < nv; k0 += 16) {
        for (int u = t; u < 16 * kTile; u += 256) {
            const int kk = u / kTile, rr = u % kTile;
            const int64_t k = k0 + kk;
            double2 a = make_double2(0.0, 0.0), b = make_double2(0.0, 0.0);
            if (k < nv) {
                const double wk = w[k];
                if (r0 + rr < n) {
                    a = X[(r0 + rr) + k * ldx];
                    a = make_double2(a.x * wk, a.y * wk);
                }
                if (c0 + rr < n) b = X[(c0 + rr) + k * ldx];
            }
            xr[kk][rr] = a;
            xc[kk][rr] = b;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < 16; ++kk) {
            double2 ra[4], cb[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) ra[a] = xr[kk][tr + 16 * a];
#pragma unroll
            for (int b = 0; b < 4; ++b) cb[b] = xc[kk][tc + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] = cfma_conj(cb[b], ra[a], acc[a][b]);  // ra conj(cb)
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int64_t r = r0 + tr + 16 * a, c = c0 + tc + 16 * b;
            if (r < n && c < n && r >= c) {
                double2* pp = P + r + c * ldp;
                *pp = cadd(*pp, acc[a][b]);
            }
        }
}

// upper triangle of P from its lower triangle; the diagonal made real
__global__ void hermitian_fill_kernel(double2* __restrict__ P, int64_t ldp, int64_t n) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    for (int64_t c = blockIdx.y; c < n; c += gridDim.y) {
        if (r < c) P[r + c * ldp] = conjd(P[c + r * ldp]);
        else if (r == c) P[r + c * ldp].y = 0.0;
    }
}

// convert a c64 block into c32 (column-major, leading dimensions given)
__global__ void to_c32_kernel(const double2* __restrict__ src, int64_t lds, float2* __restrict__ dst, int64_t ldd,
                              int64_t n, int64_t ncols) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    for (int64_t c = blockIdx.y; c < ncols; c += gridDim.y) {
        const double2 v = src[r + c * lds];
        dst[r + c * ldd] = make_float2((float)v.x, (float)v.y);
    }
}

inline unsigned grid_y(int64_t ncols) { return (unsigned)std::min<int64_t>(std::max<int64_t>(ncols, 1), 65535); }

}  // namespace

// ------------------------------------------------------------------------------------------
// Host side.
// ------------------------------------------------------------------------------------------
struct lm_eigsys {
    lm_ctx* ctx = nullptr;
    int64_t n = 0;
    double2* d_A = nullptr;     // n x n; Householder vectors below the subdiagonal after the reduction
    double2* d_tau = nullptr;   // n - 1 reflector scalars
    double* d_d = nullptr;      // tridiagonal (device copies after splitting)
    double* d_e = nullptr;
    std::vector<double> d, e;   // host copies; e zero where T splits
    double tnorm = 0.0;
    std::vector<int64_t> blk_s, blk_len;  // blocks of T
    // eigenvalues ascending, with their block and index within the block
    std::vector<double> w;
    std::vector<int64_t> w_blk, w_k;
};

namespace {

template <typename T>
int dalloc_t(lm_ctx* ctx, T** p, size_t count, const char* what) {
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(count, 1));
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return set_err(ctx, e == cudaErrorMemoryAllocation ? LM_ERR_OOM : LM_ERR_CUDA,
                       std::string("eigensolver: cannot allocate ") + what);
    }
    return LM_OK;
}

template <typename T>
int upload_vec(lm_ctx* ctx, T** dptr, const std::vector<T>& h, const char* what) {
    int rc = dalloc_t(ctx, dptr, h.size(), what);
    if (rc != LM_OK) return rc;
    if (!h.empty())
        CUDA_TRY(ctx, cudaMemcpyAsync(*dptr, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, ctx->stream),
                 "eigensolver: upload");
    return LM_OK;
}

struct DevFree {
    std::vector<void*> ptrs;
    ~DevFree() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <typename T>
    T* keep(T* p) {
        ptrs.push_back((void*)p);
        return p;
    }
};

void free_eigsys(lm_eigsys* e) {
    cudaFree(e->d_A);
    cudaFree(e->d_tau);
    cudaFree(e->d_d);
    cudaFree(e->d_e);
    e->d_A = nullptr;
    e->d_tau = nullptr;
    e->d_d = nullptr;
    e->d_e = nullptr;
}

// Householder reduction of es->d_A (filled with the dense H), then splitting and bisection.
int reduce_and_solve(lm_eigsys* es) {
    lm_ctx* ctx = es->ctx;
    const int64_t n = es->n;
    int rc = dalloc_t(ctx, &es->d_tau, (size_t)std::max<int64_t>(n - 1, 1), "reflector scalars");
    if (rc == LM_OK) rc = dalloc_t(ctx, &es->d_d, (size_t)n, "tridiagonal");
    if (rc == LM_OK) rc = dalloc_t(ctx, &es->d_e, (size_t)std::max<int64_t>(n - 1, 1), "tridiagonal");
    if (rc != LM_OK) return rc;
    DevFree tmp;
    const int64_t m0 = std::max<int64_t>(n - 1, 1);
    const int nt0 = (int)((m0 + kTile - 1) / kTile);
    double2 *d_v = nullptr, *d_p = nullptr, *d_part1 = nullptr, *d_part2 = nullptr, *d_pdot = nullptr;
    rc = dalloc_t(ctx, &d_v, (size_t)m0, "reflector");
    if (rc == LM_OK) rc = dalloc_t(ctx, &d_p, (size_t)m0, "product");
    if (rc == LM_OK) rc = dalloc_t(ctx, &d_part1, (size_t)nt0 * (size_t)m0, "partial sums");
    if (rc == LM_OK) rc = dalloc_t(ctx, &d_part2, (size_t)nt0 * (size_t)m0, "partial sums");
    if (rc == LM_OK) rc = dalloc_t(ctx, &d_pdot, (size_t)(m0 + 255) / 256, "partial dots");
    tmp.keep(d_v); tmp.keep(d_p); tmp.keep(d_part1); tmp.keep(d_part2); tmp.keep(d_pdot);
    if (rc != LM_OK) return rc;
    const size_t smem = sizeof(double2) * kTile * (kTile + 1);
    CUDA_TRY(ctx, cudaFuncSetAttribute(hemv_tiles_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
             "eigensolver: shared memory attribute");
    for (int64_t j = 0; j + 1 < n; ++j) {
        const int64_t m = n - 1 - j, o = j + 1;
        const int nt = (int)((m + kTile - 1) / kTile);
        const int64_t ntiles = (int64_t)nt * (nt + 1) / 2;
        const int nb = (int)((m + 255) / 256);
        house_kernel<<<1, 1024, 0, ctx->stream>>>(es->d_A, n, n, j, es->d_d, es->d_e, es->d_tau, d_v);
        hemv_tiles_kernel<<<(unsigned)ntiles, 256, smem, ctx->stream>>>(es->d_A, n, o, m, nt, d_v, es->d_tau + j,
                                                                       d_part1, d_part2);
        hemv_reduce_kernel<<<nb, 256, 0, ctx->stream>>>(m, nt, d_part1, d_part2, d_v, es->d_tau + j, d_p, d_pdot);
        her2_tiles_kernel<<<(unsigned)ntiles, 256, 0, ctx->stream>>>(es->d_A, n, o, m, d_v, d_p, d_pdot, nb,
                                                                     es->d_tau + j);
        ctx->launches += 4;
        if ((j & 255) == 0) CUDA_TRY(ctx, cudaGetLastError(), "eigensolver: tridiagonalisation");
    }
    CUDA_TRY(ctx, cudaGetLastError(), "eigensolver: tridiagonalisation");
    es->d.assign((size_t)n, 0.0);
    es->e.assign((size_t)std::max<int64_t>(n - 1, 0), 0.0);
    // d[n-1] is the last diagonal entry of the reduced matrix
    CUDA_TRY(ctx, cudaMemcpyAsync(es->d_d + (n - 1), es->d_A + (n - 1) + (n - 1) * n, sizeof(double),
                                  cudaMemcpyDeviceToDevice, ctx->stream),
             "eigensolver: last diagonal");
    CUDA_TRY(ctx, cudaMemcpyAsync(es->d.data(), es->d_d, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream),
             "eigensolver: download");
    if (n > 1)
        CUDA_TRY(ctx, cudaMemcpyAsync(es->e.data(), es->d_e, sizeof(double) * (n - 1), cudaMemcpyDeviceToHost,
                                      ctx->stream),
                 "eigensolver: download");
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "eigensolver: synchronize");
    for (double v : es->d)
        if (!std::isfinite(v)) return set_err(ctx, LM_ERR_NONFINITE, "eigensolver: non-finite tridiagonal");
    for (double v : es->e)
        if (!std::isfinite(v)) return set_err(ctx, LM_ERR_NONFINITE, "eigensolver: non-finite tridiagonal");
    // norm, splitting
    double tn = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        double r = fabs(es->d[(size_t)i]);
        if (i > 0) r += fabs(es->e[(size_t)i - 1]);
        if (i + 1 < n) r += fabs(es->e[(size_t)i]);
        tn = std::max(tn, r);
    }
    es->tnorm = tn;
    es->blk_s.clear();
    es->blk_len.clear();
    int64_t s0 = 0;
    for (int64_t i = 0; i + 1 < n; ++i) {
        if (fabs(es->e[(size_t)i]) <= kSplitRel * tn) {
            es->e[(size_t)i] = 0.0;
            es->blk_s.push_back(s0);
            es->blk_len.push_back(i + 1 - s0);
            s0 = i + 1;
        }
    }
    es->blk_s.push_back(s0);
    es->blk_len.push_back(n - s0);
    if (n > 1)
        CUDA_TRY(ctx, cudaMemcpyAsync(es->d_e, es->e.data(), sizeof(double) * (n - 1), cudaMemcpyHostToDevice,
                                      ctx->stream),
                 "eigensolver: upload");
    // bisection jobs
    std::vector<double> e2((size_t)std::max<int64_t>(n - 1, 1), 0.0);
    double emax2 = 0.0;
    for (int64_t i = 0; i + 1 < n; ++i) {
        e2[(size_t)i] = es->e[(size_t)i] * es->e[(size_t)i];
        emax2 = std::max(emax2, e2[(size_t)i]);
    }
    const double pivmin = DBL_MIN * std::max(1.0, emax2);
    std::vector<int64_t> js, jl, jk;
    std::vector<double> jlo, jhi;
    js.reserve((size_t)n); jl.reserve((size_t)n); jk.reserve((size_t)n); jlo.reserve((size_t)n); jhi.reserve((size_t)n);
    for (size_t b = 0; b < es->blk_s.size(); ++b) {
        const int64_t s = es->blk_s[b], len = es->blk_len[b];
        double lo = 1e300, hi = -1e300;
        for (int64_t i = s; i < s + len; ++i) {
            double r = 0.0;
            if (i > s) r += fabs(es->e[(size_t)i - 1]);
            if (i + 1 < s + len) r += fabs(es->e[(size_t)i]);
            lo = std::min(lo, es->d[(size_t)i] - r);
            hi = std::max(hi, es->d[(size_t)i] + r);
        }
        const double pad = 2.0 * DBL_EPSILON * std::max(fabs(lo), fabs(hi)) * (double)len + 2.0 * pivmin;
        for (int64_t k = 0; k < len; ++k) {
            js.push_back(s); jl.push_back(len); jk.push_back(k);
            jlo.push_back(lo - pad); jhi.push_back(hi + pad);
        }
    }
    double *d_e2 = nullptr, *d_jlo = nullptr, *d_jhi = nullptr, *d_out = nullptr;
    int64_t *d_js = nullptr, *d_jl = nullptr, *d_jk = nullptr;
    rc = upload_vec(ctx, &d_e2, e2, "bisection");
    if (rc == LM_OK) rc = upload_vec(ctx, &d_js, js, "bisection");
    if (rc == LM_OK) rc = upload_vec(ctx, &d_jl, jl, "bisection");
    if (rc == LM_OK) rc = upload_vec(ctx, &d_jk, jk, "bisection");
    if (rc == LM_OK) rc = upload_vec(ctx, &d_jlo, jlo, "bisection");
    if (rc == LM_OK) rc = upload_vec(ctx, &d_jhi, jhi, "bisection");
    if (rc == LM_OK) rc = dalloc_t(ctx, &d_out, (size_t)n, "bisection");
    tmp.keep(d_e2); tmp.keep(d_js); tmp.keep(d_jl); tmp.keep(d_jk); tmp.keep(d_jlo); tmp.keep(d_jhi); tmp.keep(d_out);
    if (rc != LM_OK) return rc;
    bisect_kernel<<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(es->d_d, d_e2, d_js, d_jl, d_jk, d_jlo, d_jhi,
                                                                       n, pivmin, d_out);
    ctx->launches++;
    CUDA_TRY(ctx, cudaGetLastError(), "eigensolver: bisection");
    std::vector<double> vals((size_t)n);
    CUDA_TRY(ctx, cudaMemcpyAsync(vals.data(), d_out, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream),
             "eigensolver: download");
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "eigensolver: synchronize");
    // eigenvalues ascending; ties keep the block order
    std::vector<int64_t> ord((size_t)n);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return vals[(size_t)a] < vals[(size_t)b]; });
    es->w.resize((size_t)n);
    es->w_blk.resize((size_t)n);
    es->w_k.resize((size_t)n);
    std::vector<int64_t> blk_of_start;
    for (int64_t i = 0; i < n; ++i) {
        const int64_t t = ord[(size_t)i];
        es->w[(size_t)i] = vals[(size_t)t];
        es->w_k[(size_t)i] = jk[(size_t)t];
        // block index from the job's start row
        const int64_t s = js[(size_t)t];
        es->w_blk[(size_t)i] = std::lower_bound(es->blk_s.begin(), es->blk_s.end(), s) - es->blk_s.begin();
    }
    return LM_OK;
}

int check_lm_state_dense(lm_ctx* ctx, const lm_state* st, int64_t n, int kind, const char* who) {
    if (!st) return set_err(ctx, LM_ERR_ARG, std::string(who) + ": null state");
    if (st->ctx != ctx) return set_err(ctx, LM_ERR_ARG, std::string(who) + ": state belongs to another context");
    if (st->n != n || st->kind != kind)
        return set_err(ctx, LM_ERR_ARG, std::string(who) + ": state shape does not match the eigensystem");
    return LM_OK;
}

// Eigenvectors of global indices idx[0..nv) (ascending eigenvalue order) into the complex n x nv
// block X (ldx): inverse iteration on T, then X = Q Z.
int eigvectors(lm_eigsys* es, const std::vector<int64_t>& idx, double2* X, int64_t ldx) {
    lm_ctx* ctx = es->ctx;
    const int64_t n = es->n, nv = (int64_t)idx.size();
    if (nv == 0) return LM_OK;
    // clusters: every requested eigenvalue with its cluster-mates (same block, consecutive
    // within the block, gaps below kClusterRel |T|), each cluster once
    const double ctol = kClusterRel * es->tnorm;
    // per block: global indices in block order
    std::vector<std::vector<int64_t>> in_blk(es->blk_s.size());
    for (int64_t i = 0; i < n; ++i) in_blk[(size_t)es->w_blk[(size_t)i]].push_back(i);
    for (auto& v : in_blk)
        std::sort(v.begin(), v.end(), [&](int64_t a, int64_t b) { return es->w_k[(size_t)a] < es->w_k[(size_t)b]; });
    std::vector<int64_t> pos_in_blk((size_t)n);
    for (auto& v : in_blk)
        for (size_t u = 0; u < v.size(); ++u) pos_in_blk[(size_t)v[u]] = (int64_t)u;
    std::vector<int64_t> cl_first, cl_count, mem_s, mem_len, mem_seed, col_mem((size_t)nv, -1);
    std::vector<double> mem_lam;
    std::vector<char> seen((size_t)n, 0);
    std::vector<int64_t> mem_of((size_t)n, -1);
    for (int64_t c = 0; c < nv; ++c) {
        const int64_t g = idx[(size_t)c];
        if (!seen[(size_t)g]) {
            const auto& bl = in_blk[(size_t)es->w_blk[(size_t)g]];
            int64_t lo = pos_in_blk[(size_t)g], hi = lo;
            while (lo > 0 && es->w[(size_t)bl[(size_t)lo]] - es->w[(size_t)bl[(size_t)lo - 1]] < ctol) --lo;
            while (hi + 1 < (int64_t)bl.size() && es->w[(size_t)bl[(size_t)hi + 1]] - es->w[(size_t)bl[(size_t)hi]] < ctol) ++hi;
            cl_first.push_back((int64_t)mem_lam.size());
            cl_count.push_back(hi - lo + 1);
            const int64_t b = es->w_blk[(size_t)g];
            for (int64_t u = lo; u <= hi; ++u) {
                const int64_t gg = bl[(size_t)u];
                seen[(size_t)gg] = 1;
                mem_of[(size_t)gg] = (int64_t)mem_lam.size();
                mem_lam.push_back(es->w[(size_t)gg]);
                mem_s.push_back(es->blk_s[(size_t)b]);
                mem_len.push_back(es->blk_len[(size_t)b]);
                mem_seed.push_back(gg);
            }
        }
        col_mem[(size_t)c] = mem_of[(size_t)g];
    }
    const int64_t nmem = (int64_t)mem_lam.size(), ncl = (int64_t)cl_first.size();
    int64_t lmax = 1;
    for (int64_t l : mem_len) lmax = std::max(lmax, l);
    DevFree tmp;
    int64_t *d_clf = nullptr, *d_clc = nullptr, *d_ms = nullptr, *d_ml = nullptr, *d_seed = nullptr, *d_col = nullptr;
    double *d_lam = nullptr, *d_vec = nullptr, *d_scr = nullptr;
    int rc = upload_vec(ctx, &d_clf, cl_first, "inverse iteration");
    if (rc == LM_OK) rc = upload_vec(ctx, &d_clc, cl_count, "inverse iteration");
    if (rc == LM_OK) rc = upload_vec(ctx, &d_ms, mem_s, "inverse iteration");
    if (rc == LM_OK) rc = upload_vec(ctx, &d_ml, mem_len, "inverse iteration");
    if (rc == LM_OK) rc = upload_vec(ctx, &d_seed, mem_seed, "inverse iteration");
    if (rc == LM_OK) rc = upload_vec(ctx, &d_col, col_mem, "inverse iteration");
    if (rc == LM_OK) rc = upload_vec(ctx, &d_lam, mem_lam, "inverse iteration");
    if (rc == LM_OK) rc = dalloc_t(ctx, &d_vec, (size_t)nmem * (size_t)lmax, "tridiagonal eigenvectors");
    if (rc == LM_OK) rc = dalloc_t(ctx, &d_scr, (size_t)ncl * 5 * (size_t)lmax, "inverse iteration scratch");
    tmp.keep(d_clf); tmp.keep(d_clc); tmp.keep(d_ms); tmp.keep(d_ml); tmp.keep(d_seed); tmp.keep(d_col);
    tmp.keep(d_lam); tmp.keep(d_vec); tmp.keep(d_scr);
    if (rc != LM_OK) return rc;
    const double pert = DBL_EPSILON * std::max(es->tnorm, DBL_MIN);
    stein_kernel<<<(unsigned)((ncl + 63) / 64), 64, 0, ctx->stream>>>(es->d_d, es->d_e, ncl, d_clf, d_clc, d_ms, d_ml,
                                                                     d_lam, d_seed, d_vec, lmax, d_scr, lmax, pert);
    scatter_vectors_kernel<<<dim3((unsigned)((n + 255) / 256), (unsigned)nv), 256, 0, ctx->stream>>>(
        n, nv, d_col, d_ms, d_ml, d_vec, lmax, X, ldx);
    ctx->launches += 2;
    CUDA_TRY(ctx, cudaGetLastError(), "eigensolver: inverse iteration");
    for (int64_t j = n - 2; j >= 0; --j) {
        apply_reflector_kernel<<<(unsigned)nv, 256, 0, ctx->stream>>>(es->d_A, n, n, j, es->d_tau, X, ldx, nv);
        ctx->launches++;
        if ((j & 255) == 0) CUDA_TRY(ctx, cudaGetLastError(), "eigensolver: back-transformation");
    }
    CUDA_TRY(ctx, cudaGetLastError(), "eigensolver: back-transformation");
    // the temporaries are freed on return: wait for the kernels that read them
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "eigensolver: synchronize");
    return LM_OK;
}

int eigsys_from_dense(lm_ctx* ctx, int64_t n, lm_eigsys** out) {
    lm_eigsys* es = *out;
    int rc = reduce_and_solve(es);
    if (rc != LM_OK) {
        free_eigsys(es);
        delete es;
        *out = nullptr;
    }
    (void)ctx;
    (void)n;
    return rc;
}

}  // namespace

extern "C" {

int lm_eigsys_create(lm_ham* h, lm_eigsys** out) {
    if (!h || !out) return LM_ERR_ARG;
    lm_ctx* ctx = h->ctx;
    *out = nullptr;
    if (!h->assembled) return set_err(ctx, LM_ERR_STATE, "lm_eigsys_create: Hamiltonian not assembled");
    cudaSetDevice(ctx->device);
    const Geom& g = h->lat->g;
    lm_eigsys* es = new lm_eigsys();
    es->ctx = ctx;
    es->n = g.N;
    int rc = dalloc_t(ctx, &es->d_A, (size_t)g.N * (size_t)g.N, "dense Hamiltonian");
    if (rc != LM_OK) {
        delete es;
        return rc;
    }
    rc = check_cuda(ctx, cudaMemsetAsync(es->d_A, 0, sizeof(double2) * (size_t)g.N * (size_t)g.N, ctx->stream),
                    "lm_eigsys_create: clear");
    if (rc == LM_OK) {
        dense_square_kernel<<<(unsigned)((g.N + 255) / 256), 256, 0, ctx->stream>>>(g, h->d_hop, h->d_onsite, es->d_A,
                                                                                   g.N);
        ctx->launches++;
        rc = check_cuda(ctx, cudaGetLastError(), "lm_eigsys_create: dense assembly");
    }
    if (rc != LM_OK) {
        free_eigsys(es);
        delete es;
        return rc;
    }
    *out = es;
    return eigsys_from_dense(ctx, g.N, out);
}

int lm_eigsys_create_ell(lm_ell* h, lm_eigsys** out) {
    if (!h || !out) return LM_ERR_ARG;
    lm_ctx* ctx = h->ctx;
    *out = nullptr;
    cudaSetDevice(ctx->device);
    lm_eigsys* es = new lm_eigsys();
    es->ctx = ctx;
    es->n = h->n;
    int rc = dalloc_t(ctx, &es->d_A, (size_t)h->n * (size_t)h->n, "dense Hamiltonian");
    if (rc != LM_OK) {
        delete es;
        return rc;
    }
    rc = check_cuda(ctx, cudaMemsetAsync(es->d_A, 0, sizeof(double2) * (size_t)h->n * (size_t)h->n, ctx->stream),
                    "lm_eigsys_create_ell: clear");
    if (rc == LM_OK) {
        dense_ell_kernel<<<(unsigned)((h->n + 255) / 256), 256, 0, ctx->stream>>>(h->n, h->w, h->d_cols, h->d_vals,
                                                                                 h->d_diag, es->d_A, h->n);
        ctx->launches++;
        rc = check_cuda(ctx, cudaGetLastError(), "lm_eigsys_create_ell: dense assembly");
    }
    if (rc != LM_OK) {
        free_eigsys(es);
        delete es;
        return rc;
    }
    *out = es;
    return eigsys_from_dense(ctx, h->n, out);
}

int lm_eigsys_destroy(lm_eigsys* e) {
    if (!e) return LM_OK;
    cudaSetDevice(e->ctx->device);
    cudaStreamSynchronize(e->ctx->stream);
    free_eigsys(e);
    delete e;
    return LM_OK;
}

int lm_eigsys_size(const lm_eigsys* e, int64_t* n) {
    if (!e || !n) return LM_ERR_ARG;
    *n = e->n;
    return LM_OK;
}

int lm_eigsys_values(const lm_eigsys* e, double* out) {
    if (!e || !out) return LM_ERR_ARG;
    std::copy(e->w.begin(), e->w.end(), out);
    return LM_OK;
}

int lm_eigsys_vectors(lm_eigsys* e, int64_t first, lm_state* out) {
    if (!e) return LM_ERR_ARG;
    lm_ctx* ctx = e->ctx;
    int rc = check_lm_state_dense(ctx, out, e->n, LM_KETS, "lm_eigsys_vectors");
    if (rc != LM_OK) return rc;
    CHECK_ARG(ctx, first >= 0 && first + out->m <= e->n, "lm_eigsys_vectors: index range outside the spectrum");
    cudaSetDevice(ctx->device);
    DevFree tmp;
    double2* X = nullptr;
    const bool direct = out->precision == LM_C64;
    for (int64_t c0 = 0; c0 < out->m; c0 += kChunk) {
        const int64_t nv = std::min<int64_t>(kChunk, out->m - c0);
        std::vector<int64_t> idx((size_t)nv);
        for (int64_t k = 0; k < nv; ++k) idx[(size_t)k] = first + c0 + k;
        if (direct) {
            rc = eigvectors(e, idx, (double2*)out->d_data + c0 * out->ld, out->ld);
        } else {
            if (!X) {
                rc = dalloc_t(ctx, &X, (size_t)e->n * (size_t)kChunk, "eigenvector chunk");
                if (rc != LM_OK) return rc;
                tmp.keep(X);
            }
            rc = eigvectors(e, idx, X, e->n);
            if (rc == LM_OK) {
                to_c32_kernel<<<dim3((unsigned)((e->n + 255) / 256), grid_y(nv)), 256, 0, ctx->stream>>>(
                    X, e->n, (float2*)out->d_data + c0 * out->ld, out->ld, e->n, nv);
                ctx->launches++;
                rc = check_cuda(ctx, cudaGetLastError(), "lm_eigsys_vectors: conversion");
            }
        }
        if (rc != LM_OK) return rc;
    }
    if (X) CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "lm_eigsys_vectors: synchronize");
    return LM_OK;
}

int lm_eigsys_projector(lm_eigsys* e, const double* weights, lm_state* out) {
    if (!e) return LM_ERR_ARG;
    lm_ctx* ctx = e->ctx;
    int rc = check_lm_state_dense(ctx, out, e->n, LM_DENSITY, "lm_eigsys_projector");
    if (rc != LM_OK) return rc;
    CHECK_ARG(ctx, weights != nullptr, "lm_eigsys_projector: null weights");
    for (int64_t k = 0; k < e->n; ++k)
        CHECK_ARG(ctx, std::isfinite(weights[k]), "lm_eigsys_projector: non-finite weight");
    cudaSetDevice(ctx->device);
    const int64_t n = e->n;
    DevFree tmp;
    double2* P = nullptr;
    int64_t ldp = out->ld;
    if (out->precision == LM_C64) {
        P = (double2*)out->d_data;
    } else {
        rc = dalloc_t(ctx, &P, (size_t)n * (size_t)n, "projector");
        if (rc != LM_OK) return rc;
        tmp.keep(P);
        ldp = n;
    }
    CUDA_TRY(ctx, cudaMemset2DAsync(P, sizeof(double2) * ldp, 0, sizeof(double2) * n, n, ctx->stream),
             "lm_eigsys_projector: clear");
    std::vector<int64_t> nz;
    for (int64_t k = 0; k < n; ++k)
        if (weights[k] != 0.0) nz.push_back(k);
    double2* X = nullptr;
    double* d_w = nullptr;
    if (!nz.empty()) {
        const int64_t cw = std::min<int64_t>(kChunk, (int64_t)nz.size());
        rc = dalloc_t(ctx, &X, (size_t)n * (size_t)cw, "eigenvector chunk");
        if (rc == LM_OK) rc = dalloc_t(ctx, &d_w, (size_t)cw, "weights");
        if (rc != LM_OK) {
            cudaFree(X);
            cudaFree(d_w);
            return rc;
        }
        tmp.keep(X);
        tmp.keep(d_w);
    }
    const int nt = (int)((n + kTile - 1) / kTile);
    const int64_t ntiles = (int64_t)nt * (nt + 1) / 2;
    std::vector<double> wc;
    for (size_t c0 = 0; c0 < nz.size(); c0 += kChunk) {
        const size_t nv = std::min<size_t>(kChunk, nz.size() - c0);
        std::vector<int64_t> idx(nz.begin() + c0, nz.begin() + c0 + nv);
        wc.assign(nv, 0.0);
        for (size_t k = 0; k < nv; ++k) wc[k] = weights[idx[k]];
        rc = eigvectors(e, idx, X, n);
        if (rc != LM_OK) return rc;
        CUDA_TRY(ctx, cudaMemcpyAsync(d_w, wc.data(), sizeof(double) * nv, cudaMemcpyHostToDevice, ctx->stream),
                 "lm_eigsys_projector: weights");
        projector_tiles_kernel<<<(unsigned)ntiles, 256, 0, ctx->stream>>>(X, n, n, (int64_t)nv, d_w, P, ldp);
        ctx->launches++;
        CUDA_TRY(ctx, cudaGetLastError(), "lm_eigsys_projector: accumulation");
        CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "lm_eigsys_projector: synchronize");  // wc reuse
    }
    hermitian_fill_kernel<<<dim3((unsigned)((n + 255) / 256), grid_y(n)), 256, 0, ctx->stream>>>(P, ldp, n);
    ctx->launches++;
    CUDA_TRY(ctx, cudaGetLastError(), "lm_eigsys_projector: fill");
    if (out->precision != LM_C64) {
        to_c32_kernel<<<dim3((unsigned)((n + 255) / 256), grid_y(n)), 256, 0, ctx->stream>>>(P, n, (float2*)out->d_data,
                                                                                             out->ld, n, n);
        ctx->launches++;
        CUDA_TRY(ctx, cudaGetLastError(), "lm_eigsys_projector: conversion");
    }
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "lm_eigsys_projector: synchronize");
    return LM_OK;
}

}  // extern "C"
