/*
 * CPU restatement of KrylovKitExp for the LatticeModels.jl evolution path.
 *
 * TEST INFRASTRUCTURE / CPU BASELINE ONLY.  The GPU library never links or calls this file;
 * only the tests and the CPU-baseline leg of bench.py load the shared object built from it.
 *
 * Restates: `step!(::KrylovKitExp, ::AbstractVector, _)` (src/evolution.jl:150-154), i.e.
 * `KrylovKit.exponentiate(H, -i*dt, psi)` on a sparse Hermitian H.  KrylovKit (compat
 * 0.4-0.9, unpinned: the reference ships no Manifest) is not vendored; for a Hermitian
 * matrix its `exponentiate` runs a Lanczos recurrence, exponentiates the projected
 * tridiagonal matrix and stops when the residual estimate falls below `tol` (default 1e-12),
 * splitting the time step when the Krylov dimension (default 30) is exhausted.  This file
 * restates that published Krylov-propagator method (Park & Light 1986; Saad 1992):
 *
 *   q1 = psi/|psi|;  H q_j = beta_{j-1} q_{j-1} + alpha_j q_j + beta_j q_{j+1}
 *   psi(dt) ~= |psi| Q_m exp(-i dt T_m) e1,   err ~= |psi| beta_m |[exp(-i dt T_m) e1]_m|
 *
 * The small tridiagonal eigenproblem is solved by cyclic Jacobi rotations.  Kets of a block
 * are independent and are distributed over OpenMP threads.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

/* y = H x for CSR H (rowptr/col 0-based, val interleaved re/im). */
static void csr_spmv(int64_t n, const int64_t *rowptr, const int64_t *col, const cplx *val,
                     const cplx *x, cplx *y) {
    for (int64_t i = 0; i < n; ++i) {
        cplx acc = 0;
        for (int64_t p = rowptr[i]; p < rowptr[i + 1]; ++p) acc += val[p] * x[col[p]];
        y[i] = acc;
    }
}

static double vnorm(int64_t n, const cplx *x) {
    double s = 0;
    for (int64_t i = 0; i < n; ++i) s += creal(x[i]) * creal(x[i]) + cimag(x[i]) * cimag(x[i]);
    return sqrt(s);
}

static cplx vdot(int64_t n, const cplx *a, const cplx *b) { /* conj(a) . b */
    cplx s = 0;
    for (int64_t i = 0; i < n; ++i) s += conj(a[i]) * b[i];
    return s;
}

/* Eigen-decomposition of a real symmetric m x m matrix A (row-major, destroyed) by cyclic
 * Jacobi rotations; eigenvalues in w, eigenvectors as columns of V (row-major). */
static void jacobi_eig(int m, double *A, double *w, double *V) {
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) V[i * m + j] = (i == j);
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0;
        for (int i = 0; i < m; ++i)
            for (int j = i + 1; j < m; ++j) off += A[i * m + j] * A[i * m + j];
        if (off < 1e-300) break;
        for (int p = 0; p < m; ++p) {
            for (int q = p + 1; q < m; ++q) {
                double apq = A[p * m + q];
                if (fabs(apq) < 1e-300) continue;
                double theta = (A[q * m + q] - A[p * m + p]) / (2 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1));
                double c = 1 / sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < m; ++k) { /* rotate columns p, q */
                    double akp = A[k * m + p], akq = A[k * m + q];
                    A[k * m + p] = c * akp - s * akq;
                    A[k * m + q] = s * akp + c * akq;
                }
                for (int k = 0; k < m; ++k) { /* rotate rows p, q */
                    double apk = A[p * m + k], aqk = A[q * m + k];
                    A[p * m + k] = c * apk - s * aqk;
                    A[q * m + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < m; ++k) {
                    double vkp = V[k * m + p], vkq = V[k * m + q];
                    V[k * m + p] = c * vkp - s * vkq;
                    V[k * m + q] = s * vkp + c * vkq;
                }
            }
        }
    }
    for (int i = 0; i < m; ++i) w[i] = A[i * m + i];
}

/* One Krylov propagation psi <- exp(-i tau H) psi.  Returns 0 on convergence, 1 when the
 * Krylov dimension is exhausted (caller halves tau).  Q holds (kdim+1) n-vectors. */
static int lanczos_expv_once(int64_t n, const int64_t *rowptr, const int64_t *col, const cplx *val,
                             double tau, cplx *psi, double tol, int kdim, cplx *Q, cplx *out) {
    double alpha[96], beta[96], T[96 * 96], w[96], V[96 * 96];
    cplx y[96];
    double b0 = vnorm(n, psi);
    if (b0 == 0) return 0;
    for (int64_t i = 0; i < n; ++i) Q[i] = psi[i] / b0;
    int m = 0;
    for (int j = 0; j < kdim; ++j) {
        cplx *qj = Q + (int64_t)j * n, *qn = Q + (int64_t)(j + 1) * n;
        csr_spmv(n, rowptr, col, val, qj, qn);
        alpha[j] = creal(vdot(n, qj, qn));
        for (int64_t i = 0; i < n; ++i) qn[i] -= alpha[j] * qj[i];
        if (j > 0) {
            cplx *qp = Q + (int64_t)(j - 1) * n;
            for (int64_t i = 0; i < n; ++i) qn[i] -= beta[j - 1] * qp[i];
        }
        /* one re-orthogonalisation pass against the whole basis (Gram-Schmidt, twice is enough) */
        for (int k = 0; k <= j; ++k) {
            cplx *qk = Q + (int64_t)k * n;
            cplx c = vdot(n, qk, qn);
            for (int64_t i = 0; i < n; ++i) qn[i] -= c * qk[i];
        }
        beta[j] = vnorm(n, qn);
        m = j + 1;
        /* exp(-i tau T_m) e1 via the eigendecomposition of T_m */
        memset(T, 0, sizeof(double) * m * m);
        for (int k = 0; k < m; ++k) {
            T[k * m + k] = alpha[k];
            if (k + 1 < m) T[k * m + k + 1] = T[(k + 1) * m + k] = beta[k];
        }
        jacobi_eig(m, T, w, V);
        for (int r = 0; r < m; ++r) {
            cplx s = 0;
            for (int k = 0; k < m; ++k) s += V[r * m + k] * cexp(-I * tau * w[k]) * V[0 * m + k];
            y[r] = s;
        }
        double err = b0 * beta[j] * cabs(y[m - 1]);
        if (err <= tol || beta[j] < 1e-300) {
            for (int64_t i = 0; i < n; ++i) out[i] = 0;
            for (int k = 0; k < m; ++k) {
                cplx *qk = Q + (int64_t)k * n;
                cplx c = b0 * y[k];
                for (int64_t i = 0; i < n; ++i) out[i] += c * qk[i];
            }
            memcpy(psi, out, sizeof(cplx) * n);
            return 0;
        }
        for (int64_t i = 0; i < n; ++i) qn[i] /= beta[j];
    }
    return 1;
}

static int lanczos_expv(int64_t n, const int64_t *rowptr, const int64_t *col, const cplx *val,
                        double dt, cplx *psi, double tol, int kdim, cplx *Q, cplx *out, int depth) {
    if (lanczos_expv_once(n, rowptr, col, val, dt, psi, tol, kdim, Q, out) == 0) return 0;
    if (depth > 20) return -1;
    /* not converged within kdim: propagate in two halves */
    if (lanczos_expv(n, rowptr, col, val, dt / 2, psi, tol / 2, kdim, Q, out, depth + 1)) return -1;
    return lanczos_expv(n, rowptr, col, val, dt / 2, psi, tol / 2, kdim, Q, out, depth + 1);
}

/* Public: propagate the m kets of a column-major n x m block (leading dimension ld) by
 * exp(-i dt H).  Returns the number of kets that failed to converge (0 = all ok). */
int lmo_krylov_block(int64_t n, const int64_t *rowptr, const int64_t *col, const double *val,
                     double dt, double *psi, int64_t ld, int64_t m, double tol, int kdim, int nthreads) {
    if (kdim < 2 || kdim > 90) return -1;
    int fails = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel reduction(+ : fails)
    {
        cplx *Q = (cplx *)malloc(sizeof(cplx) * (size_t)n * (size_t)(kdim + 1));
        cplx *out = (cplx *)malloc(sizeof(cplx) * (size_t)n);
#pragma omp for schedule(dynamic, 1)
        for (int64_t k = 0; k < m; ++k) {
            cplx *x = (cplx *)(psi) + k * ld;
            if (lanczos_expv(n, rowptr, col, (const cplx *)val, dt, x, tol, kdim, Q, out, 0)) fails += 1;
        }
        free(Q);
        free(out);
    }
    return fails;
}

/* Threads available to the OpenMP runtime (for the baseline's `cores` field). */
int lmo_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
