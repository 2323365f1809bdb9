/*
 * lmgpu.h -- C ABI of the GB300 backend for the LatticeModels.jl time-evolution path.
 *
 * The path is `Evolution(t -> tightbinding_hamiltonian(l; field), P_0)` read out through
 * `localdensity` and `DensityCurrents`.  A Julia `EvolutionSolver` subtype (or any other host
 * language through its C FFI) drives it through the calls below.  All citations are to
 * LatticeModels.jl v1.0.7, paths relative to that repository's root.
 *
 * Conventions
 *  - Every call returns an int status: LM_OK (0) or an LM_ERR_* code; `lm_last_error(ctx)`
 *    returns the message of the last failure on that context.
 *  - Host pointers are borrowed for the duration of the call only.  The library owns all
 *    device memory it allocates.  Complex numbers are interleaved (re, im) pairs.
 *  - Site indices are those of the reference: 1-based, x-major with y fastest, i.e.
 *    index = (x-1)*Ly + y.  Bonds follow the reference's NearestNeighbor(1) iteration order:
 *    every +x bond (source sites in index order), then every +y bond.
 *  - Calls on one context are ordered on that context's CUDA stream; a context is used from
 *    one host thread at a time.  There is no CPU fallback: without a usable GPU,
 *    lm_ctx_create fails.
 */
#ifndef LMGPU_H
#define LMGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LM_OK 0
#define LM_ERR_ARG 1       /* bad argument (null pointer, size, mismatched objects) */
#define LM_ERR_OOM 2       /* device allocation failed */
#define LM_ERR_CUDA 3      /* CUDA runtime error */
#define LM_ERR_TIMEOUT 4   /* a bounded device wait gave up */
#define LM_ERR_NONFINITE 5 /* non-finite value detected */
#define LM_ERR_STATE 6     /* call out of order (e.g. step before update) */
#define LM_ERR_NOTSUP 7    /* configuration outside what the backend implements */

#define LM_C64 0 /* ComplexF64 state, FP64 recurrence (the plain form) */
#define LM_C32 1 /* ComplexF32 state, FP32 recurrence with FP64 coefficients/reductions */

#define LM_KETS 0    /* N x M block of kets, column-major (each ket contiguous) */
#define LM_DENSITY 1 /* N x N density matrix, column-major */

#define LM_FIELD_LANDAU 1             /* LandauGauge(B): src/zoo/magneticfields.jl:11-15 */
#define LM_FIELD_SYMMETRIC 2          /* SymmetricGauge(B): src/zoo/magneticfields.jl:27-31 */
#define LM_FIELD_POINTFLUX_AXIAL 3    /* PointFlux(phi, p; gauge=:axial): :72-85 */
#define LM_FIELD_POINTFLUX_SINGULAR 4 /* PointFlux(phi, p; gauge=:singular): :89-104 */

typedef struct lm_ctx lm_ctx;
typedef struct lm_lattice lm_lattice;
typedef struct lm_ham lm_ham;
typedef struct lm_state lm_state;
typedef struct lm_solver lm_solver;

/* Library version (major*10000 + minor*100 + patch). */
int lm_version(void);

/* ---- context ------------------------------------------------------------------------ */
/* Creates a context on CUDA device `device` with its own stream. No reference counterpart:
 * the reference runs on the CPU (src/evolution.jl:183-196 holds no device state). */
int lm_ctx_create(int device, lm_ctx **out);
int lm_ctx_destroy(lm_ctx *ctx);
const char *lm_last_error(const lm_ctx *ctx);
int lm_ctx_synchronize(lm_ctx *ctx);
/* The context's CUDA stream (cudaStream_t), for callers that order their own work or
 * CUDA events against the library's launches. */
int lm_ctx_stream(lm_ctx *ctx, void **stream);
/* Context options.  LM_OPT_FUSED (default 1): a ComplexF32 ket-block step whose Chebyshev
 * order is at most 8 runs as one temporally blocked launch; 0 selects one launch per order
 * (same results to FP32 rounding; kept for comparison). */
#define LM_OPT_FUSED 1
/* LM_OPT_STREAM (default 1): a single lattice with even Ly, Lx >= 2K + 3 and K <= 6 runs the
 * fused step in its x-streaming form (a warp walks one ket along x with a halo only in y);
 * 0 selects the region form (a halo on both axes).  Both give bit-identical results. */
#define LM_OPT_STREAM 2
/* LM_OPT_KPM (default 1): the recurrences of lm_kpm_moments and lm_cheb_apply run in
 * double-float arithmetic (pairs of FP32 values, about 48 significant bits) on the FP32 pipe;
 * 0 selects FP64.  KPM moments agree to about 1e-15 mu_0. */
#define LM_OPT_KPM 3
/* LM_OPT_RESIDENT (default 1): in a ComplexF32 batch's fused pass, lattices of up to 4608
 * sites (one CTA; smaller ones several kets per CTA) or 9216 sites (a cluster of two CTAs)
 * keep a whole ket on chip for all K orders (K <= 40); 0 runs them in the region form.  Both
 * give bit-identical results.  Takes effect at the next lm_batch_update. */
#define LM_OPT_RESIDENT 4
int lm_ctx_set_option(lm_ctx *ctx, int option, int value);
/* Number of fused steps that ran in the x-streaming form on this context so far. */
int lm_ctx_stream_launches(lm_ctx *ctx, int64_t *n);
/* Opt-in CUDA-event timing of the Chebyshev-order launches (for measurement); events are
 * resolved lazily by lm_ctx_timing, so timing adds no host synchronisation per step. */
int lm_ctx_set_timing(lm_ctx *ctx, int enable);
int lm_ctx_timing(lm_ctx *ctx, double *order_ms, int64_t *order_launches, int64_t *launches);
int lm_ctx_reset_timing(lm_ctx *ctx);

/* ---- lattice ------------------------------------------------------------------------ */
/* SquareLattice(Lx, Ly; boundaries=(:axis1 => theta_x, :axis2 => theta_y)); `ctx` may be NULL
 * for a host-only lattice (bond and coordinate queries need no GPU).
 * Replaces SquareLattice / span_unitcells / setboundaries (src/zoo/lattices.jl:131,
 * src/lattices/bravais/lattice.jl:101-172, src/core/boundaries.jl:46-76, :219-226).
 * periodic_* = 0 gives an open axis; twist_* is the TwistedBoundary angle (0 = periodic). */
int lm_lattice_square(lm_ctx *ctx, int64_t Lx, int64_t Ly, int periodic_x, int periodic_y,
                      double twist_x, double twist_y, lm_lattice **out);
int lm_lattice_destroy(lm_lattice *lat);
/* length(l) (src/lattices/bravais/lattice.jl:34). */
int64_t lm_lattice_nsites(const lm_lattice *lat);
/* Number of NearestNeighbor(1) bonds after boundary routing (src/core/bonds.jl:415-422). */
int64_t lm_lattice_nbonds(const lm_lattice *lat);
/* Bond list in iteration order, 1-based (src/core/bonds.jl:415-422,
 * src/lattices/bravais/nearestneighbor.jl:97-131, src/core/boundaries.jl:251-289). */
int lm_lattice_bonds(const lm_lattice *lat, int64_t *src, int64_t *dst);
/* Site coordinates, x then y per site (2N doubles) (src/lattices/bravais/unitcell.jl:119-122). */
int lm_lattice_coords(const lm_lattice *lat, double *xy);

/* ---- Hamiltonian -------------------------------------------------------------------- */
/* tightbinding_hamiltonian(l; t1) with on-device assembly.  Replaces
 * construct_operator / OperatorBuilder / UniformMatrixBuilder
 * (src/operators/constructoperator.jl:136-194, src/operators/builder.jl:86-151, :274-309). */
int lm_ham_create(lm_ctx *ctx, lm_lattice *lat, double t1, lm_ham **out);
int lm_ham_destroy(lm_ham *ham);
/* Adds a gauge-field term; `amplitudes[k]` of lm_ham_assemble scales component k.
 * `auto_pbc` = 1 applies adapt_field for lattices with boundaries (point fluxes become
 * singular-gauge images, src/zoo/magneticfields.jl:237-266), as OperatorBuilder does by
 * default (src/operators/builder.jl:165-174). */
int lm_ham_add_field(lm_ham *ham, int kind, double px, double py, int auto_pbc, int *component);
/* On-site term `LatticeValue => 1` (src/operators/constructoperator.jl:21-30); NULL clears. */
int lm_ham_set_onsite(lm_ham *ham, const double *V);
/* Evaluates H(t) on the device: H[i,j] = t1*f_b*exp(-2 pi i LI(r_i, r_j)), H[j,i] = conj,
 * H[i,i] += V_i (src/operators/builder.jl:282-285, :296-309). */
int lm_ham_assemble(lm_ham *ham, const double *amplitudes, int ncomponents);
/* Stored entries of the assembled H as the reference's CSC (src/operators/builder.jl:143-151). */
int lm_ham_nnz(lm_ham *ham, int64_t *nnz);
int lm_ham_csc(lm_ham *ham, int64_t *colptr, int64_t *rowval, double *nzval);
/* Gershgorin enclosure of the spectrum of the assembled H. */
int lm_ham_bounds(lm_ham *ham, double *emin, double *emax);

/* ---- states ------------------------------------------------------------------------- */
/* Device state: a Ket block (N x M) or a density matrix (N x N).  The reference evolves
 * `Ket`/`Operator` data in place (src/evolution.jl:69-80, :188-196). */
int lm_state_create(lm_ctx *ctx, int64_t n, int64_t m, int kind, int precision, lm_state **out);
int lm_state_destroy(lm_state *st);
/* Host <-> device copies; `host` holds complex values in the state's precision,
 * column-major with leading dimension `ld` (>= n).  lm_state_upload also accepts a device
 * pointer (unified addressing): the copy then stays on the device.  From pageable memory the
 * upload has read `host` when it returns; from pinned or device memory it is asynchronous
 * (ordered on the context's stream), so keep
 * that buffer unchanged until a synchronising call (lm_ctx_synchronize, a download, a
 * readout). */
int lm_state_upload(lm_state *st, const void *host, int64_t ld);
int lm_state_download(lm_state *st, void *host, int64_t ld);
/* Device-to-device copy of `src` into `dst` (same shape, kind and precision): the state
 * copy `Evolution` makes at construction (src/evolution.jl:190-194). */
int lm_state_copy(lm_state *dst, const lm_state *src);
/* Current device buffer (it may change after a step) and its leading dimension. */
int lm_state_device_ptr(lm_state *st, void **ptr, int64_t *ld);
/* Ket weights w_m, so that P = sum_m w_m |psi_m><psi_m| for the readouts; NULL = all ones. */
int lm_state_set_weights(lm_state *st, const double *w);
/* Per-ket FP64 norms (m doubles). */
int lm_state_norms(lm_state *st, double *out);
/* Rescales every ket to the given FP64 norms (the FP32 form's periodic norm correction).
 * Stream-ordered: returns without waiting for the device; target_norms is copied during the
 * call. */
int lm_state_renormalize(lm_state *st, const double *target_norms);
/* Compensated ComplexF32 kets (enable != 0): the state keeps, beside each FP32 amplitude,
 * the residual of its last rounding (a bfloat16 pair per site: 8 significant bits of the
 * residual), and the fused Chebyshev step forms the new amplitude from the (value, residual)
 * pair with error-free FP32 transformations (Dekker TwoProd via fmaf, Knuth TwoSum).  The
 * state then carries about 32 significant bits from step to step, so the rounding walk of
 * long FP32 runs (the 400-step current) shrinks, at the cost of 8 more bytes per site-ket of
 * traffic (the residual read and written once per step).  ComplexF32 ket blocks stepped by
 * lm_solver_step through the x-streaming form: square lattices with Ly even and Lx >= 2K + 3
 * (K <= 5 with complex x-hops) and honeycomb lattices in the brick layout; other paths return
 * LM_ERR_NOTSUP.  Uploads clear the residual; copies carry it;
 * norms and renormalize use value + residual.  enable == 0 drops it. */
int lm_state_set_compensation(lm_state *st, int enable);

/* ---- evolution solver (the EvolutionSolver plugin, src/evolution.jl:5-33) ------------ */
/* ChebyshevGPU(; tol): Chebyshev propagator exp(-i H dt) with truncation `tol`. */
int lm_solver_create(lm_ctx *ctx, double tol, lm_solver **out);
int lm_solver_destroy(lm_solver *s);
/* update_solver!(solver, H, dt, force) (src/evolution.jl:83-92): recomputes the
 * propagator unless H (same object, same assembly) and dt are unchanged and force = 0. */
int lm_solver_update(lm_solver *s, lm_ham *ham, double dt, int force);
/* Fixes the spectral interval [emin, emax] of the propagator (the Gershgorin enclosure of the
 * Hamiltonian otherwise; emin = emax = 0 restores it).  With fixed bounds the propagator is
 * one polynomial in H for every parameter value, which the adjoint differentiates exactly. */
int lm_solver_set_bounds(lm_solver *s, double emin, double emax);
/* Chebyshev order chosen by the last update (number of H applications per step). */
int lm_solver_order(const lm_solver *s, int *K, double *a, double *b);
/* step!(solver, state, cache) (src/evolution.jl:69-78): psi <- U psi for kets,
 * P <- U P U^dagger for a density matrix. */
int lm_solver_step(lm_solver *s, lm_state *st);

/* Chebyshev plan (host only, needs no GPU): for x = a*|dt| >= 0 (a = spectral half-width)
 * the order K >= 2 whose neglected tail 2*sum_{k>K}|J_k(x)| is below `tol`, and the
 * coefficients c_k = (2 - delta_k0) (-i)^k J_k(x), k = 0..K, as (re, im) pairs in `coef`
 * (room for `cap` coefficients).  Returns LM_ERR_ARG when cap < K + 1. */
int lm_chebyshev_plan(double x, double tol, int cap, int *K, double *coef);

/* Allocation-free variant of lm_solver_step for a caller-owned ComplexF64 (precision LM_C64)
 * or ComplexF32 (LM_C32) ket block: `kets` is a device pointer to the n x m column-major block
 * (leading dimension ld >= n), advanced in place by exp(-i H dt) with the per-order Chebyshev
 * kernel.  It has no counterpart in the reference.  It calls no cudaMalloc/cudaFree: the
 * recurrence and accumulator buffers live in a 32 MiB static device array that every GPU
 * loading the library holds until exit, for hosts whose device memory belongs to another
 * allocator or that forbid allocation after start-up.  Limit: ld * m <= 1 Mi (ComplexF64) or
 * 2 Mi (ComplexF32), else LM_ERR_ARG.  The first call on a device sets up the array's address
 * (call it once before any stream capture); calls that overlap on the GPU share the array and
 * race. */
int lm_solver_step_noalloc(lm_solver *s, void *kets, int64_t n, int64_t m, int64_t ld, int precision);

/* ---- batches of independent lattices ------------------------------------------------ */
/* Many (Hamiltonian, state) pairs of different sizes evolved together: every step is a
 * fixed sequence of launches over the work items of all instances (ComplexF32 with K <= 8:
 * one temporally blocked launch per pass fed by an atomic work queue; otherwise K launches
 * of the per-order kernel), replayed from a CUDA graph.  The reference evolves each state
 * separately (src/evolution.jl:245-247); a batch is the same step! applied to all of them.
 * Density matrices use U P U^dagger = U (U P)^dagger (Hermitian P). */
typedef struct lm_batch lm_batch;
int lm_batch_create(lm_ctx *ctx, int kind, int precision, double tol, lm_batch **out);
int lm_batch_destroy(lm_batch *b);
/* Adds one instance (its Hamiltonian must be assembled before lm_batch_update). */
int lm_batch_add(lm_batch *b, lm_ham *ham, lm_state *st, int *index);
/* update_solver! for every instance; K = the largest order over the instances. */
int lm_batch_update(lm_batch *b, double dt);
/* step! for every instance (the states' device buffers may swap, see lm_state_device_ptr). */
int lm_batch_step(lm_batch *b);
/* 1 (default): capture the step into a CUDA graph once per buffer parity and replay it. */
int lm_batch_set_graph(lm_batch *b, int enable);
/* Column panels of `width` columns (0: off): the per-order recurrence runs in place on each
 * panel with per-lattice panel scratch (2 x n x width), and a density matrix takes in-place
 * conjugate transposes, so the batch needs no full-size recurrence buffers (~3x less memory;
 * ComplexF64 batches that would not fit otherwise).  Takes effect at the next update. */
int lm_batch_set_panel(lm_batch *b, int64_t width);
/* Pass shape: -1 auto, 0 one temporally blocked launch per pass, 1/2/3 one launch per
 * order with 2/4/8 kets per thread. */
int lm_batch_set_config(lm_batch *b, int cfg);
int lm_batch_info(lm_batch *b, int *K, int *cfg, int64_t *items, int *ninst);
/* Autotuner: times `steps` steps of every eligible pass shape on copies of the states
 * (ms_out[0..3], -1 when not eligible), keeps the fastest (*best). */
int lm_batch_tune(lm_batch *b, int steps, double *ms_out, int *best);

/* ---- adjoint (gradients of a density loss) ----------------------------------------- */
/* Co-state propagation through the Chebyshev steps for L = sum_i (rho_i(T) - target_i)^2,
 * rho_i = sum_m |psi_im|^2: gradients with respect to every on-site potential V_i and to the
 * amplitude of one field component per step (accumulated into `nslots` slots, e.g. one per
 * piecewise-constant flux interval).  No reference counterpart (the reference has no
 * derivatives); it differentiates the same step! (src/evolution.jl:69-78). */
typedef struct lm_adjoint lm_adjoint;
int lm_adjoint_create(lm_ctx *ctx, int64_t n, int64_t m, int precision, int nslots, lm_adjoint **out);
int lm_adjoint_destroy(lm_adjoint *a);
/* Zeroes the accumulated gradients. */
int lm_adjoint_reset(lm_adjoint *a);
/* Final co-state lambda = dL/dpsi* = 4 (rho - target) psi (host target, N values) and the loss. */
int lm_adjoint_seed(lm_adjoint *a, lm_state *psi, const double *target, lm_state *lambda, double *loss);
/* Gradient terms of step n (psi = psi_n, lambda = lambda_{n+1}); `s` must be updated with `ham`
 * and dt.  component >= 0 also accumulates dL/d(amplitude of that field component) into
 * gradient slot `slot`.  The caller then applies U_n^dagger to lambda (a solver updated with -dt). */
int lm_adjoint_step(lm_adjoint *a, lm_solver *s, lm_ham *ham, int component, int slot, lm_state *psi,
                    lm_state *lambda);
/* Downloads the accumulated gradients (N on-site values, nslots field amplitudes). */
int lm_adjoint_gradients(lm_adjoint *a, double *gV, double *gA);

/* ---- readouts ----------------------------------------------------------------------- */
/* localdensity(state) (src/operators/latticeutils.jl:41-45): N doubles. */
int lm_localdensity(lm_state *st, double *out);
/* DensityCurrents(H, state) on every bond, J_b = 2 Im(H[i,j] P[j,i])
 * (src/zoo/currents.jl:92-102), in lm_lattice_bonds order: nbonds doubles. */
int lm_bond_currents(lm_ham *ham, lm_state *st, double *out);
/* tr(P) = sum of the local densities, FP64 (particle number). */
int lm_trace(lm_state *st, double *out);

/* ---- general sparse Hamiltonians (other lattices, internal degrees of freedom) -------------- */
/* Any Hermitian operator that the reference's construct_operator builds
 * (src/operators/constructoperator.jl:4-47) -- HoneycombLattice, KagomeLattice, qwz and the
 * other zoo models, next-nearest hopping -- given as its SparseMatrixCSC: 1-based colptr
 * (n+1) and rowval (nnz), nzval as interleaved (re, im) pairs.  Stored on the device in ELL
 * form; LM_ERR_ARG when the matrix is not Hermitian to 1e-12 of its largest entry. */
typedef struct lm_ell lm_ell;
int lm_ell_create_csc(lm_ctx *ctx, int64_t n, const int64_t *colptr, const int64_t *rowval, const double *nzval,
                      lm_ell **out);
int lm_ell_destroy(lm_ell *h);
/* New values on the same pattern (H(t) every step). */
int lm_ell_set_values(lm_ell *h, const double *nzval);
/* Gershgorin interval of the current values. */
int lm_ell_bounds(const lm_ell *h, double *emin, double *emax);
/* update_solver!(solver, H, dt, force) for a general Hamiltonian (src/evolution.jl:83-92);
 * lm_solver_step then applies its propagator to kets or density matrices. */
/* A general lattice Hamiltonian assembled on the device from its bonds, the way the
 * reference's builder assembles it (src/operators/builder.jl:296-309,
 * src/operators/constructoperator.jl:4-47): bond b joins sites src[b] -> dst[b] (1-based)
 * with real-space endpoints xy[4b .. 4b+3] = (x1, y1, x2, y2), the destination unwrapped across
 * a periodic boundary, and base value base[2b], base[2b+1] (t1 times the boundary's twist
 * factor).  lm_ell_assemble sets H[src, dst] += base exp(-2 pi i LI(field; r1 -> r2)) and
 * H[dst, src] += its conjugate for every bond, H[i, i] = the on-site term, on the device:
 * the Hamiltonian of every step of a time-dependent field is assembled without a host
 * upload.  Field components: LM_FIELD_*, without boundary images (the reference's
 * adapt_field replication applies to the square-lattice path).  Replaces passing the
 * construct_operator CSC of HoneycombLattice / KagomeLattice / TriangularLattice models. */
int lm_ell_create_bonds(lm_ctx *ctx, int64_t n, int64_t nbonds, const int64_t *src, const int64_t *dst,
                        const double *xy, const double *base, lm_ell **out);
int lm_ell_add_field(lm_ell *ham, int kind, double px, double py, int *component);
/* n on-site values, or NULL for none (copied during the call). */
int lm_ell_set_onsite(lm_ell *ham, const double *onsite);
/* One amplitude per field component; asynchronous on the context's stream. */
int lm_ell_assemble(lm_ell *ham, const double *amplitudes, int namp);
/* Site layout of a general Hamiltonian that a temporally blocked kernel can step.
 * LM_LAYOUT_HONEYCOMB: an a x b HoneycombLattice (2ab sites) in the reference's site order
 * ((j1, j2, s) -> 2((j1-1) b + j2 - 1) + s - 1, src/lattices/bravais/unitcell.jl:113-132;
 * basis [0, 0] and [1/2, sqrt(3)/6], src/zoo/lattices.jl:145-160) with nearest-neighbour
 * bonds only; periodic_a / periodic_b: the boundaries along a a1 / b a2.  Every stored entry is
 * checked to be one of the three bonds of its site (LM_ERR_ARG otherwise).  ComplexF32 ket
 * blocks are then stepped by the x-streaming kernel as an a x 2b lattice (a >= 2K + 3;
 * otherwise, and for ComplexF64 or density matrices, the per-order ELL kernels run).
 * LM_LAYOUT_NONE drops the layout. */
#define LM_LAYOUT_NONE 0
#define LM_LAYOUT_HONEYCOMB 1
int lm_ell_set_layout(lm_ell *h, int layout, int64_t a, int64_t b, int periodic_a, int periodic_b);
int lm_ell_solver_update(lm_solver *s, lm_ell *h, double dt, int force);
/* DensityCurrents(H, state)[i, j] = 2 Im(H[i,j] P[j,i]) (src/zoo/currents.jl:92-102) for every
 * stored entry of the CSC, in its order (0 for the diagonal): nnz doubles. */
int lm_ell_currents(lm_ell *h, lm_state *st, double *out);
/* LocalOperatorCurrents(H, state, op)[i, j] (src/zoo/currents.jl:170-184) per stored entry:
 * with ndof internal states per site (matrix index = ndof (site - 1) + alpha), the entry
 * (r, c) = ((i, k), (j, beta)) contributes 2 Im(H[r,c] sum_alpha op[alpha,k] P[c, (i, alpha)]);
 * summing the entries of the (i, j) site block gives the reference's value.  Entries inside
 * one site block give 0.  op: ndof x ndof complex, column-major, interleaved re/im; NULL is
 * the identity (DensityCurrents summed per site block).  1 <= ndof <= 8, n divisible by ndof. */
int lm_ell_op_currents(lm_ell *h, lm_state *st, int ndof, const double *op, double *out);

/* ---- KPM moments (DOS / LDOS without an eigensystem; the reference computes dos and ldos
 * from an Eigensystem or GreenFunction, src/greenfunction.jl:306-339) ------------------------ */
/* mu_n = sum over the columns v of the block of <v| T_n(H~) |v>, H~ = (H - b)/a with
 * [b - a, b + a] = [emin, emax], which must enclose the spectrum (LM_ERR_NONFINITE when the
 * moments show that it does not), n = 0..nmom-1, in FP64.  vecs: a ComplexF64 ket block of
 * starting vectors (stochastic trace), or NULL for the N unit vectors (exact trace; N x N
 * scratch).  per_column = 0: out[n] sums the columns; otherwise out[j*nmom + n] holds column j
 * (with unit vectors: the local moments of site j).  Extension of the reference. */
int lm_kpm_moments(lm_ham *ham, double emin, double emax, int nmom, const lm_state *vecs, int per_column,
                   double *out);
/* out = sum_{n < ncoef} coef[n] T_n(H~) in, with real coefficients and an FP64 recurrence on
 * [emin, emax] (must enclose the spectrum).  in: an N x M state, or NULL for the identity (out
 * is then the N x N matrix f(H), e.g. the Fermi operator of densitymatrix at T > 0,
 * src/spectrum.jl:226-257, from the Chebyshev coefficients of the occupation).  out: N x M,
 * ComplexF64 or ComplexF32 (rounded at the end).  Extension of the reference (which
 * diagonalises). */
int lm_cheb_apply(lm_ham *ham, double emin, double emax, const double *coef, int ncoef, const lm_state *in,
                  lm_state *out);
/* Spectral interval by FP64 Lanczos (iters steps from a seeded random-phase vector): the
 * extreme Ritz values padded by their residuals and 1 % of the width, clipped to the
 * Gershgorin interval of lm_ham_bounds.  A tighter interval lowers the Chebyshev order;
 * pass it to lm_solver_set_bounds, lm_kpm_moments or lm_cheb_apply. */
int lm_ham_lanczos_bounds(lm_ham *ham, int iters, unsigned long long seed, double *emin, double *emax);

/* ---- eigensystem (diagonalize / densitymatrix, src/spectrum.jl:48-55, :226-257, :317-333) ---- */
/* The Hermitian eigensystem of an assembled Hamiltonian, computed on the device in FP64 with
 * the library's own kernels (Householder tridiagonalisation, bisection, inverse iteration,
 * back-transformation; no vendor eigensolver).  Replaces the reference's dense LAPACK
 * `eigen` in `diagonalize` (src/spectrum.jl:48-55).  The object holds the N x N reduced
 * matrix (16 N^2 bytes) until destroyed; every call synchronises the context's stream. */
typedef struct lm_eigsys lm_eigsys;
/* Square-lattice Hamiltonian (as last assembled) or general sparse Hamiltonian. */
int lm_eigsys_create(lm_ham *ham, lm_eigsys **out);
int lm_eigsys_create_ell(lm_ell *ham, lm_eigsys **out);
int lm_eigsys_destroy(lm_eigsys *e);
int lm_eigsys_size(const lm_eigsys *e, int64_t *n);
/* The N eigenvalues in ascending order (host array of N doubles). */
int lm_eigsys_values(const lm_eigsys *e, double *out);
/* Eigenvectors first .. first + m - 1 (ascending eigenvalue order) into the columns of a
 * ket state out (N x m, ComplexF64 or ComplexF32), each of unit norm; the sign is fixed by
 * making the largest component of the tridiagonal eigenvector positive. */
int lm_eigsys_vectors(lm_eigsys *e, int64_t first, lm_state *out);
/* out (an N x N density state) = sum_k weights[k] v_k v_k^H over the eigenvectors whose weight
 * is nonzero (weights: host array of N doubles in eigenvalue order).  With the occupations of
 * src/spectrum.jl:226-257 as weights this is densitymatrix(eigensystem; mu, T). */
int lm_eigsys_projector(lm_eigsys *e, const double *weights, lm_state *out);

/* ---- readout ring (device side of TimeSequence(f, ev(times)), src/timesequence.jl:41-43) -- */
/* Per-moment readouts computed into the slots of a device ring and downloaded asynchronously
 * into pinned host memory: pushing does not wait for the device, so an evolution loop that
 * records every step keeps the GPU busy.  (The first readout of a context, or the first of a
 * larger shape, allocates the readout's slice scratch, which synchronises the device once.)  Entry s lives in slot s % nslots; its host copy is
 * valid from lm_ring_wait(s) until entry s + nslots is pushed.  Extension of the reference:
 * it has no asynchronous readout. */
typedef struct lm_ring lm_ring;
int lm_ring_create(lm_ctx *ctx, int nslots, int64_t len, lm_ring **out);
int lm_ring_destroy(lm_ring *r);
/* localdensity(state) at time t (src/operators/latticeutils.jl:41-45); *seq = entry number. */
int lm_ring_push_localdensity(lm_ring *r, lm_state *st, double t, int64_t *seq);
/* DensityCurrents(ham, state) on every bond (src/zoo/currents.jl:92-102) at time t. */
int lm_ring_push_currents(lm_ring *r, lm_ham *ham, lm_state *st, double t, int64_t *seq);
/* LocalOperatorCurrents (lm_ell_op_currents) of a general Hamiltonian into the next slot:
 * nnz values in CSC order. */
int lm_ring_push_op_currents(lm_ring *r, lm_ell *h, lm_state *st, int ndof, const double *op, double t,
                             int64_t *seq);
/* *ready = 1 when entry seq has reached host memory (LM_ERR_ARG once it is overwritten). */
int lm_ring_ready(lm_ring *r, int64_t seq, int *ready);
/* Waits for entry seq; copies it to out (if non-null), returns the pinned view, the number
 * of values and the time stamp (each optional). */
int lm_ring_wait(lm_ring *r, int64_t seq, double *out, const double **view, int64_t *n, double *t);
/* Sequence number of the next entry. */
int lm_ring_head(const lm_ring *r, int64_t *head);

#ifdef __cplusplus
}
#endif
#endif /* LMGPU_H */
