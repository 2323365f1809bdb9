// Internal definitions shared by the lmgpu translation units (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/lmgpu.h"

namespace lmgpu {

// ------------------------------------------------------------------------------------------
// Square-lattice geometry.  Site index (0-based) s = (x-1)*Ly + (y-1) for x in 1..Lx,
// y in 1..Ly: the reference sorts Bravais pointers lexicographically
// (src/lattices/bravais/unitcell.jl:126-132), so y runs fastest.
// ------------------------------------------------------------------------------------------
struct Geom {
    int64_t Lx, Ly, N;
    int per_x, per_y;     // periodic axes
    double twist_x, twist_y;
};

// Field component as evaluated by the assembly kernel.  `amp` is the time-dependent
// amplitude (B or flux), the rest is fixed at creation.
struct FieldComp {
    int kind;             // LM_FIELD_*
    int replicate;        // point flux replicated over the 3^d boundary images (singular gauge)
    double px, py;
};

constexpr int kMaxFields = 8;

struct FieldSet {
    int n;
    FieldComp c[kMaxFields];
    double amp[kMaxFields];
};

// Largest Chebyshev order the temporally blocked kernel handles in one pass (its halo).
constexpr int kFusedMaxK = 8;
// Kets per work item of the temporally blocked kernel.
constexpr int kFusedKetsPerItem = 16;

// Per-order launch description of the Chebyshev recurrence.
enum ChebMode { CHEB_FIRST = 0, CHEB_MID = 1, CHEB_LAST = 2 };

template <typename R> struct V2;
template <> struct V2<double> { typedef double2 T; };
template <> struct V2<float> { typedef float2 T; };

struct ChebCoef {
    double s;        // real magnitude with sign: c_k = s (k even) or -i*s (k odd)
    int odd;         // parity of k
};

// Second FP32 words of the scalar constants of one FP32 step.  The FP32 kernels apply
//   per-order form: out = ph_h (c0_h T0 + c1_h T1 + g0 T0 + g1 T1 + sum_{k>=2} c_k T_k)
//   fused form:     out = ph_h (c1_h T1 + g0 T0 + g1 T1 + sum_{k>=2} c_k T_k) + a0_h T0
// with ph_h, c0_h, c1_h, a0_h the FP32 roundings of e^{-ib dt}, c_0, c_1 and e^{-ib dt} c_0;
// g0 and g1 (complex) restore the FP64 values of the T0 and T1 terms.  Without them the
// rounding of c_0 scales every step by the same factor 1 + O(1e-8), which compounds: after
// 400 steps the density is off by ~1e-5.
struct ChebLo {
    float g0_re, g0_im, g1_re, g1_im;
};
// ph = e^{-ib dt} (after any conjugation), c_0 = c0, c_1 = -i s1; fused selects the form.
ChebLo cheb_lo(double ph_re, double ph_im, double c0, double s1, bool fused);

// One lattice of a temporally blocked launch: geometry, stencil tables, in/out ket blocks,
// its first global work item and its Chebyshev coefficients (c_k = s_k or -i s_k by parity).
struct FusedInst {
    Geom g;
    const float2* hop2;
    const float* diag2;
    const float2* x;
    float2* out;
    int64_t ld, M;
    int ntx, nty;
    int64_t item_begin;
    float s[kFusedMaxK + 1];
    float ph_re, ph_im;   // e^{-ib dt}
    float a0_re, a0_im;   // e^{-ib dt} c_0
    ChebLo lo;            // fused-form second words
    uint32_t* comp;       // encoded residual plane of x, updated in place (x-streaming form only), or null
};

}  // namespace lmgpu

// ------------------------------------------------------------------------------------------
// Opaque handle bodies.
// ------------------------------------------------------------------------------------------
struct lm_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int sm_count = 0;
    std::string err;
    int timing = 0;
    int fused = 1;                      // LM_OPT_FUSED: temporally blocked c32 step enabled
    unsigned fused_attr = 0;            // bit K (+16 for real x-hops): shared-memory attribute set
    unsigned long long stream_attr = 0;       // the same for the x-streaming form (bit K + 8 mode)
    unsigned long long stream_attr_comp = 0;  // the same for its compensated-state variant
    int fused_form = 1;                 // LM_OPT_STREAM: 1 = x-streaming form where supported, 0 = region form
    int64_t stream_launches = 0;        // fused steps run in the x-streaming form
    int kpm_df = 1;                     // LM_OPT_KPM: double-float recurrence in lm_kpm_moments
    int resident = 1;                   // LM_OPT_RESIDENT: lattice-resident form in the batch's fused pass
    std::vector<double> h_norms;        // pageable staging of lm_state_renormalize's targets
    std::vector<cudaEvent_t> ev_pool;   // pairs (start, stop) of timed Chebyshev sweeps
    std::vector<int> ev_launches;       // launches covered by each recorded pair
    size_t ev_used = 0;                 // pairs recorded but not yet resolved
    double order_ms = 0.0;         // accumulated device time of Chebyshev-order launches
    int64_t order_launches = 0;
    int64_t launches = 0;          // every kernel launched by the library
    double* d_red = nullptr;       // small reduction scratch (owned)
    size_t red_cap = 0;
    double* d_ld_part = nullptr;   // per-slice partial densities of the ket readout (owned)
    size_t ld_part_cap = 0;
    int ld_slices_override = 0;    // LMGPU_READOUT_SLICES: fixed ket-slice count of the readout (0 = chosen)
    int currents_scalar = 0;       // LMGPU_CURRENTS_SCALAR=1: c32 bond currents with one site per lane
};

struct lm_lattice {
    lm_ctx* ctx = nullptr;
    lmgpu::Geom g{};
    int64_t nbonds = 0;
};

struct lm_ham {
    lm_ctx* ctx = nullptr;
    lm_lattice* lat = nullptr;
    double t1 = 1.0;
    lmgpu::FieldSet fields{};
    double* d_onsite = nullptr;     // raw on-site V (N) or null
    double vmin = 0.0, vmax = 0.0;  // on-site extrema (host-side bookkeeping)
    double2* d_hop = nullptr;       // raw H[s, s+x] (N) then H[s, s+y] (N)
    uint64_t version = 0;           // bumps on every assembly
    int assembled = 0;
    std::vector<double> last_amp;
    // pinned staging of the on-site upload: the caller's V is copied here during the call, so
    // the asynchronous copy never reads the caller's memory after lm_ham_set_onsite returns
    double* h_stage[2] = {nullptr, nullptr};
    cudaEvent_t stage_ev[2] = {nullptr, nullptr};
    int stage_next = 0;
};

struct lm_state {
    lm_ctx* ctx = nullptr;
    int64_t n = 0, m = 0, ld = 0;
    int kind = LM_KETS;
    int precision = LM_C64;
    void* d_data = nullptr;   // current state buffer
    void* d_a = nullptr;      // recurrence scratch (allocated on first use)
    void* d_y = nullptr;      // accumulator scratch
    double* d_w = nullptr;    // ket weights (m) or null (= all ones)
    size_t elem = 16;
    // compensated ComplexF32 ket block (lm_state_set_compensation): the rounding residual of
    // every element as a bfloat16 pair (res_encode), so that the state carries about 32
    // significant bits; element i of ket k at d_lo[k ld + i], updated in place by the
    // x-streaming step (null when off)
    uint32_t* d_lo = nullptr;
};

struct lm_solver {
    lm_ctx* ctx = nullptr;
    double tol = 1e-12;
    int precision_hint = -1;
    // cache key (update_solver! semantics)
    const lm_ham* ham = nullptr;
    uint64_t ham_version = ~0ull;
    double dt = 0.0;
    int valid = 0;
    // propagator
    double a = 1.0, b = 0.0;
    int K = 0;
    std::vector<lmgpu::ChebCoef> coef;  // k = 0..K
    double phase_re = 1.0, phase_im = 0.0;
    // normalised stencil tables: 2*H/a hops and 2*(V-b)/a diagonal
    double2* d_hop2 = nullptr;  double* d_diag2 = nullptr;
    float2* d_hop2f = nullptr;  float* d_diag2f = nullptr;
    int64_t tab_n = 0;
    uint64_t tab_version = 0;    // bumped whenever the tables are rewritten
    // x-streaming form: padded, packed FP32 coefficient planes (lmgpu_stream.cu)
    float4* d_spack = nullptr;
    size_t spack_f4 = 0;
    uint64_t spack_version = ~0ull;
    int bpack_valid = 0;         // d_spack holds the honeycomb brick planes of the current ELL tables
    int has_onsite = 0;
    int fixed_bounds = 0;        // lm_solver_set_bounds: use [fix_emin, fix_emax] instead of Gershgorin
    double fix_emin = 0.0, fix_emax = 0.0;
    // general sparse Hamiltonian (lm_ell_*): set by lm_ell_solver_update, cleared by
    // lm_solver_update; its normalised ELL values 2H/a (off-diagonal) and 2(H_ii - b)/a
    const lm_ell* ell = nullptr;
    uint64_t ell_version = ~0ull;
    double2* d_ev2 = nullptr;  double* d_ed2 = nullptr;
    float2* d_ev2f = nullptr;  float* d_ed2f = nullptr;
    int64_t ell_tab = 0;
};

// A general Hermitian sparse Hamiltonian in ELL form: row i holds up to w off-diagonal
// entries (column cols[k*n + i], value vals[k*n + i]; unused slots point at i with value 0)
// and its real diagonal diag[i].  Built from the reference's CSC; `map` sends every CSC
// entry to its ELL slot (k*n + i) or, for a diagonal entry, to -(i + 1).
struct lm_ell {
    lm_ctx* ctx = nullptr;
    int64_t n = 0, nnz = 0;
    int w = 0;
    int* d_cols = nullptr;
    double2* d_vals = nullptr;
    double* d_diag = nullptr;
    std::vector<int64_t> map;          // CSC entry -> ELL slot or -(row + 1) for the diagonal
    std::vector<int64_t> csc_row, csc_col;  // 0-based row / column of every CSC entry
    int* d_crow = nullptr;             // the same on the device (for the currents)
    int* d_ccol = nullptr;
    double2* d_cval = nullptr;         // CSC values on the device
    double emin = 0.0, emax = 0.0;     // Gershgorin interval
    uint64_t version = 0;
    std::vector<double2> h_vals;       // host staging of the ELL values
    std::vector<double> h_diag;
    // device assembly from a bond list (lm_ell_create_bonds): every CSC entry sums, in a fixed
    // order, the bonds that land on it (base * exp(-2 pi i LI(r_src -> r_dst)), or its
    // conjugate for the reverse entry); the diagonal adds the on-site term
    int64_t nbonds = 0;
    double* d_bxy = nullptr;           // 4 per bond: x1 y1 x2 y2 (destination unwrapped)
    double2* d_bbase = nullptr;        // base value per bond (t1 times the boundary twist)
    int64_t* d_eptr = nullptr;         // CSR over CSC entries: contributions of entry p
    int64_t* d_eterm = nullptr;        // contribution: (bond << 1) | conjugate
    int64_t* d_emap = nullptr;         // ELL slot of entry p, or -(row + 1) for the diagonal
    double* d_onsite = nullptr;        // on-site term (n) or null
    std::vector<double> h_onsite;      // its host copy (for the bounds)
    std::vector<double> rad;           // Gershgorin radius per row: sum of |base| (field-free)
    lmgpu::FieldSet fields{};
    int assembled = 0;
    // honeycomb brick layout (lm_ell_set_layout): an a x b HoneycombLattice in the reference's
    // site order, stepped by the x-streaming kernel (MODE 4) as an a x 2b lattice; per unit
    // cell the ELL value indices of its five distinct bonds (-1 = none)
    int brick = 0;
    int64_t brick_a = 0, brick_b = 0;
    int brick_px = 0, brick_py = 0;
    int* d_bmap = nullptr;
};

// Argument and CUDA-status checks that return the status from the calling C-ABI function.
#define CHECK_ARG(ctx, cond, msg)                                   \
    do {                                                            \
        if (!(cond)) return lmgpu::set_err(ctx, LM_ERR_ARG, msg);   \
    } while (0)

#define CUDA_TRY(ctx, expr, what)                                   \
    do {                                                            \
        int _rc = lmgpu::check_cuda(ctx, (expr), what);             \
        if (_rc != LM_OK) return _rc;                               \
    } while (0)

namespace lmgpu {

int set_err(lm_ctx* ctx, int code, const std::string& msg);
int check_cuda(lm_ctx* ctx, cudaError_t e, const char* what);

// Kernel launchers (lmgpu_kernels.cu).  All launch on ctx->stream and return cudaError_t.
cudaError_t launch_assemble(lm_ctx* ctx, const Geom& g, const FieldSet& f, double t1, double2* hop);
cudaError_t launch_normalise(lm_ctx* ctx, const Geom& g, const double2* hop, const double* onsite,
                             double a, double b, double2* hop2, double* diag2, float2* hop2f,
                             float* diag2f);
cudaError_t launch_cheb_order(lm_ctx* ctx, const Geom& g, int precision, int site_fast, int conj,
                              int mode, const void* hop2, const void* diag2, const void* tp, void* tq,
                              void* y, int64_t ld, int64_t m, double c0, ChebCoef ck,
                              double ph_re, double ph_im, ChebLo lo, bool xreal = false);
cudaError_t launch_scale(lm_ctx* ctx, int precision, void* x, int64_t n, int64_t m, int64_t ld,
                         double re, double im);
cudaError_t launch_localdensity(lm_ctx* ctx, int precision, int kind, const void* x, int64_t n,
                                int64_t m, int64_t ld, const double* w, double* out);
cudaError_t launch_bond_currents(lm_ctx* ctx, const Geom& g, int precision, int kind, const double2* hop,
                                 const void* x, int64_t m, int64_t ld, const double* w, double* out);
cudaError_t launch_column_norms(lm_ctx* ctx, int precision, const void* x, int64_t n, int64_t m,
                                int64_t ld, double* out);
cudaError_t launch_rescale_columns(lm_ctx* ctx, int precision, void* x, int64_t n, int64_t m,
                                   int64_t ld, const double* norms, const double* target);
// The same for a compensated ComplexF32 block: norms of hi + lo, and hi + lo rescaled and split
// again into hi and its encoded residual, both in FP32-pair arithmetic (no FP64 per element).
cudaError_t launch_column_norms_comp(lm_ctx* ctx, const float2* hi, const uint32_t* lo, int64_t n, int64_t m,
                                     int64_t ld, double* out);
cudaError_t launch_rescale_columns_comp(lm_ctx* ctx, float2* hi, uint32_t* lo, int64_t n, int64_t m, int64_t ld,
                                        const double* norms, const double* target);

// Error-free transformations (round to nearest): p + e = a b exactly; s + e = a + b exactly.
__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
    p = a * b;
    e = fmaf(a, b, -p);
}
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    const float r = a + b;
    const float bb = r - a;
    e = (a - (r - bb)) + (b - bb);
    s = r;
}

// Residual encoding of a compensated ComplexF32 amplitude (value hi + lo per real component,
// |lo| <= ulp(hi)/2): the residual pair rounded to bfloat16 (8 significant bits, the FP32
// exponent range), lo.x in bits 15..0 and lo.y in bits 31..16 of one word per site.  The
// stored residual is within 2^-9 |lo| <= 2^-10 ulp(hi) of the exact one, one conversion
// encodes a site and two bit operations decode it.
__device__ __forceinline__ unsigned res_encode(float lx, float ly) {
    unsigned w;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(w) : "f"(ly), "f"(lx));
    return w;
}
__device__ __forceinline__ float res_lo_x(unsigned w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float res_lo_y(unsigned w) { return __uint_as_float(w & 0xFFFF0000u); }
cudaError_t launch_sum(lm_ctx* ctx, const double* v, int64_t n, double* out1);
int fused_supported(int precision, int K);
int fused_supported_geom(const Geom& g);
int64_t fused_items(const Geom& g, int K, int64_t m, int* ntx, int* nty);
void fused_fill_coef(FusedInst& d, int K, const ChebCoef* coef, double ph_re, double ph_im);
// One launch over `nitems` work items of one instance (`single`) or of a device table of
// `ninst` instances pulled from the work-queue counter `d_queue` (zeroed before the launch).
cudaError_t launch_fused_table(lm_ctx* ctx, int K, bool xreal, const FusedInst* single, const FusedInst* d_table,
                               int ninst, int64_t nitems, unsigned long long* d_queue, int grid);
cudaError_t ensure_fused_attr(lm_ctx* ctx, int K, bool xreal);
// x-streaming form of the single-lattice c32 step (lmgpu_stream.cu): its preconditions, its
// packed coefficient planes (rebuilt from the FP32 tables when they change) and the launch.
bool stream_supported(const Geom& g, int K, int mode, const void* x, const void* out, int64_t ld);
int ensure_stream_pack(lm_solver* s, const Geom& g);
int ensure_brick_pack(lm_solver* s, const Geom& g, const int* d_bmap);
// Next (start, stop) event pair of the context's per-launch timing (lm_ctx_set_timing).
int timing_event_pair(lm_ctx* ctx, cudaEvent_t* e0, cudaEvent_t* e1);
cudaError_t launch_cheb_stream_c32(lm_ctx* ctx, const FusedInst& d, int K, int mode, const float4* spack);
cudaError_t launch_cheb_fused_c32(lm_ctx* ctx, const Geom& g, const float2* hop2, const float* diag2,
                                  const float2* x, float2* out, int64_t ld, int64_t m, int K, bool xreal,
                                  const ChebCoef* coef, double ph_re, double ph_im, const float4* spack = nullptr,
                                  int stream_mode = 0, uint32_t* comp = nullptr);
// Whether the x-streaming step can carry a compensation plane for this geometry and order
// (the uniform-column modes, whose shared memory leaves room for it).
bool stream_comp_supported(const Geom& g, int K, int mode);
// Every x-hop of H is real: Landau-gauge field components only (or none) and no twist across
// a periodic x axis.  The fused kernel then skips the imaginary parts of the x-hops.
bool ham_x_real(const lm_ham* h);
// ham_x_real and every hop of a lattice column equal (no twist across a periodic y axis): the
// Landau line integral of a y-bond, (x1+x2)(y2-y1)B/2, depends on x only.
bool ham_uniform_columns(const lm_ham* h);
// a, b, K, the Chebyshev coefficients and e^{-ib dt} of exp(-i H dt) on [emin, emax] (or on
// the solver's frozen interval), lmgpu_api.cu.
// K, the coefficients and the interval [b - a, b + a] for exp(-i H dt).  t_exact > 0: a is
// raised (by at most one FP32 ulp, relative 6e-8) until 2 t_exact / a is an FP32 number, so a
// hop of magnitude t_exact has no rounding error in the FP32 stencil tables.
void plan_propagator(lm_solver* s, double emin, double emax, double dt, double t_exact = 0.0);
// lm_solver_step / destroy for a solver updated with an lm_ell Hamiltonian (lmgpu_ell.cu).
int ell_solver_step(lm_solver* s, lm_state* st);
void ell_free_tables(lm_solver* s);
// A local (on-site) operator of up to 8 internal states, column-major, passed by value.
struct LocalOp {
    double2 o[64];
};
// Checks ndof / op against h and fills lop (op null: the identity); an lm_status.
int make_local_op(lm_ctx* ctx, const lm_ell* h, int ndof, const double* op, LocalOp* lop, const char* who);
// LocalOperatorCurrents per stored CSC entry of h into d_out (nnz doubles), lmgpu_ell.cu.
cudaError_t launch_ell_op_currents(lm_ctx* ctx, const lm_ell* h, const lm_state* st, int ndof, const LocalOp& lop,
                                   double* d_out);
// out = alpha (2H~) tp - tpp + w lam over an n x M ket block (tables 2H/a, 2(V-b)/a); tpp and
// lam may be null; out may alias tpp; with y non-null also y += cy out (lmgpu_adjoint.cu).
cudaError_t launch_stencil_recur(lm_ctx* ctx, const Geom& g, int precision, const void* hop2, const void* diag2,
                                 const void* tp, const void* tpp, const void* lam, void* out, int64_t ld, int64_t M,
                                 double alpha, double wre, double wim, void* y = nullptr, double cy = 0.0,
                                 bool xreal = false);
cudaError_t launch_convert(lm_ctx* ctx, int to_precision, const void* src, void* dst, int64_t n,
                           int64_t m, int64_t ld_src, int64_t ld_dst);

// Host math (lmgpu_api.cu)
int64_t bond_count(const Geom& g);
void bessel_j_all(double x, int kmax, std::vector<double>& out);
void make_coefs(const std::vector<double>& J, int K, double sgn, std::vector<ChebCoef>& out);
int ensure_accumulator(lm_state* s);
int ensure_scratch(lm_state* s);

}  // namespace lmgpu
