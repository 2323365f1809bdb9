// C ABI of the lmgpu evolution backend: handle management, host-side bookkeeping
// (bond counts, Chebyshev coefficients) and the update/step orchestration of the
// EvolutionSolver plugin (src/evolution.jl:5-33, :83-92, :69-78).
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <complex>
#include <new>
#include <string>
#include <vector>

#include "lmgpu_internal.cuh"

using namespace lmgpu;

namespace lmgpu {

int set_err(lm_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int check_cuda(lm_ctx* ctx, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return LM_OK;
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return set_err(ctx, LM_ERR_OOM, m);
    return set_err(ctx, LM_ERR_CUDA, m);
}

int64_t bond_count(const Geom& g) {
    const int64_t nbx = g.per_x ? g.N : (g.Lx - 1) * g.Ly;
    const int64_t nby = g.per_y ? g.N : g.Lx * (g.Ly - 1);
    return nbx + nby;
}

// J_0..J_kmax(x), x >= 0, by Miller's backward recurrence normalised with
// J_0 + 2 sum_k J_2k = 1 (Abramowitz & Stegun 9.1.27, 9.1.46).
void bessel_j_all(double x, int kmax, std::vector<double>& out) {
    out.assign((size_t)kmax + 1, 0.0);
    if (x == 0.0) {
        out[0] = 1.0;
        return;
    }
    int start = std::max(kmax, (int)ceil(x)) + 30 + (int)(4.0 * cbrt(x + 1.0) * 3.0);
    if (start % 2) ++start;
    std::vector<double> j((size_t)start + 2, 0.0);
    double jp1 = 0.0, jk = 1e-280, norm = 0.0;
    j[(size_t)start] = jk;
    for (int k = start; k >= 1; --k) {
        const double jm1 = (2.0 * k / x) * jk - jp1;
        j[(size_t)k - 1] = jm1;
        jp1 = jk;
        jk = jm1;
        if (fabs(jk) > 1e250) {  // rescale to stay finite
            for (int i = k - 1; i <= start; ++i) j[(size_t)i] *= 1e-250;
            jp1 *= 1e-250;
            jk *= 1e-250;
        }
    }
    norm = j[0];
    for (int k = 2; k <= start; k += 2) norm += 2.0 * j[(size_t)k];
    for (int k = 0; k <= kmax; ++k) out[(size_t)k] = j[(size_t)k] / norm;
}

}  // namespace lmgpu


static int dalloc(lm_ctx* ctx, void** p, size_t bytes, const char* what) {
    *p = nullptr;
    if (bytes == 0) return LM_OK;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return set_err(ctx, e == cudaErrorMemoryAllocation ? LM_ERR_OOM : LM_ERR_CUDA,
                       std::string("cudaMalloc(") + what + "): " + cudaGetErrorString(e));
    }
    return LM_OK;
}

namespace lmgpu {
// Allocates the accumulator buffer of a state on first use (the per-order path needs it).
int ensure_accumulator(lm_state* s) {
    if (s->d_y) return LM_OK;
    return dalloc(s->ctx, &s->d_y, s->elem * (size_t)s->ld * (size_t)s->m, "accumulator scratch");
}
// Allocates the recurrence scratch (T_{k-1}/T_k ping-pong) of a state on first use; a state
// stepped only through a panelled batch never needs it.
int ensure_scratch(lm_state* s) {
    if (s->d_a) return LM_OK;
    return dalloc(s->ctx, &s->d_a, s->elem * (size_t)s->ld * (size_t)s->m, "recurrence scratch");
}
}  // namespace lmgpu

static int ensure_red(lm_ctx* ctx, size_t n) {
    if (ctx->red_cap >= n) return LM_OK;
    if (ctx->d_red) cudaFree(ctx->d_red);
    ctx->d_red = nullptr;
    ctx->red_cap = 0;
    int rc = dalloc(ctx, (void**)&ctx->d_red, n * sizeof(double), "reduction scratch");
    if (rc == LM_OK) ctx->red_cap = n;
    return rc;
}

// Bonds of NearestNeighbor(1) in the reference's iteration order (0-based source,
// destination): every +x bond in source order, then every +y bond
// (src/core/bonds.jl:415-422, src/core/boundaries.jl:251-289).
static void for_each_bond(const Geom& g, std::vector<std::pair<int64_t, int64_t>>& out) {
    out.clear();
    for (int dir = 0; dir < 2; ++dir) {
        for (int64_t s = 0; s < g.N; ++s) {
            const int64_t xi = s / g.Ly, yi = s - xi * g.Ly;
            int64_t j;
            if (dir == 0) {
                if (xi + 1 < g.Lx) j = s + g.Ly;
                else if (g.per_x) j = yi;
                else continue;
            } else {
                if (yi + 1 < g.Ly) j = s + 1;
                else if (g.per_y) j = s - yi;
                else continue;
            }
            out.push_back({s, j});
        }
    }
}

namespace lmgpu {
// c_k = (2 - delta_k0) (-i)^k J_k(a|dt|) for k = 0..K stored as (s, parity): c_k = s (k even) or
// -i s (k odd).  sgn = -1 (dt < 0) gives exp(+i H |dt|), the conjugate coefficients.
void make_coefs(const std::vector<double>& J, int K, double sgn, std::vector<ChebCoef>& out) {
    out.assign((size_t)K + 1, ChebCoef{0.0, 0});
    for (int k = 0; k <= K; ++k) {
        const double mag = (k == 0 ? 1.0 : 2.0) * J[(size_t)k];
        const int r = k & 3;
        ChebCoef c;
        c.odd = k & 1;
        if (r == 0) c.s = mag;
        else if (r == 1) c.s = mag * sgn;       // -i mag (conjugate: +i mag = -i (-mag))
        else if (r == 2) c.s = -mag;
        else c.s = -mag * sgn;                  // +i mag = -i (-mag)
        out[(size_t)k] = c;
    }
}
bool ham_x_real(const lm_ham* h) {
    if (h->lat->g.per_x && h->lat->g.twist_x != 0.0) return false;
    for (int c = 0; c < h->fields.n; ++c)
        if (h->fields.c[c].kind != LM_FIELD_LANDAU) return false;  // (x1+x2)(y2-y1)B/2 = 0 on x-bonds
    return true;
}

bool ham_uniform_columns(const lm_ham* h) {
    return ham_x_real(h) && !(h->lat->g.per_y && h->lat->g.twist_y != 0.0);
}

ChebLo cheb_lo(double ph_re, double ph_im, double c0, double s1, bool fused) {
    typedef std::complex<double> cd;
    const cd ph(ph_re, ph_im);
    const cd phh((double)(float)ph_re, (double)(float)ph_im);
    const cd c1(0.0, -s1), c1h(0.0, -(double)(float)s1);
    const cd a0 = ph * c0;
    // the T0 coefficient the kernel applies from its FP32 words alone
    const cd t0 = fused ? cd((double)(float)(ph_re * c0), (double)(float)(ph_im * c0)) : phh * (double)(float)c0;
    const cd g0 = (a0 - t0) / phh;
    const cd g1 = (ph * c1 - phh * c1h) / phh;
    ChebLo lo;
    lo.g0_re = (float)g0.real();
    lo.g0_im = (float)g0.imag();
    lo.g1_re = (float)g1.real();
    lo.g1_im = (float)g1.imag();
    return lo;
}
}  // namespace lmgpu

// Smallest K >= 2 whose neglected tail 2 sum_{k>K} |J_k(x)| is below tol; J holds J_0..J_kmax.
static int cheb_order_for(double x, double tol, std::vector<double>& J) {
    const int kmax = (int)ceil(1.5 * x) + 60;
    bessel_j_all(x, kmax, J);
    std::vector<double> tail((size_t)kmax + 2, 0.0);
    for (int k = kmax; k >= 0; --k) tail[(size_t)k] = tail[(size_t)k + 1] + 2.0 * fabs(J[(size_t)k]);
    int K = 2;
    while (K < kmax && tail[(size_t)K + 1] > tol) ++K;
    return K;
}

extern "C" {

int lm_version(void) { return 100; }

// ------------------------------------------------------------------------------------------
// context
// ------------------------------------------------------------------------------------------
int lm_ctx_create(int device, lm_ctx** out) {
    if (!out) return LM_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return LM_ERR_CUDA;
    }
    if (device < 0 || device >= ndev) return LM_ERR_ARG;
    lm_ctx* c = new (std::nothrow) lm_ctx();
    if (!c) return LM_ERR_OOM;
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return LM_ERR_CUDA;
    }
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (const char* v = getenv("LMGPU_READOUT_SLICES")) c->ld_slices_override = std::max(0, std::min(64, atoi(v)));
    if (const char* v = getenv("LMGPU_CURRENTS_SCALAR")) c->currents_scalar = atoi(v) != 0;
    *out = c;
    return LM_OK;
}

int lm_ctx_destroy(lm_ctx* ctx) {
    if (!ctx) return LM_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->d_red) cudaFree(ctx->d_red);
    if (ctx->d_ld_part) cudaFree(ctx->d_ld_part);
    for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return LM_OK;
}

const char* lm_last_error(const lm_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int lm_ctx_synchronize(lm_ctx* ctx) {
    if (!ctx) return LM_ERR_ARG;
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    return LM_OK;
}

int lm_ctx_stream(lm_ctx* ctx, void** stream) {
    if (!ctx) return LM_ERR_ARG;
    CHECK_ARG(ctx, stream != nullptr, "lm_ctx_stream: null output");
    *stream = (void*)ctx->stream;
    return LM_OK;
}

// Folds every recorded (start, stop) pair into the accumulated timing.
static int resolve_timing(lm_ctx* ctx) {
    if (ctx->ev_used == 0) return LM_OK;
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    for (size_t i = 0; i < ctx->ev_used; ++i) {
        float ms = 0.f;
        CUDA_TRY(ctx, cudaEventElapsedTime(&ms, ctx->ev_pool[2 * i], ctx->ev_pool[2 * i + 1]), "cudaEventElapsedTime");
        ctx->order_ms += ms;
        ctx->order_launches += ctx->ev_launches[i];
    }
    ctx->ev_used = 0;
    return LM_OK;
}

// Returns the next free (start, stop) event pair, creating or resolving as needed.
static int timing_pair(lm_ctx* ctx, cudaEvent_t* e0, cudaEvent_t* e1) {
    const size_t kMaxPairs = 4096;
    if (ctx->ev_used == kMaxPairs) {
        int rc = resolve_timing(ctx);
        if (rc != LM_OK) return rc;
    }
    if (2 * ctx->ev_used + 1 >= ctx->ev_pool.size()) {
        cudaEvent_t a, b;
        CUDA_TRY(ctx, cudaEventCreate(&a), "cudaEventCreate");
        CUDA_TRY(ctx, cudaEventCreate(&b), "cudaEventCreate");
        ctx->ev_pool.push_back(a);
        ctx->ev_pool.push_back(b);
        ctx->ev_launches.push_back(0);
    }
    *e0 = ctx->ev_pool[2 * ctx->ev_used];
    *e1 = ctx->ev_pool[2 * ctx->ev_used + 1];
    return LM_OK;
}

int lm_ctx_set_option(lm_ctx* ctx, int option, int value) {
    if (!ctx) return LM_ERR_ARG;
    switch (option) {
        case LM_OPT_FUSED:
            ctx->fused = value ? 1 : 0;
            return LM_OK;
        case LM_OPT_STREAM:
            ctx->fused_form = value ? 1 : 0;
            return LM_OK;
        case LM_OPT_KPM:
            ctx->kpm_df = value ? 1 : 0;
            return LM_OK;
        case LM_OPT_RESIDENT:
            ctx->resident = value ? 1 : 0;
            return LM_OK;
        default:
            return set_err(ctx, LM_ERR_ARG, "lm_ctx_set_option: unknown option");
    }
}

int lm_ctx_stream_launches(lm_ctx* ctx, int64_t* n) {
    if (!ctx || !n) return LM_ERR_ARG;
    *n = ctx->stream_launches;
    return LM_OK;
}

int lm_ctx_set_timing(lm_ctx* ctx, int enable) {
    if (!ctx) return LM_ERR_ARG;
    ctx->timing = enable ? 1 : 0;
    return LM_OK;
}

int lm_ctx_timing(lm_ctx* ctx, double* order_ms, int64_t* order_launches, int64_t* launches) {
    if (!ctx) return LM_ERR_ARG;
    int rc = resolve_timing(ctx);
    if (rc != LM_OK) return rc;
    if (order_ms) *order_ms = ctx->order_ms;
    if (order_launches) *order_launches = ctx->order_launches;
    if (launches) *launches = ctx->launches;
    return LM_OK;
}

int lm_ctx_reset_timing(lm_ctx* ctx) {
    if (!ctx) return LM_ERR_ARG;
    int rc = resolve_timing(ctx);
    if (rc != LM_OK) return rc;
    ctx->order_ms = 0.0;
    ctx->order_launches = 0;
    ctx->launches = 0;
    return LM_OK;
}

// ------------------------------------------------------------------------------------------
// lattice
// ------------------------------------------------------------------------------------------
int lm_lattice_square(lm_ctx* ctx, int64_t Lx, int64_t Ly, int periodic_x, int periodic_y, double twist_x,
                      double twist_y, lm_lattice** out) {
    CHECK_ARG(ctx, out != nullptr, "lm_lattice_square: null output");
    *out = nullptr;
    CHECK_ARG(ctx, Lx >= 1 && Ly >= 1, "lm_lattice_square: sizes must be >= 1");
    CHECK_ARG(ctx, Lx <= (1ll << 31) && Ly <= (1ll << 31) && Lx * Ly <= (1ll << 40), "lm_lattice_square: lattice too large");
    if ((periodic_x && Lx < 2) || (periodic_y && Ly < 2))
        return set_err(ctx, LM_ERR_NOTSUP, "lm_lattice_square: a periodic axis of length 1 makes a site its own neighbour; not supported");
    CHECK_ARG(ctx, isfinite(twist_x) && isfinite(twist_y), "lm_lattice_square: non-finite twist");
    lm_lattice* l = new (std::nothrow) lm_lattice();
    if (!l) return set_err(ctx, LM_ERR_OOM, "host allocation");
    l->ctx = ctx;
    l->g.Lx = Lx;
    l->g.Ly = Ly;
    l->g.N = Lx * Ly;
    l->g.per_x = periodic_x ? 1 : 0;
    l->g.per_y = periodic_y ? 1 : 0;
    l->g.twist_x = periodic_x ? twist_x : 0.0;
    l->g.twist_y = periodic_y ? twist_y : 0.0;
    l->nbonds = bond_count(l->g);
    *out = l;
    return LM_OK;
}

int lm_lattice_destroy(lm_lattice* lat) {
    delete lat;
    return LM_OK;
}

int64_t lm_lattice_nsites(const lm_lattice* lat) { return lat ? lat->g.N : -1; }
int64_t lm_lattice_nbonds(const lm_lattice* lat) { return lat ? lat->nbonds : -1; }

int lm_lattice_bonds(const lm_lattice* lat, int64_t* src, int64_t* dst) {
    if (!lat) return LM_ERR_ARG;
    CHECK_ARG(lat->ctx, src && dst, "lm_lattice_bonds: null output");
    std::vector<std::pair<int64_t, int64_t>> bonds;
    for_each_bond(lat->g, bonds);
    for (size_t b = 0; b < bonds.size(); ++b) {
        src[b] = bonds[b].first + 1;
        dst[b] = bonds[b].second + 1;
    }
    return LM_OK;
}

int lm_lattice_coords(const lm_lattice* lat, double* xy) {
    if (!lat) return LM_ERR_ARG;
    CHECK_ARG(lat->ctx, xy != nullptr, "lm_lattice_coords: null output");
    for (int64_t s = 0; s < lat->g.N; ++s) {
        const int64_t xi = s / lat->g.Ly, yi = s - xi * lat->g.Ly;
        xy[2 * s] = (double)(xi + 1);
        xy[2 * s + 1] = (double)(yi + 1);
    }
    return LM_OK;
}

// ------------------------------------------------------------------------------------------
// Hamiltonian
// ------------------------------------------------------------------------------------------
int lm_ham_create(lm_ctx* ctx, lm_lattice* lat, double t1, lm_ham** out) {
    if (!ctx) return LM_ERR_ARG;
    CHECK_ARG(ctx, lat && out, "lm_ham_create: null argument");
    CHECK_ARG(ctx, lat->ctx == ctx, "lm_ham_create: lattice belongs to another context");
    CHECK_ARG(ctx, isfinite(t1), "lm_ham_create: non-finite t1");
    *out = nullptr;
    lm_ham* h = new (std::nothrow) lm_ham();
    if (!h) return set_err(ctx, LM_ERR_OOM, "host allocation");
    h->ctx = ctx;
    h->lat = lat;
    h->t1 = t1;
    h->fields.n = 0;
    cudaSetDevice(ctx->device);
    int rc = dalloc(ctx, (void**)&h->d_hop, sizeof(double2) * 2 * (size_t)lat->g.N, "hopping table");
    if (rc != LM_OK) {
        delete h;
        return rc;
    }
    *out = h;
    return LM_OK;
}

int lm_ham_destroy(lm_ham* h) {
    if (!h) return LM_OK;
    cudaSetDevice(h->ctx->device);
    cudaStreamSynchronize(h->ctx->stream);
    if (h->d_hop) cudaFree(h->d_hop);
    if (h->d_onsite) cudaFree(h->d_onsite);
    for (int j = 0; j < 2; ++j) {
        if (h->h_stage[j]) cudaFreeHost(h->h_stage[j]);
        if (h->stage_ev[j]) cudaEventDestroy(h->stage_ev[j]);
    }
    delete h;
    return LM_OK;
}

int lm_ham_add_field(lm_ham* h, int kind, double px, double py, int auto_pbc, int* component) {
    if (!h) return LM_ERR_ARG;
    lm_ctx* ctx = h->ctx;
    CHECK_ARG(ctx, kind >= LM_FIELD_LANDAU && kind <= LM_FIELD_POINTFLUX_SINGULAR, "lm_ham_add_field: unknown field kind");
    CHECK_ARG(ctx, isfinite(px) && isfinite(py), "lm_ham_add_field: non-finite point");
    if (h->fields.n >= kMaxFields) return set_err(ctx, LM_ERR_NOTSUP, "lm_ham_add_field: too many field components");
    FieldComp fc{};
    fc.kind = kind;
    fc.px = px;
    fc.py = py;
    const bool point = kind == LM_FIELD_POINTFLUX_AXIAL || kind == LM_FIELD_POINTFLUX_SINGULAR;
    fc.replicate = (point && auto_pbc && (h->lat->g.per_x || h->lat->g.per_y)) ? 1 : 0;
    const int idx = h->fields.n;
    h->fields.c[idx] = fc;
    h->fields.amp[idx] = 0.0;
    h->fields.n++;
    h->assembled = 0;
    if (component) *component = idx;
    return LM_OK;
}

int lm_ham_set_onsite(lm_ham* h, const double* V) {
    if (!h) return LM_ERR_ARG;
    lm_ctx* ctx = h->ctx;
    cudaSetDevice(ctx->device);
    const int64_t N = h->lat->g.N;
    if (!V) {
        if (h->d_onsite) {
            cudaStreamSynchronize(ctx->stream);
            cudaFree(h->d_onsite);
        }
        h->d_onsite = nullptr;
        h->vmin = h->vmax = 0.0;
        h->assembled = 0;
        return LM_OK;
    }
    if (!h->d_onsite) {
        int rc = dalloc(ctx, (void**)&h->d_onsite, sizeof(double) * (size_t)N, "on-site table");
        if (rc != LM_OK) return rc;
    }
    // two pinned staging slots; a slot is rewritten only after its previous copy has run
    const int j = h->stage_next;
    if (!h->h_stage[j]) {
        CUDA_TRY(ctx, cudaHostAlloc((void**)&h->h_stage[j], sizeof(double) * (size_t)N, cudaHostAllocDefault),
                 "pinned on-site staging");
        CUDA_TRY(ctx, cudaEventCreateWithFlags(&h->stage_ev[j], cudaEventDisableTiming), "cudaEventCreate");
    } else {
        CUDA_TRY(ctx, cudaEventSynchronize(h->stage_ev[j]), "on-site staging wait");
    }
    double* st = h->h_stage[j];
    double vmin = V[0], vmax = V[0];
    for (int64_t i = 0; i < N; ++i) {
        const double v = V[i];
        if (!isfinite(v)) return set_err(ctx, LM_ERR_NONFINITE, "lm_ham_set_onsite: non-finite on-site value");
        vmin = std::min(vmin, v);
        vmax = std::max(vmax, v);
        st[i] = v;
    }
    CUDA_TRY(ctx, cudaMemcpyAsync(h->d_onsite, st, sizeof(double) * (size_t)N, cudaMemcpyHostToDevice, ctx->stream),
             "upload on-site");
    CUDA_TRY(ctx, cudaEventRecord(h->stage_ev[j], ctx->stream), "cudaEventRecord");
    h->stage_next = j ^ 1;
    h->vmin = vmin;
    h->vmax = vmax;
    h->assembled = 0;
    return LM_OK;
}

int lm_ham_assemble(lm_ham* h, const double* amplitudes, int ncomponents) {
    if (!h) return LM_ERR_ARG;
    lm_ctx* ctx = h->ctx;
    CHECK_ARG(ctx, ncomponents == h->fields.n, "lm_ham_assemble: amplitude count does not match the field components");
    CHECK_ARG(ctx, ncomponents == 0 || amplitudes, "lm_ham_assemble: null amplitudes");
    for (int c = 0; c < ncomponents; ++c)
        if (!isfinite(amplitudes[c])) return set_err(ctx, LM_ERR_NONFINITE, "lm_ham_assemble: non-finite amplitude");
    // value-equal H: keep the cached assembly (the `mat == old` test of src/evolution.jl:87)
    if (h->assembled && (int)h->last_amp.size() == ncomponents &&
        std::equal(h->last_amp.begin(), h->last_amp.end(), amplitudes))
        return LM_OK;
    for (int c = 0; c < ncomponents; ++c) h->fields.amp[c] = amplitudes[c];
    cudaSetDevice(ctx->device);
    CUDA_TRY(ctx, launch_assemble(ctx, h->lat->g, h->fields, h->t1, h->d_hop), "assemble kernel");
    h->last_amp.assign(amplitudes, amplitudes + ncomponents);
    h->assembled = 1;
    h->version++;
    return LM_OK;
}

int lm_ham_nnz(lm_ham* h, int64_t* nnz) {
    if (!h) return LM_ERR_ARG;
    CHECK_ARG(h->ctx, nnz, "lm_ham_nnz: null output");
    const Geom& g = h->lat->g;
    std::vector<std::vector<int64_t>> cols((size_t)g.N);
    if (h->d_onsite)
        for (int64_t s = 0; s < g.N; ++s) cols[(size_t)s].push_back(s);
    if (h->t1 != 0.0) {
        std::vector<std::pair<int64_t, int64_t>> bonds;
        for_each_bond(g, bonds);
        for (auto& b : bonds) {
            cols[(size_t)b.second].push_back(b.first);
            cols[(size_t)b.first].push_back(b.second);
        }
    }
    int64_t n = 0;
    for (auto& c : cols) {
        std::sort(c.begin(), c.end());
        n += std::unique(c.begin(), c.end()) - c.begin();
    }
    *nnz = n;
    return LM_OK;
}

int lm_ham_csc(lm_ham* h, int64_t* colptr, int64_t* rowval, double* nzval) {
    if (!h) return LM_ERR_ARG;
    lm_ctx* ctx = h->ctx;
    CHECK_ARG(ctx, colptr && rowval && nzval, "lm_ham_csc: null output");
    if (!h->assembled) return set_err(ctx, LM_ERR_STATE, "lm_ham_csc: Hamiltonian not assembled");
    const Geom& g = h->lat->g;
    cudaSetDevice(ctx->device);
    std::vector<double2> hop((size_t)(2 * g.N));
    std::vector<double> V;
    CUDA_TRY(ctx, cudaMemcpyAsync(hop.data(), h->d_hop, sizeof(double2) * 2 * (size_t)g.N, cudaMemcpyDeviceToHost, ctx->stream),
             "download hopping");
    if (h->d_onsite) {
        V.resize((size_t)g.N);
        CUDA_TRY(ctx, cudaMemcpyAsync(V.data(), h->d_onsite, sizeof(double) * (size_t)g.N, cudaMemcpyDeviceToHost, ctx->stream),
                 "download on-site");
    }
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    // entries in the builder's insertion order: on-site first, then H[i,j] and H[j,i] per bond
    std::vector<std::vector<std::pair<int64_t, std::pair<double, double>>>> cols((size_t)g.N);
    if (h->d_onsite)
        for (int64_t s = 0; s < g.N; ++s) cols[(size_t)s].push_back({s, {V[(size_t)s], 0.0}});
    if (h->t1 != 0.0) {
        std::vector<std::pair<int64_t, int64_t>> bonds;
        for_each_bond(g, bonds);
        int64_t b = 0;
        const int64_t nbx = g.per_x ? g.N : (g.Lx - 1) * g.Ly;
        for (auto& bd : bonds) {
            const int64_t s = bd.first, j = bd.second;
            const int dir = b < nbx ? 0 : 1;
            ++b;
            const double2 v = hop[(size_t)(dir * g.N + s)];
            cols[(size_t)j].push_back({s, {v.x, v.y}});    // H[s, j]
            cols[(size_t)s].push_back({j, {v.x, -v.y}});   // H[j, s] = conj
        }
    }
    int64_t p = 0;
    colptr[0] = 1;
    for (int64_t c = 0; c < g.N; ++c) {
        auto& col = cols[(size_t)c];
        std::stable_sort(col.begin(), col.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
        size_t i = 0;
        while (i < col.size()) {
            int64_t r = col[i].first;
            double re = col[i].second.first, im = col[i].second.second;
            size_t k = i + 1;
            while (k < col.size() && col[k].first == r) {
                re += col[k].second.first;
                im += col[k].second.second;
                ++k;
            }
            rowval[p] = r + 1;
            nzval[2 * p] = re;
            nzval[2 * p + 1] = im;
            ++p;
            i = k;
        }
        colptr[c + 1] = p + 1;
    }
    return LM_OK;
}

int lm_ham_bounds(lm_ham* h, double* emin, double* emax) {
    if (!h) return LM_ERR_ARG;
    CHECK_ARG(h->ctx, emin && emax, "lm_ham_bounds: null output");
    // Gershgorin: every row holds at most 4 hops of modulus |t1| around V_i.
    const double r = 4.0 * fabs(h->t1);
    *emin = h->vmin - r;
    *emax = h->vmax + r;
    return LM_OK;
}

// ------------------------------------------------------------------------------------------
// states
// ------------------------------------------------------------------------------------------
int lm_state_create(lm_ctx* ctx, int64_t n, int64_t m, int kind, int precision, lm_state** out) {
    if (!ctx) return LM_ERR_ARG;
    CHECK_ARG(ctx, out != nullptr, "lm_state_create: null output");
    *out = nullptr;
    CHECK_ARG(ctx, kind == LM_KETS || kind == LM_DENSITY, "lm_state_create: unknown state kind");
    CHECK_ARG(ctx, precision == LM_C64 || precision == LM_C32, "lm_state_create: unknown precision");
    CHECK_ARG(ctx, n >= 1 && m >= 1, "lm_state_create: empty state");
    if (kind == LM_DENSITY) CHECK_ARG(ctx, m == n, "lm_state_create: a density matrix is square");
    lm_state* s = new (std::nothrow) lm_state();
    if (!s) return set_err(ctx, LM_ERR_OOM, "host allocation");
    s->ctx = ctx;
    s->n = n;
    s->m = m;
    s->ld = n;
    s->kind = kind;
    s->precision = precision;
    s->elem = precision == LM_C64 ? 16 : 8;
    cudaSetDevice(ctx->device);
    const size_t bytes = s->elem * (size_t)n * (size_t)m;
    int rc = dalloc(ctx, &s->d_data, bytes, "state");
    // the recurrence scratch and the accumulator are allocated on first use
    if (rc != LM_OK) {
        delete s;
        return rc;
    }
    cudaMemsetAsync(s->d_data, 0, bytes, ctx->stream);
    *out = s;
    return LM_OK;
}

int lm_state_destroy(lm_state* s) {
    if (!s) return LM_OK;
    cudaSetDevice(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    if (s->d_data) cudaFree(s->d_data);
    if (s->d_a) cudaFree(s->d_a);
    if (s->d_y) cudaFree(s->d_y);
    if (s->d_w) cudaFree(s->d_w);
    if (s->d_lo) cudaFree(s->d_lo);
    delete s;
    return LM_OK;
}

int lm_state_set_compensation(lm_state* s, int enable) {
    if (!s) return LM_ERR_ARG;
    lm_ctx* ctx = s->ctx;
    cudaSetDevice(ctx->device);
    if (!enable) {
        if (s->d_lo) {
            cudaStreamSynchronize(ctx->stream);
            cudaFree(s->d_lo);
        }
        s->d_lo = nullptr;
        return LM_OK;
    }
    CHECK_ARG(ctx, s->kind == LM_KETS && s->precision == LM_C32,
              "lm_state_set_compensation: applies to ComplexF32 ket blocks");
    if (s->d_lo) return LM_OK;
    const size_t bytes = sizeof(uint32_t) * (size_t)s->ld * (size_t)s->m;
    int rc = dalloc(ctx, (void**)&s->d_lo, bytes, "compensation plane");
    if (rc != LM_OK) return rc;
    CUDA_TRY(ctx, cudaMemsetAsync(s->d_lo, 0, bytes, ctx->stream), "clear compensation plane");
    return LM_OK;
}

int lm_state_upload(lm_state* s, const void* host, int64_t ld) {
    if (!s) return LM_ERR_ARG;
    lm_ctx* ctx = s->ctx;
    CHECK_ARG(ctx, host != nullptr, "lm_state_upload: null host buffer");
    CHECK_ARG(ctx, ld >= s->n, "lm_state_upload: leading dimension smaller than n");
    cudaSetDevice(ctx->device);
    CUDA_TRY(ctx, cudaMemcpy2DAsync(s->d_data, s->elem * (size_t)s->ld, host, s->elem * (size_t)ld, s->elem * (size_t)s->n,
                                    (size_t)s->m, cudaMemcpyDefault, ctx->stream),
             "upload state");
    if (s->d_lo)  // uploaded FP32 values are exact: no residual
        CUDA_TRY(ctx, cudaMemsetAsync(s->d_lo, 0, sizeof(uint32_t) * (size_t)s->ld * (size_t)s->m, ctx->stream),
                 "clear compensation plane");
    return LM_OK;
}

int lm_state_download(lm_state* s, void* host, int64_t ld) {
    if (!s) return LM_ERR_ARG;
    lm_ctx* ctx = s->ctx;
    CHECK_ARG(ctx, host != nullptr, "lm_state_download: null host buffer");
    CHECK_ARG(ctx, ld >= s->n, "lm_state_download: leading dimension smaller than n");
    cudaSetDevice(ctx->device);
    CUDA_TRY(ctx, cudaMemcpy2DAsync(host, s->elem * (size_t)ld, s->d_data, s->elem * (size_t)s->ld, s->elem * (size_t)s->n,
                                    (size_t)s->m, cudaMemcpyDeviceToHost, ctx->stream),
             "download state");
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    return LM_OK;
}

int lm_state_copy(lm_state* dst, const lm_state* src) {
    if (!dst || !src) return LM_ERR_ARG;
    lm_ctx* ctx = dst->ctx;
    CHECK_ARG(ctx, src->ctx == ctx, "lm_state_copy: states from different contexts");
    CHECK_ARG(ctx, dst->n == src->n && dst->m == src->m && dst->kind == src->kind && dst->precision == src->precision,
              "lm_state_copy: states differ in shape, kind or precision");
    cudaSetDevice(ctx->device);
    CUDA_TRY(ctx, cudaMemcpy2DAsync(dst->d_data, dst->elem * (size_t)dst->ld, src->d_data, src->elem * (size_t)src->ld,
                                    dst->elem * (size_t)dst->n, (size_t)dst->m, cudaMemcpyDeviceToDevice, ctx->stream),
             "copy state");
    if (dst->d_lo && src->d_lo)
        CUDA_TRY(ctx, cudaMemcpy2DAsync(dst->d_lo, sizeof(uint32_t) * (size_t)dst->ld, src->d_lo,
                                        sizeof(uint32_t) * (size_t)src->ld, sizeof(uint32_t) * (size_t)dst->n,
                                        (size_t)dst->m, cudaMemcpyDeviceToDevice, ctx->stream),
                 "copy compensation plane");
    else if (dst->d_lo)
        CUDA_TRY(ctx, cudaMemsetAsync(dst->d_lo, 0, sizeof(uint32_t) * (size_t)dst->ld * (size_t)dst->m, ctx->stream),
                 "clear compensation plane");
    return LM_OK;
}

int lm_state_device_ptr(lm_state* s, void** ptr, int64_t* ld) {
    if (!s) return LM_ERR_ARG;
    CHECK_ARG(s->ctx, ptr != nullptr, "lm_state_device_ptr: null output");
    *ptr = s->d_data;
    if (ld) *ld = s->ld;
    return LM_OK;
}

int lm_state_set_weights(lm_state* s, const double* w) {
    if (!s) return LM_ERR_ARG;
    lm_ctx* ctx = s->ctx;
    cudaSetDevice(ctx->device);
    if (!w) {
        if (s->d_w) {
            cudaStreamSynchronize(ctx->stream);
            cudaFree(s->d_w);
        }
        s->d_w = nullptr;
        return LM_OK;
    }
    CHECK_ARG(ctx, s->kind == LM_KETS, "lm_state_set_weights: weights apply to ket blocks");
    for (int64_t k = 0; k < s->m; ++k)
        if (!isfinite(w[k])) return set_err(ctx, LM_ERR_NONFINITE, "lm_state_set_weights: non-finite weight");
    if (!s->d_w) {
        int rc = dalloc(ctx, (void**)&s->d_w, sizeof(double) * (size_t)s->m, "weights");
        if (rc != LM_OK) return rc;
    }
    CUDA_TRY(ctx, cudaMemcpyAsync(s->d_w, w, sizeof(double) * (size_t)s->m, cudaMemcpyHostToDevice, ctx->stream), "upload weights");
    return LM_OK;
}

int lm_state_norms(lm_state* s, double* out) {
    if (!s) return LM_ERR_ARG;
    lm_ctx* ctx = s->ctx;
    CHECK_ARG(ctx, out != nullptr, "lm_state_norms: null output");
    cudaSetDevice(ctx->device);
    int rc = ensure_red(ctx, (size_t)s->m);
    if (rc != LM_OK) return rc;
    if (s->d_lo)
        CUDA_TRY(ctx, launch_column_norms_comp(ctx, (const float2*)s->d_data, s->d_lo, s->n, s->m, s->ld, ctx->d_red),
                 "column norms");
    else
        CUDA_TRY(ctx, launch_column_norms(ctx, s->precision, s->d_data, s->n, s->m, s->ld, ctx->d_red), "column norms");
    CUDA_TRY(ctx, cudaMemcpyAsync(out, ctx->d_red, sizeof(double) * (size_t)s->m, cudaMemcpyDeviceToHost, ctx->stream), "download norms");
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    return LM_OK;
}

int lm_state_renormalize(lm_state* s, const double* target) {
    if (!s) return LM_ERR_ARG;
    lm_ctx* ctx = s->ctx;
    CHECK_ARG(ctx, target != nullptr, "lm_state_renormalize: null target norms");
    CHECK_ARG(ctx, s->kind == LM_KETS, "lm_state_renormalize: applies to ket blocks");
    cudaSetDevice(ctx->device);
    int rc = ensure_red(ctx, 2 * (size_t)s->m);
    if (rc != LM_OK) return rc;
    // a library-owned pageable copy: the driver stages it during the call, so the caller's
    // buffer (pinned or not) is free again on return and the stream is not drained
    ctx->h_norms.assign(target, target + s->m);
    CUDA_TRY(ctx, cudaMemcpyAsync(ctx->d_red + s->m, ctx->h_norms.data(), sizeof(double) * (size_t)s->m,
                                  cudaMemcpyHostToDevice, ctx->stream),
             "upload target norms");
    if (s->d_lo) {
        CUDA_TRY(ctx, launch_column_norms_comp(ctx, (const float2*)s->d_data, s->d_lo, s->n, s->m, s->ld, ctx->d_red),
                 "column norms");
        CUDA_TRY(ctx, launch_rescale_columns_comp(ctx, (float2*)s->d_data, s->d_lo, s->n, s->m, s->ld, ctx->d_red,
                                                  ctx->d_red + s->m),
                 "rescale columns");
        return LM_OK;
    }
    CUDA_TRY(ctx, launch_column_norms(ctx, s->precision, s->d_data, s->n, s->m, s->ld, ctx->d_red), "column norms");
    CUDA_TRY(ctx, launch_rescale_columns(ctx, s->precision, s->d_data, s->n, s->m, s->ld, ctx->d_red, ctx->d_red + s->m),
             "rescale columns");
    // no host synchronisation: the target norms were staged by the (pageable) copy above
    return LM_OK;
}

// ------------------------------------------------------------------------------------------
// solver (EvolutionSolver plugin)
// ------------------------------------------------------------------------------------------
int lm_solver_create(lm_ctx* ctx, double tol, lm_solver** out) {
    if (!ctx) return LM_ERR_ARG;
    CHECK_ARG(ctx, out != nullptr, "lm_solver_create: null output");
    CHECK_ARG(ctx, tol > 0.0 && tol < 1.0, "lm_solver_create: tol must lie in (0, 1)");
    *out = nullptr;
    lm_solver* s = new (std::nothrow) lm_solver();
    if (!s) return set_err(ctx, LM_ERR_OOM, "host allocation");
    s->ctx = ctx;
    s->tol = tol;
    *out = s;
    return LM_OK;
}

static void free_tables(lm_solver* s) {
    if (s->d_hop2) cudaFree(s->d_hop2);
    if (s->d_diag2) cudaFree(s->d_diag2);
    if (s->d_hop2f) cudaFree(s->d_hop2f);
    if (s->d_diag2f) cudaFree(s->d_diag2f);
    if (s->d_spack) cudaFree(s->d_spack);
    s->d_spack = nullptr;
    s->spack_f4 = 0;
    s->spack_version = ~0ull;
    s->d_hop2 = nullptr;
    s->d_diag2 = nullptr;
    s->d_hop2f = nullptr;
    s->d_diag2f = nullptr;
    s->tab_n = 0;
}

int lm_solver_destroy(lm_solver* s) {
    if (!s) return LM_OK;
    cudaSetDevice(s->ctx->device);
    cudaStreamSynchronize(s->ctx->stream);
    free_tables(s);
    ell_free_tables(s);
    delete s;
    return LM_OK;
}

int lm_solver_update(lm_solver* s, lm_ham* h, double dt, int force) {
    if (!s) return LM_ERR_ARG;
    lm_ctx* ctx = s->ctx;
    CHECK_ARG(ctx, h != nullptr, "lm_solver_update: null Hamiltonian");
    CHECK_ARG(ctx, h->ctx == ctx, "lm_solver_update: Hamiltonian belongs to another context");
    CHECK_ARG(ctx, isfinite(dt), "lm_solver_update: non-finite dt");
    if (!h->assembled) return set_err(ctx, LM_ERR_STATE, "lm_solver_update: Hamiltonian not assembled");
    // cache hit: same H (object and assembly) and same factor -i*dt (src/evolution.jl:86-88)
    if (!force && s->valid && s->ham == h && s->ham_version == h->version &&
        fabs(dt - s->dt) <= 1.4901161193847656e-08 * std::max(fabs(dt), fabs(s->dt)))
        return LM_OK;
    cudaSetDevice(ctx->device);
    const Geom& g = h->lat->g;
    if (s->tab_n != g.N) {
        free_tables(s);
        int rc = dalloc(ctx, (void**)&s->d_hop2, sizeof(double2) * 2 * (size_t)g.N, "hop table");
        if (rc == LM_OK) rc = dalloc(ctx, (void**)&s->d_diag2, sizeof(double) * (size_t)g.N, "diag table");
        if (rc == LM_OK) rc = dalloc(ctx, (void**)&s->d_hop2f, sizeof(float2) * 2 * (size_t)g.N, "hop table f32");
        if (rc == LM_OK) rc = dalloc(ctx, (void**)&s->d_diag2f, sizeof(float) * (size_t)g.N, "diag table f32");
        if (rc != LM_OK) {
            free_tables(s);
            s->valid = 0;
            return rc;
        }
        s->tab_n = g.N;
    }
    double emin, emax;
    lm_ham_bounds(h, &emin, &emax);
    // the nearest-neighbour hop magnitude |t1| is exact in the FP32 tables: a rounded uniform
    // hop is a coherent rescaling of the kinetic energy, whose error would grow linearly with
    // the number of steps (1.4e-6 on the bond currents after 400 steps of the 256^2 Landau
    // workload, 2.7e-7 without it)
    plan_propagator(s, emin, emax, dt, fabs(h->t1));
    CUDA_TRY(ctx, launch_normalise(ctx, g, h->d_hop, h->d_onsite, s->a, s->b, s->d_hop2, s->d_diag2, s->d_hop2f,
                                   s->d_diag2f),
             "normalise kernel");
    s->tab_version++;
    s->ell = nullptr;
    s->ham = h;
    s->ham_version = h->version;
    s->dt = dt;
    s->valid = 1;
    s->has_onsite = h->d_onsite != nullptr;
    return LM_OK;
}

}  // extern "C"

namespace lmgpu {
void plan_propagator(lm_solver* s, double emin, double emax, double dt, double t_exact) {
    if (s->fixed_bounds) {
        emin = s->fix_emin;
        emax = s->fix_emax;
    }
    const double hw = 0.5 * (emax - emin);
    double a = std::max(hw * (1.0 + 1e-12) + 1e-300, 1e-12);
    if (t_exact > 0.0 && isfinite(2.0 * t_exact / a)) {
        // the largest FP32 number q <= 2 t / a, then the smallest a' >= a with t * (2 / a')
        // rounding to q in FP32 (the normalise kernel forms hop * (2 / a) in FP64, then
        // rounds); a' - a is below 1e-7 relative, so K does not change
        float q = (float)(2.0 * t_exact / a);
        if ((double)q > 2.0 * t_exact / a) q = nextafterf(q, 0.0f);
        if (q > 0.0f) {
            double a2 = 2.0 * t_exact / (double)q;
            for (int it = 0; it < 4 && (float)(t_exact * (2.0 / a2)) != q; ++it) a2 = nextafter(a2, 2.0 * a2);
            if ((float)(t_exact * (2.0 / a2)) == q && a2 >= a) a = a2;
        }
    }
    const double b = 0.5 * (emax + emin);
    std::vector<double> J;
    const int K = cheb_order_for(a * fabs(dt), s->tol, J);
    make_coefs(J, K, dt >= 0 ? 1.0 : -1.0, s->coef);
    s->phase_re = cos(b * dt);
    s->phase_im = -sin(b * dt);
    s->a = a;
    s->b = b;
    s->K = K;
}
}  // namespace lmgpu

extern "C" {

int lm_solver_order(const lm_solver* s, int* K, double* a, double* b) {
    if (!s) return LM_ERR_ARG;
    if (K) *K = s->valid ? s->K : 0;
    if (a) *a = s->a;
    if (b) *b = s->b;
    return LM_OK;
}

// One application of the Chebyshev series to the kets laid out by (site_fast, ld, m) in
// buffers S (input T0), A, Y.  The result lands in S when K is even and in A when K is
// odd; the return value says which (0 = S, 1 = A).
static int cheb_apply(lm_solver* s, const Geom& g, int precision, int site_fast, int conj, void* S, void* A,
                      void* Y, int64_t ld, int64_t m, int* where, uint32_t* comp = nullptr) {
    lm_ctx* ctx = s->ctx;
    const void* hop2 = precision == LM_C64 ? (const void*)s->d_hop2 : (const void*)s->d_hop2f;
    const void* diag2 = precision == LM_C64 ? (const void*)s->d_diag2 : (const void*)s->d_diag2f;
    const int K = s->K;
    const double c0 = s->coef[0].s;
    const double pr = s->phase_re, pi = conj ? -s->phase_im : s->phase_im;
    auto coef = [&](int k) {
        ChebCoef c = s->coef[(size_t)k];
        if (conj && c.odd) c.s = -c.s;  // conj(-i s) = -i (-s)
        return c;
    };
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (ctx->timing) {
        int rc = timing_pair(ctx, &t0, &t1);
        if (rc != LM_OK) return rc;
        CUDA_TRY(ctx, cudaEventRecord(t0, ctx->stream), "cudaEventRecord");
    }
    if (ctx->fused && site_fast && !conj && fused_supported(precision, K) && fused_supported_geom(g)) {
        // whole series in one temporally blocked pass; result lands in A
        const bool xr = ham_x_real(s->ham);
        const int mode = ham_uniform_columns(s->ham) ? 2 : (xr ? 1 : 0);
        const float4* spack = nullptr;
        if (ctx->fused_form == 1 && stream_supported(g, K, mode, S, A, ld)) {
            const int rc = ensure_stream_pack(s, g);
            if (rc != LM_OK) return rc;
            spack = s->d_spack;
        }
        if (comp && !(spack && stream_comp_supported(g, K, mode)))
            return set_err(ctx, LM_ERR_NOTSUP,
                           "lm_solver_step: a compensated state needs the x-streaming form (Ly even, Lx >= 2K + 3, "
                           "K <= 6; K <= 5 with complex x-hops)");
        CUDA_TRY(ctx, launch_cheb_fused_c32(ctx, g, (const float2*)hop2, (const float*)diag2, (const float2*)S,
                                            (float2*)A, ld, m, K, xr, s->coef.data(), pr, pi, spack, mode, comp),
                 "fused chebyshev step");
        if (ctx->timing) {
            CUDA_TRY(ctx, cudaEventRecord(t1, ctx->stream), "cudaEventRecord");
            ctx->ev_launches[ctx->ev_used] = K;
            ctx->ev_used++;
        }
        *where = 1;
        return LM_OK;
    }
    if (comp)
        return set_err(ctx, LM_ERR_NOTSUP,
                       "lm_solver_step: a compensated state needs the x-streaming form (fused step enabled)");
    const ChebLo lo = cheb_lo(pr, pi, c0, coef(1).s, false);
    const bool xr = ham_x_real(s->ham);
    CUDA_TRY(ctx, launch_cheb_order(ctx, g, precision, site_fast, conj, CHEB_FIRST, hop2, diag2, S, A, Y, ld, m, c0, coef(1), pr, pi, lo, xr),
             "chebyshev order 1");
    for (int k = 2; k <= K; ++k) {
        const void* tp = (k % 2 == 0) ? A : S;
        void* tq = (k % 2 == 0) ? S : A;
        const int mode = (k == K) ? CHEB_LAST : CHEB_MID;
        CUDA_TRY(ctx, launch_cheb_order(ctx, g, precision, site_fast, conj, mode, hop2, diag2, tp, tq, Y, ld, m, c0, coef(k), pr, pi, lo, xr),
                 "chebyshev order");
    }
    if (ctx->timing) {
        CUDA_TRY(ctx, cudaEventRecord(t1, ctx->stream), "cudaEventRecord");
        ctx->ev_launches[ctx->ev_used] = K;
        ctx->ev_used++;
    }
    *where = (K % 2 == 0) ? 0 : 1;
    return LM_OK;
}

int lm_solver_step(lm_solver* s, lm_state* st) {
    if (!s) return LM_ERR_ARG;
    lm_ctx* ctx = s->ctx;
    CHECK_ARG(ctx, st != nullptr, "lm_solver_step: null state");
    CHECK_ARG(ctx, st->ctx == ctx, "lm_solver_step: state belongs to another context");
    if (!s->valid) return set_err(ctx, LM_ERR_STATE, "lm_solver_step: update_solver must run before step");
    if (s->ell) return ell_solver_step(s, st);
    const Geom& g = s->ham->lat->g;
    CHECK_ARG(ctx, st->n == g.N, "lm_solver_step: state size does not match the lattice");
    cudaSetDevice(ctx->device);
    {
        int rc0 = ensure_scratch(st);
        if (rc0 != LM_OK) return rc0;
    }
    if (!(ctx->fused && st->kind == LM_KETS && fused_supported(st->precision, s->K) && fused_supported_geom(g))) {
        int rc0 = ensure_accumulator(st);
        if (rc0 != LM_OK) return rc0;
    }
    int where = 0;
    // psi <- U psi on the columns (kets, or the columns of P)
    int rc = cheb_apply(s, g, st->precision, 1, 0, st->d_data, st->d_a, st->d_y, st->ld, st->m, &where, st->d_lo);
    if (rc != LM_OK) return rc;
    if (where == 1) std::swap(st->d_data, st->d_a);
    if (st->kind == LM_DENSITY) {
        // P <- X U^dagger: row r of the result is conj(U) applied to row r of X
        rc = cheb_apply(s, g, st->precision, 0, 1, st->d_data, st->d_a, st->d_y, st->ld, st->m, &where);
        if (rc != LM_OK) return rc;
        if (where == 1) std::swap(st->d_data, st->d_a);
    }
    return LM_OK;
}

int lm_chebyshev_plan(double x, double tol, int cap, int* K, double* coef) {
    if (!K || !(x >= 0.0) || !isfinite(x) || !(tol > 0.0 && tol < 1.0)) return LM_ERR_ARG;
    std::vector<double> J;
    const int k = cheb_order_for(x, tol, J);
    *K = k;
    if (!coef) return LM_OK;
    if (cap < k + 1) return LM_ERR_ARG;
    for (int i = 0; i <= k; ++i) {
        const double mag = (i == 0 ? 1.0 : 2.0) * J[(size_t)i];
        const int r = i & 3;  // (-i)^i = 1, -i, -1, i
        coef[2 * i] = (r == 0) ? mag : (r == 2 ? -mag : 0.0);
        coef[2 * i + 1] = (r == 1) ? -mag : (r == 3 ? mag : 0.0);
    }
    return LM_OK;
}

// ------------------------------------------------------------------------------------------
// readouts
// ------------------------------------------------------------------------------------------
int lm_localdensity(lm_state* s, double* out) {
    if (!s) return LM_ERR_ARG;
    lm_ctx* ctx = s->ctx;
    CHECK_ARG(ctx, out != nullptr, "lm_localdensity: null output");
    cudaSetDevice(ctx->device);
    int rc = ensure_red(ctx, (size_t)s->n + 1);
    if (rc != LM_OK) return rc;
    CUDA_TRY(ctx, launch_localdensity(ctx, s->precision, s->kind, s->d_data, s->n, s->m, s->ld, s->d_w, ctx->d_red),
             "localdensity kernel");
    CUDA_TRY(ctx, cudaMemcpyAsync(out, ctx->d_red, sizeof(double) * (size_t)s->n, cudaMemcpyDeviceToHost, ctx->stream),
             "download density");
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    return LM_OK;
}

int lm_bond_currents(lm_ham* h, lm_state* s, double* out) {
    if (!h || !s) return LM_ERR_ARG;
    lm_ctx* ctx = s->ctx;
    CHECK_ARG(ctx, out != nullptr, "lm_bond_currents: null output");
    CHECK_ARG(ctx, h->ctx == ctx, "lm_bond_currents: objects from different contexts");
    CHECK_ARG(ctx, s->n == h->lat->g.N, "lm_bond_currents: state size does not match the lattice");
    if (!h->assembled) return set_err(ctx, LM_ERR_STATE, "lm_bond_currents: Hamiltonian not assembled");
    const int64_t nb = h->lat->nbonds;
    cudaSetDevice(ctx->device);
    int rc = ensure_red(ctx, (size_t)std::max<int64_t>(nb, 1));
    if (rc != LM_OK) return rc;
    if (nb == 0) return LM_OK;
    CUDA_TRY(ctx, launch_bond_currents(ctx, h->lat->g, s->precision, s->kind, h->d_hop, s->d_data, s->m, s->ld, s->d_w, ctx->d_red),
             "bond currents kernel");
    CUDA_TRY(ctx, cudaMemcpyAsync(out, ctx->d_red, sizeof(double) * (size_t)nb, cudaMemcpyDeviceToHost, ctx->stream),
             "download currents");
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    return LM_OK;
}

int lm_trace(lm_state* s, double* out) {
    if (!s) return LM_ERR_ARG;
    lm_ctx* ctx = s->ctx;
    CHECK_ARG(ctx, out != nullptr, "lm_trace: null output");
    cudaSetDevice(ctx->device);
    int rc = ensure_red(ctx, (size_t)s->n + 1);
    if (rc != LM_OK) return rc;
    CUDA_TRY(ctx, launch_localdensity(ctx, s->precision, s->kind, s->d_data, s->n, s->m, s->ld, s->d_w, ctx->d_red),
             "localdensity kernel");
    CUDA_TRY(ctx, launch_sum(ctx, ctx->d_red, s->n, ctx->d_red + s->n), "sum kernel");
    CUDA_TRY(ctx, cudaMemcpyAsync(out, ctx->d_red + s->n, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "download trace");
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream), "sync");
    return LM_OK;
}

}  // extern "C"

namespace lmgpu {
// The timing event pair of one step launch, for the step paths outside this file.
int timing_event_pair(lm_ctx* ctx, cudaEvent_t* e0, cudaEvent_t* e1) { return timing_pair(ctx, e0, e1); }
}  // namespace lmgpu
