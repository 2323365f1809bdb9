// Readout ring: per-moment observables (local densities, bond currents) computed on the
// device into the slots of a ring and copied asynchronously into pinned host memory, so that
// an evolution loop that records a readout every step never waits for the step to finish.
// This is the device side of TimeSequence(f, ev(times)) (src/timesequence.jl:41-43) for
// f = localdensity of the moment's state (src/operators/latticeutils.jl:41-45) and
// f = DensityCurrents(moment.H, moment.state) on the lattice bonds (src/zoo/currents.jl:92-102).
#include <cuda_runtime.h>

#include <string.h>

#include <new>
#include <vector>

#include "lmgpu_internal.cuh"

using namespace lmgpu;

struct lm_ring {
    lm_ctx* ctx = nullptr;
    int nslots = 0;
    int64_t len = 0;
    double* d_buf = nullptr;  // nslots x len on the device
    double* h_buf = nullptr;  // nslots x len, pinned host memory
    std::vector<cudaEvent_t> ev;
    std::vector<double> t;
    std::vector<int64_t> count;  // values held by each slot
    int64_t head = 0;            // sequence number of the next entry
};

extern "C" {

int lm_ring_create(lm_ctx* ctx, int nslots, int64_t len, lm_ring** out) {
    if (!ctx || !out) return LM_ERR_ARG;
    *out = nullptr;
    CHECK_ARG(ctx, nslots >= 1 && nslots <= 4096, "lm_ring_create: nslots must be in 1..4096");
    CHECK_ARG(ctx, len >= 1 && len <= ((int64_t)1 << 34) / nslots, "lm_ring_create: bad slot length");
    cudaSetDevice(ctx->device);
    lm_ring* r = new (std::nothrow) lm_ring();
    if (!r) return set_err(ctx, LM_ERR_OOM, "lm_ring_create: host allocation");
    r->ctx = ctx;
    r->nslots = nslots;
    r->len = len;
    const size_t bytes = sizeof(double) * (size_t)len * (size_t)nslots;
    cudaError_t e = cudaMalloc((void**)&r->d_buf, bytes);
    if (e == cudaSuccess) e = cudaHostAlloc((void**)&r->h_buf, bytes, cudaHostAllocDefault);
    r->ev.assign((size_t)nslots, nullptr);
    for (int i = 0; e == cudaSuccess && i < nslots; ++i)
        e = cudaEventCreateWithFlags(&r->ev[(size_t)i], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        cudaGetLastError();
        int rc = check_cuda(ctx, e, "lm_ring_create");
        lm_ring_destroy(r);
        return rc;
    }
    r->t.assign((size_t)nslots, 0.0);
    r->count.assign((size_t)nslots, 0);
    *out = r;
    return LM_OK;
}

int lm_ring_destroy(lm_ring* r) {
    if (!r) return LM_OK;
    cudaSetDevice(r->ctx->device);
    cudaStreamSynchronize(r->ctx->stream);
    for (cudaEvent_t e : r->ev)
        if (e) cudaEventDestroy(e);
    if (r->d_buf) cudaFree(r->d_buf);
    if (r->h_buf) cudaFreeHost(r->h_buf);
    delete r;
    return LM_OK;
}

}  // extern "C"

// Claims the next slot, runs `fill` into its device copy, queues the download and the
// slot's event.  The pinned copy of entry s - nslots is overwritten by this download.
template <typename Fill>
static int ring_push(lm_ring* r, double t, int64_t n, int64_t* seq, Fill fill) {
    lm_ctx* ctx = r->ctx;
    const int64_t s = r->head;
    const int k = (int)(s % r->nslots);
    double* d = r->d_buf + (size_t)k * (size_t)r->len;
    double* h = r->h_buf + (size_t)k * (size_t)r->len;
    CUDA_TRY(ctx, fill(d), "readout kernel");
    CUDA_TRY(ctx, cudaMemcpyAsync(h, d, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream),
             "readout download");
    CUDA_TRY(ctx, cudaEventRecord(r->ev[(size_t)k], ctx->stream), "cudaEventRecord");
    r->t[(size_t)k] = t;
    r->count[(size_t)k] = n;
    r->head = s + 1;
    if (seq) *seq = s;
    return LM_OK;
}

static int ring_entry(lm_ring* r, int64_t seq, int* k) {
    lm_ctx* ctx = r->ctx;
    CHECK_ARG(ctx, seq >= 0 && seq < r->head, "lm_ring: entry not pushed yet");
    CHECK_ARG(ctx, seq >= r->head - r->nslots, "lm_ring: entry already overwritten");
    *k = (int)(seq % r->nslots);
    return LM_OK;
}

extern "C" {

int lm_ring_push_localdensity(lm_ring* r, lm_state* st, double t, int64_t* seq) {
    if (!r) return LM_ERR_ARG;
    lm_ctx* ctx = r->ctx;
    CHECK_ARG(ctx, st != nullptr && st->ctx == ctx, "lm_ring_push_localdensity: state from another context");
    CHECK_ARG(ctx, st->n <= r->len, "lm_ring_push_localdensity: slot shorter than the lattice");
    cudaSetDevice(ctx->device);
    return ring_push(r, t, st->n, seq, [&](double* d) {
        return launch_localdensity(ctx, st->precision, st->kind, st->d_data, st->n, st->m, st->ld, st->d_w, d);
    });
}

int lm_ring_push_currents(lm_ring* r, lm_ham* h, lm_state* st, double t, int64_t* seq) {
    if (!r) return LM_ERR_ARG;
    lm_ctx* ctx = r->ctx;
    CHECK_ARG(ctx, h != nullptr && h->ctx == ctx, "lm_ring_push_currents: Hamiltonian from another context");
    CHECK_ARG(ctx, st != nullptr && st->ctx == ctx, "lm_ring_push_currents: state from another context");
    CHECK_ARG(ctx, st->n == h->lat->g.N, "lm_ring_push_currents: state size does not match the lattice");
    if (!h->assembled) return set_err(ctx, LM_ERR_STATE, "lm_ring_push_currents: Hamiltonian not assembled");
    const int64_t nb = h->lat->nbonds;
    CHECK_ARG(ctx, nb <= r->len, "lm_ring_push_currents: slot shorter than the bond list");
    cudaSetDevice(ctx->device);
    return ring_push(r, t, nb, seq, [&](double* d) {
        if (nb == 0) return cudaSuccess;
        return launch_bond_currents(ctx, h->lat->g, st->precision, st->kind, h->d_hop, st->d_data, st->m, st->ld,
                                    st->d_w, d);
    });
}

int lm_ring_push_op_currents(lm_ring* r, lm_ell* h, lm_state* st, int ndof, const double* op, double t,
                             int64_t* seq) {
    if (!r) return LM_ERR_ARG;
    lm_ctx* ctx = r->ctx;
    CHECK_ARG(ctx, h != nullptr && h->ctx == ctx, "lm_ring_push_op_currents: Hamiltonian from another context");
    CHECK_ARG(ctx, st != nullptr && st->ctx == ctx && st->n == h->n,
              "lm_ring_push_op_currents: state does not match the Hamiltonian");
    CHECK_ARG(ctx, h->nnz <= r->len, "lm_ring_push_op_currents: slot shorter than the stored entries");
    LocalOp lop;
    const int rc = make_local_op(ctx, h, ndof, op, &lop, "lm_ring_push_op_currents");
    if (rc != LM_OK) return rc;
    cudaSetDevice(ctx->device);
    return ring_push(r, t, h->nnz, seq, [&](double* d) { return launch_ell_op_currents(ctx, h, st, ndof, lop, d); });
}

int lm_ring_ready(lm_ring* r, int64_t seq, int* ready) {
    if (!r || !ready) return LM_ERR_ARG;
    int k = 0;
    int rc = ring_entry(r, seq, &k);
    if (rc != LM_OK) return rc;
    const cudaError_t e = cudaEventQuery(r->ev[(size_t)k]);
    if (e == cudaErrorNotReady) {
        *ready = 0;
        return LM_OK;
    }
    *ready = 1;
    return check_cuda(r->ctx, e, "lm_ring_ready");
}

int lm_ring_wait(lm_ring* r, int64_t seq, double* out, const double** view, int64_t* n, double* t) {
    if (!r) return LM_ERR_ARG;
    int k = 0;
    int rc = ring_entry(r, seq, &k);
    if (rc != LM_OK) return rc;
    CUDA_TRY(r->ctx, cudaEventSynchronize(r->ev[(size_t)k]), "lm_ring_wait");
    const double* h = r->h_buf + (size_t)k * (size_t)r->len;
    const int64_t cnt = r->count[(size_t)k];
    if (out) memcpy(out, h, sizeof(double) * (size_t)cnt);
    if (view) *view = h;
    if (n) *n = cnt;
    if (t) *t = r->t[(size_t)k];
    return LM_OK;
}

int lm_ring_head(const lm_ring* r, int64_t* head) {
    if (!r || !head) return LM_ERR_ARG;
    *head = r->head;
    return LM_OK;
}

}  // extern "C"
