// Allocation-free Chebyshev step.
//
// Some hosts cannot let this library call cudaMalloc: applications whose device memory is
// owned by another allocator (a pooled allocator such as CUDA.jl's or PyTorch's caching
// allocator running under a fixed memory budget, where a foreign cudaMalloc can fail or
// fragment the pool) and real-time or embedded hosts that forbid allocation after start-up.
// lm_solver_step_noalloc serves them: it advances a caller-owned ket block in place and
// keeps the Chebyshev recurrence and accumulator buffers in the file-scope device array
// below instead of allocating them.
//
// Cost and limits: every GPU that loads this library holds the array (32 MiB) until the
// process exits.  A call needs 2 * ld * m complex scratch elements (16 bytes each for
// ComplexF64, 8 for ComplexF32), so ld * m <= 1 Mi for ComplexF64 and <= 2 Mi for
// ComplexF32; larger blocks are rejected with LM_ERR_ARG.  The first call on a device looks
// up the array's device address (set-up, once per device); make that first call before any
// stream capture.  All calls share the array: calls whose
// launches overlap on the GPU (different streams or contexts) race on it and give wrong
// results.  Nothing in it has to start at zero: the first Chebyshev order overwrites both
// buffers before anything reads them, so the previous call's contents do no harm.
#include <cuda_runtime.h>

#include <mutex>

#include "lmgpu_internal.cuh"

namespace {

constexpr size_t kNoallocScratchBytes = (size_t)32 << 20;
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

constexpr int kMaxDevices = 64;
void* g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

// Device address of the scratch array on `device` (looked up once per device, with that
// device current).  In host code the symbol itself is only a host-side stand-in.
int scratch_address(lm_ctx* ctx, void** out) {
    if (ctx->device < 0 || ctx->device >= kMaxDevices)
        return lmgpu::set_err(ctx, LM_ERR_NOTSUP, "lm_solver_step_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[ctx->device]) {
        cudaError_t e = cudaSetDevice(ctx->device);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&g_scratch_ptr[ctx->device], g_noalloc_scratch);
        if (e != cudaSuccess) {
            g_scratch_ptr[ctx->device] = nullptr;
            return lmgpu::check_cuda(ctx, e, "lm_solver_step_noalloc: cudaGetSymbolAddress");
        }
    }
    *out = g_scratch_ptr[ctx->device];
    return LM_OK;
}

}  // namespace

extern "C" int lm_solver_step_noalloc(lm_solver* s, void* kets, int64_t n, int64_t m, int64_t ld, int precision) {
    using namespace lmgpu;
    if (!s) return LM_ERR_ARG;
    lm_ctx* ctx = s->ctx;
    if (!kets) return set_err(ctx, LM_ERR_ARG, "lm_solver_step_noalloc: null ket block");
    if (precision != LM_C64 && precision != LM_C32)
        return set_err(ctx, LM_ERR_ARG, "lm_solver_step_noalloc: unknown precision");
    if (!s->valid) return set_err(ctx, LM_ERR_STATE, "lm_solver_step_noalloc: update_solver must run before step");
    if (s->ell) return set_err(ctx, LM_ERR_NOTSUP, "lm_solver_step_noalloc: square-lattice Hamiltonians only");
    const Geom& g = s->ham->lat->g;
    if (n != g.N || m < 1 || ld < n)
        return set_err(ctx, LM_ERR_ARG, "lm_solver_step_noalloc: block shape does not match the lattice");
    const size_t elem = precision == LM_C64 ? 16 : 8;
    // recurrence buffer A and accumulator Y, each addressed like the caller's block (ld x m)
    const size_t per_buf = elem * (size_t)ld;
    if ((size_t)m > kNoallocScratchBytes / (2 * per_buf))
        return set_err(ctx, LM_ERR_ARG,
                       "lm_solver_step_noalloc: block too large for the 32 MiB static scratch "
                       "(needs ld*m <= 1Mi for ComplexF64, 2Mi for ComplexF32)");
    void* base = nullptr;
    int rc = scratch_address(ctx, &base);
    if (rc != LM_OK) return rc;
    rc = check_cuda(ctx, cudaSetDevice(ctx->device), "lm_solver_step_noalloc: cudaSetDevice");
    if (rc != LM_OK) return rc;
    void* A = base;
    void* Y = (unsigned char*)base + per_buf * (size_t)m;
    const void* hop2 = precision == LM_C64 ? (const void*)s->d_hop2 : (const void*)s->d_hop2f;
    const void* diag2 = precision == LM_C64 ? (const void*)s->d_diag2 : (const void*)s->d_diag2f;
    const int K = s->K;
    const double c0 = s->coef[0].s;
    const ChebLo lo = cheb_lo(s->phase_re, s->phase_im, c0, s->coef[1].s, false);
    // T_k overwrites T_{k-2}: even orders land in the caller's block, odd orders in A
    const bool xr = ham_x_real(s->ham);
    rc = check_cuda(ctx, launch_cheb_order(ctx, g, precision, 1, 0, CHEB_FIRST, hop2, diag2, kets, A, Y, ld, m, c0,
                                           s->coef[1], s->phase_re, s->phase_im, lo, xr),
                    "lm_solver_step_noalloc: order 1");
    if (rc != LM_OK) return rc;
    for (int k = 2; k <= K; ++k) {
        const void* tp = (k % 2 == 0) ? A : kets;
        void* tq = (k % 2 == 0) ? kets : A;
        const int mode = (k == K) ? CHEB_LAST : CHEB_MID;
        rc = check_cuda(ctx, launch_cheb_order(ctx, g, precision, 1, 0, mode, hop2, diag2, tp, tq, Y, ld, m, c0,
                                               s->coef[(size_t)k], s->phase_re, s->phase_im, lo, xr),
                        "lm_solver_step_noalloc: order");
        if (rc != LM_OK) return rc;
    }
    if (K % 2 == 1)  // the result is in A: copy it into the caller's block (no allocation)
        return check_cuda(ctx, cudaMemcpy2DAsync(kets, per_buf, A, per_buf, elem * (size_t)n, (size_t)m,
                                                 cudaMemcpyDeviceToDevice, ctx->stream),
                          "lm_solver_step_noalloc: copy result");
    return LM_OK;
}
