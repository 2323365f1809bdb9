// The lattice-resident form of a ComplexF32 batch's fused pass (lmgpu_resident.cu): its
// descriptor and launch interface, shared with the batch (lmgpu_batch.cu).
#pragma once
#include "lmgpu_internal.cuh"

namespace lmgpu {

// Lattice-resident form of the ComplexF32 step (lmgpu_resident.cu): a thread holds a block of
// kResC columns x kResR rows of one ket in registers for all K orders, one CTA of kResThreads
// holds a lattice of up to kResThreads blocks (G kets at a time when smaller), a cluster of two
// CTAs one of up to 2 kResThreads blocks split along x.
constexpr int kResR = 4;
constexpr int kResC = 3;
constexpr int kResThreads = 384;
constexpr int kResMaxK = 40;

struct ResidentInst {
    const float2* hop2;
    const float* diag2;
    const float2* x;
    float2* out;
    int64_t ld, M;
    int64_t item_begin, item_end;  // this instance's work items [begin, end): G kets each
    int Lx, Ly, per_x, per_y;
    int nbx, nby;   // thread blocks along x (kResC columns each) and y (kResR rows each)
    int G;          // kets per item (thread groups of nbx * nby threads); 1 on a cluster
    int nbx0;       // on a cluster: block columns held by CTA rank 0 (rank 1 holds the rest)
    int ncl;        // columns of the exchange buffer without its two halo columns
    int rs, gs;     // bytes of a row of exchange entries, (ncl + 2) 32 + 16, and of a thread group, (nby + 2) rs
    int slab;       // float2 words per ket of the staging buffer, ncl * Ly
    int smem;       // dynamic shared memory the instance needs (bytes)
    int vec;        // site pairs move as 16-byte units (even Ly and ld, 16-byte aligned x and out)
    float s[kResMaxK + 1];
    float ph_re, ph_im;   // e^{-ib dt}
    float a0_re, a0_im;   // e^{-ib dt} c_0
    ChebLo lo;            // fused-form second words
};

// Lattice-resident form (lmgpu_resident.cu).  resident_plan: whether a lattice of geometry g
// with m kets runs in it, on one CTA (*cl = 1) or a cluster of two (*cl = 2), and its layout
// in d (every field but the pointers, items and coefficients).  resident_fill_coef: the
// coefficients.  launch_resident_table: one launch over the items of a device table of ninst
// instances, pulled from the work-queue counter d_queue (zeroed before the launch); smem is the
// largest `smem` of the table; *d_err gets bit 0 when a halo exchange on a cluster timed out.
bool resident_plan(const Geom& g, int64_t m, ResidentInst& d, int* cl);
void resident_fill_coef(ResidentInst& d, int K, const ChebCoef* coef, double ph_re, double ph_im);
cudaError_t launch_resident_table(lm_ctx* ctx, int K, bool xreal, int cl, const ResidentInst* d_table, int ninst,
                                  int64_t nitems, unsigned long long* d_queue, unsigned long long* d_err,
                                  int smem);
// Sets the kernel's shared-memory attribute (outside stream capture).
cudaError_t ensure_resident_attr(lm_ctx* ctx, bool xreal, int cl);

}  // namespace lmgpu
