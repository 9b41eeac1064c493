// Per-call staging: the arrays of one per-call step move between the caller's
// page-locked host memory and the device inside the step's graph, as loads and
// stores of kernels (host memory is reached over the CPU-GPU link; on Grace
// machines NVLink-C2C), instead of one copy call per array. The caller's pointers
// and the step's small results pass through a mailbox in mapped host memory, so
// one captured graph serves every call whatever buffers the caller hands in.
#include "qtg_internal.h"

namespace qtg {
namespace {

// dst[0 .. n) = src[0 .. n) by the grid's threads, 16-byte accesses where both
// arrays are 16-byte aligned
__device__ __forceinline__ void copy_seg(double *__restrict__ dst, const double *__restrict__ src, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x, nt = (long long)gridDim.x * blockDim.x;
    if (((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15u) == 0) {
        const long long n2 = n >> 1;
        double2 *d2 = reinterpret_cast<double2 *>(dst);
        const double2 *s2 = reinterpret_cast<const double2 *>(src);
        for (long long i = t; i < n2; i += nt) d2[i] = s2[i];
        if ((n & 1) && t == 0) dst[n - 1] = src[n - 1];
    } else {
        for (long long i = t; i < n; i += nt) dst[i] = src[i];
    }
}

// The arrays a.mask names (q, p, f: nt doubles each; disp: nd) from the caller
// into the device arrays; the caller's heat into the run state.
__global__ void __launch_bounds__(256) k_stage_in(StageArgs a) {
    __shared__ const double *src[4];
    if (threadIdx.x == 0) {
        src[0] = a.box->q;
        src[1] = a.box->p;
        src[2] = a.box->f;
        src[3] = a.box->disp;
        if (blockIdx.x == 0) a.run->heat = a.box->heat_in;
    }
    __syncthreads();
    if (a.mask & STAGE_Q) copy_seg(a.q, src[0], a.nt);
    if (a.mask & STAGE_P) copy_seg(a.p, src[1], a.nt);
    if (a.mask & STAGE_F) copy_seg(a.f, src[2], a.nt);
    if (a.mask & STAGE_DISP) copy_seg(a.disp, src[3], a.nd);
}

// The arrays a.mask names back to the caller (q, p, f, fphys: nt doubles each;
// disp: nd); with STAGE_SMALL, block 0 also posts the heat, per-bead energies and
// rebuild flags, the accumulators and the status word to the mailbox, then
// clears the accumulators and the status word.
__global__ void __launch_bounds__(256) k_stage_out(StageArgs a) {
    __shared__ double *dst[5];
    if (threadIdx.x == 0) {
        dst[0] = a.box->q;
        dst[1] = a.box->p;
        dst[2] = a.box->f;
        dst[3] = a.box->fphys;
        dst[4] = a.box->disp;
    }
    __syncthreads();
    if (a.mask & STAGE_Q) copy_seg(dst[0], a.q, a.nt);
    if (a.mask & STAGE_P) copy_seg(dst[1], a.p, a.nt);
    if (a.mask & STAGE_F) copy_seg(dst[2], a.f, a.nt);
    if (a.mask & STAGE_FPHYS) copy_seg(dst[3], a.fphys, a.nt);
    if (a.mask & STAGE_DISP) copy_seg(dst[4], a.disp, a.nd);
    if ((a.mask & STAGE_SMALL) && blockIdx.x == 0) {
        for (int b = threadIdx.x; b < a.n_beads; b += blockDim.x) {
            a.box_energy[b] = a.energy[b];
            a.box_rebuilt[b] = a.rebuilt[b];
        }
        if (threadIdx.x == 0) {
            a.box->heat_out = a.run->heat;
            a.box->acc = *a.acc;
            a.box->status = *a.status;
            *a.acc = SysAcc{};
            *a.status = 0u;
        }
    }
}

}  // namespace

void launch_stage_in(const StageArgs &a, cudaStream_t s, unsigned long long *n) {
    k_stage_in<<<a.blocks, 256, 0, s>>>(a);
    if (n) *n += 1;
}

void launch_stage_out(const StageArgs &a, cudaStream_t s, unsigned long long *n) {
    k_stage_out<<<a.blocks, 256, 0, s>>>(a);
    if (n) *n += 1;
}

}  // namespace qtg
