// qtg_kwald_noalloc: the reciprocal-space Ewald sum of qtg_kwald for callers
// that cannot allocate device memory. Every piece of scratch the computation
// needs lives in one file-scope static device array; the caller passes only
// its own input and output buffers.
//
// Who needs this: code that gets its GPU memory handed to it and must not call
// cudaMalloc -- a molecular-dynamics engine or framework plugin that owns the
// device memory budget and calls force routines with preallocated buffers (an
// allocation of its own would escape the engine's accounting, or fail under
// the engine's memory cap), and loops that cannot afford allocator latency or
// fragmentation on every call. A qtg_ctx cannot serve them: qtg_create
// allocates all of its memory up front.
//
// Limits: at most QTG_NOALLOC_MAX_SITES charge sites and k_max <=
// QTG_NOALLOC_MAX_KMAX; the array is 2.76 MiB (2,895,872 bytes) and every GPU that loads the
// library holds it until the process exits.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <mutex>

#include "../../include/qtip4pf_gb300.h"
#include "qtg_internal.h"

namespace qtg {
namespace {

constexpr int NA_MAX_SITES = QTG_NOALLOC_MAX_SITES;
constexpr int NA_MAX_KMAX = QTG_NOALLOC_MAX_KMAX;
constexpr int NA_COLS = (NA_MAX_KMAX + 1) * (2 * NA_MAX_KMAX + 1);  // every (kx >= 0, ky) column
constexpr int NA_MAX_K = NA_COLS * (2 * NA_MAX_KMAX + 1);          // every kz of every column
constexpr int NA_MAX_GRP = NA_COLS * ((NA_MAX_KMAX + 1 + 3) / 4);
constexpr int NA_MAX_BATCH = NA_COLS;
constexpr int NA_SC = 8, NA_KC = 8;  // structure-factor site chunks and k-chunks the scratch holds

constexpr size_t al256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t OFF_SYS = 0;
constexpr size_t OFF_JOB = OFF_SYS + al256(sizeof(SysDev));
constexpr size_t OFF_KVEC = OFF_JOB + al256(sizeof(Job));
constexpr size_t OFF_KCOL = OFF_KVEC + al256(sizeof(KVec) * NA_MAX_K);
constexpr size_t OFF_KGRP = OFF_KCOL + al256(sizeof(KCol) * NA_COLS);
constexpr size_t OFF_KBATCH = OFF_KGRP + al256(sizeof(KGroup) * NA_MAX_GRP);
constexpr size_t OFF_SITES = OFF_KBATCH + al256(sizeof(KBatch) * NA_MAX_BATCH);
constexpr size_t OFF_PHASE = OFF_SITES + al256(4 * sizeof(double) * NA_MAX_SITES);
constexpr size_t OFF_SKP = OFF_PHASE + al256(2 * sizeof(double) * 3 * (NA_MAX_KMAX + 1) * NA_MAX_SITES);
constexpr size_t OFF_WSK = OFF_SKP + al256(2 * sizeof(double) * NA_SC * NA_MAX_K);
constexpr size_t OFF_PART = OFF_WSK + al256(2 * sizeof(double) * NA_MAX_K);
constexpr size_t OFF_STATUS = OFF_PART + al256(3 * sizeof(double) * NA_KC * NA_MAX_SITES);
constexpr size_t NA_BYTES = OFF_STATUS + 256;

// All scratch of qtg_kwald_noalloc. In host code this name is only a host-side
// stand-in for the symbol: the device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];
static_assert(NA_BYTES == 2895872, "the scratch size stated in the header and comments is out of date");

constexpr int NA_MAX_DEVICES = 64;
unsigned char *g_scratch_ptr[NA_MAX_DEVICES] = {nullptr};

struct NAParams {
    SysDev S;
    double bk[3];
    double kc_sq, quart;
    int kmax;
};

// The reference's k set (forces.cpp:251-445), FP64 products and sums rounded
// one by one as the host evaluates them: (kx,0,0) if 0 < |k|^2 < kc^2; every
// other (kx, ky, kz) if |k|^2 <= kc^2 and, for ky != 0, kx^2 + ky^2 within kc^2.
__device__ bool k_included(const NAParams &p, int kx, int ky, int kz, double *ksq_out) {
    const double rx = __dmul_rn(p.bk[0], (double)kx);
    const double ry = __dmul_rn(p.bk[1], (double)abs(ky));
    const double rz = __dmul_rn(p.bk[2], (double)abs(kz));
    const double xx = __dmul_rn(rx, rx);
    if (ky == 0 && kz == 0) {
        *ksq_out = xx;
        return xx > 0.0 && xx < p.kc_sq;
    }
    if (ky == 0) {
        const double k2 = __dadd_rn(xx, __dmul_rn(rz, rz));
        *ksq_out = k2;
        return k2 <= p.kc_sq;
    }
    const double gate = __dadd_rn(xx, __dmul_rn(ry, ry));
    if (gate > p.kc_sq) return false;
    if (kz == 0) {
        *ksq_out = gate;
        return true;
    }
    const double k2 = __dadd_rn(gate, __dmul_rn(rz, rz));
    *ksq_out = k2;
    return k2 <= p.kc_sq;
}

__device__ int block_scan_excl(int v, int *sh, int *total) {
    // 512 threads: inclusive warp scans, then a scan of the 16 warp totals
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
    }
    __syncthreads();
    if (lane == 31) sh[w] = inc;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            const int t = sh[k];
            sh[k] = run;
            run += t;
        }
        sh[32] = run;
    }
    __syncthreads();
    *total = sh[32];
    return sh[w] + inc - v;
}

// Builds the column-ordered k tables and the system / job records in the
// scratch (one block of 512 threads; every table entry is rewritten, so no
// state survives from an earlier call) and clears the status word.
__global__ void __launch_bounds__(512) k_noalloc_setup(NAParams p, unsigned char *base) {
    __shared__ int sh[33];
    KVec *kvec = reinterpret_cast<KVec *>(base + OFF_KVEC);
    KCol *kcol = reinterpret_cast<KCol *>(base + OFF_KCOL);
    KGroup *kgrp = reinterpret_cast<KGroup *>(base + OFF_KGRP);
    KBatch *kbat = reinterpret_cast<KBatch *>(base + OFF_KBATCH);
    const int width = 2 * p.kmax + 1, ncol_all = (p.kmax + 1) * width;
    const int t = threadIdx.x;
    int kx = 0, ky = 0, m = -1;
    if (t < ncol_all) {
        kx = t / width;
        ky = t % width - p.kmax;
        double ksq;
        for (int kz = 1; kz <= p.kmax; ++kz) {
            if (!k_included(p, kx, ky, kz, &ksq)) break;
            m = kz;
        }
        if (m < 0 && k_included(p, kx, ky, 0, &ksq)) m = 0;
    }
    const int n = m >= 0 ? 2 * m + 1 : 0;
    int nk, ncol, ngrp;
    const int kb = block_scan_excl(n, sh, &nk);
    const int ci = block_scan_excl(n > 0 ? 1 : 0, sh, &ncol);
    const int ng_col = m >= 0 ? (m + 4) / 4 : 0;  // groups of <= 4 |kz|
    const int gi = block_scan_excl(ng_col, sh, &ngrp);
    if (n > 0) {
        KCol c;
        c.kx = kx;
        c.ky = ky;
        c.m = m;
        c.k_begin = kb;
        kcol[ci] = c;
        for (int kz = -m; kz <= m; ++kz) {
            KVec v;
            v.kx = kx;
            v.ky = ky;
            v.kz = kz;
            v.twin = 0;
            double ksq = 0.0;
            if (k_included(p, kx, ky, kz, &ksq)) {
                v.coef = p.S.k_pref * exp(-ksq * p.quart) / ksq * (kx ? 2.0 : 1.0);
                v.gx = 2.0 * v.coef * p.bk[0] * kx;
                v.gy = 2.0 * v.coef * p.bk[1] * ky;
                v.gz = 2.0 * v.coef * p.bk[2] * kz;
            } else {
                v.coef = v.gx = v.gy = v.gz = 0.0;
            }
            kvec[kb + kz + m] = v;
        }
        for (int g = 0; g < ng_col; ++g) {
            KGroup G;
            G.col = ci;
            G.kz0 = 4 * g;
            G.n = min(4, m - G.kz0 + 1);
            G.pad = 0;
            kgrp[gi + g] = G;
        }
    }
    __syncthreads();
    if (t == 0) {
        int nb = 0, c0 = 0;
        while (c0 < ncol) {
            int c1 = c0, cnt = 0;
            while (c1 < ncol && cnt + 2 * kcol[c1].m + 1 <= 128) {
                cnt += 2 * kcol[c1].m + 1;
                ++c1;
            }
            KBatch b;
            b.c0 = c0;
            b.c1 = c1;
            b.k0 = kcol[c0].k_begin;
            b.k1 = kcol[c1 - 1].k_begin + 2 * kcol[c1 - 1].m + 1;
            kbat[nb++] = b;
            c0 = c1;
        }
        SysDev S = p.S;
        S.n_kvec = nk;
        S.n_col = ncol;
        S.n_grp = ngrp;
        S.n_batch = nb;
        S.n_grp_half = ngrp;  // FP64 only here: the full set
        S.n_batch_half = nb;
        *reinterpret_cast<SysDev *>(base + OFF_SYS) = S;
        Job J;
        J.sys = 0;
        J.bead = 0;
        J.slot = 0;
        J.mode = 0;
        J.pos_off = J.out_off = J.site_off = J.phase_off = J.sk_off = 0;
        *reinterpret_cast<Job *>(base + OFF_JOB) = J;
        *reinterpret_cast<unsigned *>(base + OFF_STATUS) = 0u;
    }
}

std::mutex g_setup_mutex;

// Once per device, with that device current: the device address of the
// scratch array and the kernels' shared-memory limits. The lock makes a first
// call made by several host threads at once set the device up once.
qtg_status scratch_for_current_device(unsigned char **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) return QTG_ERR_NODEVICE;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return QTG_ERR_CUDA;
        init_force_kernel_attributes();
        g_scratch_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch_ptr[dev];
    return QTG_OK;
}

}  // namespace
}  // namespace qtg

using namespace qtg;

extern "C" qtg_status qtg_kwald_noalloc(const double *sites, const double *charge, int n_sites,
                                        const double *box_bohr, double eps_ewald, double *f_sites,
                                        double *energy, void *cuda_stream) {
    if (!sites || !charge || !f_sites || !energy || !box_bohr) return QTG_ERR_ARG;
    if (n_sites < 3 || n_sites % 3 != 0 || n_sites > NA_MAX_SITES) return QTG_ERR_ARG;
    if (!(box_bohr[0] > 0 && box_bohr[1] > 0 && box_bohr[2] > 0)) return QTG_ERR_ARG;
    if (!(eps_ewald > 0 && eps_ewald < 1)) return QTG_ERR_ARG;
    // an error left pending by the caller's own CUDA work is theirs: report it
    // without clearing it, and launch nothing
    if (cudaPeekAtLastError() != cudaSuccess) return QTG_ERR_CUDA;
    // Ewald parameters exactly as forces.cpp:574-584 derives them
    NAParams p;
    memset(&p, 0, sizeof(p));
    SysDev &S = p.S;
    const double vol = box_bohr[0] * box_bohr[1] * box_bohr[2];
    const double acc = sqrt(-log(eps_ewald));
    const double rho = n_sites / vol;
    const double min_box = std::min(std::min(box_bohr[0], box_bohr[1]), box_bohr[2]);
    const double max_box = std::max(std::max(box_bohr[0], box_bohr[1]), box_bohr[2]);
    double kappa = 2.6 * pow(rho / vol, 1.0 / 6.0);
    double rc = acc / kappa;
    if (rc > 0.5 * min_box) {
        rc = 0.5 * min_box;
        kappa = acc / rc;
    }
    const double kc = 2.0 * acc * kappa;
    const int kmax = (int)(kc * max_box / (2.0 * PI_REF));
    if (kmax > NA_MAX_KMAX) return QTG_ERR_ARG;
    S.n_mols = n_sites / 3;
    S.n_sites = n_sites;
    S.n_dof = 3 * n_sites;
    S.k_max = kmax;
    S.kappa = kappa;
    S.k_pref = 2.0 * PI_REF / vol;
    for (int d = 0; d < 3; ++d) {
        S.box[d] = box_bohr[d];
        S.inv_box[d] = 1.0 / box_bohr[d];
        S.boxf[d] = (float)S.box[d];
        S.inv_boxf[d] = (float)S.inv_box[d];
        p.bk[d] = 2.0 * PI_REF / box_bohr[d];
    }
    set_float_consts(S);
    p.kc_sq = kc * kc;
    p.quart = 0.25 / (kappa * kappa);
    p.kmax = kmax;
    unsigned char *base = nullptr;
    const qtg_status st = scratch_for_current_device(&base);
    if (st != QTG_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    k_noalloc_setup<<<1, 512, 0, s>>>(p, base);
    EvalArgs a;
    memset(&a, 0, sizeof(a));
    a.sys = reinterpret_cast<const SysDev *>(base + OFF_SYS);
    a.jobs = reinterpret_cast<const Job *>(base + OFF_JOB);
    a.n_jobs = 1;
    a.max_mols = S.n_mols;
    a.max_kvec = NA_MAX_K;
    a.max_kmax = kmax;
    a.max_grp = NA_MAX_GRP;
    a.kz = 4;  // the groups built above hold <= 4 |kz|
    a.max_batch = NA_MAX_BATCH;
    a.pos = sites;
    a.out = f_sites;
    a.charge = charge;
    a.kvec = reinterpret_cast<const KVec *>(base + OFF_KVEC);
    a.kcol = reinterpret_cast<const KCol *>(base + OFF_KCOL);
    a.kgrp = reinterpret_cast<const KGroup *>(base + OFF_KGRP);
    a.kbatch = reinterpret_cast<const KBatch *>(base + OFF_KBATCH);
    a.sites = base + OFF_SITES;
    a.phase = base + OFF_PHASE;
    a.skp = reinterpret_cast<double2 *>(base + OFF_SKP);
    a.total_k = NA_MAX_K;
    a.wsk = base + OFF_WSK;
    a.part = reinterpret_cast<double *>(base + OFF_PART);
    a.total_sites = NA_MAX_SITES;
    a.energy = energy;
    a.status = reinterpret_cast<unsigned *>(base + OFF_STATUS);
    a.sites_are_input = 1;
    a.tune_sc = NA_SC;  // the scratch holds this many partial planes
    a.tune_kc = NA_KC;
    launch_kwald_only(a, false, s, nullptr);
    return cudaGetLastError() == cudaSuccess ? QTG_OK : QTG_ERR_CUDA;
}
