// Verlet-list skin test and rebuild (replaces neighbour.cpp:12-62 and the
// per-bead displacement test of update.cpp:354-385 / :95-123).
//
// The list is the reference's CSR half list: for each oxygen i, the oxygens
// j > i (ascending) whose minimum-image distance satisfies r^2 < r_skin^2
// strictly, with point[i] the row start; the device stepper also keeps the
// symmetric list (every j != i). Pair tests run in FP32 on positions wrapped
// into the box; a pair whose FP32 r^2 lies within a relative band of 1e-4
// around r_skin^2 is re-tested with the reference's FP64 arithmetic
// (x - L*round(x/L), then x^2+y^2+z^2, each operation rounded separately), so
// the pair set is bit-identical to the reference's. The FP32 r^2 error is below
// 2e-6 relative for coordinates within a few box lengths of the origin, far
// inside the band.
//
// Four launches over all (system, bead) jobs:
//  1. k_skin_test, a block per job: the two largest oxygen displacements since
//     the last build (update.cpp:356-385) decide whether the bead rebuilds;
//     a rebuilding bead wraps its oxygens into the box, sorts them into a cell
//     grid of side >= r_skin / 2 (boxes of at least five cells a side) and
//     zeroes its displacements.
//  2. k_list_rows (count), a warp per row i: the candidates -- the molecules of
//     the 5 x 5 x 5 cells around i's cell, or every molecule in smaller boxes --
//     are tested and marked in a per-row bitmap of all N molecules in shared
//     memory; its population (all, and j > i) gives the row's two counts.
//  3. k_list_scan, a block per rebuilding job: row starts by exclusive scans,
//     overflow check.
//  4. k_list_rows (fill): the bitmap again, read word by word in ascending j, so
//     the rows come out in the reference's order whatever order the cells gave.
// Rows spread over many blocks per bead (the build is O(N) candidates a row).
#include <algorithm>

#include "qtg_internal.h"

namespace qtg {

namespace {

constexpr float kBand = 1e-4f;
constexpr int ROWS = 8;  // warps (rows at a time) per block of k_list_rows

__device__ __forceinline__ bool pair_exact(const double *qi, const double *qj, const SysDev &S) {
    double r2 = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        double x = __dsub_rn(qi[d], qj[d]);
        double n = round(__ddiv_rn(x, S.box[d]));
        x = __dsub_rn(x, __dmul_rn(S.box[d], n));
        r2 = (d == 0) ? __dmul_rn(x, x) : __dadd_rn(r2, __dmul_rn(x, x));
    }
    return r2 < S.r_skin_sq;
}

__device__ __forceinline__ bool pair_in(const float4 a, const float4 b, const double *qi, const double *qj,
                                        const SysDev &S, float rs2) {
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    dx -= S.boxf[0] * rintf(dx * S.inv_boxf[0]);
    dy -= S.boxf[1] * rintf(dy * S.inv_boxf[1]);
    dz -= S.boxf[2] * rintf(dz * S.inv_boxf[2]);
    float r2 = dx * dx + dy * dy + dz * dz;
    if (fabsf(r2 - rs2) > kBand * rs2) return r2 < rs2;
    return pair_exact(qi, qj, S);
}

// Exclusive scan of cnt[0..n) in place; returns the total. All threads call it.
__device__ int block_exclusive_scan(int *cnt, int n, int *warp_tot) {
    const int T = blockDim.x, t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int per = (n + T - 1) / T;
    const int b0 = min(n, t * per), b1 = min(n, b0 + per);
    int loc = 0;
    for (int k = b0; k < b1; ++k) loc += cnt[k];
    int inc = loc;
    for (int o = 1; o < 32; o <<= 1) {
        int v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    if (lane == 31) warp_tot[w] = inc;
    __syncthreads();
    if (w == 0) {
        int nw = (T + 31) >> 5;
        int v = (lane < nw) ? warp_tot[lane] : 0;
        int vi = v;
        for (int o = 1; o < 32; o <<= 1) {
            int u = __shfl_up_sync(0xffffffffu, vi, o);
            if (lane >= o) vi += u;
        }
        if (lane < nw) warp_tot[lane] = vi - v;  // exclusive warp offsets
        if (lane == nw - 1) warp_tot[32] = vi;   // total
    }
    __syncthreads();
    int run = warp_tot[w] + inc - loc;
    for (int k = b0; k < b1; ++k) {
        int c = cnt[k];
        cnt[k] = run;
        run += c;
    }
    __syncthreads();
    return warp_tot[32];
}

__device__ __forceinline__ int cell_of(const float4 p, const SysDev &S) {
    int c[3];
    const float v[3] = {p.x, p.y, p.z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        c[d] = (int)(v[d] * (float)S.lc_n[d] * S.inv_boxf[d]);
        c[d] = min(max(c[d], 0), S.lc_n[d] - 1);
    }
    return (c[2] * S.lc_n[1] + c[1]) * S.lc_n[0] + c[0];
}

__global__ void __launch_bounds__(256) k_skin_test(ListArgs a) {
    const int job = blockIdx.x;
    const int sid = a.job_sys[job], bead = a.job_bead[job];
    const SysDev &S = a.sys[sid];
    const int N = S.n_mols;
    double *disp = a.disp + S.d_off + (size_t)bead * 3 * N;
    __shared__ unsigned long long red[2][33];
    __shared__ int do_build;
    int build = a.force_rebuild;
    if (!build) {
        // two largest squared displacements (update.cpp:361-375). Squared norms are
        // non-negative doubles, which order exactly as their 64-bit patterns do, so
        // the top-2 selection runs on integer compares instead of the FP64 pipe.
        unsigned long long m1 = 0ull, m2 = 0ull;
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            const double x = disp[3 * i], y = disp[3 * i + 1], z = disp[3 * i + 2];
            const unsigned long long d2 = (unsigned long long)__double_as_longlong(x * x + y * y + z * z);
            if (d2 > m1) {
                m2 = m1;
                m1 = d2;
            } else if (d2 > m2) {
                m2 = d2;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long b1 = __shfl_xor_sync(0xffffffffu, m1, o), b2 = __shfl_xor_sync(0xffffffffu, m2, o);
            const unsigned long long n1 = max(m1, b1), n2 = max(min(m1, b1), max(m2, b2));
            m1 = n1;
            m2 = n2;
        }
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
        if (lane == 0) {
            red[0][w] = m1;
            red[1][w] = m2;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long t1 = 0ull, t2 = 0ull;
            for (int k = 0; k < nw; ++k) {
                const unsigned long long b1 = red[0][k], b2 = red[1][k];
                const unsigned long long n1 = max(t1, b1), n2 = max(min(t1, b1), max(t2, b2));
                t1 = n1;
                t2 = n2;
            }
            do_build = (sqrt(__longlong_as_double((long long)t1)) + sqrt(__longlong_as_double((long long)t2)) >
                        S.skin_margin) ? 1 : 0;
        }
        __syncthreads();
        build = do_build;
    }
    // the rebuilding beads, in arrival order (each one's build is independent)
    if (threadIdx.x == 0 && build) a.rb_jobs[atomicAdd(a.rb_count, 1)] = job;
    if (!build) return;
    const double *qb = a.q + S.q_off + (size_t)bead * S.n_dof;
    float4 *wp = a.wpos + S.pt_off + (size_t)bead * N;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        float c[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double x = qb[9 * i + d];
            c[d] = (float)(x - S.box[d] * floor(x * S.inv_box[d]));
        }
        wp[i] = make_float4(c[0], c[1], c[2], 0.f);
    }
    if (S.lc_cells > 0) {
        // counting sort of the molecules into cells (any order within a cell)
        extern __shared__ int ccount[];
        __shared__ int wtot[33];
        const int nc = S.lc_cells;
        for (int c = threadIdx.x; c < nc; c += blockDim.x) ccount[c] = 0;
        __syncthreads();
        for (int i = threadIdx.x; i < N; i += blockDim.x) atomicAdd(&ccount[cell_of(wp[i], S)], 1);
        __syncthreads();
        block_exclusive_scan(ccount, nc, wtot);
        int *cs = a.cell_start + S.lc_off + (size_t)bead * (nc + 1);
        for (int c = threadIdx.x; c < nc; c += blockDim.x) cs[c] = ccount[c];
        if (threadIdx.x == 0) cs[nc] = N;
        __syncthreads();
        int *cm = a.cell_mol + S.pt_off + (size_t)bead * N;
        for (int i = threadIdx.x; i < N; i += blockDim.x) cm[atomicAdd(&ccount[cell_of(wp[i], S)], 1)] = i;
    }
    for (int k = threadIdx.x; k < 3 * N; k += blockDim.x) disp[k] = 0.0;
}

// Marks row i's neighbours (j != i) in the warp's bitmap bm[0 .. ceil(N/32)).
__device__ void row_bitmap(const ListArgs &a, const SysDev &S, int bead, int i, unsigned *bm) {
    const int N = S.n_mols, lane = threadIdx.x & 31, W = (N + 31) >> 5;
    for (int k = lane; k < W; k += 32) bm[k] = 0u;
    __syncwarp();
    const float4 *wp = a.wpos + S.pt_off + (size_t)bead * N;
    const double *qb = a.q + S.q_off + (size_t)bead * S.n_dof;
    const float rs2 = (float)S.r_skin_sq;
    const float4 pi = wp[i];
    auto test = [&](int j) {
        if (j != i && pair_in(pi, wp[j], qb + 9 * i, qb + 9 * j, S, rs2)) atomicOr(&bm[j >> 5], 1u << (j & 31));
    };
    if (S.lc_cells == 0) {
        // every molecule in order: the 32 lanes test the 32 molecules of one bitmap
        // word, which a ballot assembles (no atomics on a shared word)
        for (int j0 = 0; j0 < N; j0 += 32) {
            const int j = j0 + lane;
            const bool in = j < N && j != i && pair_in(pi, wp[j], qb + 9 * i, qb + 9 * j, S, rs2);
            const unsigned word = __ballot_sync(0xffffffffu, in);
            if (lane == 0) bm[j0 >> 5] = word;
        }
    } else {
        const int *cs = a.cell_start + S.lc_off + (size_t)bead * (S.lc_cells + 1);
        const int *cm = a.cell_mol + S.pt_off + (size_t)bead * N;
        const int ci = cell_of(pi, S);
        const int cx = ci % S.lc_n[0], cy = (ci / S.lc_n[0]) % S.lc_n[1], cz = ci / (S.lc_n[0] * S.lc_n[1]);
        for (int dz = -2; dz <= 2; ++dz)
            for (int dy = -2; dy <= 2; ++dy)
                for (int dx = -2; dx <= 2; ++dx) {
                    const int x = (cx + dx + S.lc_n[0]) % S.lc_n[0], y = (cy + dy + S.lc_n[1]) % S.lc_n[1],
                              z = (cz + dz + S.lc_n[2]) % S.lc_n[2];
                    const int c = (z * S.lc_n[1] + y) * S.lc_n[0] + x;
                    for (int k = cs[c] + lane; k < cs[c + 1]; k += 32) test(cm[k]);
                }
    }
    __syncwarp();
}

// FILL = false: the rows' counts; true: the rows' entries (after k_list_scan).
// Work items are (rebuilding job, block of ROWS rows) over the list k_skin_test
// made; a fixed grid loops over them, so a step without rebuilds costs each
// block one load of the count.
template <bool FILL>
__device__ void list_row(const ListArgs &a, int job, int i, unsigned *bms);

template <bool FILL>
__global__ void __launch_bounds__(32 * ROWS) k_list_rows(ListArgs a, int row_blocks) {
    extern __shared__ unsigned bms[];
    const int w = threadIdx.x >> 5;
    // work items (rebuilding job, block of ROWS rows); none when no bead rebuilds
    const long long n_items = (long long)(*a.rb_count) * row_blocks;
    for (long long it = blockIdx.x; it < n_items; it += gridDim.x) {
        const int job = a.rb_jobs[it / row_blocks], rb = (int)(it % row_blocks);
        const SysDev &S = a.sys[a.job_sys[job]];
        const int i = rb * ROWS + w;
        if (i >= S.n_mols) continue;
        // each warp's bitmap at a fixed stride (the launch's largest bead): the warps
        // of a block move on to the next item independently, and items of beads of
        // different sizes must not shift one warp's bitmap onto another's
        list_row<FILL>(a, job, i, bms + (size_t)w * ((a.max_mols + 31) >> 5));
        __syncwarp();
    }
}

template <bool FILL>
__device__ void list_row(const ListArgs &a, int job, int i, unsigned *bm) {
    const int sid = a.job_sys[job], bead = a.job_bead[job];
    const SysDev &S = a.sys[sid];
    const int N = S.n_mols, W = (N + 31) >> 5;
    const int lane = threadIdx.x & 31;
    row_bitmap(a, S, bead, i, bm);
    if (!FILL) {
        int full = 0, half = 0;
        for (int k = lane; k < W; k += 32) {
            const unsigned v = bm[k];
            full += __popc(v);
            // bits j > i of word k
            const unsigned gt = (k > (i >> 5)) ? 0xffffffffu : (k < (i >> 5) ? 0u : ~((2u << (i & 31)) - 1u));
            half += __popc(v & gt);
        }
        for (int o = 16; o > 0; o >>= 1) {
            full += __shfl_xor_sync(0xffffffffu, full, o);
            half += __shfl_xor_sync(0xffffffffu, half, o);
        }
        if (lane == 0) {
            a.cnt_half[S.pt_off + (size_t)bead * N + i] = half;
            a.cnt_full[S.pt_off + (size_t)bead * N + i] = full;
        }
        return;
    }
    // entries in ascending j: each lane takes one word of 32 molecules, an exclusive
    // scan of the words' populations gives its first slot
    const int *point = a.point + S.pt_off + (size_t)bead * N;
    int *list = a.list + S.ls_off + (size_t)bead * S.list_size;
    int off_h = point[i];
    int off_f = 0, cap = 2 * S.list_size;
    const int *pf = nullptr;
    int *lf = nullptr;
    if (a.point_full) {
        pf = a.point_full + S.pf_off + (size_t)bead * (N + 1);
        lf = a.list_full + S.lf_off + (size_t)bead * cap;
        off_f = pf[i];
    }
    for (int k0 = 0; k0 < W; k0 += 32) {
        const int k = k0 + lane;
        const unsigned v = k < W ? bm[k] : 0u;
        const unsigned gt = (k > (i >> 5)) ? 0xffffffffu : (k < (i >> 5) ? 0u : ~((2u << (i & 31)) - 1u));
        const unsigned vh = v & gt;
        int ch = __popc(vh), cf = __popc(v);
        int sh = ch, sf = cf;
        for (int o = 1; o < 32; o <<= 1) {
            const int uh = __shfl_up_sync(0xffffffffu, sh, o), uf = __shfl_up_sync(0xffffffffu, sf, o);
            if (lane >= o) {
                sh += uh;
                sf += uf;
            }
        }
        int at_h = off_h + sh - ch, at_f = off_f + sf - cf;
        for (unsigned m = vh; m; m &= m - 1) {
            const int j = 32 * k + __ffs(m) - 1;
            if (at_h < S.list_size) list[at_h] = j;
            ++at_h;
        }
        if (lf)
            for (unsigned m = v; m; m &= m - 1) {
                const int j = 32 * k + __ffs(m) - 1;
                if (at_f < cap) lf[at_f] = j;
                ++at_f;
            }
        off_h += __shfl_sync(0xffffffffu, sh, 31);
        off_f += __shfl_sync(0xffffffffu, sf, 31);
    }
}

__global__ void __launch_bounds__(512) k_list_scan(ListArgs a) {
    if ((int)blockIdx.x >= *a.rb_count) return;
    const int job = a.rb_jobs[blockIdx.x];
    const int sid = a.job_sys[job], bead = a.job_bead[job];
    const SysDev &S = a.sys[sid];
    const int N = S.n_mols;
    extern __shared__ int cnt[];
    __shared__ int wtot[33];
    const int *ch = a.cnt_half + S.pt_off + (size_t)bead * N;
    for (int i = threadIdx.x; i < N; i += blockDim.x) cnt[i] = ch[i];
    __syncthreads();
    const int total = block_exclusive_scan(cnt, N, wtot);
    int *point = a.point + S.pt_off + (size_t)bead * N;
    for (int i = threadIdx.x; i < N; i += blockDim.x) point[i] = cnt[i];
    if (total > S.list_size && threadIdx.x == 0) atomicOr(a.status, (unsigned)ST_LIST_OVERFLOW);
    int *list = a.list + S.ls_off + (size_t)bead * S.list_size;
    for (int k = total + threadIdx.x; k < S.list_size; k += blockDim.x) list[k] = 0;
    if (a.point_full) {
        __syncthreads();
        const int *cf = a.cnt_full + S.pt_off + (size_t)bead * N;
        for (int i = threadIdx.x; i < N; i += blockDim.x) cnt[i] = cf[i];
        __syncthreads();
        const int tot2 = block_exclusive_scan(cnt, N, wtot);
        const int cap = 2 * S.list_size;
        int *pf = a.point_full + S.pf_off + (size_t)bead * (N + 1);
        for (int i = threadIdx.x; i < N; i += blockDim.x) pf[i] = min(cnt[i], cap);
        if (threadIdx.x == 0) pf[N] = min(tot2, cap);
    }
    if (threadIdx.x == 0) {
        if (a.acc) atomicAdd(&a.acc[sid].rebuilds, 1.0);
        if (a.run) atomicAdd(&a.run[sid].list_builds, 1.0);
        a.rebuilt[S.job_base + bead] = 1;
    }
}

}  // namespace

void init_list_kernel_attributes() {
    cudaFuncSetAttribute(k_skin_test, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
    cudaFuncSetAttribute(k_list_rows<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_list_rows<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_list_scan, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

void launch_skin_rebuild(const ListArgs &a, cudaStream_t s, unsigned long long *launches) {
    if (a.n_jobs <= 0) return;
    const int W = (a.max_mols + 31) / 32;
    cudaMemsetAsync(a.rb_count, 0, sizeof(int), s);
    k_skin_test<<<a.n_jobs, 256, (size_t)LC_MAX_CELLS * sizeof(int), s>>>(a);
    const int row_blocks = (a.max_mols + ROWS - 1) / ROWS;
    const long long items = (long long)row_blocks * a.n_jobs;
    // one block an SM, or one per 16 items of a rebuild of every bead when that is
    // more (at most eight an SM): in a step without a rebuild the blocks only read the count and exit,
    // and a wide grid holds the thread slots of the force kernels running beside
    // it (1216 blocks cost the 512-water P = 32 step ~7 us)
    const int grid = (int)std::min<long long>(items, std::max<long long>(152LL, std::min<long long>(items / 16, 152LL * 8)));
    const size_t bm = (size_t)ROWS * W * sizeof(unsigned);
    k_list_rows<false><<<grid, 32 * ROWS, bm, s>>>(a, row_blocks);
    k_list_scan<<<a.n_jobs, 512, (size_t)a.max_mols * sizeof(int), s>>>(a);
    k_list_rows<true><<<grid, 32 * ROWS, bm, s>>>(a, row_blocks);
    if (launches) *launches += 4;
}

}  // namespace qtg
