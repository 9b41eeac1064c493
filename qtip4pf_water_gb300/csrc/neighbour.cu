// Verlet-list skin test and rebuild (replaces neighbour.cpp:12-62 and the
// per-bead displacement test of update.cpp:354-385 / :95-123).
//
// One block per (system, bead). The list is the reference's CSR half list:
// for each oxygen i, the oxygens j > i (ascending) whose minimum-image
// distance satisfies r^2 < r_skin^2 strictly, with point[i] the row start.
// Pair tests run in FP32 on positions wrapped into the box; a pair whose FP32
// r^2 lies within a relative band of 1e-4 around r_skin^2 is re-tested with
// the reference's FP64 arithmetic (x - L*round(x/L), then x^2+y^2+z^2, each
// operation rounded separately), so the pair set is bit-identical to the
// reference's. The FP32 r^2 error is below 2e-6 relative for coordinates
// within a few box lengths of the origin, far inside the band.
#include "qtg_internal.h"

namespace qtg {

namespace {

constexpr float kBand = 1e-4f;

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

__device__ __forceinline__ bool pair_in(int i, int j, const float4 *pos, const double *qb,
                                        const SysDev &S, float rs2) {
    float4 a = pos[i], b = pos[j];
    float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    dx -= S.boxf[0] * rintf(dx * S.inv_boxf[0]);
    dy -= S.boxf[1] * rintf(dy * S.inv_boxf[1]);
    dz -= S.boxf[2] * rintf(dz * S.inv_boxf[2]);
    float r2 = dx * dx + dy * dy + dz * dz;
    if (fabsf(r2 - rs2) > kBand * rs2) return r2 < rs2;
    return pair_exact(qb + 9 * i, qb + 9 * j, S);
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

__global__ void __launch_bounds__(512) k_skin_rebuild(ListArgs a) {
    const int job = blockIdx.x;
    const int sid = a.job_sys[job], bead = a.job_bead[job];
    const SysDev S = a.sys[sid];
    const int N = S.n_mols;
    double *disp = a.disp + S.d_off + (size_t)bead * 3 * N;
    extern __shared__ unsigned char smem[];
    __shared__ unsigned long long red[2][33];
    __shared__ int wtot[33];
    __shared__ int do_build;

    if (!a.force_rebuild) {
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
        if (!do_build) return;
    }

    const double *qb = a.q + S.q_off + (size_t)bead * S.n_dof;
    float4 *pos = reinterpret_cast<float4 *>(smem);
    int *cnt = reinterpret_cast<int *>(pos + N);
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        float c[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            double x = qb[9 * i + d];
            double w = x - S.box[d] * floor(x * S.inv_box[d]);
            c[d] = (float)w;
        }
        pos[i] = make_float4(c[0], c[1], c[2], 0.f);
    }
    __syncthreads();
    const float rs2 = (float)S.r_skin_sq;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = w; i < N; i += nw) {
        int c = 0;
        for (int j0 = i + 1; j0 < N; j0 += 32) {
            int j = j0 + lane;
            bool in = (j < N) && pair_in(i, j, pos, qb, S, rs2);
            c += __popc(__ballot_sync(0xffffffffu, in));
        }
        if (lane == 0) cnt[i] = c;
    }
    __syncthreads();
    const int total = block_exclusive_scan(cnt, N, wtot);
    int *point = a.point + S.pt_off + (size_t)bead * N;
    int *list = a.list + S.ls_off + (size_t)bead * S.list_size;
    for (int i = threadIdx.x; i < N; i += blockDim.x) point[i] = cnt[i];
    if (total > S.list_size && threadIdx.x == 0) atomicOr(a.status, (unsigned)ST_LIST_OVERFLOW);
    const unsigned lt = (1u << lane) - 1u;
    for (int i = w; i < N; i += nw) {
        int off = cnt[i];
        for (int j0 = i + 1; j0 < N; j0 += 32) {
            int j = j0 + lane;
            bool in = (j < N) && pair_in(i, j, pos, qb, S, rs2);
            unsigned m = __ballot_sync(0xffffffffu, in);
            int at = off + __popc(m & lt);
            if (in && at < S.list_size) list[at] = j;
            off += __popc(m);
        }
    }
    for (int k = total + threadIdx.x; k < S.list_size; k += blockDim.x) list[k] = 0;
    if (a.point_full) {
        // the symmetric list: every j != i with the same pair test (which is exactly
        // antisymmetric under i <-> j), ascending j; capacity 2 list_size per bead
        __syncthreads();
        for (int i = w; i < N; i += nw) {
            int c = 0;
            for (int j0 = 0; j0 < N; j0 += 32) {
                const int j = j0 + lane;
                const bool in = (j < N) && (j != i) && pair_in(i, j, pos, qb, S, rs2);
                c += __popc(__ballot_sync(0xffffffffu, in));
            }
            if (lane == 0) cnt[i] = c;
        }
        __syncthreads();
        const int tot2 = block_exclusive_scan(cnt, N, wtot);
        const int cap = 2 * S.list_size;
        int *pf = a.point_full + S.pf_off + (size_t)bead * (N + 1);
        int *lf = a.list_full + S.lf_off + (size_t)bead * cap;
        for (int i = threadIdx.x; i < N; i += blockDim.x) pf[i] = min(cnt[i], cap);
        if (threadIdx.x == 0) pf[N] = min(tot2, cap);
        for (int i = w; i < N; i += nw) {
            int off = cnt[i];
            for (int j0 = 0; j0 < N; j0 += 32) {
                const int j = j0 + lane;
                const bool in = (j < N) && (j != i) && pair_in(i, j, pos, qb, S, rs2);
                const unsigned m = __ballot_sync(0xffffffffu, in);
                const int at = off + __popc(m & lt);
                if (in && at < cap) lf[at] = j;
                off += __popc(m);
            }
        }
    }
    for (int k = threadIdx.x; k < 3 * N; k += blockDim.x) disp[k] = 0.0;
    if (threadIdx.x == 0 && a.acc) atomicAdd(&a.acc[sid].rebuilds, 1.0);
    if (threadIdx.x == 0 && a.run) atomicAdd(&a.run[sid].list_builds, 1.0);
    if (threadIdx.x == 0) a.rebuilt[S.job_base + bead] = 1;
}

}  // namespace

void init_list_kernel_attributes() {
    cudaFuncSetAttribute(k_skin_rebuild, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

void launch_skin_rebuild(const ListArgs &a, cudaStream_t s, unsigned long long *launches) {
    if (a.n_jobs <= 0) return;
    size_t smem = (size_t)a.max_mols * (sizeof(float4) + sizeof(int));
    k_skin_rebuild<<<a.n_jobs, 512, smem, s>>>(a);
    if (launches) ++*launches;
}

}  // namespace qtg
