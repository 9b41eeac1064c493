// Learned centroid-force correction for centroid molecular dynamics.
//
// A per-molecule network maps local symmetry-function descriptors of the
// molecule's three atoms to the correction (mean constrained-PIMD centroid force
// minus the classical qTIP4P/F force) on those atoms, expressed in the
// molecule's own frame. This file holds its device side:
//
//   k_descriptors   Behler-Parrinello radial (G2) and angular (G5) symmetry
//                   functions within 6 A, 32 per atom, one warp per molecule
//   k_mlp_fwd       the network's forward pass on the tensor cores: BF16
//                   operands in shared memory, tcgen05.mma into FP32
//                   accumulators in tensor memory, bias + SiLU epilogues
//   k_mlp_train     forward and backward of one batch: the loss gradient, the
//                   weight and bias gradients (all on tcgen05), per-CTA partial
//                   sums reduced in a fixed order
//   k_adam          FP32 master weights, Adam, BF16 copies for the next pass
//   k_frames / k_apply_correction   molecular frames and the lab-frame force
//
// Nothing here has a counterpart in the reference; the reference's own CMD
// correction is a tabulated spline (forces.cpp:452-466), which this replaces.

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "qtg_internal.h"
#include "qtip4pf_gb300.h"

namespace qtg {
namespace {

// ---- symmetry-function descriptors ---------------------------------------------
// Behler & Parrinello, Phys. Rev. Lett. 98, 146401 (2007); Behler, J. Chem. Phys.
// 134, 074106 (2011), eq. 27 (the angular form without r_jk terms). Cutoff
// f_c(r) = (cos(pi r / R_c) + 1) / 2 for r < R_c.
//   G2_i = sum_{j != i, species s} exp(-eta r_ij^2) f_c(r_ij)
//   G5_i = 2^(1 - zeta) sum_{j < k, pair class c} (1 + lambda cos theta_jik)^zeta
//          exp(-eta (r_ij^2 + r_ik^2)) f_c(r_ij) f_c(r_ik)
// Layout of the 32 values of an atom:
//   0..7    G2, neighbours O, eta = G2_ETA[0..7]
//   8..15   G2, neighbours H
//   16..23  G5, neighbour pair of one species (OO or HH), the eight G5 sets below
//   24..31  G5, mixed neighbour pair (OH)
// G5 without r_jk separates over the neighbours: with w_j = exp(-eta r_ij^2)
// f_c(r_ij), u_j the unit vector to j and cos theta_jik = u_j . u_k, the
// moments W = sum w, V = sum w u, M = sum w u u^T and Q = sum w^2 of a species
// set give its pair sums
//   sum_{j<k} w_j w_k = (W^2 - Q) / 2,  sum w_j w_k cos = (|V|^2 - Q) / 2,
//   sum w_j w_k cos^2 = (|M|_F^2 - Q) / 2,
// and the mixed (O, H) pairs W_O W_H, V_O . V_H, <M_O, M_H>_F; (1 + lambda cos)^zeta
// for zeta = 1, 2 is a combination of those three. The cost is per neighbour,
// not per neighbour pair.
// Atoms are O, H1, H2 of each molecule in the reference's order; every atom
// within R_c counts, the atom's own molecule included.
constexpr int ND = QTG_DESC_PER_ATOM;
constexpr int NB_MAX = 256;  // neighbours within R_c kept per atom
__constant__ float G2_ETA[8] = {0.001f, 0.01f, 0.03f, 0.06f, 0.15f, 0.3f, 0.7f, 1.5f};  // 1/A^2
// G5 sets, in this order: (zeta, lambda) = (1, +1), (1, -1), (2, +1), (2, -1) with
// eta = 0.005 / A^2, then the same four with eta = 0.02 / A^2

constexpr float BOHR_A = 0.529177210903f;

__device__ __forceinline__ float fcut(float r, float rc) { return 0.5f * (cospif(r / rc) + 1.0f); }

struct DescArgs {
    const double *pos;  // [n_conf][9N] bohr
    int n_conf, n_mols;
    double box[3];      // bohr
    float4 *wrapped;    // scratch [n_conf][3N]: atoms wrapped into the box, A
    float *desc;        // [n_conf][3N][32]
    float rc_ang;       // cutoff, A
    unsigned *status;
};

// Atoms wrapped into [0, L) and converted to FP32 Angstrom once, so that the
// neighbour scan runs in FP32 (w = species: 0 = O, 1 = H).
__global__ void k_wrap_atoms(DescArgs a) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int na = 3 * a.n_mols;
    if (g >= (long long)a.n_conf * na) return;
    const double *r = a.pos + 3 * g;
    float v[3];
    for (int d = 0; d < 3; ++d) {
        const double L = a.box[d], t = r[d] / L;
        v[d] = (float)((t - floor(t)) * L) * BOHR_A;
    }
    a.wrapped[g] = make_float4(v[0], v[1], v[2], (g % na) % 3 ? 1.f : 0.f);
}

// One warp per molecule. The lanes first scan the molecules' oxygens and keep
// the molecules whose O lies within R_c + CAND_MARGIN of this molecule's O
// (an atom within R_c of one of this molecule's atoms belongs to such a
// molecule: every H lies within CAND_MARGIN / 2 of its O); then, for each of
// the three atoms in turn, the candidates' atoms within R_c are compacted into
// shared memory (ballot + prefix), G2 and the G5 moments are summed over them
// (each lane over its share of the neighbours, for all of them and for the H
// ones; the O sums are the difference), the sums are reduced over the warp and
// lane 0 forms the 32 values. The two G5 widths share one Gaussian
// (exp(-0.02 s) = exp(-0.005 s)^4).
constexpr int DW = 4;            // warps per block
constexpr int CAND_MAX = 256;    // candidate molecules kept per molecule
constexpr float CAND_MARGIN = 3.2f;  // A
__global__ void __launch_bounds__(32 * DW) k_descriptors(DescArgs a) {
    __shared__ int cand[DW][CAND_MAX];
    __shared__ float4 nb[DW][NB_MAX];   // (dx, dy, dz, r) in A, minimum image
    __shared__ float nfc[DW][NB_MAX];   // f_c(r)
    __shared__ unsigned char sp[DW][NB_MAX];
    __shared__ float red[DW][64];       // the warp's 64 totals of an atom
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int N = a.n_mols, na = 3 * N;
    const long long g = (long long)blockIdx.x * DW + warp;  // global molecule index over configurations
    if (g >= (long long)a.n_conf * N) return;
    const int conf = (int)(g / N), mol = (int)(g - (long long)conf * N);
    const float4 *w = a.wrapped + (size_t)conf * na;
    const float L[3] = {(float)a.box[0] * BOHR_A, (float)a.box[1] * BOHR_A, (float)a.box[2] * BOHR_A};
    const float IL[3] = {1.f / L[0], 1.f / L[1], 1.f / L[2]};
    const float rc = a.rc_ang, rc2 = rc * rc, irc = 1.f / rc;
    const float rcand = rc + CAND_MARGIN, rcand2 = rcand * rcand;
    auto disp = [&](const float4 &x, const float4 &y) {  // minimum-image y - x
        float3 d;
        d.x = y.x - x.x;
        d.y = y.y - x.y;
        d.z = y.z - x.z;
        d.x = fmaf(-L[0], rintf(d.x * IL[0]), d.x);
        d.y = fmaf(-L[1], rintf(d.y * IL[1]), d.y);
        d.z = fmaf(-L[2], rintf(d.z * IL[2]), d.z);
        return d;
    };
    // candidate molecules
    const float4 om = w[3 * mol];
    int nc = 0;
    for (int j0 = 0; j0 < N; j0 += 32) {
        const int j = j0 + lane;
        bool in = false;
        if (j < N) {
            const float3 d = disp(om, w[3 * j]);
            in = d.x * d.x + d.y * d.y + d.z * d.z < rcand2;
        }
        const unsigned m = __ballot_sync(0xffffffffu, in);
        const int at = nc + __popc(m & ((1u << lane) - 1u));
        if (in && at < CAND_MAX) cand[warp][at] = j;
        nc += __popc(m);
    }
    if (nc > CAND_MAX) {
        if (lane == 0) atomicOr(a.status, (unsigned)ST_DESC_OVERFLOW);
        nc = CAND_MAX;
    }
    __syncwarp();
    for (int atom = 0; atom < 3; ++atom) {
        const int i = 3 * mol + atom;
        const float4 xi = w[i];
        int n = 0;
        for (int c0 = 0; c0 < 3 * nc; c0 += 32) {
            const int c = c0 + lane;
            bool in = false;
            float4 d4 = make_float4(0.f, 0.f, 0.f, 0.f);
            float spj = 0.f;
            if (c < 3 * nc) {
                const int j = 3 * cand[warp][c / 3] + c % 3;
                if (j != i) {
                    const float4 xj = w[j];
                    const float3 d = disp(xi, xj);
                    const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
                    in = r2 < rc2;
                    d4 = make_float4(d.x, d.y, d.z, sqrtf(r2));
                    spj = xj.w;
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, in);
            const int at = n + __popc(m & ((1u << lane) - 1u));
            if (in && at < NB_MAX) {
                nb[warp][at] = d4;
                nfc[warp][at] = fcut(d4.w, rc);
                sp[warp][at] = (unsigned char)(spj > 0.5f);
            }
            n += __popc(m);
        }
        if (n > NB_MAX) {
            if (lane == 0) atomicOr(a.status, (unsigned)ST_DESC_OVERFLOW);
            n = NB_MAX;
        }
        __syncwarp();
        // per lane: G2 of all neighbours and of the H ones; the G5 moments
        // W, V (3), M (xx, yy, zz, xy, xz, yz), Q of the two widths, all and H
        constexpr int NM = 11;
        float g2a[8], g2h[8], mo[2][2][NM];
#pragma unroll
        for (int k = 0; k < 8; ++k) g2a[k] = g2h[k] = 0.f;
#pragma unroll
        for (int e = 0; e < 2; ++e)
#pragma unroll
            for (int t = 0; t < 2; ++t)
#pragma unroll
                for (int k = 0; k < NM; ++k) mo[e][t][k] = 0.f;
        for (int jj = lane; jj < n; jj += 32) {
            const float4 d = nb[warp][jj];
            const float r2 = d.w * d.w, fc = nfc[warp][jj];
            const float h = sp[warp][jj] ? 1.f : 0.f;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const float v = __expf(-G2_ETA[k] * r2) * fc;
                g2a[k] += v;
                g2h[k] = fmaf(h, v, g2h[k]);
            }
            const float ir = 1.f / d.w, ux = d.x * ir, uy = d.y * ir, uz = d.z * ir;
            const float e1 = __expf(-0.005f * r2), e2 = e1 * e1;
            const float wv[2] = {e1 * fc, e2 * e2 * fc};
#pragma unroll
            for (int e = 0; e < 2; ++e)
#pragma unroll
                for (int t = 0; t < 2; ++t) {
                    const float w = t ? h * wv[e] : wv[e];
                    const float wx = w * ux, wy = w * uy, wz = w * uz;
                    float *m = mo[e][t];
                    m[0] += w;
                    m[1] += wx;
                    m[2] += wy;
                    m[3] += wz;
                    m[4] = fmaf(wx, ux, m[4]);
                    m[5] = fmaf(wy, uy, m[5]);
                    m[6] = fmaf(wz, uz, m[6]);
                    m[7] = fmaf(wx, uy, m[7]);
                    m[8] = fmaf(wx, uz, m[8]);
                    m[9] = fmaf(wy, uz, m[9]);
                    m[10] = fmaf(w, wv[e], m[10]);
                }
        }
        // warp sums of the 60 values by a reduce-scatter: at the step of offset o
        // each lane keeps one half of its vector (the upper one if lane & o),
        // sends the other half to lane ^ o and adds what it receives; after the
        // five steps lane l holds the totals of values 2l and 2l + 1
        float v[64];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            v[k] = g2a[k];
            v[8 + k] = g2h[k];
        }
#pragma unroll
        for (int e = 0; e < 2; ++e)
#pragma unroll
            for (int t = 0; t < 2; ++t)
#pragma unroll
                for (int k = 0; k < NM; ++k) v[16 + NM * (2 * e + t) + k] = mo[e][t][k];
#pragma unroll
        for (int k = 16 + 4 * NM; k < 64; ++k) v[k] = 0.f;
#pragma unroll
        for (int o = 16, len = 64; o > 0; o >>= 1, len >>= 1) {
            const bool up = lane & o;
#pragma unroll
            for (int k = 0; k < len / 2; ++k) {
                const float send = up ? v[k] : v[k + len / 2];
                const float keep = up ? v[k + len / 2] : v[k];
                v[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
            }
        }
        red[warp][2 * lane] = v[0];
        red[warp][2 * lane + 1] = v[1];
        __syncwarp();
        if (lane == 0) {
            const float *tot = red[warp];
            float *out = a.desc + ((size_t)conf * na + i) * ND;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                out[k] = tot[k] - tot[8 + k];
                out[8 + k] = tot[8 + k];
            }
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                float so[NM];  // the O moments: all minus H
                const float *sa = tot + 16 + NM * (2 * e), *sh = tot + 16 + NM * (2 * e + 1);
#pragma unroll
                for (int k = 0; k < NM; ++k) so[k] = sa[k] - sh[k];
                // same-species pair sums (OO + HH) and mixed ones (OH) of 1, cos, cos^2
                auto frob = [](const float *x, const float *y) {
                    return x[4] * y[4] + x[5] * y[5] + x[6] * y[6] + 2.f * (x[7] * y[7] + x[8] * y[8] + x[9] * y[9]);
                };
                auto dot3 = [](const float *x, const float *y) { return x[1] * y[1] + x[2] * y[2] + x[3] * y[3]; };
                const float p0 = 0.5f * ((so[0] * so[0] - so[10]) + (sh[0] * sh[0] - sh[10]));
                const float p1 = 0.5f * ((dot3(so, so) - so[10]) + (dot3(sh, sh) - sh[10]));
                const float p2 = 0.5f * ((frob(so, so) - so[10]) + (frob(sh, sh) - sh[10]));
                const float x0 = so[0] * sh[0], x1 = dot3(so, sh), x2 = frob(so, sh);
                // (zeta, lambda) = (1, +1), (1, -1), (2, +1), (2, -1):
                // 1 + c, 1 - c, (1 + 2c + c^2) / 2, (1 - 2c + c^2) / 2
                float *g = out + 16 + 4 * e;
                g[0] = p0 + p1;
                g[1] = p0 - p1;
                g[2] = 0.5f * (p0 + 2.f * p1 + p2);
                g[3] = 0.5f * (p0 - 2.f * p1 + p2);
                g[8] = x0 + x1;
                g[9] = x0 - x1;
                g[10] = 0.5f * (x0 + 2.f * x1 + x2);
                g[11] = 0.5f * (x0 - 2.f * x1 + x2);
            }
        }
        __syncwarp();
    }
}

}  // namespace
}  // namespace qtg

namespace qtg {
namespace {

// ---- tensor-core building blocks (tcgen05, sm_100 family) ----------------------
// Operand tiles live in shared memory in the no-swizzle K-major layout: the tile
// is cut into core matrices of 8 rows x 16 bytes (8 BF16 values along K), each
// stored as 128 contiguous bytes; the core matrices of a row group follow one
// another along K (leading-dimension offset 128 B) and the row groups follow
// one another (stride offset K * 16 B).
__device__ __forceinline__ uint32_t kmaj_off(int r, int k, int K) {
    return (uint32_t)((r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
// shared-memory matrix descriptor: start, leading and stride byte offsets (>> 4),
// descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// instruction descriptor of kind::f16: BF16 A and B (K-major), FP32 D, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar));
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count));
}
// bounded wait for the mbarrier phase; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (int it = 0; it < (1 << 20); ++it) {
        uint32_t ok;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}
__device__ __forceinline__ void tmem_alloc(uint32_t slot_saddr, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot_saddr), "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}
// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
}
__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }

// ---- the network ------------------------------------------------------------------
constexpr int TM = 128;                    // molecules per tile (MMA M)
constexpr int DIN = QTG_MLP_IN, DH = QTG_MLP_HIDDEN, DOUT = QTG_MLP_OUT_PAD;
constexpr uint32_t IDESC_H = idesc_bf16(TM, DH), IDESC_O = idesc_bf16(TM, DOUT);
constexpr uint32_t FWD_COLS = 256;        // TMEM columns: layer 1 at 0, layer 2 at 64, layer 3 at 128

struct MlpArgs {
    const __nv_bfloat16 *w1, *w2, *w3;  // [DH][DIN], [DH][DH], [DOUT][DH], row-major (out x in)
    const float *b1, *b2, *b3;
    const __nv_bfloat16 *x;  // [m][DIN]
    int m;
    float *y;                // [m][DOUT]
    unsigned *status;
};

// shared-memory plan of the forward kernel (byte offsets from a 1024-aligned base)
constexpr uint32_t F_W1 = 0, F_W2 = F_W1 + DH * DIN * 2, F_W3 = F_W2 + DH * DH * 2, F_X = F_W3 + DOUT * DH * 2,
                   F_H1 = F_X + TM * DIN * 2, F_H2 = F_H1 + TM * DH * 2, F_B = F_H2 + TM * DH * 2,
                   F_MISC = F_B + (2 * DH + DOUT) * 4, F_END = F_MISC + 64;

// copy a row-major BF16 matrix [rows][K] into a K-major operand tile (16-byte chunks)
__device__ __forceinline__ void load_tile(uint8_t *tile, const __nv_bfloat16 *src, int rows, int K, int row0,
                                          int max_rows) {
    const int chunks = rows * (K / 8);
    for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
        const int r = c / (K / 8), kg = c - r * (K / 8);
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (row0 + r < max_rows) v = *reinterpret_cast<const uint4 *>(src + (size_t)(row0 + r) * K + kg * 8);
        *reinterpret_cast<uint4 *>(tile + kmaj_off(r, kg * 8, K)) = v;
    }
}

// bias + SiLU on this thread's row of a 64-column accumulator, into a BF16 A tile;
// z keeps the pre-activations
__device__ __forceinline__ void epilogue_silu(uint32_t tmem_row, const float *bias, uint8_t *tile, int r,
                                              float *z) {
#pragma unroll
    for (int c = 0; c < DH; c += 16) tmem_ld16(tmem_row + c, z + c);
#pragma unroll
    for (int kg = 0; kg < DH / 8; ++kg) {
        float h[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            z[kg * 8 + t] += bias[kg * 8 + t];
            h[t] = silu(z[kg * 8 + t]);
        }
        *reinterpret_cast<uint4 *>(tile + kmaj_off(r, kg * 8, DH)) =
            make_uint4(pack_bf16(h[0], h[1]), pack_bf16(h[2], h[3]), pack_bf16(h[4], h[5]), pack_bf16(h[6], h[7]));
    }
}

// layer GEMM: D[128 x N] = A[128 x K] B^T, both K-major tiles; issued by one thread
__device__ __forceinline__ void gemm(uint32_t d_tmem, const uint8_t *a, const uint8_t *b, int K, uint32_t idesc) {
    const uint32_t sa = smem_u32(a), sb = smem_u32(b), sbo = (uint32_t)K * 16;
    for (int kk = 0; kk < K / 16; ++kk)
        mma_bf16(d_tmem, sdesc(sa + kk * 256, 128, sbo), sdesc(sb + kk * 256, 128, sbo), idesc, kk > 0 ? 1u : 0u);
}

// One CTA of 128 threads per tile of 128 molecules (persistent over tiles);
// thread r owns row r of the tile, which is TMEM lane r.
__global__ void __launch_bounds__(TM) k_mlp_fwd(MlpArgs a) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *sm = reinterpret_cast<uint8_t *>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    float *b1 = reinterpret_cast<float *>(sm + F_B), *b2 = b1 + DH, *b3 = b2 + DH;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + F_MISC);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + F_MISC + 8);
    const int tid = threadIdx.x, warp = tid >> 5;
    load_tile(sm + F_W1, a.w1, DH, DIN, 0, DH);
    load_tile(sm + F_W2, a.w2, DH, DH, 0, DH);
    load_tile(sm + F_W3, a.w3, DOUT, DH, 0, DOUT);
    for (int k = tid; k < DH; k += TM) {
        b1[k] = a.b1[k];
        b2[k] = a.b2[k];
    }
    if (tid < DOUT) b3[tid] = a.b3[tid];
    if (tid == 0) mbar_init(smem_u32(mbar), 1);
    if (warp == 0) tmem_alloc(smem_u32(tslot), FWD_COLS);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot, lane_base = (uint32_t)(warp * 32) << 16;
    uint32_t phase = 0;
    bool ok = true;
    const int n_tiles = (a.m + TM - 1) / TM;
    for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x) {
        const int m0 = t * TM;
        load_tile(sm + F_X, a.x, TM, DIN, m0, a.m);
        float z[DH];
        const uint8_t *ain[3] = {sm + F_X, sm + F_H1, sm + F_H2};
        const uint8_t *bw[3] = {sm + F_W1, sm + F_W2, sm + F_W3};
        const int kin[3] = {DIN, DH, DH};
        const uint32_t dcol[3] = {0u, 64u, 128u};
        for (int layer = 0; layer < 3 && ok; ++layer) {
            fence_async_smem();
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
            if (tid == 0) {
                gemm(tmem + dcol[layer], ain[layer], bw[layer], kin[layer], layer < 2 ? IDESC_H : IDESC_O);
                mma_commit(smem_u32(mbar));
            }
            ok = mbar_wait(smem_u32(mbar), phase);
            phase ^= 1u;
            ok = __syncthreads_and(ok);
            if (!ok) break;
            tc_fence_after();
            const uint32_t row = tmem + lane_base + dcol[layer];
            if (layer == 0) epilogue_silu(row, b1, sm + F_H1, tid, z);
            else if (layer == 1) epilogue_silu(row, b2, sm + F_H2, tid, z);
            else {
                float o[DOUT];
                tmem_ld16(row, o);
                if (m0 + tid < a.m) {
                    float4 *dst = reinterpret_cast<float4 *>(a.y + (size_t)(m0 + tid) * DOUT);
#pragma unroll
                    for (int c = 0; c < DOUT; c += 4)
                        dst[c / 4] = make_float4(o[c] + b3[c], o[c + 1] + b3[c + 1], o[c + 2] + b3[c + 2],
                                                 o[c + 3] + b3[c + 3]);
                }
            }
        }
    }
    if (!ok) {
        if (tid == 0) atomicOr(a.status, (unsigned)ST_MMA_TIMEOUT);
        mbar_wait(smem_u32(mbar), phase ^ 1u);  // bounded: let an MMA still in flight finish
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, FWD_COLS);
}

}  // namespace
}  // namespace qtg

namespace qtg {
namespace {

// ---- training: forward + backward of one batch on the tensor cores ---------------
// Flat parameter vector (FP32 masters, gradients, Adam moments):
//   w1 [64][96] | w2 [64][64] | w3 [16][64] | b1 [64] | b2 [64] | b3 [16]
constexpr int P_W1 = 0, P_W2 = P_W1 + DH * DIN, P_W3 = P_W2 + DH * DH, P_B1 = P_W3 + DOUT * DH, P_B2 = P_B1 + DH,
              P_B3 = P_B2 + DH, NPAR = P_B3 + DOUT;
constexpr int NPART = NPAR + 1;  // per-CTA partial: gradients, then the loss sum
static_assert(NPAR == QTG_MLP_NPARAMS, "parameter count");

// Weight gradients are formed as G^T = A^T dZ with A^T (features x molecules) the
// A operand and dZ^T (outputs x molecules) the B operand, both K-major along the
// molecules of the tile (K = 128). The A^T tiles carry one more row of ones
// after the features, so the accumulator lane after the last feature holds the
// bias gradient. Lanes past that read whatever follows in shared memory and are
// never used.
constexpr uint32_t IDESC_GT_H = idesc_bf16(TM, DH), IDESC_GT_O = idesc_bf16(TM, DOUT);
constexpr uint32_t TRAIN_COLS = 512;
constexpr uint32_t C_Z1 = 0, C_Z2 = 64, C_Y = 128, C_DH2 = 160, C_DH1 = 224, C_GW1 = 288, C_GW2 = 352, C_GW3 = 416;

// shared-memory plan (byte offsets from a 1024-aligned base); the three A^T tiles
// come first so that their unused tail rows stay inside the allocation
constexpr int RG = TM * 16;  // bytes per 8-row group of a K = 128 tile
constexpr uint32_t T_XT = 0, T_H1T = T_XT + 13 * RG, T_H2T = T_H1T + 9 * RG, T_W1 = T_H2T + 9 * RG,
                   T_W2 = T_W1 + DH * DIN * 2, T_W3 = T_W2 + DH * DH * 2, T_W3T = T_W3 + DOUT * DH * 2,
                   T_W2T = T_W3T + DH * DOUT * 2, T_X = T_W2T + DH * DH * 2, T_H1 = T_X + TM * DIN * 2,
                   T_H2 = T_H1 + TM * DH * 2, T_DZ3 = T_H2 + TM * DH * 2, T_DZ2 = T_DZ3 + TM * DOUT * 2,
                   T_DZ3T = T_DZ2 + TM * DH * 2, T_DZ2T = T_DZ3T + DOUT * TM * 2, T_DZ1T = T_DZ2T + DH * TM * 2,
                   T_B = T_DZ1T + DH * TM * 2, T_MISC = T_B + (2 * DH + DOUT) * 4, T_END = T_MISC + 64;
static_assert(T_H2T + 16 * RG <= T_END, "A^T tails must stay inside the allocation");

struct TrainArgs {
    const __nv_bfloat16 *w1, *w2, *w3;
    const float *b1, *b2, *b3;
    const __nv_bfloat16 *x;  // [m][DIN]
    const float *t;          // targets [m][DOUT] (the first QTG_MLP_OUT count)
    int m;
    float grad_scale;        // dL/dy = grad_scale (y - t): 2 / (rows of the whole batch x outputs)
    float *partial;          // [gridDim.x][NPART]
    unsigned *status;
};

__device__ __forceinline__ void st_bf16(uint8_t *tile, uint32_t off, float v) {
    *reinterpret_cast<__nv_bfloat16 *>(tile + off) = __float2bfloat16_rn(v);
}
__device__ __forceinline__ float dsilu(float z) {
    const float s = 1.0f / (1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}
// copy the transposed (k, n) view of a row-major [rows][cols] BF16 matrix into a
// K-major B tile: element (n, k) = src[k][n]
__device__ __forceinline__ void load_tile_t(uint8_t *tile, const __nv_bfloat16 *src, int rows, int cols, int K) {
    for (int e = threadIdx.x; e < rows * cols; e += blockDim.x) {
        const int k = e / cols, n = e - k * cols;
        *reinterpret_cast<__nv_bfloat16 *>(tile + kmaj_off(n, k, K)) = src[e];
    }
}

__global__ void __launch_bounds__(TM, 1) k_mlp_train(TrainArgs a) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *sm = reinterpret_cast<uint8_t *>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    float *b1 = reinterpret_cast<float *>(sm + T_B), *b2 = b1 + DH, *b3 = b2 + DH;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + T_MISC);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + T_MISC + 8);
    float *red = reinterpret_cast<float *>(sm + T_MISC + 16);  // 4 warp sums
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    load_tile(sm + T_W1, a.w1, DH, DIN, 0, DH);
    load_tile(sm + T_W2, a.w2, DH, DH, 0, DH);
    load_tile(sm + T_W3, a.w3, DOUT, DH, 0, DOUT);
    // dH2 = dZ3 W3: B element (i, o) = W3[o][i] (K = 16 outputs); dH1 = dZ2 W2: B element (i, o) = W2[o][i]
    load_tile_t(sm + T_W3T, a.w3, DOUT, DH, DOUT);
    load_tile_t(sm + T_W2T, a.w2, DH, DH, DH);
    for (int k = tid; k < DH; k += TM) {
        b1[k] = a.b1[k];
        b2[k] = a.b2[k];
    }
    if (tid < DOUT) b3[tid] = a.b3[tid];
    // rows of ones after the features of the A^T tiles (bias gradients)
    st_bf16(sm + T_XT, kmaj_off(DIN, tid, TM), 1.0f);
    st_bf16(sm + T_H1T, kmaj_off(DH, tid, TM), 1.0f);
    st_bf16(sm + T_H2T, kmaj_off(DH, tid, TM), 1.0f);
    if (tid == 0) mbar_init(smem_u32(mbar), 1);
    if (warp == 0) tmem_alloc(smem_u32(tslot), TRAIN_COLS);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot, lrow = tmem + ((uint32_t)(warp * 32) << 16);
    uint32_t phase = 0;
    bool ok = true;
    float loss = 0.f;
    int my_tiles = 0;
    const int n_tiles = (a.m + TM - 1) / TM;
    // one synchronised MMA stage: operands visible to the tensor cores, issue, wait
    auto stage = [&](auto issue) {
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            issue();
            mma_commit(smem_u32(mbar));
        }
        bool w = mbar_wait(smem_u32(mbar), phase);
        phase ^= 1u;
        ok = __syncthreads_and(w);
        tc_fence_after();
    };
    for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x, ++my_tiles) {
        const int m0 = t * TM, r = tid;
        const bool valid = m0 + r < a.m;
        const uint32_t gacc = my_tiles > 0 ? 1u : 0u;
        // inputs: K-major X and transposed X^T
        load_tile(sm + T_X, a.x, TM, DIN, m0, a.m);
        for (int kg = 0; kg < DIN / 8; ++kg) {
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (valid) v = *reinterpret_cast<const uint4 *>(a.x + (size_t)(m0 + r) * DIN + kg * 8);
            const __nv_bfloat16 *h = reinterpret_cast<const __nv_bfloat16 *>(&v);
#pragma unroll
            for (int e = 0; e < 8; ++e)
                *reinterpret_cast<__nv_bfloat16 *>(sm + T_XT + kmaj_off(kg * 8 + e, r, TM)) = h[e];
        }
        // layer 1
        stage([&] { gemm(tmem + C_Z1, sm + T_X, sm + T_W1, DIN, IDESC_H); });
        if (!ok) break;
        for (int c = 0; c < DH; c += 16) {
            float z[16];
            tmem_ld16(lrow + C_Z1 + c, z);
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                const float h = silu(z[e] + b1[c + e]);
                st_bf16(sm + T_H1, kmaj_off(r, c + e, DH), h);
                st_bf16(sm + T_H1T, kmaj_off(c + e, r, TM), h);
            }
        }
        // layer 2
        stage([&] { gemm(tmem + C_Z2, sm + T_H1, sm + T_W2, DH, IDESC_H); });
        if (!ok) break;
        for (int c = 0; c < DH; c += 16) {
            float z[16];
            tmem_ld16(lrow + C_Z2 + c, z);
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                const float h = silu(z[e] + b2[c + e]);
                st_bf16(sm + T_H2, kmaj_off(r, c + e, DH), h);
                st_bf16(sm + T_H2T, kmaj_off(c + e, r, TM), h);
            }
        }
        // layer 3 and the loss gradient dZ3 = grad_scale (y - t) on the valid outputs
        stage([&] { gemm(tmem + C_Y, sm + T_H2, sm + T_W3, DH, IDESC_O); });
        if (!ok) break;
        {
            float y[16];
            tmem_ld16(lrow + C_Y, y);
#pragma unroll
            for (int o = 0; o < DOUT; ++o) {
                float d = 0.f;
                if (valid && o < QTG_MLP_OUT) {
                    d = y[o] + b3[o] - a.t[(size_t)(m0 + r) * DOUT + o];
                    loss += d * d;
                }
                const float g = a.grad_scale * d;
                st_bf16(sm + T_DZ3, kmaj_off(r, o, DOUT), g);
                st_bf16(sm + T_DZ3T, kmaj_off(o, r, TM), g);
            }
        }
        // dH2 = dZ3 W3 and dW3^T += H2^T dZ3
        stage([&] {
            gemm(tmem + C_DH2, sm + T_DZ3, sm + T_W3T, DOUT, IDESC_H);
            const uint32_t sa = smem_u32(sm + T_H2T), sb = smem_u32(sm + T_DZ3T);
            for (int kk = 0; kk < TM / 16; ++kk)
                mma_bf16(tmem + C_GW3, sdesc(sa + kk * 256, 128, TM * 16), sdesc(sb + kk * 256, 128, TM * 16),
                         IDESC_GT_O, (gacc || kk > 0) ? 1u : 0u);
        });
        if (!ok) break;
        for (int c = 0; c < DH; c += 16) {
            float dh[16], z[16];
            tmem_ld16(lrow + C_DH2 + c, dh);
            tmem_ld16(lrow + C_Z2 + c, z);
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                const float g = valid ? dh[e] * dsilu(z[e] + b2[c + e]) : 0.f;
                st_bf16(sm + T_DZ2, kmaj_off(r, c + e, DH), g);
                st_bf16(sm + T_DZ2T, kmaj_off(c + e, r, TM), g);
            }
        }
        // dH1 = dZ2 W2 and dW2^T += H1^T dZ2
        stage([&] {
            gemm(tmem + C_DH1, sm + T_DZ2, sm + T_W2T, DH, IDESC_H);
            const uint32_t sa = smem_u32(sm + T_H1T), sb = smem_u32(sm + T_DZ2T);
            for (int kk = 0; kk < TM / 16; ++kk)
                mma_bf16(tmem + C_GW2, sdesc(sa + kk * 256, 128, TM * 16), sdesc(sb + kk * 256, 128, TM * 16),
                         IDESC_GT_H, (gacc || kk > 0) ? 1u : 0u);
        });
        if (!ok) break;
        for (int c = 0; c < DH; c += 16) {
            float dh[16], z[16];
            tmem_ld16(lrow + C_DH1 + c, dh);
            tmem_ld16(lrow + C_Z1 + c, z);
#pragma unroll
            for (int e = 0; e < 16; ++e)
                st_bf16(sm + T_DZ1T, kmaj_off(c + e, r, TM), valid ? dh[e] * dsilu(z[e] + b1[c + e]) : 0.f);
        }
        // dW1^T += X^T dZ1
        stage([&] {
            const uint32_t sa = smem_u32(sm + T_XT), sb = smem_u32(sm + T_DZ1T);
            for (int kk = 0; kk < TM / 16; ++kk)
                mma_bf16(tmem + C_GW1, sdesc(sa + kk * 256, 128, TM * 16), sdesc(sb + kk * 256, 128, TM * 16),
                         IDESC_GT_H, (gacc || kk > 0) ? 1u : 0u);
        });
    }
    // per-CTA partial: weight and bias gradients from the accumulators, the loss sum
    float *part = a.partial + (size_t)blockIdx.x * NPART;
    if (ok) {
        const int i = tid;  // accumulator lane = input feature (or the bias row)
        for (int c = 0; c < DH; c += 16) {
            float g[16];
            if (my_tiles > 0) tmem_ld16(lrow + C_GW1 + c, g);
            else
                for (int e = 0; e < 16; ++e) g[e] = 0.f;
            for (int e = 0; e < 16; ++e) {
                if (i < DIN) part[P_W1 + (c + e) * DIN + i] = g[e];
                else if (i == DIN) part[P_B1 + c + e] = g[e];
            }
            if (my_tiles > 0) tmem_ld16(lrow + C_GW2 + c, g);
            for (int e = 0; e < 16; ++e) {
                if (i < DH) part[P_W2 + (c + e) * DH + i] = g[e];
                else if (i == DH) part[P_B2 + c + e] = g[e];
            }
        }
        float g[16];
        if (my_tiles > 0) tmem_ld16(lrow + C_GW3, g);
        else
            for (int e = 0; e < 16; ++e) g[e] = 0.f;
        for (int o = 0; o < DOUT; ++o) {
            const float v = o < QTG_MLP_OUT ? g[o] : 0.f;
            if (i < DH) part[P_W3 + o * DH + i] = v;
            else if (i == DH) part[P_B3 + o] = v;
        }
        for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
        if (lane == 0) red[warp] = loss;
        __syncthreads();
        if (tid == 0) part[NPAR] = red[0] + red[1] + red[2] + red[3];
    } else {
        if (tid == 0) atomicOr(a.status, (unsigned)ST_MMA_TIMEOUT);
        mbar_wait(smem_u32(mbar), phase ^ 1u);  // bounded: let an MMA still in flight finish
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, TRAIN_COLS);
}

// Sum of the per-CTA partials in CTA order (deterministic).
__global__ void k_reduce_partials(const float *partial, int n_cta, float *out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= NPART) return;
    float s = 0.f;
    for (int c = 0; c < n_cta; ++c) s += partial[(size_t)c * NPART + e];
    out[e] = s;
}

// Adam (Kingma & Ba, 2015) on the FP32 master parameters, then the BF16 copies
// of the weights the tensor-core kernels read.
__global__ void k_adam(float *w, float *m1, float *m2, const float *g, int n, float lr, float beta1, float beta2,
                       float eps, float bc1, float bc2, __nv_bfloat16 *wbf, int n_bf) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const float ge = g[e];
    const float a = beta1 * m1[e] + (1.f - beta1) * ge, b = beta2 * m2[e] + (1.f - beta2) * ge * ge;
    m1[e] = a;
    m2[e] = b;
    const float v = w[e] - lr * (a / bc1) / (sqrtf(b / bc2) + eps);
    w[e] = v;
    if (e < n_bf) wbf[e] = __float2bfloat16_rn(v);
}

}  // namespace
}  // namespace qtg

namespace qtg {
namespace {

// ---- deployment: the correction inside a force evaluation ------------------------
// Molecular frame of a water with its H atoms labelled (a, b): e1 along the
// bisector d_a + d_b, e2 along d_a - d_b made orthogonal to e1, e3 = e1 x e2,
// with d = r_H - r_O (minimum image). Swapping the labels maps (e1, e2, e3) to
// (e1, -e2, -e3). frames: float[N][9] = e1, e2, e3 of labelling (H1, H2).
__global__ void k_frames(const double *pos, int n_mols, double bx, double by, double bz, float *frames) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n_mols) return;
    const double *r = pos + 9 * m;
    const double L[3] = {bx, by, bz};
    double d1[3], d2[3];
    for (int k = 0; k < 3; ++k) {
        d1[k] = r[3 + k] - r[k];
        d2[k] = r[6 + k] - r[k];
        d1[k] -= L[k] * rint(d1[k] / L[k]);
        d2[k] -= L[k] * rint(d2[k] / L[k]);
    }
    float e1[3], e2[3], e3[3];
    float n1 = 0.f, n2 = 0.f, pj = 0.f;
    for (int k = 0; k < 3; ++k) {
        e1[k] = (float)(d1[k] + d2[k]);
        n1 += e1[k] * e1[k];
    }
    n1 = rsqrtf(n1);
    for (int k = 0; k < 3; ++k) {
        e1[k] *= n1;
        e2[k] = (float)(d1[k] - d2[k]);
        pj += e2[k] * e1[k];
    }
    for (int k = 0; k < 3; ++k) {
        e2[k] -= pj * e1[k];
        n2 += e2[k] * e2[k];
    }
    n2 = rsqrtf(n2);
    for (int k = 0; k < 3; ++k) e2[k] *= n2;
    e3[0] = e1[1] * e2[2] - e1[2] * e2[1];
    e3[1] = e1[2] * e2[0] - e1[0] * e2[2];
    e3[2] = e1[0] * e2[1] - e1[1] * e2[0];
    float *f = frames + 9 * m;
    for (int k = 0; k < 3; ++k) {
        f[k] = e1[k];
        f[3 + k] = e2[k];
        f[6 + k] = e3[k];
    }
}

// Network inputs of every molecule in both labellings: rows m (O, H1, H2) and
// N + m (O, H2, H1), each value normalised as (g - mean) * inv_std, in BF16.
__global__ void k_mol_features(const float *desc, int n_mols, const float *norm, __nv_bfloat16 *feat) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 2LL * n_mols * DIN) return;
    const int row = (int)(e / DIN), c = (int)(e - (long long)row * DIN);
    const int m = row % n_mols, swap = row >= n_mols;
    int atom = c / ND;  // 0 = O, 1 = first H, 2 = second H of this labelling
    if (swap && atom > 0) atom = 3 - atom;
    const float g = desc[((size_t)3 * m + atom) * ND + (c % ND)];
    feat[e] = __float2bfloat16_rn((g - norm[c]) * norm[DIN + c]);
}

// Lab-frame correction, symmetrised over the two labellings, added to the
// forces: for atom a of the molecule, F_a += s * (R_ab y_ab[a] + R_ba y_ba[a']) / 2
// with R the frame matrices and y scaled by the output scale s.
__global__ void k_apply_correction(const float *frames, const float *y, int n_mols, float out_scale, double *f) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n_mols) return;
    const float *e = frames + 9 * m;
    const float *ya = y + (size_t)m * DOUT, *yb = y + (size_t)(n_mols + m) * DOUT;
    for (int a = 0; a < 3; ++a) {
        const int ab = (a == 0) ? 0 : (3 - a);  // the same atom's slot in the swapped labelling
        const float c1 = ya[3 * a], c2 = ya[3 * a + 1], c3 = ya[3 * a + 2];
        const float s1 = yb[3 * ab], s2 = yb[3 * ab + 1], s3 = yb[3 * ab + 2];
        for (int k = 0; k < 3; ++k) {
            const float v = 0.5f * ((c1 + s1) * e[k] + (c2 - s2) * e[3 + k] + (c3 - s3) * e[6 + k]);
            f[9 * m + 3 * a + k] += (double)(out_scale * v);
        }
    }
}

}  // namespace

void launch_surrogate_prepare(const SurrogateRun &r, cudaStream_t s, unsigned long long *launches) {
    const int N = r.n_mols;
    DescArgs d;
    d.pos = r.pos;
    d.n_conf = 1;
    d.n_mols = N;
    for (int k = 0; k < 3; ++k) d.box[k] = r.box[k];
    d.desc = r.desc;
    d.wrapped = r.wrapped;
    d.rc_ang = 6.0f;
    d.status = r.status;
    k_wrap_atoms<<<(3 * N + 255) / 256, 256, 0, s>>>(d);
    k_descriptors<<<(N + DW - 1) / DW, 32 * DW, 0, s>>>(d);
    const long long nf = 2LL * N * DIN;
    k_mol_features<<<(unsigned)((nf + 255) / 256), 256, 0, s>>>(r.desc, N, r.norm, r.feat);
    MlpArgs a;
    a.w1 = r.wbf;
    a.w2 = r.wbf + DH * DIN;
    a.w3 = r.wbf + DH * DIN + DH * DH;
    a.b1 = r.bias;
    a.b2 = r.bias + DH;
    a.b3 = r.bias + 2 * DH;
    a.x = r.feat;
    a.m = 2 * N;
    a.y = r.y;
    a.status = r.status;
    const int tiles = (2 * N + TM - 1) / TM;
    k_mlp_fwd<<<tiles < 2 * r.n_sm ? tiles : 2 * r.n_sm, TM, (size_t)F_END + 1024, s>>>(a);
    k_frames<<<(N + 127) / 128, 128, 0, s>>>(r.pos, N, r.box[0], r.box[1], r.box[2], r.frames);
    if (launches) *launches += 5;
}

void launch_surrogate_apply(const SurrogateRun &r, cudaStream_t s, unsigned long long *launches) {
    k_apply_correction<<<(r.n_mols + 127) / 128, 128, 0, s>>>(r.frames, r.y, r.n_mols, r.out_scale, r.f);
    if (launches) *launches += 1;
}

void init_surrogate_kernel_attributes() {
    cudaFuncSetAttribute(k_mlp_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(F_END + 1024));
}

}  // namespace qtg

// ---- C ABI -----------------------------------------------------------------------
namespace {
__device__ unsigned g_surrogate_status;  // error bits of the surrogate kernels (bounded waits, overflows)

unsigned *status_word() {
    static void *addr[64] = {nullptr};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    if (!addr[dev] && cudaGetSymbolAddress(&addr[dev], g_surrogate_status) != cudaSuccess) addr[dev] = nullptr;
    return static_cast<unsigned *>(addr[dev]);
}

size_t fwd_smem() { return (size_t)qtg::F_END + 1024; }
size_t train_smem() { return (size_t)qtg::T_END + 1024; }

int grid_for(int tiles, int per_sm) {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return tiles < per_sm * sms ? tiles : per_sm * sms;
}
}  // namespace

extern "C" {

qtg_status qtg_sym_descriptors(const double *pos, int n_conf, int n_mols, const double *box_bohr, float *desc,
                               void *stream) {
    if (!pos || !desc || !box_bohr || n_conf < 0 || n_mols <= 0) return QTG_ERR_ARG;
    const double rc_bohr = 6.0 / 0.529177210903;
    for (int d = 0; d < 3; ++d)
        if (!(box_bohr[d] > 2.0 * rc_bohr)) return QTG_ERR_ARG;  // minimum image needs L > 2 R_c
    if (n_conf == 0) return QTG_OK;
    unsigned *st = status_word();
    if (!st) return QTG_ERR_CUDA;
    qtg::DescArgs a;
    a.pos = pos;
    a.n_conf = n_conf;
    a.n_mols = n_mols;
    for (int d = 0; d < 3; ++d) a.box[d] = box_bohr[d];
    a.desc = desc;
    a.rc_ang = 6.0f;
    a.status = st;
    const long long atoms = (long long)n_conf * 3 * n_mols;
    const long long blocks = ((long long)n_conf * n_mols + qtg::DW - 1) / qtg::DW;
    if (blocks > 0x7fffffffLL) return QTG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    void *wrapped = nullptr;  // stream-ordered scratch: the wrapped FP32 atoms
    if (cudaMallocAsync(&wrapped, sizeof(float4) * (size_t)atoms, s) != cudaSuccess) return QTG_ERR_CUDA;
    a.wrapped = static_cast<float4 *>(wrapped);
    qtg::k_wrap_atoms<<<(unsigned)((atoms + 255) / 256), 256, 0, s>>>(a);
    qtg::k_descriptors<<<(unsigned)blocks, 32 * qtg::DW, 0, s>>>(a);
    const cudaError_t e = cudaGetLastError();
    cudaFreeAsync(wrapped, s);
    return e == cudaSuccess ? QTG_OK : QTG_ERR_CUDA;
}

qtg_status qtg_mlp_forward(const qtg_mlp_weights *w, const void *x_bf16, int m, float *y, void *stream) {
    if (!w || !w->w1 || !w->w2 || !w->w3 || !w->b1 || !w->b2 || !w->b3 || !x_bf16 || !y || m < 0) return QTG_ERR_ARG;
    if (m == 0) return QTG_OK;
    unsigned *st = status_word();
    if (!st) return QTG_ERR_CUDA;
    static bool attr[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !attr[dev]) {
        if (cudaFuncSetAttribute(qtg::k_mlp_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fwd_smem()) !=
            cudaSuccess)
            return QTG_ERR_CUDA;
        attr[dev] = true;
    }
    qtg::MlpArgs a;
    a.w1 = static_cast<const __nv_bfloat16 *>(w->w1);
    a.w2 = static_cast<const __nv_bfloat16 *>(w->w2);
    a.w3 = static_cast<const __nv_bfloat16 *>(w->w3);
    a.b1 = w->b1;
    a.b2 = w->b2;
    a.b3 = w->b3;
    a.x = static_cast<const __nv_bfloat16 *>(x_bf16);
    a.m = m;
    a.y = y;
    a.status = st;
    const int tiles = (m + qtg::TM - 1) / qtg::TM;
    qtg::k_mlp_fwd<<<grid_for(tiles, 2), qtg::TM, fwd_smem(), (cudaStream_t)stream>>>(a);
    return cudaGetLastError() == cudaSuccess ? QTG_OK : QTG_ERR_CUDA;
}

qtg_status qtg_mlp_train_batch(const qtg_mlp_weights *w, const void *x_bf16, const float *t, int m, float grad_scale,
                               float *partial, int max_ctas, float *grad_out, void *stream) {
    if (!w || !w->w1 || !w->w2 || !w->w3 || !w->b1 || !w->b2 || !w->b3 || !x_bf16 || !t || !partial || !grad_out ||
        m <= 0 || max_ctas <= 0)
        return QTG_ERR_ARG;
    unsigned *st = status_word();
    if (!st) return QTG_ERR_CUDA;
    static bool attr[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && !attr[dev]) {
        if (cudaFuncSetAttribute(qtg::k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem()) !=
            cudaSuccess)
            return QTG_ERR_CUDA;
        attr[dev] = true;
    }
    qtg::TrainArgs a;
    a.w1 = static_cast<const __nv_bfloat16 *>(w->w1);
    a.w2 = static_cast<const __nv_bfloat16 *>(w->w2);
    a.w3 = static_cast<const __nv_bfloat16 *>(w->w3);
    a.b1 = w->b1;
    a.b2 = w->b2;
    a.b3 = w->b3;
    a.x = static_cast<const __nv_bfloat16 *>(x_bf16);
    a.t = t;
    a.m = m;
    a.grad_scale = grad_scale;
    a.partial = partial;
    a.status = st;
    const int tiles = (m + qtg::TM - 1) / qtg::TM;
    int grid = grid_for(tiles, 1);
    if (grid > max_ctas) grid = max_ctas;
    cudaStream_t s = (cudaStream_t)stream;
    qtg::k_mlp_train<<<grid, qtg::TM, train_smem(), s>>>(a);
    qtg::k_reduce_partials<<<(qtg::NPART + 255) / 256, 256, 0, s>>>(partial, grid, grad_out);
    return cudaGetLastError() == cudaSuccess ? QTG_OK : QTG_ERR_CUDA;
}

qtg_status qtg_adam_step(float *params, float *m1, float *m2, const float *grad, int n, int step, float lr,
                         float beta1, float beta2, float eps, void *w_bf16, int n_bf16, void *stream) {
    if (!params || !m1 || !m2 || !grad || n <= 0 || step <= 0 || n_bf16 < 0 || n_bf16 > n || (n_bf16 && !w_bf16))
        return QTG_ERR_ARG;
    const float bc1 = 1.f - powf(beta1, (float)step), bc2 = 1.f - powf(beta2, (float)step);
    qtg::k_adam<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(params, m1, m2, grad, n, lr, beta1, beta2, eps,
                                                                    bc1, bc2, static_cast<__nv_bfloat16 *>(w_bf16),
                                                                    n_bf16);
    return cudaGetLastError() == cudaSuccess ? QTG_OK : QTG_ERR_CUDA;
}

qtg_status qtg_surrogate_status(unsigned *bits, int clear) {
    if (!bits) return QTG_ERR_ARG;
    unsigned *st = status_word();
    if (!st) return QTG_ERR_CUDA;
    if (cudaDeviceSynchronize() != cudaSuccess) return QTG_ERR_CUDA;
    if (cudaMemcpy(bits, st, sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess) return QTG_ERR_CUDA;
    if (clear && cudaMemset(st, 0, sizeof(unsigned)) != cudaSuccess) return QTG_ERR_CUDA;
    return QTG_OK;
}

}  // extern "C"
