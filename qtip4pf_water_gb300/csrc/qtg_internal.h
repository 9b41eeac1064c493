// Internal definitions shared by the CUDA translation units of libqtipgpu.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace qtg {

// The reference's truncated pi (qtip4pfparams.h:45). It enters theta_eq,
// sqrt(pi), 2 pi / L and sin(k pi / P), so FP64 parity needs the same value.
constexpr double PI_REF = 3.14159265359;

// qTIP4P/F parameters in atomic units, derived on the host exactly as
// qtip4pfparams.h:41-133 derives them (same constants, same operation order).
struct Consts {
    double angs2bohr, fs2au, K2au, mo, mh;
    double r_cut, r_cut_sq, r_skin, r_skin_sq;
    double gamma_vs, epslj, sigmalj6, sigmalj12, e_cut;
    double roheq, ar2, ar3, ar4fac, Dr, theta_eq, ktheta, qo, qh;
    float ljf[6];  // FP32 Lennard-Jones constants: sigma^6, sigma^12, 4 eps, 24 eps, e_cut, r_cut^2
};

// Per-system constants (one per replica), resident in device memory.
struct SysDev {
    int n_mols, n_beads, n_sites, n_dof, list_size, k_max, n_kvec, kvec_off;
    int propagator, thermostat, job_base, cols_per_block;
    int cw_begin, cw_count;  // the system's column-work blocks: slots cw_begin .. cw_begin + cw_count - 1
    int n_kvec_ref;              // the reference's k-vector count (n_kvec includes c_k = 0 fillers)
    int col_off, n_col, grp_off, n_grp, batch_off, n_batch;
    // the mixed MODE-0 k-space kernels skip the kx = 0, ky < 0 columns (S(-k) =
    // conj S(k) for real charges; their kx = 0, ky > 0 partners count twice):
    // those columns come last, so the kept groups, batches and k entries are prefixes
    int n_grp_half, n_batch_half, n_kvec_half, n_col_half;
    int centroid_fixed;          // 1: the centroid is held fixed (centroid-constrained PIMD)
    // Verlet-list build: cell grid of side >= r_skin / 2 (lc_n cells a side, lc_cells in
    // all; 0 cells: boxes under five cells a side scan every molecule), cell starts of
    // bead b at lc_off + b (lc_cells + 1)
    int lc_n[3], lc_cells;
    long long lc_off;
    int lj_tie_mask;             // bit d: half of box side d lies within r_cut (a half-box tie can matter)
    long long nm_off;   // doubles: P x P bead->normal-mode matrix C (y = C x)
    long long mode_off; // ModeCoef entries: P per system
    long long q_off;    // doubles: system block [P][9N] in q/p/f/fphys/aux arrays
    long long d_off;    // doubles: [P][3N] block in disp
    long long pt_off;   // ints: [P][N] block in point
    long long ls_off;   // ints: [P][list_size] block in list
    long long pf_off;   // ints: [P][N+1] block in point_full (symmetric list row starts)
    long long lf_off;   // ints: [P][2 list_size] block in list_full
    long long chg_off;  // doubles: [3N] in charge
    long long mass_off; // doubles: [9N] in mass
    double box[3], inv_box[3];
    double kappa, rc_sq, ewald_pref, k_pref, self_energy;
    double r_cut_sq, r_skin_sq, skin_margin;
    double beta, beta_n, omega_psq, dt, halfdt, eps_sc, c1_centroid, inv_sqrt_beta_n;
    double inv_p, sqrt_inv_p, half_omega_psq, half_nd_beta;  // 1/P, sqrt(1/P), omega_P^2 / 2, n_dof / (2 beta)
    double c2n_centroid;  // PILE-L centroid: sqrt(1 - c1_centroid^2) / sqrt(beta_P)
    float boxf[3], inv_boxf[3];
    float kappaf, rc_sqf, ewald_preff, kappa_sqf;
    float kbf[3];   // 2 pi / L_d, the reciprocal-lattice steps
    // real space (FP32): fixf[d] = L_d / 2^32, one unit of a 32-bit fixed-point box
    // fraction; ka = 0.3275911 kappa (Abramowitz & Stegun 7.1.26), cex = -kappa^2
    // log2(e). A cubic box (fix_cubic) also has the constants in fixed-point units
    // (u = L / 2^32): r_c^2 / u^2, cex u^2, ka u, the Ewald prefactor times u, 1 / u^2
    // and 1 / u, so the pair loop needs no scaling of its integer differences.
    float fixf[3], kaf, cexf;
    double fix_scale[3];  // 2^32 / L_d: a coordinate times this, rounded, is its box fraction in fixed point
    int fix_cubic;
    float rc2u, cexu, kau, prefu, s2u, invu;
    unsigned long long seed;
};

// The FP32 constants above, from the FP64 ones (host).
inline void set_float_consts(SysDev &S) {
    const double two32 = 2.3283064365386963e-10, pi = PI_REF;
    for (int d = 0; d < 3; ++d) {
        S.kbf[d] = (float)(2.0 * pi * S.inv_box[d]);
        S.fixf[d] = (float)(S.box[d] * two32);
        S.fix_scale[d] = S.inv_box[d] * 4294967296.0;
    }
    S.kaf = (float)(0.3275911 * S.kappa);
    S.cexf = (float)(-S.kappa * S.kappa * 1.4426950408889634);
    S.fix_cubic = S.box[0] == S.box[1] && S.box[1] == S.box[2];
    const double u = S.box[0] * two32;
    S.rc2u = (float)(S.rc_sq / (u * u));
    S.cexu = (float)(-S.kappa * S.kappa * 1.4426950408889634 * u * u);
    S.kau = (float)(0.3275911 * S.kappa * u);
    S.prefu = (float)(S.ewald_pref * u);
    S.s2u = (float)(1.0 / (u * u));
    S.invu = (float)(1.0 / u);
}

// Per normal mode k of a system: free ring-polymer frequency and the
// sqrt-Cayley / PILE coefficients (update.cpp:301-320, thermostat.cpp:117-123).
struct ModeCoef {
    double w2;     // omega_k^2 = (2 / beta_P hbar)^2 sin^2(k pi / P)
    double scale;  // 1 / sqrt(1 + omega_k^2 dt^2 / 4)
    double c1;     // exp(-dt gamma_k), gamma_k = (4 / beta_P hbar) sin(k pi / P)
    double c2;     // sqrt(1 - c1^2)
    double cq;     // scale dt / 2: a half Cayley step is q' = scale q + cq p / m
    double cp;     //   and p' = scale p - cp m q, with cp = scale omega_k^2 dt / 2
    double c2n;    // c2 / sqrt(beta_P), the PILE noise amplitude per sqrt(m)
};

// One reciprocal-lattice vector k = 2 pi (kx/Lx, ky/Ly, kz/Lz) of the set
// forces.cpp:251-445 visits, with c_k = (2 pi / V) exp(-k^2/4 kappa^2) / k^2
// (doubled for kx > 0) and g = 2 c_k k.
struct KVec {
    int kx, ky, kz;
    int twin;  // 1: kx = 0, ky > 0 (stands for its conjugate partner too in the mixed half set)
    double coef, gx, gy, gz;
};

// Reciprocal-space vectors are stored in columns of fixed (kx, ky) with kz
// running over [-m, m]; points of a column outside the reference's set carry
// c_k = 0. A column's vectors are contiguous in the KVec table.
struct KCol {
    int kx, ky, m, k_begin;
};
// Structure-factor work item: up to 4 consecutive |kz| of one column, starting
// at kz0 >= 0; each |kz| stands for the pair kz = +|kz|, -|kz|.
struct KGroup {
    int col, kz0, n, pad;
};
// Reciprocal-force work item: whole columns [c0, c1) holding k in [k0, k1), k1 - k0 <= 128.
struct KBatch {
    int c0, c1, k0, k1;
};

// One force evaluation ("job"): one configuration of one system.
struct Job {
    int sys;   // system index
    int bead;  // bead whose Verlet list (point/list slice) the LJ term uses
    int slot;  // scratch slot (per-job scratch arrays are indexed by slot)
    int mode;  // 0 = forces; 1 = directional derivative of the Ewald forces
    long long pos_off;  // doubles: the job's 9N positions, relative to the position base
    long long out_off;  // doubles: the job's 9N forces, relative to the output base
    long long site_off; // elements: 3N sites in the site scratch (per slot)
    long long phase_off;// complex elements: phase table (3 * (kmax+1) * 3N) per slot
    long long sk_off;   // complex elements: S(k) per slot
};

// Per-system, per-step accumulators (zeroed by the step-finalize kernel).
struct SysAcc {
    double kin;      // sum_b p^2 / 2m after the closing kick
    double spring;   // sum_b 1/2 m w_P^2 (q_b - q_{b+1})^2
    double kcv_tq;   // -sum (q_b - qbar) . fphys_b over the estimator's beads
    double k0;       // centroid normal-mode kinetic energy entering the next O step
    double sc_extra; // SC: sum over odd beads of fsq / (3 w_P^2)
    double rebuilds; // Verlet lists rebuilt this step
    double pad[2];
};

// Per-system persistent thermostat / RNG state.
struct SysRun {
    double heat;        // accumulated thermostat heat (update.cpp:325)
    double alpha;       // centroid rescale factor for the next O step (PILE-G)
    double cf_samples;  // steps accumulated into the mean centroid force
    double list_builds; // Verlet-list rebuilds of any bead since creation (never reset)
    double R_draw, g2_draw;  // PILE-G centroid draws made ahead by k_ring's draw blocks ...
    unsigned long long draw_step_plus1;  // ... for step draw_step_plus1 - 1 (0: none made)
};

// Status word written by kernels (bit flags), read by the host after a sync.
enum StatusBits : unsigned {
    ST_LIST_OVERFLOW = 1u,
    ST_NONFINITE = 2u,
    ST_GAMMA_LIMIT = 4u,
    ST_DESC_OVERFLOW = 8u,   // an atom had more neighbours within the descriptor cutoff than kept
    ST_MMA_TIMEOUT = 16u,    // a tensor-core completion wait ran out of its iteration limit
    ST_RLIST_OVERFLOW = 32u, // a real-space pair-list row needed more than rl_cap entries
};

// ---- device helpers ---------------------------------------------------------
#ifdef __CUDACC__

// Programmatic dependent launch: a kernel launched with launch_pdl may start
// before the kernel ahead of it in the stream has finished (once that kernel's
// blocks have all called pdl_launch_dependents, or exited); it must call pdl_wait
// before it reads anything that kernel writes. Both are no-ops for a kernel
// launched the ordinary way.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... Params, typename... Args>
inline void launch_pdl(void (*kern)(Params...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, args...);
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float warp_sum(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum; every thread must call it. `sh` needs blockDim.x/32 doubles.
__device__ __forceinline__ double block_sum(double v, double *sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = 0.0;
    if (w == 0) {
        t = (lane < nw) ? sh[lane] : 0.0;
        t = warp_sum(t);
    }
    return t;  // valid in warp 0 (lane 0)
}

// Fixed-order sum of per-block values over the column-work blocks of one system
// (every thread of the block calls it, after the kernel's last __syncthreads).
// Each block stores its NV values (v, read by thread 0) at its slot; the block
// that arrives last on the system's ticket sums all the system's slots in slot
// order (thread t the slots t, t + blockDim.x, ..., all NV values at once, then a
// fixed shuffle-and-shared-memory tree), adds the NV totals to dst[k] and re-arms
// the ticket. The totals therefore do not depend on the order the blocks ran in.
// Returns true in that last block (the totals are visible to its warp 0).
template <int NV>
__device__ bool ordered_system_sum(const double *v, int slot, int cw_begin, int cw_count, double *part,
                                   unsigned *ticket, double *const *dst) {
    __shared__ int last;
    __shared__ double red[NV][32];
    if (threadIdx.x == 0) {
        for (int k = 0; k < NV; ++k) part[(size_t)slot * NV + k] = v[k];
        __threadfence();
        last = atomicAdd(ticket, 1u) == (unsigned)(cw_count - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double t[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) t[k] = 0.0;
    for (int j = threadIdx.x; j < cw_count; j += blockDim.x) {
        const double *pj = part + (size_t)(cw_begin + j) * NV;
#pragma unroll
        for (int k = 0; k < NV; ++k) t[k] += __ldcg(pj + k);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        t[k] = warp_sum(t[k]);
        if (lane == 0) red[k][w] = t[k];
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const double u = warp_sum(lane < nw ? red[k][lane] : 0.0);
            if (lane == 0) *dst[k] += u;
        }
        if (lane == 0) *ticket = 0u;
    }
    return true;
}

// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror & Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC'11): ten rounds of
// (hi,lo) = M * x multiplications with a Weyl-sequence key schedule.
struct Philox4 {
    uint32_t v[4];
};

__device__ __forceinline__ Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                 uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(M0, c0), lo0 = M0 * c0;
        uint32_t hi1 = __umulhi(M1, c2), lo1 = M1 * c2;
        uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += W0;
        k1 += W1;
    }
    Philox4 o;
    o.v[0] = c0;
    o.v[1] = c1;
    o.v[2] = c2;
    o.v[3] = c3;
    return o;
}

// Uniform double in (0, 1) from two 32-bit words (53 significant bits).
__device__ __forceinline__ double u01_from(uint32_t a, uint32_t b) {
    unsigned long long x = ((unsigned long long)a << 21) ^ (unsigned long long)(b >> 11);
    x &= ((1ull << 53) - 1ull);
    return ((double)x + 0.5) * (1.0 / 9007199254740992.0);
}

// Two standard normals (Box-Muller) from one Philox block.
__device__ __forceinline__ double2 normal2(const Philox4 &r) {
    double u1 = u01_from(r.v[0], r.v[1]);
    double u2 = u01_from(r.v[2], r.v[3]);
    double rad = sqrt(-2.0 * log(u1));
    double s, c;
    sincospi(2.0 * u2, &s, &c);
    return make_double2(rad * c, rad * s);
}

// RNG stream tags (third counter word's high byte) keep draws independent.
enum RngTag : uint32_t { RNG_MODES = 1u, RNG_CENTROID = 2u, RNG_GAMMA = 3u };

#endif  // __CUDACC__

// ---- launch interface between translation units ----------------------------

// Column work item of the normal-mode / propagation kernels: a block handles
// cols_per_block dof columns of one system (all beads of each column).
struct ColWork {
    int sys, col0, ncols;
    int slot;  // index of this block in the context's column-work list
};

enum RingFlags : int {
    RF_KICK = 1,    // p += dt/2 f before the transform
    RF_FWD = 2,     // bead -> normal-mode transform of q, p
    RF_CAYLEY = 4,  // sqrt-Cayley free ring-polymer half steps around the O step
    RF_THERMO = 8,  // O step (PILE-G centroid rescale or PILE-L / mode Langevin)
    RF_BACK = 16,   // normal-mode -> bead transform
    RF_DISP = 32,   // track oxygen displacements in bead space
    RF_VV = 64,     // classical velocity-Verlet drift q += dt p / m (P = 1)
};

struct FinalizeArgs {
    const SysDev *sys;
    int n_sys;
    const double *energy;    // base-job energies (job_base + bead)
    SysAcc *acc;
    SysRun *run;
    double *est;             // ring buffer [max_records][n_sys][8]
    int max_records;
    unsigned long long *step;
    unsigned long long *records;
    unsigned *status;
    const double *noise;     // optional caller noise for the centroid draw (system 0 only)
    int record;              // 1: write an estimator record and count a step
    int draw_alpha;          // 1: draw the next PILE-G centroid factor
    int sys_begin, sys_end;  // systems handled
    int pile_g;              // 1: draw alpha whatever the system's thermostat
    int pre_drawn;           // 1: this step's k_ring already made the centroid draws (SysRun)
    unsigned *ticket;        // fused into k_end_step: systems finished (the last advances the counters)
};

struct RingArgs {
    const SysDev *sys;
    const ColWork *work;
    int n_work;
    int flags;
    double *q, *p;
    const double *f;
    double *disp;
    const double *mass;
    const double *inv_mass;  // 1 / m per dof
    const double *sqrt_mass; // sqrt(m) per dof
    const double *nm;        // bead -> normal-mode matrices
    const ModeCoef *modes;
    SysRun *run;
    SysAcc *acc;
    const double *noise;     // optional caller noise [R, g2, xi(mode 1..P-1, dof)] (one system)
    const unsigned long long *step;
    const double *fphys;     // end step: physical forces for the virial estimator
    int kick;                // end step: 1 = apply the closing kick, 0 = estimators only
    int kcv_all_beads;       // end step: -1 = by propagator, 0 = even beads, 1 = all beads
    int max_p;               // largest bead count (shared-memory sizing)
    int pile_g;              // 1: O step is PILE-G whatever the system's thermostat
    double *cf_acc;          // end step: sum over steps of the bead-averaged force, per dof
                             // (systems with a fixed centroid; indexed like mass)
    unsigned *status;        // ring draw blocks: ST_GAMMA_LIMIT
    double *cw_part;         // per column-work slot: block partials of the system sums (4 doubles)
    unsigned *cw_ticket;     // per system: blocks arrived at the system sums of the running kernel
    int fuse_fin;            // end step: the last block of each system also runs its finalize (fin)
    FinalizeArgs fin;
    const struct CallBox *box;  // centroid alpha: staged per-call step -- p and f come from the
                                // caller's arrays named in this mailbox (device address)
    int n_draw;              // ring: extra blocks that make the PILE-G centroid draws at the
                             // current step of systems draw_sys0 .. draw_sys0 + n_draw - 1
                             // while the ring work runs (0: none)
    int draw_sys0;
    // end step of a staged per-call step: the kicked momenta also go to the caller's
    // array named in this mailbox, and the block that completes the system's sums
    // posts the small results there (heat, energies, rebuild flags, accumulators,
    // status), then clears the accumulators and the status word
    struct CallBox *post_box;
    double *post_energy;       // device address of the mailbox's energy[]
    int *post_rebuilt;         // device address of its rebuilt[]
    const double *sys_energy;  // the system's per-bead energies
    const int *sys_rebuilt;    // the system's per-bead rebuild flags
};


struct ScArgs {
    const SysDev *sys;
    const int *job_sys, *job_bead;  // odd beads (prepare) or all base jobs (finish)
    int n_jobs;
    const double *q, *fphys, *mass, *inv_mass;
    double *qdisp;      // displaced positions (q + d at bead b, q - d at bead b-1)
    double *dirv;       // direction f/m at bead b (mixed mode)
    const double *fdisp;   // FP64: F(q+d) at b, F(q-d) at b-1; mixed: dF_ewald at b
    const double *fsr;     // mixed: short-range F(q+d) at b, F(q-d) at b-1
    double *f;
    double *sc_scale;   // per base job: s (the finite-difference step scale)
    SysAcc *acc;
    int mixed;
    int max_dof;
    int force_sc;       // finish: 1 = Suzuki-Chin assembly whatever the propagator
};

struct ReduceArgs {   // tier-1 estimators
    const SysDev *sys;
    int sysi;
    const double *q, *p, *f, *mass, *nm;
    double *out;      // out[0..]
    int trotter;
};

// propagate.cu
void launch_ring(const RingArgs &a, cudaStream_t s, unsigned long long *n);
void launch_end_step(const RingArgs &a, cudaStream_t s, unsigned long long *n);
void launch_finalize(const FinalizeArgs &a, cudaStream_t s, unsigned long long *n);
void launch_sc_prepare(const ScArgs &a, cudaStream_t s, unsigned long long *n);
void launch_sc_finish(const ScArgs &a, cudaStream_t s, unsigned long long *n);
void launch_transform(const SysDev *sys, int sysi, int P, const double *nm_sys, double *a, int length,
                      int forwards, cudaStream_t s, unsigned long long *n);
void launch_centroid_ke(const RingArgs &a, cudaStream_t s, unsigned long long *n);
// Bussi global rescale of system sys (one block)
void launch_bussi(const RingArgs &a, int sys, cudaStream_t s, unsigned long long *n);
// per-call PIMD steps: k0 after the opening kick, the centroid draws and alpha of system sys
void launch_centroid_alpha(const RingArgs &a, int sys, cudaStream_t s, unsigned long long *n);
// sum_k sum_j (p_kj^2 / 2 m_j + m_j w_k^2 q_kj^2 / 2) of normal-mode arrays -> out[0], out[1]
void launch_nm_energy(const SysDev *sys, int sysi, int P, int n_dof, const double *q, const double *p,
                      const double *mass, const ModeCoef *modes, double *out, cudaStream_t s,
                      unsigned long long *n);

// Chunking limits of the force kernels' second grid dimension.
constexpr int MAX_RJ = 16;   // real-space j-chunks
constexpr int MAX_KC = 16;   // reciprocal-space k-chunks
constexpr int MAX_SC = 32;   // structure-factor site chunks
constexpr int HALF_MAX_TILES = 64;  // half-interaction real space: beads of at most 64 x 32 sites
constexpr int HALF_MAX_CH = 8;      // its stationary-side chunks
constexpr int MAX_RPLANES = HALF_MAX_CH + HALF_MAX_TILES / 2 > MAX_RJ ? HALF_MAX_CH + HALF_MAX_TILES / 2 : MAX_RJ;
constexpr int MAX_PART = MAX_RPLANES + MAX_KC + 1;  // partial site-force planes
// Real-space pair list (mixed form, beads beyond the half-interaction kernel):
// the distance from its molecule's M site (bohr) within which every charge site
// of a configuration must lie for one minimum image per molecule pair to serve
// its nine site pairs, and the list's skin (bohr).
constexpr float RL_SPREAD = 3.0f;
constexpr float RL_SKIN = 2.0f;

struct EvalArgs {
    const SysDev *sys;     // device array
    const Job *jobs;       // device array, n_jobs entries
    int n_jobs;
    int max_mols;          // largest N over the jobs' systems (grid sizing)
    int max_kvec;          // largest k-vector count
    int max_kmax;
    int kz;                  // |kz| values per structure-factor group (3 or 4)
    const double *pos;     // position base (jobs' pos_off are relative to it)
    double *out;           // force output base
    double *out_prop;      // mixed, optional: the same forces also written here (the propagating
                           // force of Trotter / classical systems, saving the assembly copy)
    const double *dir;     // tangent direction base (mode 1 jobs), same offsets as pos
    const double *charge;
    const int *point, *list;
    const int *point_full, *list_full;  // symmetric lists built by the stepper's rebuild
    int lj_full;                        // 1: Lennard-Jones over the symmetric list (no atomics)
    int lj_list;                        // mixed, symmetric lists valid: k_lj over them instead of every pair
    const KVec *kvec;
    const KCol *kcol;
    const KGroup *kgrp;
    const KBatch *kbatch;
    const int *kpk;        // per k (as kvec): kz >= 0: (packed slot in its force batch) << 8 | kz; kz < 0: -1
    const int4 *kfc;       // per column (as kcol): kx, ky, m, packed slot of its kz = 0 (FP32 k-force)
    const float2 *kfb;     // per column: (2 pi / L_x) kx, (2 pi / L_y) ky in FP32
    float4 *wpk;           // per k slot: the packed +-kz weights P1, P2 of k_kforce_f32 (k_sk_reduce)
    int max_grp, max_batch;
    void *sites;           // 4 reals per site (x, y, z, q), per slot
    int4 *sites_fix;       // mixed: per site the box fractions of x, y, z as 32-bit fixed point
                           // (so a wrapped integer difference is the minimum image) and q's bits
    void *opos;            // wrapped oxygen positions, 4 reals per molecule, per slot
    float4 *ljf;           // dense Lennard-Jones oxygen forces, per molecule, per slot (lj_plane)
    int lj_plane;          // 1: k_lj_dense writes ljf and k_combine_f32 adds it to the O force
    float *intra;          // mixed: intramolecular site and atom forces, 18 floats per molecule and slot
    int intra_plane;       // 1: k_intra_f32 wrote intra (and the energy) and k_combine_f32 adds it
    void *phase;           // complex phase tables, per slot
    void *tan_sites;       // tangent of the site positions (mode 1), per slot
    double *part;          // partial site forces [MAX_PART][total_sites][3]
    // mixed: the half-interaction real space's site forces as 64-bit fixed point
    // (units of 2^-40 Hartree/bohr, [total_sites][3]; zeroed by k_prep_f32, summed by
    // integer atomics, so the sum does not depend on their order), read by
    // k_combine_f32 when real_fix is set
    long long *rfix;
    int real_fix;
    long long total_sites; // sites summed over all slots (plane stride of part)
    double2 *skp;          // partial S(k) [MAX_SC][total_k]
    double2 *dskp;         // partial dS(k) along the tangent direction
    void *wsk, *wdsk;      // 2 c_k S(k) and 2 c_k dS(k), working precision, per slot
    long long total_k;     // k-vectors summed over all slots (plane stride of skp)
    double *energy;        // per slot
    unsigned *status;
    int n_rj, n_sc, n_kc;  // chunk counts, chosen by the launcher
    // real-space pair list, per slot (rl_on: the mixed real space runs over it)
    int rl_on, rl_cap;     // rl_cap: entries a row holds
    unsigned short *rl_list;  // [slot molecule][rl_cap]: molecules j with a site pair within r_c + RL_SKIN at the build
    int *rl_cnt;           // entries per slot molecule
    float4 *rl_ref;        // per slot site: the positions the list was built at (NaN: never built)
    int *rl_jobs, *rl_count;  // the launch's jobs whose list is rebuilt, and their number
    int *rl_wide;          // per slot: a site lies beyond RL_SPREAD of its M site (minimum image per site pair)
    uint4 *rl_state;       // per slot: the displacement test's merge state (zero between launches)
    int tune_rj, tune_sc, tune_kc;  // chunk counts fixed by the autotuner (0: launcher heuristic)
    int sites_are_input;   // 1: positions are charge sites (M,H1,H2) -> reciprocal space only
    int sr_only;           // 1: only the short-range terms (LJ, intramolecular,
                           //    same-molecule Ewald), in FP64; Ewald partials ignored
    int mode;              // 0 = forces, 1 = directional derivative of the Ewald forces
    Consts c;
};

// splines.cu: tabulated pair corrections (forces.cpp:452-466, :634-691). One
// table per pair type: coefficients c_{-1} .. c_n at coef[coef_off ..], knots
// start + i / inv_step, pairs with r^2 < cut_sq.
struct SplineType {
    long long coef_off;
    int n, pad;
    double start, inv_step, cut_sq;
};
struct PairSplines {
    SplineType t[3];  // O-O, O-H, H-H
    int on, pad;
};
struct SplineArgs {
    const SysDev *sys;
    const Job *jobs;
    int n_jobs, max_mols;
    const double *pos;          // position base (jobs' pos_off)
    double *out, *out_prop;     // force bases the spline forces are added to (out_prop optional)
    double *energy;             // per slot
    const PairSplines *tables;  // per system
    const double *coef;
};
void launch_pair_splines(const SplineArgs &a, bool mixed, cudaStream_t s, unsigned long long *launches);
bool bspline_coefficients(const double *y, int n, double h, double dl, double dr, double *c);

// surrogate.cu: the learned centroid correction of one P = 1 system, added to
// its forces inside a force evaluation (descriptors, features, tensor-core
// forward pass, frames, lab-frame correction)
struct SurrogateRun {
    const double *pos;            // [9N] positions of the system
    double *f;                    // [9N] forces to correct
    int n_mols, n_sm;
    double box[3];
    const __nv_bfloat16 *wbf;     // w1 | w2 | w3, BF16
    const float *bias;            // b1 | b2 | b3
    const float *norm;            // input mean [96] | inverse standard deviation [96]
    float out_scale;
    float *desc, *y, *frames;     // scratch: [3N][32], [2N][16], [N][9]
    float4 *wrapped;              // scratch: [3N] atoms wrapped into the box (A, FP32)
    __nv_bfloat16 *feat;          // scratch: [2N][96]
    unsigned *status;
};
// The correction in two parts: prepare (wrapped atoms, descriptors, features,
// the network, the molecular frames: positions only, so it may run beside the
// force evaluation) and apply (the lab-frame correction added to f).
void launch_surrogate_prepare(const SurrogateRun &r, cudaStream_t s, unsigned long long *launches);
void launch_surrogate_apply(const SurrogateRun &r, cudaStream_t s, unsigned long long *launches);
void init_surrogate_kernel_attributes();

// forces.cu: individual Ewald kernels (for timing)
void launch_ewald_kernel(const EvalArgs &a, bool mixed, const char *name, cudaStream_t s);
void launch_fp32_probe(float *out, int blocks, int iters, cudaStream_t s);
void launch_fp64_probe(double *out, int blocks, int iters, cudaStream_t s);

// forces.cu
void launch_eval_fp64(const EvalArgs &a, cudaStream_t s, unsigned long long *launches);
// Side streams and events for a forked mixed evaluation: after k_prep, the
// reciprocal-space chain (k_ksk, k_sk_reduce, k_kforce_f32) runs on side[0] and
// the dense Lennard-Jones on side[1] beside the real-space kernel; both join
// before k_combine_f32. (Captured into a graph, these become parallel branches.)
struct Forks {
    cudaStream_t side[2];
    cudaEvent_t fork, join[2];
    cudaEvent_t lists_ready;  // set: the Verlet-list rebuild runs beside the forces; the list LJ waits for it
};
void launch_eval_mixed(const EvalArgs &a, cudaStream_t s, unsigned long long *launches,
                       const Forks *forks = nullptr);
void launch_kwald_only(const EvalArgs &a, bool mixed, cudaStream_t s, unsigned long long *launches);

// one-time kernel attribute set-up (shared-memory limits); called at context creation
void init_force_kernel_attributes();
void init_list_kernel_attributes();
void init_propagate_kernel_attributes();

// neighbour.cu
struct ListArgs {
    const SysDev *sys;
    const int *job_sys, *job_bead;  // one (system, bead) per block
    int n_jobs;
    const double *q;
    double *disp;
    int *point, *list;
    int *point_full, *list_full;  // may be null: only the half list is built
    SysAcc *acc;
    SysRun *run;        // cumulative rebuild count per system (may be null)
    int *rebuilt;       // per base job (system's job_base + bead): set to 1 by a rebuild
    unsigned *status;
    int force_rebuild;  // 1: rebuild unconditionally (initial build / per-call API)
    int max_mols;
    // build scratch, indexed like point (pt_off + bead N) unless noted
    int *rb_jobs;       // the launch's rebuilding jobs (launch-local indices), rb_count of them
    int *rb_count;      // zeroed before every launch
    float4 *wpos;       // oxygen positions wrapped into the box (FP32)
    int *cnt_half, *cnt_full;  // per-row neighbour counts
    int *cell_start;    // per bead lc_cells + 1 (lc_off)
    int *cell_mol;      // molecules by cell
};
void launch_skin_rebuild(const ListArgs &a, cudaStream_t s, unsigned long long *launches);
constexpr int LC_MAX_CELLS = 8000;  // cells of the Verlet-list build's grid (20 a side at most)

// stage.cu: the per-call mailbox and the kernels that move a per-call step's
// arrays between the caller's page-locked host memory and the device
struct CallBox {
    // the caller's arrays of this call (device-accessible host memory; stage kernels)
    double *q, *p, *f, *fphys, *disp;
    double heat_in, heat_out;
    SysAcc acc;
    unsigned status;
    int pad;
    // followed by double energy[max_p] and int rebuilt[max_p]
};
struct StageArgs {
    CallBox *box;            // device address of the mailbox
    double *box_energy;      // device address of its energy[]
    int *box_rebuilt;        // device address of its rebuilt[]
    double *q, *p, *f, *fphys, *disp;  // the system's device arrays
    long long nt, nd;        // doubles in q (p, f, fphys) and in disp
    SysRun *run;             // the system's run state (heat)
    const double *energy;    // the system's per-bead energies
    const int *rebuilt;      // the system's per-bead rebuild flags
    SysAcc *acc;             // the system's step accumulators (cleared by stage out)
    unsigned *status;        // context status word (copied, then cleared, by stage out)
    int n_beads;
    int blocks;              // grid size
    unsigned mask;           // stage out: STAGE_* arrays to write back
};
enum StageParts : unsigned {
    STAGE_Q = 1u, STAGE_P = 2u, STAGE_F = 4u, STAGE_FPHYS = 8u, STAGE_DISP = 16u,
    STAGE_SMALL = 32u,  // heat, energies, rebuild flags, accumulators, status
};
void launch_stage_in(const StageArgs &a, cudaStream_t s, unsigned long long *n);
void launch_stage_out(const StageArgs &a, cudaStream_t s, unsigned long long *n);

}  // namespace qtg
