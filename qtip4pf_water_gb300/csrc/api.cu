// Host side of libqtipgpu: context, parameter derivation, job tables, the C ABI.
//
// All device memory is allocated in qtg_create; no later call allocates.
// A context holds any number of independent systems (replicas) of uneven
// size, laid out back to back in every array; each force-evaluation launch
// covers a table of jobs (system, bead) so all replicas advance together.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "../../include/qtip4pf_gb300.h"
#include "qtg_internal.h"

using namespace qtg;

namespace {

// ---- qTIP4P/F constants (qtip4pfparams.h:41-133, same values and order) ----
Consts make_consts() {
    Consts K;
    const double me = 9.10938356e-31, kb = 1.38064852e-23, Na = 6.0221409e23;
    const double eh = 4.3597447222071e-18, kcal2au = 1.5936e-3;
    const double mhgmol = 1.0080, mogmol = 15.9994, hbar_SI = 1.054571817e-34;
    K.angs2bohr = 1.0 / 0.529177210903;
    K.mo = 0.001 * mogmol / (Na * me);
    K.mh = 0.001 * mhgmol / (Na * me);
    K.K2au = kb / eh;
    const double au2fs = hbar_SI * 1e15 / eh;
    K.fs2au = 1.0 / au2fs;
    K.r_cut = 9.0 * K.angs2bohr;
    K.r_cut_sq = K.r_cut * K.r_cut;
    K.r_skin = 1.30 * K.r_cut;
    K.r_skin_sq = K.r_skin * K.r_skin;
    K.gamma_vs = 0.73612;
    K.epslj = 0.1852 * kcal2au;
    const double sigmalj = 3.1589 * K.angs2bohr;
    K.sigmalj6 = pow(sigmalj, 6.0);
    K.sigmalj12 = K.sigmalj6 * K.sigmalj6;
    K.e_cut = 4.0 * K.epslj * (pow((sigmalj / K.r_cut), 12.0) - pow((sigmalj / K.r_cut), 6.0));
    K.roheq = 0.9419 * K.angs2bohr;
    const double ar = 2.287 / K.angs2bohr;
    K.ar2 = ar * ar;
    K.ar3 = K.ar2 * ar;
    K.ar4fac = 7.0 * K.ar3 * ar / 12.0;
    K.Dr = 116.09 * kcal2au;
    K.theta_eq = 107.4 * PI_REF / 180.0;
    K.ktheta = 87.85 * kcal2au;
    K.qo = -1.1128;
    K.qh = -0.5 * K.qo;
    K.ljf[0] = (float)K.sigmalj6;
    K.ljf[1] = (float)K.sigmalj12;
    K.ljf[2] = (float)(4.0 * K.epslj);
    K.ljf[3] = (float)(24.0 * K.epslj);
    K.ljf[4] = (float)K.e_cut;
    K.ljf[5] = (float)K.r_cut_sq;
    return K;
}

// The k-vectors forces.cpp:251-445 visits, in its order.
void enumerate_k(const SysDev &S, double kc_sq, std::vector<KVec> &out) {
    double bk[3];
    for (int d = 0; d < 3; ++d) bk[d] = 2.0 * PI_REF / S.box[d];
    const double quart = 0.25 / (S.kappa * S.kappa);
    const int km = S.k_max;
    auto push = [&](int a, int b, int c, double ksq) {
        KVec v;
        v.kx = a;
        v.ky = b;
        v.kz = c;
        v.twin = (a == 0 && b > 0) ? 1 : 0;
        v.coef = S.k_pref * exp(-ksq * quart) / ksq * (a ? 2.0 : 1.0);
        v.gx = 2.0 * v.coef * bk[0] * a;
        v.gy = 2.0 * v.coef * bk[1] * b;
        v.gz = 2.0 * v.coef * bk[2] * c;
        out.push_back(v);
    };
    for (int kx = 0; kx <= km; ++kx) {
        const double rx = bk[0] * kx;
        double ksq = rx * rx;
        if (ksq > 0.0 && ksq < kc_sq) push(kx, 0, 0, ksq);
        for (int kz = 1; kz <= km; ++kz) {
            const double rz = bk[2] * kz;
            ksq = rx * rx + rz * rz;
            if (ksq > kc_sq) break;
            push(kx, 0, kz, ksq);
            push(kx, 0, -kz, ksq);
        }
        for (int ky = 1; ky <= km; ++ky) {
            const double ry = bk[1] * ky;
            ksq = rx * rx + ry * ry;
            if (ksq > kc_sq) break;
            push(kx, ky, 0, ksq);
            push(kx, -ky, 0, ksq);
            for (int kz = 1; kz <= km; ++kz) {
                const double rz = bk[2] * kz;
                ksq = rx * rx + ry * ry + rz * rz;
                if (ksq > kc_sq) break;
                push(kx, ky, kz, ksq);
                push(kx, ky, -kz, ksq);
                push(kx, -ky, kz, ksq);
                push(kx, -ky, -kz, ksq);
            }
        }
    }
}

// Orthonormal bead -> normal-mode matrix in FFTW halfcomplex order with
// fourier.cpp:39-51's scaling (sqrt(1/P) for k = 0 and k = P/2, sqrt(2/P) else).
void nm_matrix(int P, std::vector<double> &C) {
    C.assign((size_t)P * P, 0.0);
    const double two_pi = 6.283185307179586476925286766559;
    for (int b = 0; b < P; ++b) C[b] = sqrt(1.0 / P);
    for (int k = 1; 2 * k < P; ++k)
        for (int b = 0; b < P; ++b) {
            const double ang = two_pi * (double)(((long)b * k) % P) / (double)P;
            C[(size_t)k * P + b] = sqrt(2.0 / P) * cos(ang);
            C[(size_t)(P - k) * P + b] = -sqrt(2.0 / P) * sin(ang);
        }
    if (P % 2 == 0 && P > 1)
        for (int b = 0; b < P; ++b) C[(size_t)(P / 2) * P + b] = sqrt(1.0 / P) * ((b % 2 == 0) ? 1.0 : -1.0);
}

// Reorder the k-vectors into columns of fixed (kx, ky) with contiguous kz in
// [-m, m] (fillers with c_k = 0 where the reference's set has a hole), and
// build the structure-factor groups (<= 8 kz of one column) and the force
// batches (whole columns, <= 128 vectors).
void build_columns(const std::vector<KVec> &kv, std::vector<KVec> &kord, std::vector<KCol> &cols,
                   std::vector<KBatch> &bats, std::vector<int> &kpk, int *n_col_half_out, int *n_batch_half,
                   int *n_kvec_half) {
    std::map<std::pair<int, int>, std::map<int, KVec>> by;
    for (const KVec &v : kv) by[{v.kx, v.ky}][v.kz] = v;
    // the kx = 0, ky < 0 columns last (the mixed half set leaves them out)
    std::vector<const std::pair<const std::pair<int, int>, std::map<int, KVec>> *> order;
    for (auto &col : by)
        if (!(col.first.first == 0 && col.first.second < 0)) order.push_back(&col);
    const int n_col_half = (int)order.size();
    for (auto &col : by)
        if (col.first.first == 0 && col.first.second < 0) order.push_back(&col);
    *n_col_half_out = n_col_half;
    *n_kvec_half = 0;
    for (const auto *colp : order) {
        const auto &col = *colp;
        if ((int)cols.size() == n_col_half) *n_kvec_half = (int)kord.size();
        int m = 0;
        for (auto &e : col.second) m = std::max(m, std::abs(e.first));
        KCol c;
        c.kx = col.first.first;
        c.ky = col.first.second;
        c.m = m;
        c.k_begin = (int)kord.size();
        for (int kz = -m; kz <= m; ++kz) {
            auto it = col.second.find(kz);
            if (it != col.second.end()) {
                kord.push_back(it->second);
            } else {
                KVec f;
                f.kx = c.kx;
                f.ky = c.ky;
                f.kz = kz;
                f.twin = 0;
                f.coef = f.gx = f.gy = f.gz = 0.0;
                kord.push_back(f);
            }
        }
        cols.push_back(c);
    }
    if ((int)cols.size() == n_col_half) *n_kvec_half = (int)kord.size();
    // force batches of whole columns (<= 128 vectors), none straddling the half-set end
    int c0 = 0;
    *n_batch_half = 0;
    while (c0 < (int)cols.size()) {
        if (c0 == n_col_half) *n_batch_half = (int)bats.size();
        const int c_end = c0 < n_col_half ? n_col_half : (int)cols.size();
        int c1 = c0, n = 0;
        while (c1 < c_end && n + 2 * cols[c1].m + 1 <= 128) {
            n += 2 * cols[c1].m + 1;
            ++c1;
        }
        KBatch b;
        b.c0 = c0;
        b.c1 = c1;
        b.k0 = cols[c0].k_begin;
        b.k1 = cols[c1 - 1].k_begin + 2 * cols[c1 - 1].m + 1;
        bats.push_back(b);
        c0 = c1;
    }
    if (c0 == n_col_half) *n_batch_half = (int)bats.size();
    // the FP32 k-force kernel's packing: per batch, the columns' |kz| = 0 .. m in
    // consecutive slots; the kz >= 0 entry of each pair names its slot and |kz|
    kpk.assign(kord.size(), -1);
    for (const KBatch &b : bats) {
        int slot = 0;
        for (int c = b.c0; c < b.c1; ++c) {
            for (int az = 0; az <= cols[c].m; ++az) kpk[cols[c].k_begin + cols[c].m + az] = ((slot + az) << 8) | az;
            slot += cols[c].m + 1;
        }
    }
}

struct Table {  // a device job table plus its host copy
    std::vector<Job> h;
    Job *d = nullptr;
};

}  // namespace

struct qtg_ctx {
    int device = 0;
    int precision = QTG_FP64;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    // a second stream and fork / join events: inside the captured per-call step, the
    // stage-out of arrays that are final early runs beside the later kernels
    cudaStream_t side_stream = nullptr;
    // learned corrections: their positions-only part runs on this branch beside the forces
    cudaStream_t sur_stream = nullptr;
    cudaEvent_t sur_fork = nullptr, sur_join = nullptr;
    cudaEvent_t ev_fork[2] = {nullptr, nullptr}, ev_join = nullptr;
    Forks forks{};            // branches of a mixed force evaluation (real | k-space | LJ)
    float4 *ljf = nullptr;    // dense LJ oxygen forces per molecule and slot
    float *intra = nullptr;   // intramolecular forces, 18 floats per molecule and slot
    int4 *sites_fix = nullptr;  // fixed-point site fractions per slot (half-interaction real space)
    long long *rfix = nullptr;  // fixed-point real-space site forces per slot (half-interaction real space)
    // real-space pair list (mixed contexts with beads beyond the half-interaction
    // kernel in boxes with r_c + 2 RL_SPREAD <= L/2): rl_ok marks the context
    // eligible, rl_form 0 runs the real space over the list there, 1 over all pairs
    bool rl_ok = false;
    int rl_form = 0, rl_cap = 0;
    unsigned short *rl_list = nullptr;
    int *rl_cnt = nullptr, *rl_jobs = nullptr, *rl_count = nullptr, *rl_wide = nullptr;
    uint4 *rl_state = nullptr;
    float4 *rl_ref = nullptr;
    std::string err;
    Consts K;
    std::vector<qtg_system_desc> desc;
    std::vector<SysDev> sys_h;
    std::vector<double> kc_sq;
    std::vector<int> cw_begin, cw_count;  // column work ranges per system
    SysDev *sys_d = nullptr;
    int n_sys = 0;
    size_t total_dof = 0, total_disp = 0, total_point = 0, total_list = 0, total_sites = 0;
    size_t total_nm = 0, total_modes = 0, total_kvec = 0, total_phase = 0, total_slots = 0;
    int max_mols = 0, max_kvec = 0, max_kmax = 0, max_p = 1, max_dof = 0;
    bool any_sc = false, mixed = false;
    // state
    double *q = nullptr, *p = nullptr, *f = nullptr, *fphys = nullptr, *disp = nullptr;
    int *point = nullptr, *list = nullptr, *point_full = nullptr, *list_full = nullptr;
    int *rebuilt = nullptr;  // per base job: 1 after a rebuild of that bead's lists (per-call steps clear it)
    // mapped, page-locked mailbox of the per-call steps: the caller's array
    // pointers for the stage kernels, and the step's small results, which arrive
    // by asynchronous copies or stage-kernel stores and resolve with one stream
    // synchronisation (host addresses; *_d: the same memory seen from the device)
    CallBox *box = nullptr, *box_d = nullptr;
    double *box_energy = nullptr, *box_energy_d = nullptr;  // [max_p] per-bead energies
    int *box_rebuilt = nullptr, *box_rebuilt_d = nullptr;    // [max_p] per-bead rebuild flags
    size_t total_point_full = 0, total_list_full = 0;
    // Verlet-list build scratch
    size_t total_cells = 0;
    int *cnt_half = nullptr, *cnt_full = nullptr, *cell_start = nullptr, *cell_mol = nullptr;
    int *rb_jobs = nullptr, *rb_count = nullptr;
    float4 *wpos = nullptr;
    double *charge = nullptr, *mass = nullptr, *inv_mass = nullptr, *sqrt_mass = nullptr;
    double *cf_acc = nullptr;  // mean-centroid-force sums of constrained systems, per dof (like mass)
    size_t n_cf = 0;
    double *qdisp = nullptr, *fdisp = nullptr, *fsr = nullptr, *dirv = nullptr, *sc_scale = nullptr;
    double *stage = nullptr;  // per-call staging (total_dof doubles)
    double *noise = nullptr;  // per-call noise (2 + (Pmax-1) * 9Nmax)
    size_t noise_len = 0;
    KVec *kvec = nullptr;
    int *kpk = nullptr;  // FP32 k-force packing code per k (see build_columns)
    int4 *kfc = nullptr;     // per column: kx, ky, m, packed slot of kz = 0
    float2 *kfb = nullptr;   // per column: FP32 reciprocal-lattice components of kx, ky
    float4 *wpk = nullptr;   // packed +-kz force weights, 2 per k slot
    KCol *kcol = nullptr;
    KGroup *kgrp = nullptr;
    KBatch *kbatch = nullptr;
    int max_grp = 0, max_batch = 0;
    int kz = 4;  // |kz| values per structure-factor group (3 or 4, chosen at creation)
    double *nm = nullptr;
    ModeCoef *modes = nullptr;
    // per-slot scratch
    void *sites = nullptr, *tan_sites = nullptr, *phase = nullptr, *opos = nullptr;
    double *part = nullptr;           // [MAX_PART][total_sites][3]
    double2 *skp = nullptr, *dskp = nullptr;  // [MAX_SC][total_k]
    double2 *wsk = nullptr, *wdsk = nullptr;  // [total_k] (sized for FP64)
    size_t total_k = 0;
    double *energy = nullptr;      // per slot: energies of the base evaluations
    double *energy_aux = nullptr;  // per slot: displaced / derivative evaluations
    // job tables
    Table base, fd, tan, fd_sc, tan_sc;
    std::vector<int> fd_begin, fd_count, tan_begin, tan_count;  // per system
    int *base_sys = nullptr, *base_bead = nullptr;  // (system, bead) of every base job
    int *odd_sys = nullptr, *odd_bead = nullptr;    // odd beads of even-P systems
    std::vector<int> odd_begin, odd_count;
    int n_odd = 0;
    int *sc_sys = nullptr, *sc_bead = nullptr;      // odd beads of SC systems (stepper)
    int n_sc_odd = 0;
    ColWork *colwork = nullptr;
    int n_colwork = 0;
    double *cw_part = nullptr;    // [n_colwork][4] block partials of the ordered system sums
    unsigned *fin_ticket = nullptr;  // systems closed by a fused end step
    unsigned *cw_ticket = nullptr;  // [n_sys] arrival tickets of those sums
    // run state
    SysAcc *acc = nullptr;
    SysRun *run = nullptr;
    double *est = nullptr;
    int max_records = 4096;
    unsigned long long *step = nullptr, *records = nullptr;
    unsigned *status = nullptr;
    double *red_out = nullptr;  // small reduction output
    bool forces_ready = false;
    int tune[3] = {0, 0, 0};  // real-space j-chunks, structure-factor site chunks, k-chunks (0: heuristic)
    struct Surrogate {        // learned centroid correction attached to a P = 1 system
        int sys = -1;
        float out_scale = 1.f;
        __nv_bfloat16 *wbf = nullptr, *feat = nullptr;
        float *bias = nullptr, *norm = nullptr, *desc = nullptr, *y = nullptr, *frames = nullptr;
        float4 *wrapped = nullptr;
    };
    std::vector<Surrogate> surrogates;
    // tabulated pair corrections: per-system tables (device), their coefficients,
    // the host copy of both, and whether any system carries one
    PairSplines *spl = nullptr;
    double *spl_coef = nullptr;
    std::vector<PairSplines> spl_h;
    std::vector<std::vector<double>> spl_coef_h;  // per system: the three types' coefficients back to back
    bool spl_any = false;
    void *flush_buf = nullptr;  // qtg_flush_l2's buffer
    int flush_val = 1;
    int n_sm = 148;
    unsigned long long h2d_bytes = 0, d2h_bytes = 0;  // host <-> device traffic of the per-call entries
    // per-call ring-polymer steps captured as graphs, by (system, NVT, caller noise): graph, kernels in it
    std::map<int, std::pair<cudaGraphExec_t, unsigned long long>> call_graphs;
    std::vector<std::vector<double>> last_mass, last_charge;  // per system: the arrays last uploaded
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    unsigned long long graph_kernels[2] = {0, 0};
    unsigned long long launches = 0;
};

namespace {

qtg_status fail(qtg_ctx *c, qtg_status st, const std::string &msg) {
    if (c) c->err = msg;
    return st;
}

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(ctx, QTG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <typename T>
cudaError_t dalloc(T **p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e == cudaSuccess) e = cudaMemset(*p, 0, n * sizeof(T));
    return e;
}

EvalArgs eval_args(qtg_ctx *c, const Job *jobs, int n_jobs, const double *pos, double *out, int mode, int sr_only) {
    EvalArgs a;
    memset(&a, 0, sizeof(a));
    a.sys = c->sys_d;
    a.jobs = jobs;
    a.n_jobs = n_jobs;
    a.max_mols = c->max_mols;
    a.max_kvec = c->max_kvec;
    a.max_kmax = c->max_kmax;
    a.pos = pos;
    a.out = out;
    a.dir = c->dirv;
    a.charge = c->charge;
    a.point = c->point;
    a.list = c->list;
    a.point_full = c->point_full;
    a.list_full = c->list_full;
    a.kvec = c->kvec;
    a.kcol = c->kcol;
    a.kgrp = c->kgrp;
    a.kbatch = c->kbatch;
    a.kpk = c->kpk;
    a.kfc = c->kfc;
    a.kfb = c->kfb;
    a.wpk = c->wpk;
    a.max_grp = c->max_grp;
    a.kz = c->kz;
    a.max_batch = c->max_batch;
    a.sites = c->sites;
    a.sites_fix = c->sites_fix;
    a.rfix = c->rfix;
    a.opos = c->opos;
    a.ljf = c->ljf;
    a.intra = c->intra;
    a.phase = c->phase;
    a.tan_sites = c->tan_sites;
    a.part = c->part;
    a.total_sites = (long long)c->total_sites;
    a.skp = c->skp;
    a.dskp = c->dskp;
    a.wsk = c->wsk;
    a.wdsk = c->wdsk;
    a.total_k = (long long)c->total_k;
    a.energy = c->energy;
    a.status = c->status;
    a.mode = mode;
    a.sr_only = sr_only;
    a.tune_rj = c->tune[0];
    a.tune_sc = c->tune[1];
    a.tune_kc = c->tune[2];
    a.rl_on = (c->rl_ok && c->rl_form == 0) ? 1 : 0;
    a.rl_cap = c->rl_cap;
    a.rl_list = c->rl_list;
    a.rl_cnt = c->rl_cnt;
    a.rl_ref = c->rl_ref;
    a.rl_jobs = c->rl_jobs;
    a.rl_count = c->rl_count;
    a.rl_wide = c->rl_wide;
    a.rl_state = c->rl_state;
    a.c = c->K;
    return a;
}

EvalArgs aux_args(qtg_ctx *c, const Job *jobs, int n_jobs, const double *pos, double *out, int mode, int sr_only) {
    EvalArgs a = eval_args(c, jobs, n_jobs, pos, out, mode, sr_only);
    a.energy = c->energy_aux;
    return a;
}

// A force evaluation; with tabulated pair corrections attached, their forces and
// energies are added to the evaluation's output afterwards (forces and
// short-range finite-difference evaluations alike; not to the Ewald-derivative
// jobs of mode 1, nor to reciprocal-space-only calls).
void launch_eval(qtg_ctx *c, const EvalArgs &a) {
    if (c->mixed) launch_eval_mixed(a, c->stream, &c->launches, &c->forks);
    else launch_eval_fp64(a, c->stream, &c->launches);
    if (c->spl_any && a.mode == 0 && !a.sites_are_input) {
        SplineArgs s;
        s.sys = c->sys_d;
        s.jobs = a.jobs;
        s.n_jobs = a.n_jobs;
        s.max_mols = a.max_mols;
        s.pos = a.pos;
        s.out = a.out;
        s.out_prop = a.out_prop;
        s.energy = a.energy;
        s.tables = c->spl;
        s.coef = c->spl_coef;
        launch_pair_splines(s, c->mixed, c->stream, &c->launches);
    }
}

RingArgs ring_args(qtg_ctx *c, int sys, int flags) {
    RingArgs r;
    memset(&r, 0, sizeof(r));
    r.sys = c->sys_d;
    if (sys < 0) {
        r.work = c->colwork;
        r.n_work = c->n_colwork;
    } else {
        r.work = c->colwork + c->cw_begin[sys];
        r.n_work = c->cw_count[sys];
    }
    r.flags = flags;
    r.q = c->q;
    r.p = c->p;
    r.f = c->f;
    r.fphys = c->fphys;
    r.disp = c->disp;
    r.mass = c->mass;
    r.inv_mass = c->inv_mass;
    r.sqrt_mass = c->sqrt_mass;
    r.nm = c->nm;
    r.modes = c->modes;
    r.run = c->run;
    r.acc = c->acc;
    r.step = c->step;
    r.kcv_all_beads = -1;
    r.max_p = c->max_p;
    r.cf_acc = c->cf_acc;
    r.status = c->status;
    r.cw_part = c->cw_part;
    r.cw_ticket = c->cw_ticket;
    return r;
}

FinalizeArgs fin_args(qtg_ctx *c, int sys, int record, int draw_alpha) {
    FinalizeArgs f;
    memset(&f, 0, sizeof(f));
    f.sys = c->sys_d;
    f.n_sys = c->n_sys;
    f.energy = c->energy;
    f.acc = c->acc;
    f.run = c->run;
    f.est = c->est;
    f.max_records = c->max_records;
    f.step = c->step;
    f.records = c->records;
    f.status = c->status;
    f.record = record;
    f.draw_alpha = draw_alpha;
    f.sys_begin = sys < 0 ? 0 : sys;
    f.sys_end = sys < 0 ? c->n_sys : sys + 1;
    return f;
}

ScArgs sc_args(qtg_ctx *c) {
    ScArgs s;
    memset(&s, 0, sizeof(s));
    s.sys = c->sys_d;
    s.q = c->q;
    s.fphys = c->fphys;
    s.mass = c->mass;
    s.inv_mass = c->inv_mass;
    s.qdisp = c->qdisp;
    s.dirv = c->dirv;
    s.fdisp = c->fdisp;
    s.fsr = c->fsr;
    s.f = c->f;
    s.sc_scale = c->sc_scale;
    s.acc = c->acc;
    s.mixed = c->mixed ? 1 : 0;
    s.max_dof = c->max_dof;
    return s;
}

ListArgs list_args(qtg_ctx *c, int first_job, int n_jobs, int force) {
    ListArgs l;
    memset(&l, 0, sizeof(l));
    l.sys = c->sys_d;
    l.job_sys = c->base_sys + first_job;
    l.job_bead = c->base_bead + first_job;
    l.n_jobs = n_jobs;
    l.q = c->q;
    l.disp = c->disp;
    l.point = c->point;
    l.list = c->list;
    l.point_full = c->point_full;
    l.list_full = c->list_full;
    l.acc = c->acc;
    l.run = c->run;
    l.rebuilt = c->rebuilt;
    l.rb_jobs = c->rb_jobs;
    l.rb_count = c->rb_count;
    l.wpos = c->wpos;
    l.cnt_half = c->cnt_half;
    l.cnt_full = c->cnt_full;
    l.cell_start = c->cell_start;
    l.cell_mol = c->cell_mol;
    l.status = c->status;
    l.force_rebuild = force;
    l.max_mols = c->max_mols;
    return l;
}

// Mixed contexts whose beads are beyond the half-interaction real-space kernel,
// with the stepper's symmetric Verlet lists: the Lennard-Jones term runs over the
// list (k_lj) instead of every O-O pair (k_lj_dense, O(N^2) a bead).
bool lj_list_ok(const qtg_ctx *c) {
    return c->mixed && c->point_full && (3 * c->max_mols + 31) / 32 > HALF_MAX_TILES;
}

// Forces of the given systems (sys < 0: all): physical forces into fphys, the
// propagating force into f (SC assembly for SC systems or force_sc; copy for
// Trotter). Positions are read from q.
void enqueue_forces(qtg_ctx *c, int sys, bool force_sc) {
    const int jb = sys < 0 ? 0 : c->sys_h[sys].job_base;
    const int nj = sys < 0 ? (int)c->base.h.size() : c->sys_h[sys].n_beads;
    // the device-resident stepper (sys < 0) maintains the symmetric lists itself;
    // per-call entries work on the caller's half lists, except that the mixed
    // evaluation of the physical forces takes the dense Lennard-Jones kernel as
    // the stepper does (every O-O pair inside r_cut: the pairs a valid Verlet list
    // holds). The Suzuki-Chin finite-difference terms stay FP64 and list-based.
    const int full = sys < 0 ? 1 : 0;
    EvalArgs base = eval_args(c, c->base.d + jb, nj, c->q, c->fphys, 0, 0);
    base.lj_full = (full || c->mixed) ? 1 : 0;
    base.lj_list = (full && lj_list_ok(c)) ? 1 : 0;
    // mixed, second-order assembly for every system in the evaluation: the combine
    // writes the propagating force too, and the assembly kernel is not launched
    bool all_trotter = c->mixed && !force_sc;
    for (int k = (sys < 0 ? 0 : sys); all_trotter && k < (sys < 0 ? c->n_sys : sys + 1); ++k)
        all_trotter = c->sys_h[k].propagator != QTG_SUZUKI_CHIN;
    for (const auto &g : c->surrogates)  // a learned correction is added to fphys after the combine
        if (sys < 0 || g.sys == sys) all_trotter = false;
    if (all_trotter) base.out_prop = c->f;
    // learned centroid corrections of the systems that carry one (P = 1): the
    // descriptors, the network and the frames need the positions only and run
    // on their own branch beside the force evaluation; the correction is added
    // to fphys after the combine
    std::vector<SurrogateRun> runs;
    for (const auto &g : c->surrogates) {
        if (sys >= 0 && g.sys != sys) continue;
        const SysDev &S = c->sys_h[g.sys];
        SurrogateRun r;
        r.pos = c->q + S.q_off;
        r.f = c->fphys + S.q_off;
        r.n_mols = S.n_mols;
        r.n_sm = c->n_sm;
        for (int k = 0; k < 3; ++k) r.box[k] = S.box[k];
        r.wbf = g.wbf;
        r.bias = g.bias;
        r.norm = g.norm;
        r.out_scale = g.out_scale;
        r.desc = g.desc;
        r.y = g.y;
        r.frames = g.frames;
        r.feat = g.feat;
        r.wrapped = g.wrapped;
        r.status = c->status;
        runs.push_back(r);
    }
    if (!runs.empty()) {
        cudaEventRecord(c->sur_fork, c->stream);
        cudaStreamWaitEvent(c->sur_stream, c->sur_fork, 0);
        for (const auto &r : runs) launch_surrogate_prepare(r, c->sur_stream, &c->launches);
        cudaEventRecord(c->sur_join, c->sur_stream);
    }
    launch_eval(c, base);
    if (!runs.empty()) {
        cudaStreamWaitEvent(c->stream, c->sur_join, 0);
        for (const auto &r : runs) launch_surrogate_apply(r, c->stream, &c->launches);
    }
    // odd beads that need the Suzuki-Chin force gradient
    const int *osys, *obead;
    const Job *fdj, *tanj;
    int n_odd, fdn, tn;
    if (sys < 0) {
        osys = c->sc_sys;
        obead = c->sc_bead;
        n_odd = c->n_sc_odd;
        fdj = c->fd_sc.d;
        fdn = (int)c->fd_sc.h.size();
        tanj = c->tan_sc.d;
        tn = (int)c->tan_sc.h.size();
    } else {
        const bool sc = force_sc || c->sys_h[sys].propagator == QTG_SUZUKI_CHIN;
        osys = c->odd_sys + c->odd_begin[sys];
        obead = c->odd_bead + c->odd_begin[sys];
        n_odd = sc ? c->odd_count[sys] : 0;
        fdj = c->fd.d + c->fd_begin[sys];
        fdn = sc ? c->fd_count[sys] : 0;
        tanj = c->tan.d + c->tan_begin[sys];
        tn = sc ? c->tan_count[sys] : 0;
    }
    ScArgs sa = sc_args(c);
    sa.force_sc = force_sc ? 1 : 0;
    if (n_odd > 0) {
        sa.job_sys = osys;
        sa.job_bead = obead;
        sa.n_jobs = n_odd;
        launch_sc_prepare(sa, c->stream, &c->launches);
        if (c->mixed) {
            launch_eval(c, aux_args(c, tanj, tn, c->q, c->fdisp, 1, 0));
            EvalArgs sr = aux_args(c, fdj, fdn, c->qdisp, c->fsr, 0, 1);
            sr.lj_full = full;
            launch_eval(c, sr);
        } else {
            EvalArgs fd = aux_args(c, fdj, fdn, c->qdisp, c->fdisp, 0, 0);
            fd.lj_full = full;
            launch_eval(c, fd);
        }
    }
    sa.job_sys = c->base_sys + jb;
    sa.job_bead = c->base_bead + jb;
    sa.n_jobs = nj;
    if (!all_trotter) launch_sc_finish(sa, c->stream, &c->launches);
}

// Whether the Verlet-list rebuild of a step can run beside its force evaluation:
// nothing in a mixed second-order evaluation reads the lists (the dense
// Lennard-Jones takes every pair inside r_cut); FP64 evaluations and the
// Suzuki-Chin finite-difference terms do.
bool rebuild_beside_forces(const qtg_ctx *c, int sys) {
    if (!c->mixed) return false;
    for (int k = (sys < 0 ? 0 : sys); k < (sys < 0 ? c->n_sys : sys + 1); ++k)
        if (c->sys_h[k].propagator == QTG_SUZUKI_CHIN) return false;
    return true;
}

void enqueue_step(qtg_ctx *c, int sys, int nvt, int ext_noise, bool pile_g) {
    RingArgs r = ring_args(c, sys, RF_KICK | RF_FWD | RF_CAYLEY | RF_BACK | RF_DISP | (nvt ? RF_THERMO : 0));
    r.noise = ext_noise ? c->noise : nullptr;
    r.pile_g = pile_g ? 1 : 0;
    // the finalize below draws from (seed, system, step) only: its draws are made
    // here by extra ring blocks, off the step's critical path. NVE steps draw and
    // set the next centroid factor too, so that an NVT step after NVE steps
    // rescales with the factor of its own step (draws at the step before it and
    // the current centroid kinetic energy), never a stale one.
    const bool ahead = sys < 0 && !ext_noise;
    r.n_draw = ahead ? c->n_sys : 0;
    launch_ring(r, c->stream, &c->launches);
    const int jb = sys < 0 ? 0 : c->sys_h[sys].job_base;
    const int nj = sys < 0 ? (int)c->base.h.size() : c->sys_h[sys].n_beads;
    const bool beside = rebuild_beside_forces(c, sys);
    if (beside) {  // on the side stream, joined before the closing kick
        cudaEventRecord(c->ev_fork[0], c->stream);
        cudaStreamWaitEvent(c->side_stream, c->ev_fork[0], 0);
        launch_skin_rebuild(list_args(c, jb, nj, 0), c->side_stream, &c->launches);
        cudaEventRecord(c->ev_join, c->side_stream);
        c->forks.lists_ready = c->ev_join;  // a Lennard-Jones term over the lists waits for them
    } else {
        launch_skin_rebuild(list_args(c, jb, nj, 0), c->stream, &c->launches);
    }
    enqueue_forces(c, sys, false);
    c->forks.lists_ready = nullptr;
    if (beside) cudaStreamWaitEvent(c->stream, c->ev_join, 0);
    FinalizeArgs fa = fin_args(c, sys, 1, 1);
    fa.noise = nullptr;
    fa.pile_g = pile_g ? 1 : 0;
    fa.pre_drawn = ahead ? 1 : 0;
    RingArgs e = ring_args(c, sys, 0);
    e.kick = 1;
    // the step's close (estimator record, next centroid factor, counters) runs in
    // the end step's block that finishes each system
    e.fuse_fin = 1;
    e.fin = fa;
    e.fin.ticket = c->fin_ticket;
    launch_end_step(e, c->stream, &c->launches);
}

qtg_status check_sys(qtg_ctx *ctx, int sys) {
    if (!ctx) return QTG_ERR_ARG;
    if (sys < 0 || sys >= ctx->n_sys) return fail(ctx, QTG_ERR_ARG, "system index out of range");
    return QTG_OK;
}

// the error a nonzero device status word stands for
qtg_status status_error(qtg_ctx *ctx, unsigned st) {
    if (st) {
        if (st & ST_LIST_OVERFLOW) return fail(ctx, QTG_ERR_LIST_OVERFLOW, "Verlet list exceeded list_size");
        if (st & ST_NONFINITE) return fail(ctx, QTG_ERR_NONFINITE, "non-finite energy or force");
        if (st & ST_GAMMA_LIMIT) return fail(ctx, QTG_ERR_NONFINITE, "gamma variate iteration limit reached");
        if (st & ST_DESC_OVERFLOW) return fail(ctx, QTG_ERR_ARG, "more than 256 atoms within the descriptor cutoff");
        if (st & ST_MMA_TIMEOUT) return fail(ctx, QTG_ERR_CUDA, "tensor-core completion wait ran out");
        if (st & ST_RLIST_OVERFLOW)
            return fail(ctx, QTG_ERR_LIST_OVERFLOW, "real-space pair list row exceeded its capacity");
    }
    return QTG_OK;
}

qtg_status sync_status(qtg_ctx *ctx) {
    CK(cudaStreamSynchronize(ctx->stream));
    unsigned st = 0;
    CK(cudaMemcpy(&st, ctx->status, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (st) CK(cudaMemset(ctx->status, 0, sizeof(unsigned)));
    return status_error(ctx, st);
}

#define CKS(expr)                            \
    do {                                     \
        qtg_status s_ = (expr);              \
        if (s_ != QTG_OK) return s_;         \
    } while (0)

cudaError_t up(qtg_ctx *c, void *dst, const void *src, size_t bytes) {
    c->h2d_bytes += bytes;
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream);
}
cudaError_t down(qtg_ctx *c, void *dst, const void *src, size_t bytes) {
    c->d2h_bytes += bytes;
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream);
}

qtg_status refresh_sys(qtg_ctx *ctx, int sys) {
    CK(cudaMemcpyAsync(ctx->sys_d + sys, &ctx->sys_h[sys], sizeof(SysDev), cudaMemcpyHostToDevice, ctx->stream));
    return QTG_OK;
}

// masses, their inverses and square roots (the kernels multiply instead of dividing)
qtg_status upload_masses(qtg_ctx *ctx, int sys, const double *mass) {
    const SysDev &S = ctx->sys_h[sys];
    if (ctx->last_mass.size() != ctx->sys_h.size()) ctx->last_mass.resize(ctx->sys_h.size());
    std::vector<double> &last = ctx->last_mass[sys];
    if (last.size() == (size_t)S.n_dof && memcmp(last.data(), mass, sizeof(double) * S.n_dof) == 0) return QTG_OK;
    last.assign(mass, mass + S.n_dof);
    ctx->h2d_bytes += 2 * sizeof(double) * S.n_dof;  // 1/m and sqrt(m)
    std::vector<double> im(S.n_dof), sm(S.n_dof);
    for (int k = 0; k < S.n_dof; ++k) {
        im[k] = 1.0 / mass[k];
        sm[k] = sqrt(mass[k]);
    }
    CK(up(ctx, ctx->mass + S.mass_off, mass, sizeof(double) * S.n_dof));
    CK(cudaMemcpyAsync(ctx->inv_mass + S.mass_off, im.data(), sizeof(double) * S.n_dof, cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaMemcpyAsync(ctx->sqrt_mass + S.mass_off, sm.data(), sizeof(double) * S.n_dof, cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));  // the host vectors go out of scope
    return QTG_OK;
}

qtg_status upload_charges(qtg_ctx *ctx, int sys, const double *charge) {
    SysDev &S = ctx->sys_h[sys];
    if (ctx->last_charge.size() != ctx->sys_h.size()) ctx->last_charge.resize(ctx->sys_h.size());
    std::vector<double> &last = ctx->last_charge[sys];
    if (last.size() == (size_t)S.n_sites && memcmp(last.data(), charge, sizeof(double) * S.n_sites) == 0)
        return QTG_OK;
    last.assign(charge, charge + S.n_sites);
    double self = 0.0;
    for (int i = 0; i < S.n_sites; ++i) self += 0.5 * S.ewald_pref * charge[i] * charge[i];
    S.self_energy = self;
    CK(up(ctx, ctx->charge + S.chg_off, charge, sizeof(double) * S.n_sites));
    return refresh_sys(ctx, sys);
}

}  // namespace

// ============================================================================
namespace {

// Drops the captured step graphs, so that the next qtg_run_steps captures
// the step again with the current launch shapes.
void drop_graphs(qtg_ctx *ctx) {
    for (int i = 0; i < 2; ++i) {
        if (ctx->graph[i]) cudaGraphExecDestroy(ctx->graph[i]);
        ctx->graph[i] = nullptr;
        ctx->graph_kernels[i] = 0;
    }
    for (auto &g : ctx->call_graphs) cudaGraphExecDestroy(g.second.first);
    ctx->call_graphs.clear();
}

void free_surrogate(qtg_ctx::Surrogate &g) {
    void *ptrs[] = {g.wbf, g.feat, g.bias, g.norm, g.desc, g.y, g.frames, g.wrapped};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    g = qtg_ctx::Surrogate();
}

// Average duration (ms) of `iters` launches of `fn` on the context's stream.
template <typename F>
qtg_status time_on_stream(qtg_ctx *ctx, int iters, F fn, double *ms_out) {
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    fn();  // warm-up
    CK(cudaEventRecord(e0, ctx->stream));
    for (int i = 0; i < iters; ++i) fn();
    CK(cudaEventRecord(e1, ctx->stream));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms_out = (double)ms / iters;
    return QTG_OK;
}

}  // namespace

// Throughput of a dependent-FMA probe filling every SM (eight blocks of 256
// threads an SM, eight chains a thread), after one short untimed launch.
template <typename T, typename L>
qtg_status fma_peak(double *tflops, int iters, L launch) {
    if (!tflops) return QTG_ERR_ARG;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return QTG_ERR_NODEVICE;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return QTG_ERR_NODEVICE;
    T *out = nullptr;
    if (cudaMalloc(&out, sizeof(T)) != cudaSuccess) return QTG_ERR_CUDA;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8;
    launch(out, blocks, 256);
    cudaEventRecord(e0, nullptr);
    launch(out, blocks, iters);
    cudaEventRecord(e1, nullptr);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess || ms <= 0.f) return QTG_ERR_CUDA;
    const double flops = 2.0 * 8.0 * (double)iters * blocks * 256.0;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return QTG_OK;
}

extern "C" {

const char *qtg_status_string(int s) {
    switch (s) {
        case QTG_OK: return "ok";
        case QTG_ERR_ARG: return "invalid argument";
        case QTG_ERR_CUDA: return "CUDA error";
        case QTG_ERR_LIST_OVERFLOW: return "Verlet list overflow";
        case QTG_ERR_NONFINITE: return "non-finite value";
        case QTG_ERR_STATE: return "invalid state";
        case QTG_ERR_NODEVICE: return "no sm_103 device";
        default: return "unknown status";
    }
}

const char *qtg_last_error(const qtg_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

qtg_status qtg_create(const qtg_system_desc *systems, int n_systems, int precision, qtg_ctx **out) {
    if (!out || !systems || n_systems <= 0) return QTG_ERR_ARG;
    *out = nullptr;
    if (precision != QTG_FP64 && precision != QTG_MIXED) return QTG_ERR_ARG;
    for (int s = 0; s < n_systems; ++s) {
        const qtg_system_desc &d = systems[s];
        if (d.n_mols < 2 || d.n_beads < 1 || d.n_beads > 128) return QTG_ERR_ARG;
        if (d.n_beads > 1 && (d.n_beads % 2) && d.propagator == QTG_SUZUKI_CHIN) return QTG_ERR_ARG;
        if (!(d.box_bohr[0] > 0 && d.box_bohr[1] > 0 && d.box_bohr[2] > 0)) return QTG_ERR_ARG;
        if (!(d.temp_K > 0) || !(d.dt_fs > 0) || !(d.eps_ewald > 0 && d.eps_ewald < 1)) return QTG_ERR_ARG;
        if (d.propagator != QTG_SUZUKI_CHIN && d.propagator != QTG_TROTTER) return QTG_ERR_ARG;
        if (d.thermostat < 0 || d.thermostat > 2) return QTG_ERR_ARG;
        if (d.thermostat == QTG_THERMO_PILE_L && !(d.tau0_fs > 0)) return QTG_ERR_ARG;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return QTG_ERR_NODEVICE;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) return QTG_ERR_NODEVICE;
    if (prop.major != 10 || prop.minor != 3) return QTG_ERR_NODEVICE;

    qtg_ctx *ctx = new qtg_ctx();
    ctx->device = dev;
    ctx->precision = precision;
    ctx->mixed = precision == QTG_MIXED;
    ctx->K = make_consts();
    ctx->n_sys = n_systems;
    ctx->desc.assign(systems, systems + n_systems);
    const Consts &K = ctx->K;
    std::vector<KVec> kall;
    std::vector<int> kpk_all;
    std::vector<int4> kfc_all;
    std::vector<float2> kfb_all;
    std::vector<KCol> call;
    std::vector<KGroup> gall;
    std::vector<KBatch> ball;
    std::vector<double> nm_all;
    std::vector<ModeCoef> mode_all;
    std::vector<double> chg_all, mass_all;
    long long q_off = 0, d_off = 0, pt_off = 0, ls_off = 0, chg_off = 0, mass_off = 0, pf_off = 0, lf_off = 0;
    long long lc_off = 0;
    long long nm_off = 0, mode_off = 0;
    int job_base = 0;
    for (int s = 0; s < n_systems; ++s) {
        const qtg_system_desc &d = systems[s];
        SysDev S;
        memset(&S, 0, sizeof(S));
        const int N = d.n_mols, P = d.n_beads;
        S.n_mols = N;
        S.n_beads = P;
        S.n_sites = 3 * N;
        S.n_dof = 9 * N;
        S.propagator = d.propagator;
        S.thermostat = d.thermostat;
        S.job_base = job_base;
        S.cols_per_block = 256 / P;
        S.seed = d.seed;
        for (int k = 0; k < 3; ++k) {
            S.box[k] = d.box_bohr[k];
            S.inv_box[k] = 1.0 / d.box_bohr[k];
            S.boxf[k] = (float)S.box[k];
            S.inv_boxf[k] = (float)S.inv_box[k];
        }
        // two images of an O-O pair tied in dimension d are both L_d / 2 away in d: the
        // tie can change the Lennard-Jones cutoff decision only when (L_d / 2)^2 is not
        // clearly above r_cut^2
        S.lj_tie_mask = 0;
        for (int k = 0; k < 3; ++k)
            if (0.25 * S.box[k] * S.box[k] < 1.001 * K.r_cut_sq) S.lj_tie_mask |= 1 << k;
        // water.cpp:76-157 with the box given directly
        S.beta = 1.0 / (K.K2au * d.temp_K);
        S.beta_n = S.beta / P;
        S.inv_sqrt_beta_n = 1.0 / sqrt(S.beta_n);
        const double omega_p = 1.0 / S.beta_n;
        S.omega_psq = omega_p * omega_p;
        S.inv_p = 1.0 / P;
        S.sqrt_inv_p = sqrt(1.0 / P);
        S.half_omega_psq = 0.5 * S.omega_psq;
        S.half_nd_beta = 0.5 * S.n_dof / S.beta;
        S.dt = d.dt_fs * K.fs2au;
        S.halfdt = 0.5 * S.dt;
        S.eps_sc = d.eps_sc;
        const double vol = S.box[0] * S.box[1] * S.box[2];
        const double rho_ox = N / vol;
        S.list_size = (int)std::round(4.0 * K.r_skin * K.r_skin * K.r_skin * N * rho_ox);
        const double acc = sqrt(-log(d.eps_ewald));
        const double rho = (3 * N) / vol;
        const double min_box = std::min(std::min(S.box[0], S.box[1]), S.box[2]);
        const double max_box = std::max(std::max(S.box[0], S.box[1]), S.box[2]);
        S.k_pref = 2.0 * PI_REF / vol;
        // forces.cpp:574-584
        double kappa = 2.6 * pow(rho / vol, 1.0 / 6.0);
        double rc = acc / kappa;
        if (rc > 0.5 * min_box) {
            rc = 0.5 * min_box;
            kappa = acc / rc;
        }
        S.kappa = kappa;
        S.rc_sq = rc * rc;
        const double kc = 2.0 * acc * kappa;
        S.k_max = (int)(kc * max_box / (2.0 * PI_REF));
        S.ewald_pref = 2.0 * kappa / sqrt(PI_REF);
        S.kappaf = (float)kappa;
        S.kappa_sqf = (float)(kappa * kappa);
        S.rc_sqf = (float)S.rc_sq;
        S.ewald_preff = (float)S.ewald_pref;
        set_float_consts(S);
        S.r_cut_sq = K.r_cut_sq;
        S.r_skin_sq = K.r_skin_sq;
        S.skin_margin = K.r_skin - K.r_cut;
        S.c1_centroid = d.thermostat == QTG_THERMO_PILE_L ? exp(-S.dt / (d.tau0_fs * K.fs2au)) : 0.0;
        S.c2n_centroid = sqrt(1.0 - S.c1_centroid * S.c1_centroid) * S.inv_sqrt_beta_n;
        std::vector<KVec> kv, kord;
        std::vector<KCol> cols;
        std::vector<KBatch> bats;
        enumerate_k(S, kc * kc, kv);
        std::vector<int> kp;
        build_columns(kv, kord, cols, bats, kp, &S.n_col_half, &S.n_batch_half, &S.n_kvec_half);
        kpk_all.insert(kpk_all.end(), kp.begin(), kp.end());
        for (const KCol &c : cols) {
            kfc_all.push_back(make_int4(c.kx, c.ky, c.m, kp[c.k_begin + c.m] >> 8));
            kfb_all.push_back(make_float2(S.kbf[0] * (float)c.kx, S.kbf[1] * (float)c.ky));
        }
        S.n_kvec_ref = (int)kv.size();
        S.n_kvec = (int)kord.size();
        S.kvec_off = (int)kall.size();
        S.col_off = (int)call.size();
        S.n_col = (int)cols.size();
        S.batch_off = (int)ball.size();
        S.n_batch = (int)bats.size();
        kall.insert(kall.end(), kord.begin(), kord.end());
        call.insert(call.end(), cols.begin(), cols.end());
        ball.insert(ball.end(), bats.begin(), bats.end());
        ctx->max_batch = std::max(ctx->max_batch, S.n_batch);
        ctx->kc_sq.push_back(kc * kc);
        S.q_off = q_off;
        S.d_off = d_off;
        S.pt_off = pt_off;
        S.ls_off = ls_off;
        S.pf_off = pf_off;
        S.lf_off = lf_off;
        // Verlet-list cell grid: side >= r_skin / 2 (with a margin over the FP32 pair
        // test's band), five or more cells a side, at most 20
        {
            const double cell_min = 0.5 * K.r_skin * (1.0 + 1e-3);
            bool cells = true;
            for (int k = 0; k < 3; ++k) {
                S.lc_n[k] = std::min(20, (int)std::floor(S.box[k] / cell_min));
                cells = cells && S.lc_n[k] >= 5;
            }
            S.lc_cells = cells ? S.lc_n[0] * S.lc_n[1] * S.lc_n[2] : 0;
            if (!cells) S.lc_n[0] = S.lc_n[1] = S.lc_n[2] = 1;
            S.lc_off = lc_off;
            lc_off += (long long)P * (S.lc_cells + 1);
        }
        S.chg_off = chg_off;
        S.mass_off = mass_off;
        S.nm_off = nm_off;
        S.mode_off = mode_off;
        q_off += (long long)P * 9 * N;
        d_off += (long long)P * 3 * N;
        pt_off += (long long)P * N;
        ls_off += (long long)P * S.list_size;
        pf_off += (long long)P * (N + 1);
        lf_off += (long long)P * 2 * S.list_size;
        chg_off += 3 * N;
        mass_off += 9 * N;
        nm_off += (long long)P * P;
        mode_off += P;
        job_base += P;
        std::vector<double> C;
        nm_matrix(P, C);
        nm_all.insert(nm_all.end(), C.begin(), C.end());
        const double piovern = PI_REF / P;
        const double pref = 2.0 / S.beta_n, pref_sq = pref * pref, gpref = 4.0 / S.beta_n;
        for (int k = 0; k < P; ++k) {
            ModeCoef mc;
            const double sn = sin(k * piovern);
            mc.w2 = pref_sq * sn * sn;
            mc.scale = 1.0 / sqrt(1.0 + 0.25 * mc.w2 * S.dt * S.dt);
            const double gk = gpref * sin(k * PI_REF / P);
            mc.c1 = exp(-S.dt * gk);
            mc.c2 = sqrt(1.0 - mc.c1 * mc.c1);
            mc.cq = mc.scale * S.halfdt;
            mc.cp = mc.scale * S.halfdt * mc.w2;
            mc.c2n = mc.c2 * S.inv_sqrt_beta_n;
            mode_all.push_back(mc);
        }
        for (int m = 0; m < N; ++m) {
            chg_all.push_back(K.qo);
            chg_all.push_back(K.qh);
            chg_all.push_back(K.qh);
            for (int a = 0; a < 3; ++a)
                for (int k = 0; k < 3; ++k) mass_all.push_back(a == 0 ? K.mo : K.mh);
        }
        double self = 0.0;
        for (int i = 0; i < 3 * N; ++i) self += 0.5 * S.ewald_pref * chg_all[S.chg_off + i] * chg_all[S.chg_off + i];
        S.self_energy = self;
        ctx->sys_h.push_back(S);
        ctx->max_mols = std::max(ctx->max_mols, N);
        ctx->max_kvec = std::max(ctx->max_kvec, S.n_kvec);
        ctx->max_kmax = std::max(ctx->max_kmax, S.k_max);
        ctx->max_p = std::max(ctx->max_p, P);
        ctx->max_dof = std::max(ctx->max_dof, 9 * N);
        if (d.propagator == QTG_SUZUKI_CHIN && P > 1) ctx->any_sc = true;
    }
    // Structure-factor groups: runs of <= kz |kz| values of one column (each |kz|
    // standing for +kz and -kz), one thread each, 128 threads a block. The width
    // (3 or 4) is the one whose launch does less work by a simple model: whole
    // blocks of threads, each paying the column factor (~7 instructions a site) and
    // ~9 a |kz| (mixed, the three-multiplication form: ~8 and ~5), over every
    // system's half set, sites and beads.
    {
        const double per_col = ctx->mixed ? 8.0 : 7.0, per_kz = ctx->mixed ? 5.0 : 9.0;
        double cost[2] = {0.0, 0.0};
        for (int w = 0; w < 2; ++w) {
            const int kz = 3 + w;
            for (const SysDev &S : ctx->sys_h) {
                long long g = 0;
                for (int c = 0; c < S.n_col_half; ++c) g += (call[S.col_off + c].m + kz) / kz;
                cost[w] += (double)((g + 127) / 128 * 128) * (per_col + per_kz * kz) * S.n_sites * S.n_beads;
            }
        }
        ctx->kz = cost[0] < cost[1] ? 3 : 4;
        for (SysDev &S : ctx->sys_h) {
            S.grp_off = (int)gall.size();
            for (int c = 0; c < S.n_col; ++c) {
                if (c == S.n_col_half) S.n_grp_half = (int)gall.size() - S.grp_off;
                const int m = call[S.col_off + c].m;
                for (int az0 = 0; az0 <= m; az0 += ctx->kz) {
                    KGroup g;
                    g.col = c;
                    g.kz0 = az0;
                    g.n = std::min(ctx->kz, m - az0 + 1);
                    g.pad = 0;
                    gall.push_back(g);
                }
            }
            S.n_grp = (int)gall.size() - S.grp_off;
            if (S.n_col_half == S.n_col) S.n_grp_half = S.n_grp;
            ctx->max_grp = std::max(ctx->max_grp, S.n_grp);
        }
    }
    ctx->total_dof = (size_t)q_off;
    ctx->total_disp = (size_t)d_off;
    ctx->total_point = (size_t)pt_off;
    ctx->total_list = (size_t)ls_off;
    ctx->total_point_full = (size_t)pf_off;
    ctx->total_cells = (size_t)lc_off;
    ctx->total_list_full = (size_t)lf_off;
    ctx->total_nm = (size_t)nm_off;
    ctx->total_modes = (size_t)mode_off;
    ctx->total_kvec = kall.size();

    // scratch slots: one per base job (bead), sized for its system
    std::vector<long long> slot_site, slot_phase, slot_sk;
    long long so = 0, po = 0, ko = 0;
    for (int s = 0; s < n_systems; ++s) {
        const SysDev &S = ctx->sys_h[s];
        for (int b = 0; b < S.n_beads; ++b) {
            slot_site.push_back(so);
            slot_phase.push_back(po);
            slot_sk.push_back(ko);
            so += S.n_sites;
            po += (long long)3 * (S.k_max + 1) * S.n_sites;
            ko += S.n_kvec;
        }
    }
    ctx->total_slots = slot_site.size();
    ctx->total_sites = (size_t)so;
    ctx->total_phase = (size_t)po;
    ctx->total_k = (size_t)ko;
    auto mkjob = [&](int s, int b, int slot, int mode, long long pos_off) {
        Job j;
        j.sys = s;
        j.bead = b;
        j.slot = slot;
        j.mode = mode;
        j.pos_off = pos_off;
        j.out_off = pos_off;
        j.site_off = slot_site[slot];
        j.phase_off = slot_phase[slot];
        j.sk_off = slot_sk[slot];
        return j;
    };
    std::vector<int> bsys, bbead, osys, obead, scs, scb;
    for (int s = 0; s < n_systems; ++s) {
        const SysDev &S = ctx->sys_h[s];
        ctx->fd_begin.push_back((int)ctx->fd.h.size());
        ctx->tan_begin.push_back((int)ctx->tan.h.size());
        ctx->odd_begin.push_back((int)osys.size());
        for (int b = 0; b < S.n_beads; ++b) {
            ctx->base.h.push_back(mkjob(s, b, S.job_base + b, 0, S.q_off + (long long)b * S.n_dof));
            bsys.push_back(s);
            bbead.push_back(b);
        }
        if (S.n_beads % 2 == 0) {
            for (int b = 1; b < S.n_beads; b += 2) {
                ctx->fd.h.push_back(mkjob(s, b, S.job_base + b, 0, S.q_off + (long long)b * S.n_dof));
                ctx->fd.h.push_back(mkjob(s, b, S.job_base + b - 1, 0, S.q_off + (long long)(b - 1) * S.n_dof));
                ctx->tan.h.push_back(mkjob(s, b, S.job_base + b, 1, S.q_off + (long long)b * S.n_dof));
                osys.push_back(s);
                obead.push_back(b);
                if (S.propagator == QTG_SUZUKI_CHIN) {
                    scs.push_back(s);
                    scb.push_back(b);
                    ctx->fd_sc.h.push_back(ctx->fd.h[ctx->fd.h.size() - 2]);
                    ctx->fd_sc.h.push_back(ctx->fd.h[ctx->fd.h.size() - 1]);
                    ctx->tan_sc.h.push_back(ctx->tan.h.back());
                }
            }
        }
        ctx->fd_count.push_back((int)ctx->fd.h.size() - ctx->fd_begin[s]);
        ctx->tan_count.push_back((int)ctx->tan.h.size() - ctx->tan_begin[s]);
        ctx->odd_count.push_back((int)osys.size() - ctx->odd_begin[s]);
    }
    ctx->n_odd = (int)osys.size();
    ctx->n_sc_odd = (int)scs.size();
    std::vector<ColWork> cw;
    for (int s = 0; s < n_systems; ++s) {
        SysDev &S = ctx->sys_h[s];
        ctx->cw_begin.push_back((int)cw.size());
        for (int c0 = 0; c0 < S.n_dof; c0 += S.cols_per_block) {
            ColWork w;
            w.sys = s;
            w.col0 = c0;
            w.ncols = std::min(S.cols_per_block, S.n_dof - c0);
            w.slot = (int)cw.size();
            cw.push_back(w);
        }
        ctx->cw_count.push_back((int)cw.size() - ctx->cw_begin[s]);
        S.cw_begin = ctx->cw_begin[s];
        S.cw_count = ctx->cw_count[s];
    }
    ctx->n_colwork = (int)cw.size();
    ctx->noise_len = 2 + (size_t)(ctx->max_p - 1) * ctx->max_dof;

    init_force_kernel_attributes();
    init_list_kernel_attributes();
    init_propagate_kernel_attributes();
    {
        int dev = 0;
        if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&ctx->n_sm, cudaDevAttrMultiProcessorCount, dev);
    }
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
    ctx->stream = ctx->own_stream;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->side_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->sur_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->sur_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->sur_join, cudaEventDisableTiming);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&ctx->ev_fork[k], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaStreamCreateWithFlags(&ctx->forks.side[k], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->forks.fork, cudaEventDisableTiming);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&ctx->forks.join[k], cudaEventDisableTiming);
#define AL(ptr, n)                                  \
    if (e == cudaSuccess) e = dalloc(&(ptr), (n));
    AL(ctx->sys_d, n_systems);
    AL(ctx->q, ctx->total_dof);
    AL(ctx->p, ctx->total_dof);
    AL(ctx->f, ctx->total_dof);
    AL(ctx->fphys, ctx->total_dof);
    AL(ctx->qdisp, ctx->total_dof);
    AL(ctx->fdisp, ctx->total_dof);
    AL(ctx->fsr, ctx->total_dof);
    AL(ctx->dirv, ctx->total_dof);
    AL(ctx->stage, ctx->total_dof);
    AL(ctx->disp, ctx->total_disp);
    AL(ctx->point, ctx->total_point);
    AL(ctx->list, ctx->total_list);
    AL(ctx->point_full, ctx->total_point_full);
    AL(ctx->wpos, ctx->total_point);
    AL(ctx->cnt_half, ctx->total_point);
    AL(ctx->cnt_full, ctx->total_point);
    AL(ctx->cell_mol, ctx->total_point);
    AL(ctx->cell_start, ctx->total_cells);
    AL(ctx->list_full, ctx->total_list_full);
    AL(ctx->charge, chg_all.size());
    AL(ctx->mass, mass_all.size());
    AL(ctx->inv_mass, mass_all.size());
    AL(ctx->sqrt_mass, mass_all.size());
    AL(ctx->cf_acc, mass_all.size());
    ctx->n_cf = mass_all.size();
    AL(ctx->sc_scale, ctx->total_slots);
    AL(ctx->noise, ctx->noise_len);
    AL(ctx->kvec, kall.size());
    AL(ctx->kpk, kpk_all.size());
    AL(ctx->kfc, kfc_all.size());
    AL(ctx->kfb, kfb_all.size());
    AL(ctx->kcol, call.size());
    AL(ctx->kgrp, gall.size());
    AL(ctx->kbatch, ball.size());
    AL(ctx->nm, nm_all.size());
    AL(ctx->modes, mode_all.size());
    {
        // sized for the FP64 element types: 4 doubles per site, 2 per phase entry
        double *tmp = nullptr;
        AL(tmp, 4 * ctx->total_sites);
        ctx->sites = tmp;
        tmp = nullptr;
        AL(tmp, 4 * ctx->total_sites);
        ctx->tan_sites = tmp;
        tmp = nullptr;
        AL(tmp, 2 * ctx->total_phase);
        ctx->phase = tmp;
    }
    {
        double *tmp = nullptr;
        AL(tmp, 4 * (ctx->total_sites / 3));
        ctx->opos = tmp;
    }
    AL(ctx->ljf, ctx->total_sites / 3);
    AL(ctx->intra, 6 * ctx->total_sites);
    AL(ctx->sites_fix, ctx->total_sites);
    if (ctx->mixed) AL(ctx->rfix, 3 * ctx->total_sites);
    {
        // real-space pair list: rows hold the molecules whose M sites lie within
        // r_c + RL_SKIN + 2 RL_SPREAD (the prefilter radius of k_rlist_rows), at the
        // mean density and 15 % above it, plus 32
        ctx->rl_ok = ctx->mixed && (3 * ctx->max_mols + 31) / 32 > HALF_MAX_TILES;
        for (const SysDev &S : ctx->sys_h) {
            const double rc = sqrt(S.rc_sq), min_box = std::min(std::min(S.box[0], S.box[1]), S.box[2]);
            if (rc + 2.0 * RL_SPREAD > 0.5 * min_box || S.n_mols > 65535) ctx->rl_ok = false;
            const double R = rc + RL_SKIN + 2.0 * RL_SPREAD;
            const double nb = 1.15 * (4.0 / 3.0) * PI_REF * R * R * R * S.n_mols / (S.box[0] * S.box[1] * S.box[2]);
            const int cap = std::min(S.n_mols - 1, (int)std::ceil(nb) + 32);
            ctx->rl_cap = std::max(ctx->rl_cap, (cap + 7) / 8 * 8);
        }
        if (ctx->rl_ok) {
            const size_t n_jobs_max = std::max(std::max(ctx->base.h.size(), ctx->fd.h.size()), ctx->tan.h.size());
            AL(ctx->rl_list, (ctx->total_sites / 3) * (size_t)ctx->rl_cap);
            AL(ctx->rl_cnt, ctx->total_sites / 3);
            AL(ctx->rl_ref, ctx->total_sites);
            AL(ctx->rl_jobs, n_jobs_max);
            AL(ctx->rl_count, 1);
            AL(ctx->rl_wide, ctx->total_slots);
            AL(ctx->rl_state, ctx->total_slots);
            // NaN reference positions: the first evaluation of every slot builds its list
            if (e == cudaSuccess) e = cudaMemset(ctx->rl_ref, 0xff, sizeof(float4) * ctx->total_sites);
        }
    }
    AL(ctx->part, (size_t)MAX_PART * 3 * ctx->total_sites);
    AL(ctx->skp, (size_t)MAX_SC * ctx->total_k);
    AL(ctx->dskp, (size_t)MAX_SC * ctx->total_k);
    AL(ctx->wsk, ctx->total_k);
    AL(ctx->wpk, 2 * ctx->total_k);
    AL(ctx->wdsk, ctx->total_k);
    AL(ctx->energy, ctx->total_slots);
    AL(ctx->energy_aux, ctx->total_slots);
    AL(ctx->base.d, ctx->base.h.size());
    AL(ctx->rebuilt, ctx->base.h.size());
    AL(ctx->rb_jobs, ctx->base.h.size());
    AL(ctx->rb_count, 1);
    if (e == cudaSuccess) {
        void *pin = nullptr;
        const size_t bytes = sizeof(CallBox) + (sizeof(double) + sizeof(int)) * ctx->max_p;
        e = cudaHostAlloc(&pin, bytes, cudaHostAllocMapped);
        void *pin_d = nullptr;
        if (e == cudaSuccess) e = cudaHostGetDevicePointer(&pin_d, pin, 0);
        if (e == cudaSuccess) {
            memset(pin, 0, bytes);
            ctx->box = static_cast<CallBox *>(pin);
            ctx->box_energy = reinterpret_cast<double *>(ctx->box + 1);
            ctx->box_rebuilt = reinterpret_cast<int *>(ctx->box_energy + ctx->max_p);
            ctx->box_d = static_cast<CallBox *>(pin_d);
            ctx->box_energy_d = reinterpret_cast<double *>(ctx->box_d + 1);
            ctx->box_rebuilt_d = reinterpret_cast<int *>(ctx->box_energy_d + ctx->max_p);
        }
    }
    AL(ctx->fd.d, ctx->fd.h.size());
    AL(ctx->tan.d, ctx->tan.h.size());
    AL(ctx->fd_sc.d, ctx->fd_sc.h.size());
    AL(ctx->tan_sc.d, ctx->tan_sc.h.size());
    AL(ctx->base_sys, bsys.size());
    AL(ctx->base_bead, bbead.size());
    AL(ctx->odd_sys, osys.size());
    AL(ctx->odd_bead, obead.size());
    AL(ctx->sc_sys, scs.size());
    AL(ctx->sc_bead, scb.size());
    AL(ctx->colwork, cw.size());
    AL(ctx->cw_part, 4 * cw.size());
    AL(ctx->cw_ticket, n_systems);
    AL(ctx->fin_ticket, 1);
    AL(ctx->acc, n_systems);
    AL(ctx->run, n_systems);
    AL(ctx->est, (size_t)ctx->max_records * n_systems * 8);
    AL(ctx->step, 1);
    AL(ctx->records, 1);
    AL(ctx->status, 1);
    AL(ctx->red_out, 8);
#undef AL
    auto cp = [&](void *dst, const void *src, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    };
    cp(ctx->sys_d, ctx->sys_h.data(), sizeof(SysDev) * n_systems);
    cp(ctx->charge, chg_all.data(), sizeof(double) * chg_all.size());
    cp(ctx->mass, mass_all.data(), sizeof(double) * mass_all.size());
    {
        std::vector<double> im(mass_all.size()), sm(mass_all.size());
        for (size_t k = 0; k < mass_all.size(); ++k) {
            im[k] = 1.0 / mass_all[k];
            sm[k] = sqrt(mass_all[k]);
        }
        cp(ctx->inv_mass, im.data(), sizeof(double) * im.size());
        cp(ctx->sqrt_mass, sm.data(), sizeof(double) * sm.size());
    }
    cp(ctx->kvec, kall.data(), sizeof(KVec) * kall.size());
    cp(ctx->kpk, kpk_all.data(), sizeof(int) * kpk_all.size());
    cp(ctx->kfc, kfc_all.data(), sizeof(int4) * kfc_all.size());
    cp(ctx->kfb, kfb_all.data(), sizeof(float2) * kfb_all.size());
    cp(ctx->kcol, call.data(), sizeof(KCol) * call.size());
    cp(ctx->kgrp, gall.data(), sizeof(KGroup) * gall.size());
    cp(ctx->kbatch, ball.data(), sizeof(KBatch) * ball.size());
    cp(ctx->nm, nm_all.data(), sizeof(double) * nm_all.size());
    cp(ctx->modes, mode_all.data(), sizeof(ModeCoef) * mode_all.size());
    cp(ctx->base.d, ctx->base.h.data(), sizeof(Job) * ctx->base.h.size());
    cp(ctx->fd.d, ctx->fd.h.data(), sizeof(Job) * ctx->fd.h.size());
    cp(ctx->tan.d, ctx->tan.h.data(), sizeof(Job) * ctx->tan.h.size());
    cp(ctx->fd_sc.d, ctx->fd_sc.h.data(), sizeof(Job) * ctx->fd_sc.h.size());
    cp(ctx->tan_sc.d, ctx->tan_sc.h.data(), sizeof(Job) * ctx->tan_sc.h.size());
    cp(ctx->base_sys, bsys.data(), sizeof(int) * bsys.size());
    cp(ctx->base_bead, bbead.data(), sizeof(int) * bbead.size());
    cp(ctx->odd_sys, osys.data(), sizeof(int) * osys.size());
    cp(ctx->odd_bead, obead.data(), sizeof(int) * obead.size());
    cp(ctx->sc_sys, scs.data(), sizeof(int) * scs.size());
    cp(ctx->sc_bead, scb.data(), sizeof(int) * scb.size());
    cp(ctx->colwork, cw.data(), sizeof(ColWork) * cw.size());
    if (e == cudaSuccess) {
        std::vector<SysRun> runs(n_systems);
        for (auto &r : runs) {
            r.heat = 0.0;
            r.alpha = 1.0;
            r.cf_samples = r.list_builds = r.R_draw = r.g2_draw = 0.0;
            r.draw_step_plus1 = 0ull;
        }
        cp(ctx->run, runs.data(), sizeof(SysRun) * n_systems);
        if (e == cudaSuccess) e = cudaMemset(ctx->cf_acc, 0, sizeof(double) * ctx->n_cf);
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        ctx->err = std::string("allocation/upload failed: ") + cudaGetErrorString(e);
        qtg_destroy(ctx);
        return QTG_ERR_CUDA;
    }
    *out = ctx;
    return QTG_OK;
}

void qtg_destroy(qtg_ctx *ctx) {
    if (!ctx) return;
    for (int i = 0; i < 2; ++i)
        if (ctx->graph[i]) cudaGraphExecDestroy(ctx->graph[i]);
    void *ptrs[] = {ctx->sys_d, ctx->q, ctx->p, ctx->f, ctx->fphys, ctx->qdisp, ctx->fdisp, ctx->fsr,
                    ctx->dirv, ctx->stage, ctx->disp, ctx->point, ctx->list, ctx->point_full, ctx->list_full,
                    ctx->charge, ctx->mass, ctx->inv_mass, ctx->sqrt_mass, ctx->cf_acc,
                    ctx->sc_scale, ctx->noise, ctx->kvec, ctx->kcol, ctx->kgrp, ctx->kbatch, ctx->nm, ctx->modes, ctx->sites, ctx->tan_sites,
                    ctx->phase, ctx->opos, ctx->part, ctx->skp, ctx->dskp, ctx->wsk, ctx->wdsk, ctx->energy, ctx->energy_aux,
                    ctx->base.d, ctx->fd.d, ctx->tan.d, ctx->fd_sc.d, ctx->tan_sc.d, ctx->base_sys, ctx->base_bead, ctx->odd_sys, ctx->odd_bead, ctx->sc_sys,
                    ctx->sc_bead, ctx->colwork, ctx->acc, ctx->run, ctx->est, ctx->step, ctx->records,
                    ctx->status, ctx->red_out, ctx->rebuilt, ctx->cw_part, ctx->cw_ticket, ctx->kpk, ctx->ljf, ctx->fin_ticket, ctx->sites_fix, ctx->intra, ctx->kfc, ctx->kfb, ctx->wpk,
                    ctx->wpos, ctx->cnt_half, ctx->cnt_full, ctx->cell_start, ctx->cell_mol,
                    ctx->rb_jobs, ctx->rb_count, ctx->rl_list, ctx->rl_cnt, ctx->rl_ref, ctx->rl_jobs, ctx->rl_count, ctx->rl_wide, ctx->rl_state, ctx->rfix};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (ctx->box) cudaFreeHost(ctx->box);
    for (auto &g : ctx->surrogates) free_surrogate(g);
    if (ctx->spl) cudaFree(ctx->spl);
    if (ctx->spl_coef) cudaFree(ctx->spl_coef);
    if (ctx->flush_buf) cudaFree(ctx->flush_buf);
    for (auto &g : ctx->call_graphs) cudaGraphExecDestroy(g.second.first);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    if (ctx->side_stream) cudaStreamDestroy(ctx->side_stream);
    if (ctx->sur_stream) cudaStreamDestroy(ctx->sur_stream);
    for (cudaEvent_t ev : {ctx->ev_fork[0], ctx->ev_fork[1], ctx->ev_join, ctx->forks.fork, ctx->forks.join[0],
                           ctx->forks.join[1], ctx->sur_fork, ctx->sur_join})
        if (ev) cudaEventDestroy(ev);
    for (cudaStream_t st : {ctx->forks.side[0], ctx->forks.side[1]})
        if (st) cudaStreamDestroy(st);
    delete ctx;
}

qtg_status qtg_set_stream(qtg_ctx *ctx, void *stream) {
    if (!ctx) return QTG_ERR_ARG;
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return QTG_OK;
}

qtg_status qtg_system_info_get(const qtg_ctx *ctx, int sys, qtg_system_info *out) {
    if (!ctx || !out || sys < 0 || sys >= ctx->n_sys) return QTG_ERR_ARG;
    const SysDev &S = ctx->sys_h[sys];
    out->n_mols = S.n_mols;
    out->n_beads = S.n_beads;
    out->n_dof = S.n_dof;
    out->list_size = S.list_size;
    out->k_max = S.k_max;
    out->n_kvectors = S.n_kvec_ref;
    out->kappa = S.kappa;
    out->rc = sqrt(S.rc_sq);
    out->kc = sqrt(ctx->kc_sq[sys]);
    out->dt = S.dt;
    out->beta_n = S.beta_n;
    out->omega_psq = S.omega_psq;
    return QTG_OK;
}

qtg_status qtg_kernel_launches(const qtg_ctx *ctx, uint64_t *out) {
    if (!ctx || !out) return QTG_ERR_ARG;
    *out = ctx->launches;
    return QTG_OK;
}

qtg_status qtg_set_charges(qtg_ctx *ctx, int sys, const double *charge) {
    CKS(check_sys(ctx, sys));
    if (!charge) return fail(ctx, QTG_ERR_ARG, "null charge array");
    CKS(upload_charges(ctx, sys, charge));
    return sync_status(ctx);
}

qtg_status qtg_set_centroid_fixed(qtg_ctx *ctx, int sys, int fixed) {
    CKS(check_sys(ctx, sys));
    ctx->sys_h[sys].centroid_fixed = fixed ? 1 : 0;
    CK(cudaMemcpyAsync(ctx->sys_d + sys, &ctx->sys_h[sys], sizeof(SysDev), cudaMemcpyHostToDevice, ctx->stream));
    return sync_status(ctx);
}

qtg_status qtg_reset_centroid_force(qtg_ctx *ctx, int sys) {
    CKS(check_sys(ctx, sys));
    const SysDev &S = ctx->sys_h[sys];
    CK(cudaMemsetAsync(ctx->cf_acc + S.mass_off, 0, sizeof(double) * S.n_dof, ctx->stream));
    CK(cudaMemsetAsync(&ctx->run[sys].cf_samples, 0, sizeof(double), ctx->stream));
    return sync_status(ctx);
}

qtg_status qtg_get_centroid_force(qtg_ctx *ctx, int sys, double *f_mean, double *n_samples) {
    CKS(check_sys(ctx, sys));
    if (!f_mean || !n_samples) return fail(ctx, QTG_ERR_ARG, "null output");
    const SysDev &S = ctx->sys_h[sys];
    std::vector<double> acc(S.n_dof);
    double ns = 0.0;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(acc.data(), ctx->cf_acc + S.mass_off, sizeof(double) * S.n_dof, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&ns, &ctx->run[sys].cf_samples, sizeof(double), cudaMemcpyDeviceToHost));
    for (int i = 0; i < S.n_dof; ++i) f_mean[i] = ns > 0.0 ? acc[i] / ns : 0.0;
    *n_samples = ns;
    return QTG_OK;
}

qtg_status qtg_get_constants(qtg_constants *out) {
    if (!out) return QTG_ERR_ARG;
    const Consts K = make_consts();
    out->angs2bohr = K.angs2bohr;
    out->fs2au = K.fs2au;
    out->K2au = K.K2au;
    out->mo = K.mo;
    out->mh = K.mh;
    out->qo = K.qo;
    out->qh = K.qh;
    out->gamma_vs = K.gamma_vs;
    out->epslj = K.epslj;
    out->sigmalj6 = K.sigmalj6;
    out->sigmalj12 = K.sigmalj12;
    out->e_cut = K.e_cut;
    out->r_cut = K.r_cut;
    out->r_skin = K.r_skin;
    out->roheq = K.roheq;
    out->ar2 = K.ar2;
    out->ar3 = K.ar3;
    out->ar4fac = K.ar4fac;
    out->Dr = K.Dr;
    out->theta_eq = K.theta_eq;
    out->ktheta = K.ktheta;
    out->pi = PI_REF;
    return QTG_OK;
}

qtg_status qtg_register_host(void *ptr, size_t bytes) {
    if (!ptr || bytes == 0) return QTG_ERR_ARG;
    const cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterPortable | cudaHostRegisterMapped);
    if (e == cudaErrorHostMemoryAlreadyRegistered) {
        cudaGetLastError();
        return QTG_OK;
    }
    return e == cudaSuccess ? QTG_OK : QTG_ERR_CUDA;
}

qtg_status qtg_unregister_host(void *ptr) {
    if (!ptr) return QTG_ERR_ARG;
    const cudaError_t e = cudaHostUnregister(ptr);
    if (e == cudaErrorHostMemoryNotRegistered) {
        cudaGetLastError();
        return QTG_OK;
    }
    return e == cudaSuccess ? QTG_OK : QTG_ERR_CUDA;
}

qtg_status qtg_set_pair_splines(qtg_ctx *ctx, int sys, const qtg_pair_spline *oo, const qtg_pair_spline *oh,
                                const qtg_pair_spline *hh) {
    CKS(check_sys(ctx, sys));
    const qtg_pair_spline *in[3] = {oo, oh, hh};
    const bool on = oo || oh || hh;
    PairSplines T;
    memset(&T, 0, sizeof(T));
    std::vector<double> coef;
    for (int t = 0; t < 3; ++t) {
        if (!in[t]) continue;
        const qtg_pair_spline &p = *in[t];
        if (!p.values || p.n < 5 || !(p.step > 0) || !(p.cut_sq >= 0) || !std::isfinite(p.start))
            return fail(ctx, QTG_ERR_ARG, "pair spline: need >= 5 values, a positive step, a cutoff");
        // a pair inside the cutoff must lie on the table (as the reference's
        // cutoffs do: cut = start + step (n - 1))
        const double end = p.start + p.step * (p.n - 1);
        if (p.cut_sq > end * end * (1.0 + 1e-12))
            return fail(ctx, QTG_ERR_ARG, "pair spline: cutoff beyond the last knot");
        const size_t off = coef.size();
        coef.resize(off + (size_t)p.n + 2);
        if (!bspline_coefficients(p.values, p.n, p.step, p.left_deriv, p.right_deriv, coef.data() + off))
            return fail(ctx, QTG_ERR_ARG, "pair spline: coefficient solve failed");
        T.t[t].coef_off = (long long)off;  // relative to the system's block, rebased below
        T.t[t].n = p.n;
        T.t[t].start = p.start;
        T.t[t].inv_step = 1.0 / p.step;
        T.t[t].cut_sq = p.cut_sq;
    }
    T.on = on ? 1 : 0;
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->spl_h.empty()) {
        ctx->spl_h.assign(ctx->n_sys, PairSplines{});
        ctx->spl_coef_h.assign(ctx->n_sys, {});
    }
    ctx->spl_h[sys] = T;
    ctx->spl_coef_h[sys] = coef;
    // all systems' tables back to back, offsets rebased
    std::vector<PairSplines> all = ctx->spl_h;
    std::vector<double> cf;
    bool any = false;
    for (int k = 0; k < ctx->n_sys; ++k) {
        for (int t = 0; t < 3; ++t) all[k].t[t].coef_off += (long long)cf.size();
        cf.insert(cf.end(), ctx->spl_coef_h[k].begin(), ctx->spl_coef_h[k].end());
        any = any || all[k].on;
    }
    if (ctx->spl) cudaFree(ctx->spl);
    if (ctx->spl_coef) cudaFree(ctx->spl_coef);
    ctx->spl = nullptr;
    ctx->spl_coef = nullptr;
    CK(cudaMalloc(&ctx->spl, sizeof(PairSplines) * ctx->n_sys));
    CK(cudaMalloc(&ctx->spl_coef, sizeof(double) * std::max<size_t>(cf.size(), 1)));
    CK(cudaMemcpy(ctx->spl, all.data(), sizeof(PairSplines) * ctx->n_sys, cudaMemcpyHostToDevice));
    if (!cf.empty()) CK(cudaMemcpy(ctx->spl_coef, cf.data(), sizeof(double) * cf.size(), cudaMemcpyHostToDevice));
    ctx->spl_any = any;
    drop_graphs(ctx);
    ctx->forces_ready = false;
    return QTG_OK;
}

qtg_status qtg_detach_surrogate(qtg_ctx *ctx, int sys) {
    CKS(check_sys(ctx, sys));
    CK(cudaStreamSynchronize(ctx->stream));
    for (size_t i = 0; i < ctx->surrogates.size(); ++i)
        if (ctx->surrogates[i].sys == sys) {
            free_surrogate(ctx->surrogates[i]);
            ctx->surrogates.erase(ctx->surrogates.begin() + (long)i);
            drop_graphs(ctx);
            break;
        }
    return QTG_OK;
}

qtg_status qtg_attach_surrogate(qtg_ctx *ctx, int sys, const qtg_mlp_weights *w, const float *norm, float out_scale) {
    CKS(check_sys(ctx, sys));
    if (!w || !w->w1 || !w->w2 || !w->w3 || !w->b1 || !w->b2 || !w->b3 || !norm)
        return fail(ctx, QTG_ERR_ARG, "null surrogate array");
    const SysDev &S = ctx->sys_h[sys];
    if (S.n_beads != 1) return fail(ctx, QTG_ERR_ARG, "the centroid correction applies to P = 1 (centroid) systems");
    const double rc = 6.0 / 0.529177210903;
    for (int d = 0; d < 3; ++d)
        if (!(S.box[d] > 2.0 * rc)) return fail(ctx, QTG_ERR_ARG, "box sides must exceed twice the 6 A cutoff");
    CKS(qtg_detach_surrogate(ctx, sys));
    init_surrogate_kernel_attributes();
    qtg_ctx::Surrogate g;
    g.sys = sys;
    g.out_scale = out_scale;
    const int N = S.n_mols, n1 = QTG_MLP_HIDDEN * QTG_MLP_IN, n2 = QTG_MLP_HIDDEN * QTG_MLP_HIDDEN,
              n3 = QTG_MLP_OUT_PAD * QTG_MLP_HIDDEN;
    cudaError_t e = cudaSuccess;
    auto al = [&](void **p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    };
    al((void **)&g.wbf, sizeof(__nv_bfloat16) * (n1 + n2 + n3));
    al((void **)&g.bias, sizeof(float) * (2 * QTG_MLP_HIDDEN + QTG_MLP_OUT_PAD));
    al((void **)&g.norm, sizeof(float) * 2 * QTG_MLP_IN);
    al((void **)&g.desc, sizeof(float) * 3 * N * QTG_DESC_PER_ATOM);
    al((void **)&g.feat, sizeof(__nv_bfloat16) * 2 * N * QTG_MLP_IN);
    al((void **)&g.y, sizeof(float) * 2 * N * QTG_MLP_OUT_PAD);
    al((void **)&g.frames, sizeof(float) * 9 * N);
    al((void **)&g.wrapped, sizeof(float4) * 3 * N);
    auto cp = [&](void *dst, const void *src, size_t bytes, cudaMemcpyKind k) {
        if (e == cudaSuccess) e = cudaMemcpy(dst, src, bytes, k);
    };
    cp(g.wbf, w->w1, sizeof(__nv_bfloat16) * n1, cudaMemcpyDeviceToDevice);
    cp(g.wbf + n1, w->w2, sizeof(__nv_bfloat16) * n2, cudaMemcpyDeviceToDevice);
    cp(g.wbf + n1 + n2, w->w3, sizeof(__nv_bfloat16) * n3, cudaMemcpyDeviceToDevice);
    cp(g.bias, w->b1, sizeof(float) * QTG_MLP_HIDDEN, cudaMemcpyDeviceToDevice);
    cp(g.bias + QTG_MLP_HIDDEN, w->b2, sizeof(float) * QTG_MLP_HIDDEN, cudaMemcpyDeviceToDevice);
    cp(g.bias + 2 * QTG_MLP_HIDDEN, w->b3, sizeof(float) * QTG_MLP_OUT_PAD, cudaMemcpyDeviceToDevice);
    cp(g.norm, norm, sizeof(float) * 2 * QTG_MLP_IN, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        free_surrogate(g);
        return fail(ctx, QTG_ERR_CUDA, std::string("surrogate attach: ") + cudaGetErrorString(e));
    }
    ctx->surrogates.push_back(g);
    drop_graphs(ctx);
    ctx->forces_ready = false;
    return QTG_OK;
}

qtg_status qtg_set_masses(qtg_ctx *ctx, int sys, const double *mass) {
    CKS(check_sys(ctx, sys));
    if (!mass) return fail(ctx, QTG_ERR_ARG, "null mass array");
    CKS(upload_masses(ctx, sys, mass));
    return sync_status(ctx);
}

// ---- tier 1 ------------------------------------------------------------------------

qtg_status qtg_neighbour_list(qtg_ctx *ctx, int sys, const double *pos, int *point, int *list, double *disp,
                              int bead) {
    CKS(check_sys(ctx, sys));
    const SysDev &S = ctx->sys_h[sys];
    if (!pos || !point || !list || !disp || bead < 0 || bead >= S.n_beads) return fail(ctx, QTG_ERR_ARG, "bad argument");
    const size_t nd = S.n_dof;
    CK(up(ctx, ctx->q + S.q_off + bead * nd, pos + bead * nd, sizeof(double) * nd));
    launch_skin_rebuild(list_args(ctx, S.job_base + bead, 1, 1), ctx->stream, &ctx->launches);
    CK(down(ctx, point + (size_t)bead * S.n_mols, ctx->point + S.pt_off + (size_t)bead * S.n_mols, sizeof(int) * S.n_mols));
    CK(down(ctx, list + (size_t)bead * S.list_size, ctx->list + S.ls_off + (size_t)bead * S.list_size,
            sizeof(int) * S.list_size));
    CK(down(ctx, disp + (size_t)bead * 3 * S.n_mols, ctx->disp + S.d_off + (size_t)bead * 3 * S.n_mols,
            sizeof(double) * 3 * S.n_mols));
    CK(cudaMemsetAsync(ctx->acc + sys, 0, sizeof(SysAcc), ctx->stream));
    return sync_status(ctx);
}

static qtg_status upload_lists(qtg_ctx *ctx, int sys, const int *point, const int *list, int bead_lo, int bead_hi) {
    const SysDev &S = ctx->sys_h[sys];
    const int nb = bead_hi - bead_lo;
    CK(up(ctx, ctx->point + S.pt_off + (size_t)bead_lo * S.n_mols, point + (size_t)bead_lo * S.n_mols,
          sizeof(int) * S.n_mols * nb));
    CK(up(ctx, ctx->list + S.ls_off + (size_t)bead_lo * S.list_size, list + (size_t)bead_lo * S.list_size,
          sizeof(int) * (size_t)S.list_size * nb));
    return QTG_OK;
}

qtg_status qtg_get_forces(qtg_ctx *ctx, int sys, const double *pos, double *f, const double *charge,
                          const int *point, const int *list, int bead, double *energy) {
    CKS(check_sys(ctx, sys));
    const SysDev &S = ctx->sys_h[sys];
    if (!pos || !f || !point || !list || bead < 0 || bead >= S.n_beads) return fail(ctx, QTG_ERR_ARG, "bad argument");
    const size_t nd = S.n_dof;
    if (charge) CKS(upload_charges(ctx, sys, charge));
    CK(up(ctx, ctx->q + S.q_off + bead * nd, pos + bead * nd, sizeof(double) * nd));
    CKS(upload_lists(ctx, sys, point, list, bead, bead + 1));
    const int jb = S.job_base + bead;
    launch_eval(ctx, eval_args(ctx, ctx->base.d + jb, 1, ctx->q, ctx->fphys, 0, 0));
    CK(down(ctx, f + bead * nd, ctx->fphys + S.q_off + bead * nd, sizeof(double) * nd));
    double e = 0.0;
    CK(down(ctx, &e, ctx->energy + jb, sizeof(double)));
    CKS(sync_status(ctx));
    if (energy) *energy = e;
    return QTG_OK;
}

qtg_status qtg_kwald(qtg_ctx *ctx, int sys, const double *sites, double *f_sites, const double *charge, int bead,
                     double *energy) {
    CKS(check_sys(ctx, sys));
    const SysDev &S = ctx->sys_h[sys];
    if (!sites || !f_sites || bead < 0 || bead >= S.n_beads) return fail(ctx, QTG_ERR_ARG, "bad argument");
    const size_t nd = S.n_dof;
    if (charge) CKS(upload_charges(ctx, sys, charge));
    // sites in qdisp, the caller's site forces in stage (the k-space forces are added)
    CK(up(ctx, ctx->qdisp + S.q_off + bead * nd, sites + bead * nd, sizeof(double) * nd));
    CK(up(ctx, ctx->stage + S.q_off + bead * nd, f_sites + bead * nd, sizeof(double) * nd));
    const int jb = S.job_base + bead;
    EvalArgs a = eval_args(ctx, ctx->base.d + jb, 1, ctx->qdisp, ctx->stage, 0, 0);
    a.sites_are_input = 1;
    launch_kwald_only(a, ctx->mixed, ctx->stream, &ctx->launches);
    CK(down(ctx, f_sites + bead * nd, ctx->stage + S.q_off + bead * nd, sizeof(double) * nd));
    double e = 0.0;
    CK(down(ctx, &e, ctx->energy + jb, sizeof(double)));
    CKS(sync_status(ctx));
    if (energy) *energy = e;
    return QTG_OK;
}

static qtg_status read_energies(qtg_ctx *ctx, int sys, double *vsum, double *veven, double *sc_extra) {
    const SysDev &S = ctx->sys_h[sys];
    std::vector<double> e(S.n_beads);
    SysAcc acc;
    CK(down(ctx, e.data(), ctx->energy + S.job_base, sizeof(double) * S.n_beads));
    CK(down(ctx, &acc, ctx->acc + sys, sizeof(SysAcc)));
    CKS(sync_status(ctx));
    CK(cudaMemsetAsync(ctx->acc + sys, 0, sizeof(SysAcc), ctx->stream));
    double vs = 0.0, ve = 0.0;
    for (int b = 0; b < S.n_beads; ++b) {
        vs += e[b];
        if (b % 2 == 0) ve += e[b];
    }
    *vsum = vs;
    *veven = ve;
    *sc_extra = acc.sc_extra;
    return QTG_OK;
}

qtg_status qtg_force_eval_sc(qtg_ctx *ctx, int sys, const double *pos, double *f, const double *charge,
                             const double *mass, const int *point, const int *list, double *sc_pot, double *fphys,
                             double *energy) {
    CKS(check_sys(ctx, sys));
    const SysDev &S = ctx->sys_h[sys];
    if (!pos || !f || !point || !list || !fphys || S.n_beads % 2) return fail(ctx, QTG_ERR_ARG, "bad argument");
    const size_t nt = (size_t)S.n_beads * S.n_dof;
    if (charge) CKS(upload_charges(ctx, sys, charge));
    if (mass) CKS(upload_masses(ctx, sys, mass));
    CK(up(ctx, ctx->q + S.q_off, pos, sizeof(double) * nt));
    CKS(upload_lists(ctx, sys, point, list, 0, S.n_beads));
    CK(cudaMemsetAsync(ctx->acc + sys, 0, sizeof(SysAcc), ctx->stream));
    enqueue_forces(ctx, sys, true);
    CK(down(ctx, f, ctx->f + S.q_off, sizeof(double) * nt));
    CK(down(ctx, fphys, ctx->fphys + S.q_off, sizeof(double) * nt));
    double vs, ve, extra;
    CKS(read_energies(ctx, sys, &vs, &ve, &extra));
    if (sc_pot) *sc_pot = 2.0 * ve / S.n_beads;
    if (energy) *energy = (2.0 * ve + 4.0 * (vs - ve) + extra) / 3.0;
    return QTG_OK;
}

qtg_status qtg_force_eval_trotter(qtg_ctx *ctx, int sys, const double *pos, double *f, const double *charge,
                                  const int *point, const int *list, double *pot, double *energy) {
    CKS(check_sys(ctx, sys));
    const SysDev &S = ctx->sys_h[sys];
    if (!pos || !f || !point || !list) return fail(ctx, QTG_ERR_ARG, "bad argument");
    const size_t nt = (size_t)S.n_beads * S.n_dof;
    if (charge) CKS(upload_charges(ctx, sys, charge));
    CK(up(ctx, ctx->q + S.q_off, pos, sizeof(double) * nt));
    CKS(upload_lists(ctx, sys, point, list, 0, S.n_beads));
    launch_eval(ctx, eval_args(ctx, ctx->base.d + S.job_base, S.n_beads, ctx->q, ctx->fphys, 0, 0));
    CK(down(ctx, f, ctx->fphys + S.q_off, sizeof(double) * nt));
    double vs, ve, extra;
    CKS(read_energies(ctx, sys, &vs, &ve, &extra));
    if (pot) *pot = vs / S.n_beads;
    if (energy) *energy = vs;
    return QTG_OK;
}

qtg_status qtg_ftransform(qtg_ctx *ctx, int sys, double *a, int length, int forwards) {
    CKS(check_sys(ctx, sys));
    const SysDev &S = ctx->sys_h[sys];
    if (!a || length <= 0 || length > S.n_dof) return fail(ctx, QTG_ERR_ARG, "bad argument");
    const size_t nt = (size_t)S.n_beads * length;
    double *buf = ctx->stage + S.q_off;
    CK(up(ctx, buf, a, sizeof(double) * nt));
    launch_transform(ctx->sys_d, sys, S.n_beads, ctx->nm + S.nm_off, buf, length, forwards, ctx->stream,
                     &ctx->launches);
    CK(down(ctx, a, buf, sizeof(double) * nt));
    return sync_status(ctx);
}

qtg_status qtg_pile_g(qtg_ctx *ctx, int sys, double *p, const double *mass, const double *noise, double *heat) {
    CKS(check_sys(ctx, sys));
    const SysDev &S = ctx->sys_h[sys];
    if (!p) return fail(ctx, QTG_ERR_ARG, "bad argument");
    const size_t nt = (size_t)S.n_beads * S.n_dof;
    if (mass) CKS(upload_masses(ctx, sys, mass));
    CK(up(ctx, ctx->p + S.q_off, p, sizeof(double) * nt));
    if (noise) CK(up(ctx, ctx->noise, noise, sizeof(double) * (2 + (size_t)(S.n_beads - 1) * S.n_dof)));
    CK(cudaMemsetAsync(ctx->acc + sys, 0, sizeof(SysAcc), ctx->stream));
    CK(cudaMemsetAsync(&ctx->run[sys].heat, 0, sizeof(double), ctx->stream));
    RingArgs r = ring_args(ctx, sys, RF_THERMO);
    r.pile_g = 1;
    r.noise = noise ? ctx->noise : nullptr;
    launch_centroid_ke(r, ctx->stream, &ctx->launches);
    FinalizeArgs fa = fin_args(ctx, sys, 0, 1);
    fa.pile_g = 1;
    fa.noise = noise ? ctx->noise : nullptr;
    launch_finalize(fa, ctx->stream, &ctx->launches);
    launch_ring(r, ctx->stream, &ctx->launches);
    CK(down(ctx, p, ctx->p + S.q_off, sizeof(double) * nt));
    double h = 0.0;
    CK(down(ctx, &h, &ctx->run[sys].heat, sizeof(double)));
    CKS(sync_status(ctx));
    if (heat) *heat = -h;
    return QTG_OK;
}

qtg_status qtg_bussi(qtg_ctx *ctx, int sys, double *p, const double *mass, const double *noise, double *heat) {
    CKS(check_sys(ctx, sys));
    const SysDev &S = ctx->sys_h[sys];
    if (!p) return fail(ctx, QTG_ERR_ARG, "bad argument");
    if (mass) CKS(upload_masses(ctx, sys, mass));
    CK(up(ctx, ctx->p + S.q_off, p, sizeof(double) * S.n_dof));
    if (noise) CK(up(ctx, ctx->noise, noise, sizeof(double) * 2));
    RingArgs r = ring_args(ctx, sys, 0);
    r.noise = noise ? ctx->noise : nullptr;
    launch_bussi(r, sys, ctx->stream, &ctx->launches);
    CK(down(ctx, p, ctx->p + S.q_off, sizeof(double) * S.n_dof));
    double h = 0.0;
    CK(down(ctx, &h, &ctx->run[sys].heat, sizeof(double)));
    CKS(sync_status(ctx));
    if (heat) *heat = h;
    return QTG_OK;
}

qtg_status qtg_get_kcv(qtg_ctx *ctx, int sys, const double *q, const double *f, double *out) {
    CKS(check_sys(ctx, sys));
    const SysDev &S = ctx->sys_h[sys];
    if (!q || !f || !out) return fail(ctx, QTG_ERR_ARG, "bad argument");
    const size_t nt = (size_t)S.n_beads * S.n_dof;
    CK(up(ctx, ctx->q + S.q_off, q, sizeof(double) * nt));
    CK(up(ctx, ctx->fphys + S.q_off, f, sizeof(double) * nt));
    CK(cudaMemsetAsync(ctx->acc + sys, 0, sizeof(SysAcc), ctx->stream));
    RingArgs e = ring_args(ctx, sys, 0);
    e.kick = 0;
    e.kcv_all_beads = 0;  // even beads only, as path_integrals.cpp:37-44
    e.f = ctx->fphys;
    launch_end_step(e, ctx->stream, &ctx->launches);
    SysAcc acc;
    CK(down(ctx, &acc, ctx->acc + sys, sizeof(SysAcc)));
    CKS(sync_status(ctx));
    CK(cudaMemsetAsync(ctx->acc + sys, 0, sizeof(SysAcc), ctx->stream));
    *out = 0.5 * S.n_dof / S.beta + acc.kcv_tq / S.n_beads;
    return sync_status(ctx);
}

qtg_status qtg_get_conserved(qtg_ctx *ctx, int sys, double *q, double *p, const double *mass, double energy,
                             double *out) {
    CKS(check_sys(ctx, sys));
    const SysDev &S = ctx->sys_h[sys];
    if (!q || !p || !out) return fail(ctx, QTG_ERR_ARG, "bad argument");
    const size_t nt = (size_t)S.n_beads * S.n_dof;
    if (mass) CKS(upload_masses(ctx, sys, mass));
    CK(up(ctx, ctx->q + S.q_off, q, sizeof(double) * nt));
    CK(up(ctx, ctx->p + S.q_off, p, sizeof(double) * nt));
    CK(cudaMemsetAsync(ctx->red_out, 0, 2 * sizeof(double), ctx->stream));
    launch_transform(ctx->sys_d, sys, S.n_beads, ctx->nm + S.nm_off, ctx->q + S.q_off, S.n_dof, 1, ctx->stream,
                     &ctx->launches);
    launch_transform(ctx->sys_d, sys, S.n_beads, ctx->nm + S.nm_off, ctx->p + S.q_off, S.n_dof, 1, ctx->stream,
                     &ctx->launches);
    launch_nm_energy(ctx->sys_d, sys, S.n_beads, S.n_dof, ctx->q, ctx->p, ctx->mass, ctx->modes, ctx->red_out,
                     ctx->stream, &ctx->launches);
    launch_transform(ctx->sys_d, sys, S.n_beads, ctx->nm + S.nm_off, ctx->q + S.q_off, S.n_dof, 0, ctx->stream,
                     &ctx->launches);
    launch_transform(ctx->sys_d, sys, S.n_beads, ctx->nm + S.nm_off, ctx->p + S.q_off, S.n_dof, 0, ctx->stream,
                     &ctx->launches);
    double r[2];
    CK(down(ctx, r, ctx->red_out, 2 * sizeof(double)));
    CK(down(ctx, q, ctx->q + S.q_off, sizeof(double) * nt));
    CK(down(ctx, p, ctx->p + S.q_off, sizeof(double) * nt));
    CKS(sync_status(ctx));
    *out = energy + r[0] + r[1];
    return QTG_OK;
}

// Inputs of a per-call step. The physical forces are not among them: the
// reference's step overwrites fphys whole before reading it (force_eval_sc_nospline,
// forces.cpp:721, through get_forces_nospline, which zeroes its output at
// forces.cpp:483). The caller's Verlet lists go up only when a kernel of the step
// reads them (lists_read): the list-based Lennard-Jones of FP64 evaluations and of
// the Suzuki-Chin finite-difference terms, not the dense kernel of a mixed
// evaluation. A rebuild rewrites a bead's lists whole on the device either way.
static bool step_reads_lists(const qtg_ctx *ctx, int sys) {
    return !ctx->mixed || ctx->sys_h[sys].propagator == QTG_SUZUKI_CHIN;
}
static qtg_status upload_dynamic(qtg_ctx *ctx, int sys, const double *q, const double *p, const double *mass,
                                 const double *f, const double *charge, const int *point, const int *list,
                                 const double *disp) {
    const SysDev &S = ctx->sys_h[sys];
    const size_t nt = (size_t)S.n_beads * S.n_dof;
    if (charge) CKS(upload_charges(ctx, sys, charge));
    if (mass) CKS(upload_masses(ctx, sys, mass));
    CK(up(ctx, ctx->q + S.q_off, q, sizeof(double) * nt));
    CK(up(ctx, ctx->p + S.q_off, p, sizeof(double) * nt));
    CK(up(ctx, ctx->f + S.q_off, f, sizeof(double) * nt));
    CK(up(ctx, ctx->disp + S.d_off, disp, sizeof(double) * S.n_beads * 3 * S.n_mols));
    if (!step_reads_lists(ctx, sys)) return QTG_OK;
    return upload_lists(ctx, sys, point, list, 0, S.n_beads);
}

static qtg_status download_dynamic(qtg_ctx *ctx, int sys, double *q, double *p, double *f, double *fphys, int *point,
                                   int *list, double *disp) {
    const SysDev &S = ctx->sys_h[sys];
    const size_t nt = (size_t)S.n_beads * S.n_dof;
    CK(down(ctx, q, ctx->q + S.q_off, sizeof(double) * nt));
    CK(down(ctx, p, ctx->p + S.q_off, sizeof(double) * nt));
    CK(down(ctx, f, ctx->f + S.q_off, sizeof(double) * nt));
    if (fphys) CK(down(ctx, fphys, ctx->fphys + S.q_off, sizeof(double) * nt));
    CK(down(ctx, disp, ctx->disp + S.d_off, sizeof(double) * S.n_beads * 3 * S.n_mols));
    if (point) CK(down(ctx, point, ctx->point + S.pt_off, sizeof(int) * S.n_beads * S.n_mols));
    if (list) CK(down(ctx, list, ctx->list + S.ls_off, sizeof(int) * (size_t)S.n_beads * S.list_size));
    return QTG_OK;
}

// Whether the five state arrays of a per-call step can move by stage-kernel
// loads and stores: each must start in page-locked host memory that the device
// can address and that was not registered read-only, and no two may overlap (the
// copy path writes them back in a fixed order, the stage kernel all at once).
// The device addresses go to d*. The callers' arrays hold nt doubles (q, p, f,
// fphys) and nd (disp), as the reference's do.
static bool stageable(qtg_ctx *ctx, double *q, double *p, double *f, double *fphys, double *disp, size_t nt,
                      size_t nd, double **dq, double **dp, double **df, double **dfp, double **dd) {
    if (!ctx->box_d) return false;
    double *h[5] = {q, p, f, fphys, disp};
    double **d[5] = {dq, dp, df, dfp, dd};
    const size_t n[5] = {nt, nt, nt, nt, nd};
    for (int k = 0; k < 5; ++k) {
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, h[k]) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (at.type != cudaMemoryTypeHost || !at.devicePointer) return false;
        unsigned flags = 0;
        if (cudaHostGetFlags(&flags, h[k]) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (flags & cudaHostRegisterReadOnly) return false;
        *d[k] = static_cast<double *>(at.devicePointer);
        for (int j = 0; j < k; ++j)
            if (h[j] < h[k] + n[k] && h[k] < h[j] + n[j]) return false;
    }
    return true;
}

// The point and list arrays of a per-call step go back to the caller bead by
// bead, for the beads whose skin test rebuilt them during the call (the
// reference's neighbour_list writes a bead's point and list only when it
// rebuilds them, update.cpp:380-383); the caller's arrays of the other beads stay
// as they are. Reads the flags that the mailbox received before the stream was
// last synchronised.
static qtg_status download_rebuilt_lists(qtg_ctx *ctx, int sys, int *point, int *list) {
    const SysDev &S = ctx->sys_h[sys];
    bool any = false;
    for (int b = 0; b < S.n_beads; ++b) {
        if (!ctx->box_rebuilt[b]) continue;
        any = true;
        CK(down(ctx, point + (size_t)b * S.n_mols, ctx->point + S.pt_off + (size_t)b * S.n_mols,
                sizeof(int) * S.n_mols));
        CK(down(ctx, list + (size_t)b * S.list_size, ctx->list + S.ls_off + (size_t)b * S.list_size,
                sizeof(int) * S.list_size));
    }
    if (any) CK(cudaStreamSynchronize(ctx->stream));
    return QTG_OK;
}

// clear the per-bead rebuild flags of a per-call step
static cudaError_t clear_rebuilt(qtg_ctx *ctx, int sys) {
    const SysDev &S = ctx->sys_h[sys];
    return cudaMemsetAsync(ctx->rebuilt + S.job_base, 0, sizeof(int) * S.n_beads, ctx->stream);
}

// The small results of a per-call step -- the heat (heat: PIMD steps), per-bead
// energies and rebuild flags, the step's accumulators and the status word -- go
// to the pinned mailbox by asynchronous copies, after which the accumulators and
// the status word are cleared on the device. One stream synchronisation then
// resolves them all.
static cudaError_t post_small_results(qtg_ctx *ctx, int sys, bool heat) {
    const SysDev &S = ctx->sys_h[sys];
    cudaError_t e = cudaSuccess;
    auto chk = [&e](cudaError_t r) {
        if (e == cudaSuccess) e = r;
    };
    if (heat) chk(down(ctx, &ctx->box->heat_out, &ctx->run[sys].heat, sizeof(double)));
    chk(down(ctx, ctx->box_energy, ctx->energy + S.job_base, sizeof(double) * S.n_beads));
    chk(down(ctx, ctx->box_rebuilt, ctx->rebuilt + S.job_base, sizeof(int) * S.n_beads));
    chk(down(ctx, &ctx->box->acc, ctx->acc + sys, sizeof(SysAcc)));
    chk(down(ctx, &ctx->box->status, ctx->status, sizeof(unsigned)));
    chk(cudaMemsetAsync(ctx->acc + sys, 0, sizeof(SysAcc), ctx->stream));
    chk(cudaMemsetAsync(ctx->status, 0, sizeof(unsigned), ctx->stream));
    return e;
}

qtg_status qtg_update_class(qtg_ctx *ctx, int sys, double *q, double *p, const double *mass, double *f,
                            const double *charge, int *point, int *list, double *disp, double *energy) {
    CKS(check_sys(ctx, sys));
    const SysDev &S = ctx->sys_h[sys];
    if (S.n_beads != 1 || !q || !p || !f || !point || !list || !disp) return fail(ctx, QTG_ERR_ARG, "bad argument");
    CKS(upload_dynamic(ctx, sys, q, p, mass, f, charge, point, list, disp));
    CK(clear_rebuilt(ctx, sys));
    CK(cudaMemsetAsync(ctx->acc + sys, 0, sizeof(SysAcc), ctx->stream));
    launch_ring(ring_args(ctx, sys, RF_KICK | RF_VV | RF_DISP), ctx->stream, &ctx->launches);
    launch_skin_rebuild(list_args(ctx, S.job_base, 1, 0), ctx->stream, &ctx->launches);
    EvalArgs ea = eval_args(ctx, ctx->base.d + S.job_base, 1, ctx->q, ctx->fphys, 0, 0);
    ea.lj_full = ctx->mixed ? 1 : 0;  // mixed: the dense Lennard-Jones, as in enqueue_forces
    launch_eval(ctx, ea);
    // P = 1: the propagating force is the physical force
    CK(cudaMemcpyAsync(ctx->f + S.q_off, ctx->fphys + S.q_off, sizeof(double) * S.n_dof, cudaMemcpyDeviceToDevice,
                       ctx->stream));
    RingArgs e = ring_args(ctx, sys, 0);
    e.kick = 1;
    launch_end_step(e, ctx->stream, &ctx->launches);
    CKS(download_dynamic(ctx, sys, q, p, f, nullptr, nullptr, nullptr, disp));
    CK(post_small_results(ctx, sys, false));
    CK(cudaStreamSynchronize(ctx->stream));
    CKS(status_error(ctx, ctx->box->status));
    CKS(download_rebuilt_lists(ctx, sys, point, list));
    if (energy) *energy = ctx->box_energy[0];
    return QTG_OK;
}

qtg_status qtg_update_pimd(qtg_ctx *ctx, int sys, double *q, double *p, const double *mass, double *f, double *fphys,
                           const double *charge, int *point, int *list, double *disp, int is_nvt, const double *noise,
                           double *heat, double *pot, double *energy) {
    CKS(check_sys(ctx, sys));
    const SysDev &S = ctx->sys_h[sys];
    if (!q || !p || !f || !fphys || !point || !list || !disp) return fail(ctx, QTG_ERR_ARG, "bad argument");
    const size_t nt = (size_t)S.n_beads * S.n_dof, nd = (size_t)S.n_beads * 3 * S.n_mols;
    // q, p, f, fphys and disp in page-locked, mapped, writable and disjoint host
    // memory move inside the step's graph by the stage kernels; anything else by
    // copy calls
    double *dq = nullptr, *dp = nullptr, *df = nullptr, *dfp = nullptr, *dd = nullptr;
    const bool staged = !noise && stageable(ctx, q, p, f, fphys, disp, nt, nd, &dq, &dp, &df, &dfp, &dd);
    ctx->box->heat_in = heat ? *heat : 0.0;  // the previous call's synchronisation freed the slot
    if (staged) {
        if (charge) CKS(upload_charges(ctx, sys, charge));
        if (mass) CKS(upload_masses(ctx, sys, mass));
        if (step_reads_lists(ctx, sys)) CKS(upload_lists(ctx, sys, point, list, 0, S.n_beads));
        ctx->box->q = dq;
        ctx->box->p = dp;
        ctx->box->f = df;
        ctx->box->fphys = dfp;
        ctx->box->disp = dd;
        ctx->h2d_bytes += sizeof(double) * (3 * nt + nd + 1);
        ctx->d2h_bytes += sizeof(double) * (4 * nt + nd + 1 + S.n_beads) + sizeof(int) * S.n_beads +
                          sizeof(SysAcc) + sizeof(unsigned);
    } else {
        CKS(upload_dynamic(ctx, sys, q, p, mass, f, charge, point, list, disp));
        if (noise) CK(up(ctx, ctx->noise, noise, sizeof(double) * (2 + (size_t)(S.n_beads - 1) * S.n_dof)));
        CK(up(ctx, &ctx->run[sys].heat, &ctx->box->heat_in, sizeof(double)));
    }
    StageArgs sg;
    memset(&sg, 0, sizeof(sg));
    sg.box = ctx->box_d;
    sg.box_energy = ctx->box_energy_d;
    sg.box_rebuilt = ctx->box_rebuilt_d;
    sg.q = ctx->q + S.q_off;
    sg.p = ctx->p + S.q_off;
    sg.f = ctx->f + S.q_off;
    sg.fphys = ctx->fphys + S.q_off;
    sg.disp = ctx->disp + S.d_off;
    sg.nt = (long long)nt;
    sg.nd = (long long)nd;
    sg.run = ctx->run + sys;
    sg.energy = ctx->energy + S.job_base;
    sg.rebuilt = ctx->rebuilt + S.job_base;
    sg.acc = ctx->acc + sys;
    sg.status = ctx->status;
    sg.n_beads = S.n_beads;
    sg.blocks = std::max(1, std::min(8 * ctx->n_sm, (int)((4 * nt + nd + 255) / 256)));
    // the step's device work (update.cpp:271-401), the same for every call of this
    // (system, NVT, caller noise, staging): captured once as a graph and replayed
    auto step = [&]() -> cudaError_t {
        cudaError_t err = cudaSuccess;
        // staged NVT: the centroid-alpha kernel moves p and f in as it reads them,
        // while q and disp come in on the side stream
        const bool split_in = staged && is_nvt;
        if (staged && !split_in) {
            StageArgs si = sg;
            si.mask = STAGE_Q | STAGE_P | STAGE_F | STAGE_DISP;
            launch_stage_in(si, ctx->stream, &ctx->launches);
        }
        if (split_in) {
            err = cudaEventRecord(ctx->ev_fork[0], ctx->stream);
            if (err == cudaSuccess) err = cudaStreamWaitEvent(ctx->side_stream, ctx->ev_fork[0], 0);
            StageArgs si = sg;
            si.mask = STAGE_Q | STAGE_DISP;
            launch_stage_in(si, ctx->side_stream, &ctx->launches);
            if (err == cudaSuccess) err = cudaEventRecord(ctx->ev_join, ctx->side_stream);
        }
        if (err == cudaSuccess) err = cudaMemsetAsync(ctx->acc + sys, 0, sizeof(SysAcc), ctx->stream);
        if (err == cudaSuccess) err = clear_rebuilt(ctx, sys);
        if (is_nvt) {
            // centroid kinetic energy after the opening kick, the centroid draws and alpha
            RingArgs e = ring_args(ctx, sys, 0);
            e.noise = noise ? ctx->noise : nullptr;
            e.box = split_in ? ctx->box_d : nullptr;
            launch_centroid_alpha(e, sys, ctx->stream, &ctx->launches);
        }
        if (split_in && err == cudaSuccess) err = cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0);
        RingArgs r = ring_args(ctx, sys, RF_KICK | RF_FWD | RF_CAYLEY | RF_BACK | RF_DISP | (is_nvt ? RF_THERMO : 0));
        r.noise = noise ? ctx->noise : nullptr;
        r.pile_g = 1;
        // one extra block draws the next call's centroid variates beside the ring work
        r.n_draw = noise ? 0 : 1;
        r.draw_sys0 = sys;
        launch_ring(r, ctx->stream, &ctx->launches);
        if (err == cudaSuccess) err = cudaMemsetAsync(ctx->acc + sys, 0, sizeof(SysAcc), ctx->stream);
        // the rebuild runs on the side stream beside the forces where they do not
        // read the lists; staged, q and disp go back after it on that stream (both
        // final there), f and fphys after the forces, each beside the kernels that follow
        const bool beside = rebuild_beside_forces(ctx, sys);
        auto fork = [&](int k) {
            if (err == cudaSuccess) err = cudaEventRecord(ctx->ev_fork[k], ctx->stream);
            if (err == cudaSuccess) err = cudaStreamWaitEvent(ctx->side_stream, ctx->ev_fork[k], 0);
        };
        auto stage_out_side = [&](unsigned mask) {
            StageArgs so = sg;
            so.mask = mask;
            so.blocks = std::min(sg.blocks, 2 * ctx->n_sm);
            launch_stage_out(so, ctx->side_stream, &ctx->launches);
        };
        if (beside) {
            fork(0);
            launch_skin_rebuild(list_args(ctx, S.job_base, S.n_beads, 0), ctx->side_stream, &ctx->launches);
            if (staged) stage_out_side(STAGE_Q | STAGE_DISP);
        } else {
            launch_skin_rebuild(list_args(ctx, S.job_base, S.n_beads, 0), ctx->stream, &ctx->launches);
            if (staged) {
                fork(0);
                stage_out_side(STAGE_Q | STAGE_DISP);
            }
        }
        enqueue_forces(ctx, sys, false);
        if (staged) {
            fork(1);
            stage_out_side(STAGE_F | STAGE_FPHYS);
        }
        RingArgs e = ring_args(ctx, sys, 0);
        e.kick = 1;
        if (staged) {  // the end step writes p back and posts the small results itself
            e.post_box = sg.box;
            e.post_energy = sg.box_energy;
            e.post_rebuilt = sg.box_rebuilt;
            e.sys_energy = sg.energy;
            e.sys_rebuilt = sg.rebuilt;
        }
        launch_end_step(e, ctx->stream, &ctx->launches);
        if (staged || beside) {
            if (err == cudaSuccess) err = cudaEventRecord(ctx->ev_join, ctx->side_stream);
            if (err == cudaSuccess) err = cudaStreamWaitEvent(ctx->stream, ctx->ev_join, 0);
        }
        return err;
    };
    const int key = sys * 8 + (staged ? 4 : 0) + (is_nvt ? 2 : 0) + (noise ? 1 : 0);
    auto it = ctx->call_graphs.find(key);
    if (it == ctx->call_graphs.end()) {
        cudaGraph_t graph;
        const unsigned long long before = ctx->launches;
        CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        const cudaError_t se = step();
        const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
        if (se != cudaSuccess || ce != cudaSuccess)
            return fail(ctx, QTG_ERR_CUDA, std::string("step capture: ") + cudaGetErrorString(se != cudaSuccess ? se : ce));
        const unsigned long long kernels = ctx->launches - before;
        ctx->launches = before;
        cudaGraphExec_t exec;
        const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) return fail(ctx, QTG_ERR_CUDA, std::string("step graph: ") + cudaGetErrorString(ie));
        it = ctx->call_graphs.emplace(key, std::make_pair(exec, kernels)).first;
    }
    CK(cudaGraphLaunch(it->second.first, ctx->stream));
    ctx->launches += it->second.second;
    if (!staged) {
        CKS(download_dynamic(ctx, sys, q, p, f, fphys, nullptr, nullptr, disp));
        CK(post_small_results(ctx, sys, true));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    CKS(status_error(ctx, ctx->box->status));
    CKS(download_rebuilt_lists(ctx, sys, point, list));
    double vs = 0.0, ve = 0.0;
    for (int b = 0; b < S.n_beads; ++b) {
        vs += ctx->box_energy[b];
        if (b % 2 == 0) ve += ctx->box_energy[b];
    }
    const double extra = ctx->box->acc.sc_extra;
    if (heat) *heat = ctx->box->heat_out;
    if (S.propagator == QTG_SUZUKI_CHIN) {
        if (pot) *pot = 2.0 * ve / S.n_beads;
        if (energy) *energy = (2.0 * ve + 4.0 * (vs - ve) + extra) / 3.0;
    } else {
        if (pot) *pot = vs / S.n_beads;
        if (energy) *energy = vs;
    }
    return QTG_OK;
}

// ---- tier 2 ------------------------------------------------------------------------

qtg_status qtg_set_state(qtg_ctx *ctx, int sys, const double *q, const double *p) {
    CKS(check_sys(ctx, sys));
    const SysDev &S = ctx->sys_h[sys];
    if (!q) return fail(ctx, QTG_ERR_ARG, "null positions");
    const size_t nt = (size_t)S.n_beads * S.n_dof;
    CK(up(ctx, ctx->q + S.q_off, q, sizeof(double) * nt));
    if (p) CK(up(ctx, ctx->p + S.q_off, p, sizeof(double) * nt));
    else CK(cudaMemsetAsync(ctx->p + S.q_off, 0, sizeof(double) * nt, ctx->stream));
    ctx->forces_ready = false;
    return sync_status(ctx);
}

qtg_status qtg_get_state(qtg_ctx *ctx, int sys, double *q, double *p, double *f, double *fphys, double *disp) {
    CKS(check_sys(ctx, sys));
    const SysDev &S = ctx->sys_h[sys];
    const size_t nt = (size_t)S.n_beads * S.n_dof;
    if (q) CK(down(ctx, q, ctx->q + S.q_off, sizeof(double) * nt));
    if (p) CK(down(ctx, p, ctx->p + S.q_off, sizeof(double) * nt));
    if (f) CK(down(ctx, f, ctx->f + S.q_off, sizeof(double) * nt));
    if (fphys) CK(down(ctx, fphys, ctx->fphys + S.q_off, sizeof(double) * nt));
    if (disp) CK(down(ctx, disp, ctx->disp + S.d_off, sizeof(double) * S.n_beads * 3 * S.n_mols));
    return sync_status(ctx);
}

qtg_status qtg_init_forces(qtg_ctx *ctx) {
    if (!ctx) return QTG_ERR_ARG;
    CK(cudaMemsetAsync(ctx->disp, 0, sizeof(double) * ctx->total_disp, ctx->stream));
    CK(cudaMemsetAsync(ctx->acc, 0, sizeof(SysAcc) * ctx->n_sys, ctx->stream));
    launch_skin_rebuild(list_args(ctx, 0, (int)ctx->base.h.size(), 1), ctx->stream, &ctx->launches);
    CK(cudaMemsetAsync(ctx->acc, 0, sizeof(SysAcc) * ctx->n_sys, ctx->stream));
    enqueue_forces(ctx, -1, false);
    RingArgs e = ring_args(ctx, -1, 0);
    e.kick = 0;
    launch_end_step(e, ctx->stream, &ctx->launches);
    launch_finalize(fin_args(ctx, -1, 1, 1), ctx->stream, &ctx->launches);
    CKS(sync_status(ctx));
    ctx->forces_ready = true;
    return QTG_OK;
}

qtg_status qtg_run_steps(qtg_ctx *ctx, int n_steps, int is_nvt) {
    if (!ctx || n_steps < 0) return QTG_ERR_ARG;
    if (!ctx->forces_ready) return fail(ctx, QTG_ERR_STATE, "qtg_init_forces must precede qtg_run_steps");
    const int g = is_nvt ? 1 : 0;
    if (!ctx->graph[g]) {
        cudaGraph_t graph;
        unsigned long long before = ctx->launches;
        CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        enqueue_step(ctx, -1, is_nvt, 0, false);
        cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
        if (e != cudaSuccess) return fail(ctx, QTG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        ctx->graph_kernels[g] = ctx->launches - before;
        ctx->launches = before;
        e = cudaGraphInstantiate(&ctx->graph[g], graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(ctx, QTG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
    for (int i = 0; i < n_steps; ++i) {
        CK(cudaGraphLaunch(ctx->graph[g], ctx->stream));
        ctx->launches += ctx->graph_kernels[g];
    }
    return QTG_OK;
}

qtg_status qtg_sync(qtg_ctx *ctx) {
    if (!ctx) return QTG_ERR_ARG;
    return sync_status(ctx);
}

qtg_status qtg_get_estimators(qtg_ctx *ctx, int sys, double *out, int max_records, int *n_records) {
    CKS(check_sys(ctx, sys));
    if (!out || max_records < 0 || !n_records) return fail(ctx, QTG_ERR_ARG, "bad argument");
    unsigned long long nrec = 0;
    CK(cudaStreamSynchronize(ctx->stream));
    CK(cudaMemcpy(&nrec, ctx->records, sizeof(nrec), cudaMemcpyDeviceToHost));
    const unsigned long long avail = std::min<unsigned long long>(nrec, (unsigned long long)ctx->max_records);
    const unsigned long long n = std::min<unsigned long long>(avail, (unsigned long long)max_records);
    std::vector<double> all((size_t)ctx->max_records * ctx->n_sys * 8);
    CK(cudaMemcpy(all.data(), ctx->est, sizeof(double) * all.size(), cudaMemcpyDeviceToHost));
    for (unsigned long long i = 0; i < n; ++i) {
        const unsigned long long r = nrec - n + i;
        const double *src = all.data() + ((size_t)(r % ctx->max_records) * ctx->n_sys + sys) * 8;
        memcpy(out + i * 8, src, 8 * sizeof(double));
    }
    *n_records = (int)n;
    return QTG_OK;
}

qtg_status qtg_time_kernel(qtg_ctx *ctx, const char *name, int iters, double *avg_ms) {
    if (!ctx || !name || iters <= 0 || !avg_ms) return QTG_ERR_ARG;
    const std::string n(name);
    const bool ewald = n == "prep" || n == "real" || n == "ksk" || n == "sk_reduce" || n == "kforce" ||
                       n == "combine" || n == "lj";
    if (!ewald && n != "rebuild" && n != "ring" && n != "end_step") return fail(ctx, QTG_ERR_ARG, "unknown kernel name");
    const int nj = (int)ctx->base.h.size();
    EvalArgs a = eval_args(ctx, ctx->base.d, nj, ctx->q, ctx->fphys, 0, 0);
    a.lj_full = 1;  // as the stepper evaluates
    a.lj_list = lj_list_ok(ctx) ? 1 : 0;
    launch_eval(ctx, a);  // fills every scratch array the single kernels read
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    RingArgs r = ring_args(ctx, -1, RF_KICK | RF_FWD | RF_CAYLEY | RF_BACK | RF_DISP);
    RingArgs es = ring_args(ctx, -1, 0);
    es.kick = 0;
    for (int pass = 0; pass < 2; ++pass) {  // pass 0 warms up
        CK(cudaEventRecord(e0, ctx->stream));
        for (int i = 0; i < (pass ? iters : 1); ++i) {
            if (ewald) launch_ewald_kernel(a, ctx->mixed, name, ctx->stream);
            else if (n == "rebuild") launch_skin_rebuild(list_args(ctx, 0, nj, 1), ctx->stream, nullptr);
            else if (n == "ring") launch_ring(r, ctx->stream, nullptr);
            else launch_end_step(es, ctx->stream, nullptr);
        }
        CK(cudaEventRecord(e1, ctx->stream));
        CK(cudaEventSynchronize(e1));
    }
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CK(cudaMemsetAsync(ctx->acc, 0, sizeof(SysAcc) * ctx->n_sys, ctx->stream));
    *avg_ms = (double)ms / iters;
    ctx->forces_ready = false;
    return sync_status(ctx);
}

qtg_status qtg_set_tuning(qtg_ctx *ctx, int n_rj, int n_sc, int n_kc) {
    if (!ctx || n_rj < 0 || n_sc < 0 || n_kc < 0 || n_rj > MAX_RJ || n_sc > MAX_SC || n_kc > MAX_KC)
        return fail(ctx, QTG_ERR_ARG, "chunk counts must lie in [0, 16], [0, 32], [0, 16] (0: heuristic)");
    ctx->tune[0] = n_rj;
    ctx->tune[1] = n_sc;
    ctx->tune[2] = n_kc;
    drop_graphs(ctx);
    return QTG_OK;
}

qtg_status qtg_get_tuning(qtg_ctx *ctx, int *n_rj, int *n_sc, int *n_kc) {
    if (!ctx || !n_rj || !n_sc || !n_kc) return QTG_ERR_ARG;
    *n_rj = ctx->tune[0];
    *n_sc = ctx->tune[1];
    *n_kc = ctx->tune[2];
    return QTG_OK;
}

qtg_status qtg_set_real_space(qtg_ctx *ctx, int form) {
    if (!ctx || form < 0 || form > 1) return fail(ctx, QTG_ERR_ARG, "real-space form must be 0 (pair list) or 1 (all pairs)");
    ctx->rl_form = form;
    drop_graphs(ctx);
    return QTG_OK;
}

qtg_status qtg_get_real_space(qtg_ctx *ctx, int *form, int *list_eligible) {
    if (!ctx || !form || !list_eligible) return QTG_ERR_ARG;
    *form = ctx->rl_form;
    *list_eligible = ctx->rl_ok ? 1 : 0;
    return QTG_OK;
}

qtg_status qtg_transfer_bytes(qtg_ctx *ctx, unsigned long long *h2d, unsigned long long *d2h) {
    if (!ctx || !h2d || !d2h) return QTG_ERR_ARG;
    *h2d = ctx->h2d_bytes;
    *d2h = ctx->d2h_bytes;
    return QTG_OK;
}

qtg_status qtg_autotune(qtg_ctx *ctx, int iters, double *ms_heuristic, double *ms_tuned) {
    if (!ctx || iters <= 0) return QTG_ERR_ARG;
    const int nj = (int)ctx->base.h.size();
    // lists for the current positions (the FP64 Lennard-Jones reads them)
    CK(cudaMemsetAsync(ctx->disp, 0, sizeof(double) * ctx->total_disp, ctx->stream));
    launch_skin_rebuild(list_args(ctx, 0, nj, 1), ctx->stream, &ctx->launches);
    ctx->forces_ready = false;  // the timing runs overwrite the forces
    // a candidate's time: the fastest of three timed runs of iters evaluations
    // (differences between candidates are a few per cent, near the run-to-run
    // spread of a single run)
    auto eval_ms = [&](const int *t, double *ms) {
        for (int k = 0; k < 3; ++k) ctx->tune[k] = t[k];
        EvalArgs a = eval_args(ctx, ctx->base.d, nj, ctx->q, ctx->fphys, 0, 0);
        a.lj_full = 1;
        a.lj_list = lj_list_ok(ctx) ? 1 : 0;
        double best = 0.0;
        for (int r = 0; r < 3; ++r) {
            double m = 0.0;
            const qtg_status st = time_on_stream(ctx, iters, [&] { launch_eval(ctx, a); }, &m);
            if (st != QTG_OK) return st;
            best = r == 0 ? m : std::min(best, m);
        }
        *ms = best;
        return QTG_OK;
    };
    // each count governs one kernel: k_real (n_rj), k_ksk (n_sc), k_kforce (n_kc), 0
    // the launcher's heuristic. The force kernels run concurrently (forked branches
    // of one evaluation), so candidates are compared by the time of the whole force
    // evaluation: coordinate descent from the heuristic, one count at a time.
    static const int cand_rk[] = {0, 1, 2, 3, 4, 6, 8, 12, 16};       // k_real, k_kforce
    static const int cand_sc[] = {0, 1, 2, 4, 6, 8, 12, 16, 24, 32};  // k_ksk
    int best[3] = {0, 0, 0};
    double best_ms = 0.0;
    if (ctx->rl_ok) {
        // the real-space form first (pair list or all pairs, heuristic counts); the
        // list's first evaluation builds it, the timed ones find it valid
        double ms_form[2];
        for (int f = 0; f < 2; ++f) {
            ctx->rl_form = f;
            CKS(eval_ms(best, &ms_form[f]));
            CKS(eval_ms(best, &ms_form[f]));
        }
        ctx->rl_form = ms_form[1] < ms_form[0] ? 1 : 0;
    }
    CKS(eval_ms(best, &best_ms));  // fills the scratch arrays, warms the kernels
    CKS(eval_ms(best, &best_ms));
    for (int sweep = 0; sweep < 2; ++sweep) {
        bool moved = false;
        for (int k = 0; k < 3; ++k) {
            const int *cand = k == 1 ? cand_sc : cand_rk;
            const int n_cand = k == 1 ? (int)(sizeof(cand_sc) / sizeof(int)) : (int)(sizeof(cand_rk) / sizeof(int));
            for (int ci = 0; ci < n_cand; ++ci) {
                if (cand[ci] == best[k]) continue;
                int t[3] = {best[0], best[1], best[2]};
                t[k] = cand[ci];
                double ms;
                CKS(eval_ms(t, &ms));
                if (ms < best_ms) {
                    best_ms = ms;
                    best[k] = cand[ci];
                    moved = true;
                }
            }
        }
        if (!moved) break;
    }
    // a fresh measurement of both decides between the descent's counts and the heuristic
    const int zero[3] = {0, 0, 0};
    double t0 = 0.0, t1 = 0.0;
    CKS(eval_ms(zero, &t0));
    CKS(eval_ms(best, &t1));
    const int *pick = t1 < t0 ? best : zero;
    for (int k = 0; k < 3; ++k) ctx->tune[k] = pick[k];
    if (ms_heuristic) *ms_heuristic = t0;
    if (ms_tuned) *ms_tuned = t1 < t0 ? t1 : t0;
    drop_graphs(ctx);
    CK(cudaMemsetAsync(ctx->acc, 0, sizeof(SysAcc) * ctx->n_sys, ctx->stream));
    return sync_status(ctx);
}

qtg_status qtg_fp32_peak(double *tflops) {
    return fma_peak<float>(tflops, 1 << 16, [](float *o, int b, int it) { launch_fp32_probe(o, b, it, nullptr); });
}

qtg_status qtg_fp64_peak(double *tflops) {
    return fma_peak<double>(tflops, 1 << 11, [](double *o, int b, int it) { launch_fp64_probe(o, b, it, nullptr); });
}

qtg_status qtg_flush_l2(qtg_ctx *ctx) {
    if (!ctx) return QTG_ERR_ARG;
    constexpr size_t bytes = (size_t)256 << 20;
    if (!ctx->flush_buf) CK(cudaMalloc(&ctx->flush_buf, bytes));
    CK(cudaMemsetAsync(ctx->flush_buf, ctx->flush_val++ & 0xff, bytes, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return QTG_OK;
}

qtg_status qtg_reset_estimators(qtg_ctx *ctx) {
    if (!ctx) return QTG_ERR_ARG;
    CK(cudaMemsetAsync(ctx->records, 0, sizeof(unsigned long long), ctx->stream));
    return sync_status(ctx);
}

}  // extern "C"
