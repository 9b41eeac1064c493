/* qtip4pf_gb300 -- C ABI of the GB300 (sm_103a) force and ring-polymer
 * propagation library for flexible qTIP4P/F water.
 *
 * Two tiers, both plain C (pointers and sizes; no C++ or torch types):
 *
 *  1. Per-call entries that take HOST arrays in the reference's layouts and
 *     mirror one reference function each (copy in, compute on the GPU, copy
 *     out, synchronise). Each declaration names the reference interface it
 *     replaces (rayseashyn/qtip4pf_water, file:line).
 *  2. A device-resident stepper: state lives in HBM, each MD step is one CUDA
 *     graph replay, and estimators are read back on demand.
 *
 * Layouts (the reference's, indexing.h:6-24), per system:
 *   positions q, momenta p, forces f   double[P][9N]  [bead][mol][O,H1,H2][x,y,z]
 *   Verlet list                        int point[P][N], int list[P][list_size]
 *   oxygen displacements               double[P][3N]
 *   charges double[3N] (per site), masses double[9N] (per degree of freedom)
 * Units: Hartree atomic units throughout (qtip4pfparams.h:43-61).
 *
 * Every entry returns a qtg_status (0 = success). On failure the message is
 * available from qtg_last_error(ctx). No entry aborts the process. */
#ifndef QTIP4PF_GB300_H
#define QTIP4PF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct qtg_ctx qtg_ctx;

typedef enum {
    QTG_OK = 0,
    QTG_ERR_ARG = 1,           /* bad argument or system index */
    QTG_ERR_CUDA = 2,          /* a CUDA runtime call failed */
    QTG_ERR_LIST_OVERFLOW = 3, /* a Verlet list needed more than list_size entries */
    QTG_ERR_NONFINITE = 4,     /* NaN/Inf in forces or energies */
    QTG_ERR_STATE = 5,         /* call made in the wrong state (e.g. no forces yet) */
    QTG_ERR_NODEVICE = 6       /* no usable sm_103 device */
} qtg_status;

typedef enum {
    QTG_FP64 = 0,  /* every force term in FP64 (parity mode) */
    QTG_MIXED = 1  /* Ewald terms in FP32 with FP64 accumulation; LJ, intramolecular,
                      integration, normal modes and thermostat in FP64 */
} qtg_precision;

typedef enum {
    QTG_SUZUKI_CHIN = 0, /* fourth-order SC forces (forces.cpp:698-789); P even */
    QTG_TROTTER = 1      /* second-order: every bead weight 1 (also P = 1) */
} qtg_propagator;

typedef enum {
    QTG_THERMO_NONE = 0,   /* NVE */
    QTG_THERMO_PILE_G = 1, /* centroid global rescale + mode Langevin (thermostat.cpp:64-133) */
    QTG_THERMO_PILE_L = 2  /* centroid Langevin with time constant tau0 + mode Langevin */
} qtg_thermostat;

/* One independent system (replica). box in bohr; dt in fs. */
typedef struct qtg_system_desc {
    int n_mols;
    int n_beads;
    double box_bohr[3];
    double temp_K;
    double dt_fs;
    double eps_ewald;  /* config.txt eps_ewald: acc = sqrt(-ln eps) (water.cpp:148) */
    double eps_sc;     /* config.txt epsilon_sc (forces.cpp:754) */
    int propagator;    /* qtg_propagator */
    int thermostat;    /* qtg_thermostat */
    double tau0_fs;    /* centroid time constant for QTG_THERMO_PILE_L */
    uint64_t seed;     /* counter-based RNG key for this system */
} qtg_system_desc;

/* Derived per-system parameters, as the reference derives them
 * (water.cpp:76-157, forces.cpp:574-584). */
typedef struct qtg_system_info {
    int n_mols, n_beads, n_dof, list_size, k_max, n_kvectors;
    double kappa, rc, kc, dt, beta_n, omega_psq;
} qtg_system_info;

/* ---- context --------------------------------------------------------------- */
/* Creates a context on the current CUDA device holding n_systems systems.
 * All device memory is allocated here; no later call allocates. */
qtg_status qtg_create(const qtg_system_desc *systems, int n_systems, int precision, qtg_ctx **out);
void qtg_destroy(qtg_ctx *ctx);
const char *qtg_last_error(const qtg_ctx *ctx);
const char *qtg_status_string(int status);
/* Work is issued on this stream (a cudaStream_t passed as void*; NULL = the
 * context's own stream). */
qtg_status qtg_set_stream(qtg_ctx *ctx, void *cuda_stream);
qtg_status qtg_system_info_get(const qtg_ctx *ctx, int sys, qtg_system_info *out);
/* Number of this library's kernels launched since the context was created. */
qtg_status qtg_kernel_launches(const qtg_ctx *ctx, uint64_t *out);
/* Replace the default per-site charges / per-dof masses of one system. */
qtg_status qtg_set_charges(qtg_ctx *ctx, int sys, const double *charge);
qtg_status qtg_set_masses(qtg_ctx *ctx, int sys, const double *mass);

/* ---- tier 1: per-call entries mirroring the reference ---------------------- */
/* neighbour.cpp:12-62  void neighbour_list(pos, point, list, disp, bead)
 * Bit-identical CSR list; the bead's disp slice is zeroed. */
qtg_status qtg_neighbour_list(qtg_ctx *ctx, int sys, const double *pos, int *point, int *list,
                              double *disp, int bead);
/* forces.cpp:468-630  double get_forces_nospline(pos, f, charge, point, list, bead)
 * Writes the bead's slice of f and the bead's potential energy. */
qtg_status qtg_get_forces(qtg_ctx *ctx, int sys, const double *pos, double *f,
                          const double *charge, const int *point, const int *list, int bead,
                          double *energy);
/* forces.cpp:180-448  double kwald(charge_pos, force, charge, k_max, kappa, k_cut_sq, bead)
 * sites: the bead's charge sites (M, H1, H2); f_sites receives += k-space forces. */
qtg_status qtg_kwald(qtg_ctx *ctx, int sys, const double *sites, double *f_sites,
                     const double *charge, int bead, double *energy);
/* forces.cpp:698-789  double force_eval_sc_nospline(pos, f, charge, mass, point, list,
 *                                                  sc_pot, fphys) */
qtg_status qtg_force_eval_sc(qtg_ctx *ctx, int sys, const double *pos, double *f,
                             const double *charge, const double *mass, const int *point,
                             const int *list, double *sc_pot, double *fphys, double *energy);
/* Second-order assembly (no reference counterpart): f = fphys = -dV/dq per bead,
 * *energy = sum_b V_b, *pot = sum_b V_b / P. */
qtg_status qtg_force_eval_trotter(qtg_ctx *ctx, int sys, const double *pos, double *f,
                                  const double *charge, const int *point, const int *list,
                                  double *pot, double *energy);
/* fourier.cpp:12-69  void ftransform(a, length, is_forwards)  (a: double[P][length]) */
qtg_status qtg_ftransform(qtg_ctx *ctx, int sys, double *a, int length, int forwards);
/* thermostat.cpp:64-133  double pile_g(p, mass, rng), on normal-mode momenta.
 * noise = [R, g2, xi(mode 1..P-1, dof 0..9N-1)] supplied by the caller, or NULL to
 * draw from the system's counter-based generator. *heat receives the return value. */
qtg_status qtg_pile_g(qtg_ctx *ctx, int sys, double *p, const double *mass,
                      const double *noise, double *heat);
/* thermostat.cpp:12-60  double bussi(p, mass, rng): global rescale of the first
 * n_dof momenta (bead 0; the reference's classical system) to the canonical
 * kinetic-energy distribution at the system's temperature. noise = [R, g2] (R the
 * normal draw, g2 the combined chi-square draw of n_dof - 1 degrees of freedom)
 * from the caller, or NULL to draw from the system's counter-based generator.
 * *heat receives the return value (kinetic energy before minus after). */
qtg_status qtg_bussi(qtg_ctx *ctx, int sys, double *p, const double *mass, const double *noise,
                     double *heat);
/* path_integrals.cpp:29-48  double get_kcv(q, f) */
qtg_status qtg_get_kcv(qtg_ctx *ctx, int sys, const double *q, const double *f, double *out);
/* path_integrals.cpp:55-81  double get_conserved(q, p, mass, energy); like the
 * reference, q and p are round-tripped through the normal-mode transform in place. */
qtg_status qtg_get_conserved(qtg_ctx *ctx, int sys, double *q, double *p, const double *mass,
                             double energy, double *out);
/* update.cpp:78-137  double update_trajectory_class_nospline(q, p, mass, f, charge,
 *                                                           point, list, disp)
 * Per-call steps (this and qtg_update_pimd): q, p, f and disp are read and written
 * back; point and list are written back only for the beads whose lists the skin
 * test rebuilt during the call, as the reference's neighbour_list writes them.
 * In QTG_MIXED the Lennard-Jones term of the physical forces runs over every O-O
 * pair inside r_cut (the pairs a valid Verlet list holds), so a mixed Trotter or
 * classical step does not read the caller's point and list; QTG_FP64 steps and
 * the Suzuki-Chin finite-difference terms read them as the reference does.
 * When q, p, f, (fphys,) disp lie in page-locked host memory the device can
 * address (cudaHostAlloc / cudaHostRegister without the read-only flag) and do
 * not overlap, qtg_update_pimd moves them inside its captured step graph (the
 * step's kernels read and write the caller's memory directly); otherwise by copy
 * calls. Results are the same bits either way. */
qtg_status qtg_update_class(qtg_ctx *ctx, int sys, double *q, double *p, const double *mass,
                            double *f, const double *charge, int *point, int *list, double *disp,
                            double *energy);
/* update.cpp:271-401  double update_sc_nospline(q, p, mass, f, fphys, charge, point, list,
 *                                               disp, rng, is_nvt, heat, sc_pot)
 * The system's propagator decides the force assembly (SC or Trotter). noise as for
 * qtg_pile_g (NULL = counter-based generator). *heat is updated in place. fphys is
 * output only: the reference's step overwrites it before reading it. */
qtg_status qtg_update_pimd(qtg_ctx *ctx, int sys, double *q, double *p, const double *mass,
                           double *f, double *fphys, const double *charge, int *point,
                           int *list, double *disp, int is_nvt, const double *noise,
                           double *heat, double *pot, double *energy);

/* ---- tier 2: device-resident stepping -------------------------------------- */
/* Upload a system's positions and momenta (double[P][9N] each; p may be NULL = 0). */
qtg_status qtg_set_state(qtg_ctx *ctx, int sys, const double *q, const double *p);
/* Download state; any pointer may be NULL. f is the propagating force (SC or
 * Trotter), fphys the physical force -dV/dq per bead. */
qtg_status qtg_get_state(qtg_ctx *ctx, int sys, double *q, double *p, double *f, double *fphys,
                         double *disp);
/* Build every Verlet list and evaluate the initial forces of every system
 * (simulation.cpp:838-874). Must precede qtg_run_steps. */
qtg_status qtg_init_forces(qtg_ctx *ctx);
/* Advance every system n_steps steps (each a CUDA graph replay), NVT if is_nvt.
 * Estimators of every step are recorded on the device. Asynchronous on the
 * context's stream: call qtg_sync to wait and collect device-side errors. */
qtg_status qtg_run_steps(qtg_ctx *ctx, int n_steps, int is_nvt);
qtg_status qtg_sync(qtg_ctx *ctx);
/* Per-step estimator records of one system since the last reset, oldest first.
 * Record layout (QTG_EST_FIELDS doubles): see QTG_EST_* indices. */
#define QTG_EST_FIELDS 8
#define QTG_EST_POT 0       /* potential estimator: SC sc_pot, Trotter sum V_b / P */
#define QTG_EST_KCV 1       /* centroid-virial kinetic energy estimator */
#define QTG_EST_CONSERVED 2 /* ring-polymer Hamiltonian + heat (path_integrals.cpp:55-81) */
#define QTG_EST_HEAT 3      /* accumulated thermostat heat (update.cpp:325) */
#define QTG_EST_KIN 4       /* bead-space kinetic energy sum p^2/2m */
#define QTG_EST_VTOT 5      /* force-eval return value (SC tot_energy, Trotter sum V_b) */
#define QTG_EST_REBUILDS 6  /* Verlet-list rebuilds performed this step (all beads) */
#define QTG_EST_STEP 7      /* step index */
qtg_status qtg_get_estimators(qtg_ctx *ctx, int sys, double *out, int max_records, int *n_records);
qtg_status qtg_reset_estimators(qtg_ctx *ctx);

/* ---- without device allocation --------------------------------------------- */
/* No counterpart in the reference: the reciprocal-space Ewald sum of qtg_kwald
 * (FP64) for callers that cannot allocate device memory -- engines and plugins
 * that own the GPU memory budget and pass preallocated buffers to their force
 * routines (an allocation of their own would escape that budget or fail under
 * its cap). It calls no cudaMalloc/cudaFree and needs no qtg_ctx: all scratch
 * lives in one static device array of 2.76 MiB (2,895,872 bytes) that every GPU loading the
 * library holds until exit.
 *   sites   device, double[3 n_sites]: charge sites (M, H1, H2 per molecule)
 *   charge  device, double[n_sites]
 *   box     host, double[3] (bohr); eps_ewald as config.txt (kappa, k_max and
 *           the k set derived as forces.cpp:574-584, :251-445)
 *   f_sites device, double[3 n_sites]: the k-space forces are ADDED
 *   energy  device, one double: the k-space energy is WRITTEN
 * Limits: n_sites <= QTG_NOALLOC_MAX_SITES, k_max <= QTG_NOALLOC_MAX_KMAX;
 * anything larger returns QTG_ERR_ARG. Work is queued on `cuda_stream` and the
 * call returns without waiting. The first call on a device looks up the array's
 * device address (once per device, that device current) and should therefore
 * come before any stream capture; that set-up is locked, so first calls from
 * several host threads are safe. Every call shares the array, so calls that
 * overlap on the GPU (other streams, other host threads) race; each call
 * rebuilds every table it reads, so nothing carries over between calls. An
 * error already pending from the caller's own CUDA work is returned as
 * QTG_ERR_CUDA, uncleared, and nothing is launched. */
#define QTG_NOALLOC_MAX_SITES 1536
#define QTG_NOALLOC_MAX_KMAX 12
qtg_status qtg_kwald_noalloc(const double *sites, const double *charge, int n_sites,
                             const double *box_bohr, double eps_ewald, double *f_sites,
                             double *energy, void *cuda_stream);

/* ---- measurement helpers (no reference counterpart) ------------------------ */
/* Average duration (ms, CUDA events on the context's stream) of `iters`
 * back-to-back launches of one kernel of the force / step pipeline over every
 * system, after one full force evaluation. name: "prep", "real", "ksk",
 * "kforce", "combine", "lj", "rebuild", "ring", "end_step". Overwrites the
 * context's forces and may move its state: call after the measured run. */
qtg_status qtg_time_kernel(qtg_ctx *ctx, const char *name, int iters, double *avg_ms);
/* Writes a device buffer larger than the L2 cache (256 MiB, allocated on the
 * first call and kept) on the context's stream and waits for it: timing loops
 * call it between timed calls so that no call finds its data in L2. */
qtg_status qtg_flush_l2(qtg_ctx *ctx);
/* FP32 fused-multiply-add throughput of the current device (TFLOP/s, 2 flops
 * per FMA) from a dependent-chain kernel filling every SM. */
qtg_status qtg_fp32_peak(double *tflops);
/* The same for FP64 fused multiply-adds (the bound of the FP64 form and of the
 * FP64 normal-mode / integrator kernels). */
qtg_status qtg_fp64_peak(double *tflops);

/* ---- host-side helpers of the drop-in --------------------------------------- */
/* The qTIP4P/F constants in atomic units, derived as qtip4pfparams.h:41-133
 * derives them (same values, same operation order): for host code that has to
 * agree with the library to the last bit (the drop-in's per-pair helpers). */
typedef struct qtg_constants {
    double angs2bohr, fs2au, K2au, mo, mh, qo, qh, gamma_vs;
    double epslj, sigmalj6, sigmalj12, e_cut, r_cut, r_skin;
    double roheq, ar2, ar3, ar4fac, Dr, theta_eq, ktheta, pi;
} qtg_constants;
qtg_status qtg_get_constants(qtg_constants *out);
/* Page-locks and maps a caller's host array (cudaHostRegister, portable and
 * mapped) so that per-call steps move it inside their graph instead of by copy
 * calls; an array already registered is accepted as it is. The caller keeps the
 * memory registered until qtg_unregister_host or process exit. No counterpart
 * in the reference (its arrays are plain new[] memory). */
qtg_status qtg_register_host(void *ptr, size_t bytes);
qtg_status qtg_unregister_host(void *ptr);

/* ---- starting configurations (host) ----------------------------------------- */
/* initialise.cpp:19-95  initialise_fcc(): nx x ny x nz fcc cells of 4 waters at
 * density rho (g/cm^3; cell side as water.cpp:90-97), every molecule at the
 * equilibrium geometry in one orientation; pos: double[n_beads][9 n_mols] with
 * n_mols = 4 nx ny nz, every bead identical; box_bohr (may be NULL) receives
 * the box. */
qtg_status qtg_lattice_fcc(int nx, int ny, int nz, double rho_g_cm3, int n_beads, double *pos, double *box_bohr);
/* initialise.cpp:137-541  initialise_orth(rng, outfile): proton-disordered ice Ih
 * in nx x ny x nz orthorhombic cells of 8 waters (water.cpp:99-108), obeying
 * the ice rules with zero dipole moment, drawn from std::mt19937(seed) in the
 * reference's order (the same seed gives the reference's configuration);
 * n_mols = 8 nx ny nz. */
qtg_status qtg_lattice_ice_ih(int nx, int ny, int nz, double rho_g_cm3, int n_beads, unsigned int seed,
                              double *pos, double *box_bohr);

/* ---- tabulated pair corrections ("fast-CMD" splines) ------------------------ */
/* Replaces the spline part of get_forces_wspline / force_eval_sc_wspline
 * (forces.cpp:452-466, :634-691, :791-882): every atom pair of a configuration
 * whose minimum-image separation r has r^2 < cut_sq for its type adds s(r) to
 * the energy and -s'(r) r_ij / r to atom i (+ to atom j). s is the clamped
 * uniform cubic B-spline interpolant of values[0 .. n-1] on the knots
 * start + i step (the construction of boost::math::cubic_b_spline, which the
 * reference builds from oo/oh/hh_spline.txt with start 0 and step 0.01 bohr,
 * simulation.cpp:36-116); an end slope given as NaN is estimated by five-point
 * one-sided differences. Units: bohr and Hartree. */
typedef struct qtg_pair_spline {
    const double *values; /* host, n >= 5 values at the knots */
    int n;
    double start, step;   /* first knot and spacing (bohr) */
    double left_deriv, right_deriv; /* end slopes (Hartree / bohr), NaN: estimated */
    double cut_sq;        /* pairs with r^2 < cut_sq; at most (start + step (n-1))^2 */
} qtg_pair_spline;
/* Attaches (any table non-NULL) or removes (all NULL) the tables of one
 * system; a NULL type adds nothing. Every later force evaluation of the system
 * -- tier-1 entries, per-call steps, the device stepper, the Suzuki-Chin
 * displaced evaluations -- includes them (the reference's *_wspline
 * functions). Allocates the tables; qtg_init_forces must precede the next
 * qtg_run_steps. */
qtg_status qtg_set_pair_splines(qtg_ctx *ctx, int sys, const qtg_pair_spline *oo, const qtg_pair_spline *oh,
                                const qtg_pair_spline *hh);

/* ---- centroid-constrained PIMD (no reference counterpart) ------------------- */
/* With the centroid fixed, the device stepper holds each atom's bead centroid
 * where it is (the centroid normal mode carries no momentum and is not
 * thermostatted) while the internal modes evolve, and every step adds the
 * bead-averaged physical force (1/P) sum_b F_b to a per-dof sum: its mean is
 * the constrained-PIMD mean centroid force, the target of the learned centroid
 * correction. Trotter systems; qtg_get_centroid_force returns the mean
 * (double[9N], reference layout) and the number of steps in it. */
qtg_status qtg_set_centroid_fixed(qtg_ctx *ctx, int sys, int fixed);
qtg_status qtg_reset_centroid_force(qtg_ctx *ctx, int sys);
qtg_status qtg_get_centroid_force(qtg_ctx *ctx, int sys, double *f_mean, double *n_samples);

/* ---- learned centroid correction (no reference counterpart) ------------------ */
/* A per-molecule network maps Behler-Parrinello symmetry functions of the
 * molecule's three atoms (G2 and G5 within 6 A, QTG_DESC_PER_ATOM per atom,
 * O H1 H2 concatenated: QTG_MLP_IN inputs) through two hidden layers of
 * QTG_MLP_HIDDEN SiLU units to the centroid-force correction of its three atoms
 * in the molecule's frame (QTG_MLP_OUT values, padded to QTG_MLP_OUT_PAD). It
 * replaces the reference's tabulated CMD spline (forces.cpp:452-466). These
 * entries take DEVICE pointers and queue work on `stream` without waiting. */
#define QTG_DESC_PER_ATOM 32
#define QTG_MLP_IN 96
#define QTG_MLP_HIDDEN 64
#define QTG_MLP_OUT 9
#define QTG_MLP_OUT_PAD 16
typedef struct qtg_mlp_weights {
    const void *w1, *w2, *w3;    /* BF16, row-major [out][in]: [64][96], [64][64], [16][64] (rows 9..15 zero) */
    const float *b1, *b2, *b3;   /* FP32: [64], [64], [16] */
} qtg_mlp_weights;
/* Symmetry functions of every atom of n_conf configurations of n_mols waters
 * (pos: double[n_conf][9N] bohr, orthorhombic box with every side above 12 A):
 * desc float[n_conf][3N][32]. */
qtg_status qtg_sym_descriptors(const double *pos, int n_conf, int n_mols, const double *box_bohr, float *desc,
                               void *stream);
/* Forward pass on the tensor cores: x BF16 [m][96] -> y float[m][16]. */
qtg_status qtg_mlp_forward(const qtg_mlp_weights *w, const void *x_bf16, int m, float *y, void *stream);
/* Training. Parameters are one FP32 vector of QTG_MLP_NPARAMS values:
 * w1 [64][96] | w2 [64][64] | w3 [16][64] | b1 [64] | b2 [64] | b3 [16].
 * qtg_mlp_train_batch runs the forward and backward pass of m rows (x BF16
 * [m][96], targets t float[m][16], the first QTG_MLP_OUT used) on the tensor
 * cores with dL/dy = grad_scale (y - t), and writes the summed gradients and the
 * summed squared error: grad_out float[QTG_MLP_NPARAMS + 1]. partial is scratch
 * of max_ctas x (QTG_MLP_NPARAMS + 1) floats; the sum over CTAs is taken in a
 * fixed order. qtg_adam_step applies Adam to the FP32 parameters and refreshes
 * the BF16 copies of its first n_bf16 entries (the weights). */
#define QTG_MLP_NPARAMS 11408
qtg_status qtg_mlp_train_batch(const qtg_mlp_weights *w, const void *x_bf16, const float *t, int m, float grad_scale,
                               float *partial, int max_ctas, float *grad_out, void *stream);
qtg_status qtg_adam_step(float *params, float *m1, float *m2, const float *grad, int n, int step, float lr,
                         float beta1, float beta2, float eps, void *w_bf16, int n_bf16, void *stream);
/* Surrogate centroid molecular dynamics: a trained network attached to a P = 1
 * system (its positions are centroids) adds the learned correction to that
 * system's forces in every force evaluation, inside the step graph. The
 * context copies the weights (device pointers in `w`) and the input
 * normalisation (host float[192]: mean[96] then 1/std[96]) into memory of its
 * own; out_scale multiplies the network's outputs (Hartree/bohr). A
 * qtg_init_forces must follow. */
qtg_status qtg_attach_surrogate(qtg_ctx *ctx, int sys, const qtg_mlp_weights *w, const float *norm, float out_scale);
qtg_status qtg_detach_surrogate(qtg_ctx *ctx, int sys);
/* Synchronises the device and returns the surrogate kernels' error bits (8: an
 * atom had more than 256 neighbours within 6 A; 16: a tensor-core completion
 * wait ran out), clearing them when `clear` is set. */
qtg_status qtg_surrogate_status(unsigned *bits, int clear);

/* Bytes the context has copied host -> device and device -> host since it was
 * created (every entry that takes host arrays counts what it moves). The
 * per-call steps skip what is provably unchanged: masses and charges equal to
 * the last ones uploaded, and the Verlet list on the way back unless the skin
 * test rebuilt it during the call (no reference counterpart). */
qtg_status qtg_transfer_bytes(qtg_ctx *ctx, unsigned long long *h2d, unsigned long long *d2h);

/* ---- launch-shape autotuner (no reference counterpart) ---------------------- */
/* The three dominant force kernels split their work into chunks whose counts
 * set the grid sizes: real-space j-chunks (k_real, 1..16), structure-factor
 * site chunks (k_ksk, 1..32) and k-vector chunks (k_kforce, 1..16). By default a
 * heuristic sizes each grid for about 12 blocks per SM over all of the
 * context's systems. qtg_autotune times every candidate count of each kernel
 * on the context's own batch (iters launches each), then keeps the tuned
 * triple if a whole force evaluation with it beats the heuristic, and reports
 * both evaluation times (ms). Call it after qtg_set_state and before
 * qtg_init_forces: it rebuilds the Verlet lists and overwrites the forces, so
 * a qtg_init_forces must follow. A changed shape takes effect at the next
 * step graph capture. qtg_set_tuning fixes the counts by hand (0: heuristic). */
qtg_status qtg_autotune(qtg_ctx *ctx, int iters, double *ms_heuristic, double *ms_tuned);
qtg_status qtg_set_tuning(qtg_ctx *ctx, int n_rj, int n_sc, int n_kc);
qtg_status qtg_get_tuning(qtg_ctx *ctx, int *n_rj, int *n_sc, int *n_kc);
/* Real-space form of the mixed precision (no reference counterpart; the reference
 * visits every site pair, forces.cpp:589-608). In contexts whose beads are too
 * large for the half-interaction kernel (more than 2048 charge sites) and whose
 * boxes satisfy r_c + 6 bohr <= L/2 ("list eligible"), form 0 (the default) finds
 * the site pairs within r_c through a per-configuration list of molecule pairs
 * (rebuilt by a site displacement test with a 2 bohr skin); form 1 evaluates every
 * site pair. Both give the same pair set. qtg_autotune keeps the faster form of
 * an eligible context. A changed form takes effect at the next step graph capture. */
qtg_status qtg_set_real_space(qtg_ctx *ctx, int form);
qtg_status qtg_get_real_space(qtg_ctx *ctx, int *form, int *list_eligible);

#ifdef __cplusplus
}
#endif
#endif
