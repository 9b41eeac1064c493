// Ring-polymer propagation on GB300 (replaces update.cpp:78-137 / :271-401,
// fourier.cpp:12-69, thermostat.cpp:12-133 and the reductions of
// path_integrals.cpp:29-81). All arithmetic here is FP64.
//
// A block owns cols_per_block degree-of-freedom columns of one system and all
// P beads of each: thread (k, c) holds bead / normal mode k of column c. The
// orthonormal bead <-> normal-mode matrix (fourier.cpp's FFTW halfcomplex order
// and scaling) is staged in shared memory and applied as a batched P x P
// matrix product on the column tile, so the B kick, forward transform, the two
// sqrt-Cayley half steps, the O step and the backward transform of a step are
// one kernel with one read and one write of q and p.
#include <math.h>

#include "qtg_internal.h"

namespace qtg {

namespace {

__device__ __forceinline__ void philox_key(const SysDev &S, int sys, uint32_t tag, uint32_t *k0,
                                           uint32_t *k1) {
    *k0 = (uint32_t)S.seed ^ ((uint32_t)sys * 0x85EBCA6Bu);
    *k1 = (uint32_t)(S.seed >> 32) ^ (tag * 0xC2B2AE35u);
}

// Standard normal from one Philox block, Box-Muller in FP32 (thermostat noise).
__device__ __forceinline__ double normal_f32(const Philox4 &r) {
    float u1 = ((float)(r.v[0] >> 8) + 0.5f) * (1.0f / 16777216.0f);
    float u2 = ((float)(r.v[1] >> 8) + 0.5f) * (1.0f / 16777216.0f);
    float s, c;
    sincospif(2.0f * u2, &s, &c);
    return (double)(sqrtf(-2.0f * logf(u1)) * c);
}

// Gamma(shape) by Marsaglia & Tsang, "A simple method for generating gamma
// variables" (ACM TOMS 26, 2000), for shape >= 1, with a bounded number of
// candidates. Candidate `it` is drawn from Philox counters (2 it, 2 it + 1), so
// the candidates are independent of one another: the 32 lanes of a warp test
// 32 of them at once and the first accepted one (lowest `it`, found by ballot)
// is the value the sequential loop would return. Called by a whole warp.
__device__ double gamma_mt_warp(double shape, const SysDev &S, int sys, unsigned long long st, bool *ok) {
    const int lane = threadIdx.x & 31;
    const double d = shape - 1.0 / 3.0, cc = 1.0 / sqrt(9.0 * d);
    uint32_t k0, k1;
    philox_key(S, sys, RNG_GAMMA, &k0, &k1);
    for (uint32_t base = 0; base < 64; base += 32) {
        const uint32_t it = base + (uint32_t)lane;
        const double x = normal2(philox4x32_10(2 * it, 0u, (uint32_t)st, (uint32_t)(st >> 32), k0, k1)).x;
        double v = 1.0 + cc * x;
        bool acc = false;
        if (v > 0.0) {
            v = v * v * v;
            const Philox4 r = philox4x32_10(2 * it + 1, 0u, (uint32_t)st, (uint32_t)(st >> 32), k0, k1);
            const double u = u01_from(r.v[0], r.v[1]);
            acc = (u < 1.0 - 0.0331 * x * x * x * x) || (log(u) < 0.5 * x * x + d * (1.0 - v + log(v)));
        }
        const unsigned hit = __ballot_sync(0xffffffffu, acc);
        if (hit) return __shfl_sync(0xffffffffu, d * v, __ffs(hit) - 1);
    }
    *ok = false;
    return shape;
}

// The PILE-G centroid draws of a step (called by a whole warp): R ~ N(0, 1) and
// g2 ~ chi^2 with (n_dof - 1) degrees of freedom -- both branches of
// thermostat.cpp:102-110 draw exactly this distribution -- from Philox counters
// of (seed, system, step), so they do not depend on where they are made.
__device__ void centroid_draw(const SysDev &S, int sys, unsigned long long st, double *R, double *g2,
                              unsigned *status) {
    uint32_t k0, k1;
    philox_key(S, sys, RNG_CENTROID, &k0, &k1);
    *R = normal2(philox4x32_10(0u, 0u, (uint32_t)st, (uint32_t)(st >> 32), k0, k1)).x;
    bool ok = true;
    *g2 = 2.0 * gamma_mt_warp(0.5 * (S.n_dof - 1), S, sys, st, &ok);
    if (!ok && (threadIdx.x & 31) == 0) atomicOr(status, (unsigned)ST_GAMMA_LIMIT);
}

__global__ void __launch_bounds__(256) k_ring(RingArgs a) {
    if ((int)blockIdx.x < a.n_draw) {
        // draw blocks (the first ones, so that they start with the first wave): the
        // PILE-G centroid draws at the current step, made while the ring work runs
        const int sys = a.draw_sys0 + blockIdx.x;
        const SysDev &S = a.sys[sys];
        if (threadIdx.x >= 32 || !(S.thermostat == 1 || a.pile_g)) return;
        double R, g2;
        const unsigned long long st = *a.step;
        centroid_draw(S, sys, st, &R, &g2, a.status);
        if (threadIdx.x == 0) {
            a.run[sys].R_draw = R;
            a.run[sys].g2_draw = g2;
            a.run[sys].draw_step_plus1 = st + 1;
        }
        return;
    }
    const ColWork W = a.work[blockIdx.x - a.n_draw];
    const SysDev &S = a.sys[W.sys];
    const int P = S.n_beads, C = S.cols_per_block;
    const int k = threadIdx.x / C, c = threadIdx.x - k * C;
    const bool act = (k < P) && (c < W.ncols);
    const int col = W.col0 + c;
    const int flags = a.flags;
    extern __shared__ double sh[];
    double *Cm = sh;
    double *Xq = Cm + P * P;
    double *Xp = Xq + P * C;
    double *Zq = Xp + P * C;  // folded sums / differences, then back-transformed values
    double *Zp = Zq + P * C;
    __shared__ double hred[256];
    // Rows 0..P/2 of C are symmetric in b <-> P-b and rows P/2+1..P-1 are
    // antisymmetric (zero at b = 0 and b = P/2), so each transform is applied to
    // s_b = x_b + x_{P-b} and d_b = x_b - x_{P-b}, b = 1..h: half the FMAs.
    const int h = (P - 1) / 2, half = P / 2;
    const bool even = (P % 2) == 0;
    if (flags & (RF_FWD | RF_BACK))
        for (int t = threadIdx.x; t < P * P; t += blockDim.x) Cm[t] = a.nm[S.nm_off + t];
    const long long at = S.q_off + (long long)k * S.n_dof + col;
    double qb = 0.0, pb = 0.0;
    const double m = act ? a.mass[S.mass_off + col] : 1.0;
    const double im = act ? a.inv_mass[S.mass_off + col] : 1.0;
    if (act) {
        qb = a.q[at];
        pb = a.p[at];
        if (flags & RF_KICK) pb += S.halfdt * a.f[at];
    }
    const double q_old = qb;
    double yq = qb, yp = pb;
    // P divisible by 4 (P >= 8): the rows are also symmetric about b = P/4 -- cos rows k
    // have C[k][P/2 - b] = (-1)^k C[k][b], sin rows of frequency j = P - k have
    // C[k][P/2 - b] = (-1)^(j+1) C[k][b] -- so a second fold halves the FMAs again
    const bool fold2 = (P % 4) == 0 && P >= 8;
    const int q4 = P / 4;
    if ((flags & RF_FWD) && fold2) {
        if (k < P) {
            Xq[k * C + c] = qb;
            Xp[k * C + c] = pb;
        }
        __syncthreads();
        // folded inputs, index j (x C + c): ss_b, sd_b, ds_b, dd_b (b = 1 .. q4 - 1) at
        // j = b - 1 + {0, 1, 2, 3} (q4 - 1), then s_q4, d_q4, x_0 + x_P/2, x_0 - x_P/2
        if (k < q4 && c < W.ncols) {
            for (int u = 0; u < 2; ++u) {
                const double *X = u ? Xp : Xq;
                double *Z = u ? Zp : Zq;
                if (k == 0) {
                    const double a0 = X[c], ah = X[half * C + c], a4 = X[q4 * C + c], a3 = X[(P - q4) * C + c];
                    Z[(4 * q4 - 4) * C + c] = a4 + a3;
                    Z[(4 * q4 - 3) * C + c] = a4 - a3;
                    Z[(4 * q4 - 2) * C + c] = a0 + ah;
                    Z[(4 * q4 - 1) * C + c] = a0 - ah;
                } else {
                    const double x1 = X[k * C + c], x2 = X[(P - k) * C + c];
                    const double x3 = X[(half - k) * C + c], x4 = X[(half + k) * C + c];
                    const double s1 = x1 + x2, s2 = x3 + x4, d1 = x1 - x2, d2 = x3 - x4;
                    Z[(k - 1) * C + c] = s1 + s2;
                    Z[(q4 - 1 + k - 1) * C + c] = s1 - s2;
                    Z[(2 * q4 - 2 + k - 1) * C + c] = d1 + d2;
                    Z[(3 * q4 - 3 + k - 1) * C + c] = d1 - d2;
                }
            }
        }
        __syncthreads();
        if (act) {
            const double *row = Cm + k * P;
            const bool sym = k <= half;
            const int par = sym ? (k & 1) : ((P - k) & 1);
            // cos rows: ss (k even) or sd (k odd); sin rows: ds (j odd) or dd (j even)
            const int base = sym ? (par ? q4 - 1 : 0) : (par ? 2 * q4 - 2 : 3 * q4 - 3);
            const int mid = sym ? 4 * q4 - 4 : 4 * q4 - 3;
            const int end = par ? 4 * q4 - 1 : 4 * q4 - 2;
            double sq = sym ? row[0] * Zq[end * C + c] : 0.0;
            double sp = sym ? row[0] * Zp[end * C + c] : 0.0;
            for (int b = 1; b < q4; ++b) {
                sq += row[b] * Zq[(base + b - 1) * C + c];
                sp += row[b] * Zp[(base + b - 1) * C + c];
            }
            yq = sq + row[q4] * Zq[mid * C + c];
            yp = sp + row[q4] * Zp[mid * C + c];
        }
        __syncthreads();
    } else
    if (flags & RF_FWD) {
        if (k < P) {
            Xq[k * C + c] = qb;
            Xp[k * C + c] = pb;
        }
        __syncthreads();
        if (k >= 1 && k <= h) {
            const double aq = Xq[k * C + c], bq = Xq[(P - k) * C + c];
            const double ap = Xp[k * C + c], bp = Xp[(P - k) * C + c];
            Zq[(k - 1) * C + c] = aq + bq;
            Zq[(h + k - 1) * C + c] = aq - bq;
            Zp[(k - 1) * C + c] = ap + bp;
            Zp[(h + k - 1) * C + c] = ap - bp;
        }
        __syncthreads();
        if (act) {
            const double *row = Cm + k * P;
            double sq, sp;
            if (k <= half) {  // symmetric row
                sq = row[0] * Xq[c];
                sp = row[0] * Xp[c];
                if (even && half > 0 && k <= half) {
                    sq += row[half] * Xq[half * C + c];
                    sp += row[half] * Xp[half * C + c];
                }
                for (int b = 1; b <= h; ++b) {
                    sq += row[b] * Zq[(b - 1) * C + c];
                    sp += row[b] * Zp[(b - 1) * C + c];
                }
            } else {  // antisymmetric row
                sq = 0.0;
                sp = 0.0;
                for (int b = 1; b <= h; ++b) {
                    sq += row[b] * Zq[(h + b - 1) * C + c];
                    sp += row[b] * Zp[(h + b - 1) * C + c];
                }
            }
            yq = sq;
            yp = sp;
        }
        __syncthreads();
    }
    double heat = 0.0;
    // centroid-constrained PIMD: the centroid normal mode carries no momentum, so
    // the free ring-polymer step (omega_0 = 0) leaves the centroid where it is
    const bool fixed0 = S.centroid_fixed && k == 0 && (flags & RF_FWD);
    if (fixed0) yp = 0.0;
    if (act) {
        if (flags & RF_VV) {
            // update.cpp:87-91
            const double dq = yp * S.dt * im;
            if ((flags & RF_DISP) && (col % 9) < 3) a.disp[S.d_off + 3 * (col / 9) + (col % 9)] += dq;
            yq += dq;
        }
        const ModeCoef mc = a.modes[S.mode_off + k];
        // half sqrt-Cayley step (update.cpp:301-320): q' = scale (q + dt/2 p / m),
        // p' = scale (p - dt/2 omega_k^2 m q), with the mode's products precomputed
        const double cqi = mc.cq * im, cpm = mc.cp * m;
        if (flags & RF_CAYLEY) {
            const double nq = fma(cqi, yp, mc.scale * yq);
            yp = fma(-cpm, yq, mc.scale * yp);
            yq = nq;
        }
        if ((flags & RF_THERMO) && (S.thermostat != 0 || a.pile_g) && !fixed0) {
            const double before = yp;
            if (k == 0 && (S.thermostat == 1 || a.pile_g)) {
                yp *= a.run[W.sys].alpha;  // PILE-G centroid (thermostat.cpp:88-104)
            } else {
                double c1 = mc.c1, c2n = mc.c2n;
                if (k == 0) {  // PILE-L centroid
                    c1 = S.c1_centroid;
                    c2n = S.c2n_centroid;
                }
                double xi;
                if (a.noise && k > 0) {
                    xi = a.noise[2 + (size_t)(k - 1) * S.n_dof + col];
                } else {
                    uint32_t k0, k1;
                    philox_key(S, W.sys, RNG_MODES, &k0, &k1);
                    const unsigned long long st = *a.step;
                    xi = normal_f32(philox4x32_10((uint32_t)col, (uint32_t)k, (uint32_t)st,
                                                  (uint32_t)(st >> 32), k0, k1));
                }
                // thermostat.cpp:131-136: sqrt(m / beta_P) c2 xi
                yp = fma(c1, yp, a.sqrt_mass[S.mass_off + col] * c2n * xi);
            }
            // kinetic energy change p'^2 / 2m - p^2 / 2m
            heat = 0.5 * im * (yp - before) * (yp + before);
        }
        if (flags & RF_CAYLEY) {
            const double nq = fma(cqi, yp, mc.scale * yq);
            yp = fma(-cpm, yq, mc.scale * yp);
            yq = nq;
        }
    }
    double qn = yq, pn = yp;
    if ((flags & RF_BACK) && fold2) {
        if (k < P) {
            Xq[k * C + c] = yq;
            Xp[k * C + c] = yp;
        }
        __syncthreads();
        // thread t = k < 2 (q4 + 1): quantity t / (q4 + 1) (q, p), column entry
        // b = t % (q4 + 1); cos rows split by the parity of k (E, O), sin rows by the
        // parity of j (Be, Bo): A_b = E + O, A_P/2-b = E - O, B_b = Bo + Be,
        // B_P/2-b = Bo - Be, and x_b = A_b + B_b, x_P-b = A_b - B_b (likewise at P/2 - b)
        if (k < 2 * (q4 + 1) && c < W.ncols) {
            const int u = k / (q4 + 1), b = k - u * (q4 + 1);
            const double *X = u ? Xp : Xq;
            double *Z = u ? Zp : Zq;
            double E = 0.0, O = 0.0, Be = 0.0, Bo = 0.0;
            for (int r = 0; r <= half; r += 2) E += Cm[r * P + b] * X[r * C + c];
            for (int r = 1; r < half; r += 2) O += Cm[r * P + b] * X[r * C + c];
            for (int j = 2; j < half; j += 2) Be += Cm[(P - j) * P + b] * X[(P - j) * C + c];
            for (int j = 1; j < half; j += 2) Bo += Cm[(P - j) * P + b] * X[(P - j) * C + c];
            const double A1 = E + O, A2 = E - O, B1 = Bo + Be, B2 = Bo - Be;
            Z[b * C + c] = A1 + B1;
            if (b > 0) Z[(P - b) * C + c] = A1 - B1;
            if (b < q4) {
                Z[(half - b) * C + c] = A2 + B2;
                if (b > 0) Z[(half + b) * C + c] = A2 - B2;
            }
        }
        __syncthreads();
        if (act) {
            qn = Zq[k * C + c];
            pn = Zp[k * C + c];
        }
    } else
    if (flags & RF_BACK) {
        if (k < P) {
            Xq[k * C + c] = yq;
            Xp[k * C + c] = yp;
        }
        __syncthreads();
        // thread b <= P/2 forms A_b (symmetric rows) and B_b (antisymmetric rows);
        // x_b = A_b + B_b and x_{P-b} = A_b - B_b
        if (k <= half && k < P && c < W.ncols) {
            double aq = Cm[k] * Xq[c], ap = Cm[k] * Xp[c];
            if (even && half > 0) {
                aq += Cm[half * P + k] * Xq[half * C + c];
                ap += Cm[half * P + k] * Xp[half * C + c];
            }
            double bq = 0.0, bp = 0.0;
            for (int j = 1; j <= h; ++j) {
                const double cs = Cm[j * P + k], sn = Cm[(P - j) * P + k];
                aq += cs * Xq[j * C + c];
                ap += cs * Xp[j * C + c];
                bq += sn * Xq[(P - j) * C + c];
                bp += sn * Xp[(P - j) * C + c];
            }
            Zq[k * C + c] = aq + bq;
            Zp[k * C + c] = ap + bp;
            if (k > 0 && 2 * k != P) {
                Zq[(P - k) * C + c] = aq - bq;
                Zp[(P - k) * C + c] = ap - bp;
            }
        }
        __syncthreads();
        if (act) {
            qn = Zq[k * C + c];
            pn = Zp[k * C + c];
        }
    }
    if (act) {
        a.q[at] = qn;
        a.p[at] = pn;
        if ((flags & RF_DISP) && !(flags & RF_VV) && (col % 9) < 3)
            a.disp[S.d_off + (long long)k * 3 * S.n_mols + 3 * (col / 9) + (col % 9)] += qn - q_old;
    }
    if (flags & RF_THERMO) {
        // one warp sums the block's values (8 a lane), then one 5-level shuffle
        // reduction; the blocks' sums go to the system's heat in slot order
        __shared__ double bsum;
        hred[threadIdx.x] = heat;
        __syncthreads();
        if (threadIdx.x < 32) {
            double t = 0.0;
            for (int k = threadIdx.x; k < (int)blockDim.x; k += 32) t += hred[k];
            t = warp_sum(t);
            if (threadIdx.x == 0) bsum = t;
        }
        __syncthreads();
        double *const dst[1] = {&a.run[W.sys].heat};
        ordered_system_sum<1>(&bsum, W.slot, S.cw_begin, S.cw_count, a.cw_part, a.cw_ticket + W.sys, dst);
    }
}

// Closing kick and the per-step estimator partial sums (bead space).
__device__ void finalize_system(const FinalizeArgs &a, int s, unsigned long long st, unsigned long long rec);

__global__ void __launch_bounds__(256) k_end_step(RingArgs a) {
    const ColWork W = a.work[blockIdx.x];
    const SysDev &S = a.sys[W.sys];
    const int P = S.n_beads, C = S.cols_per_block;
    const int b = threadIdx.x / C, c = threadIdx.x - b * C;
    const bool act = (b < P) && (c < W.ncols);
    const int col = W.col0 + c;
    extern __shared__ double sh[];
    double *Xq = sh;
    double *Xp = Xq + P * C;
    double *Xf = Xp + P * C;  // physical forces (centroid-constrained systems)
    __shared__ double qbar[256];
    const bool cf = a.kick && S.centroid_fixed && a.cf_acc;
    __shared__ double red4[4][256];
    __shared__ double2 cpart[256];  // [b][c], b < min(8, P): bead-sum partials of (q, p + dt/2 f)
    const long long at = S.q_off + (long long)b * S.n_dof + col;
    double qb = 0.0, pb = 0.0, fb = 0.0, fpb = 0.0;
    const double m = act ? a.mass[S.mass_off + col] : 1.0;
    const double im = act ? a.inv_mass[S.mass_off + col] : 1.0;
    __shared__ double *p_out;  // staged per-call step: the caller's momentum array
    if (threadIdx.x == 0) p_out = a.post_box ? a.post_box->p : nullptr;
    if (act) {
        qb = a.q[at];
        pb = a.p[at];
    }
    pdl_wait();  // the forces of the evaluation ahead
    __syncthreads();
    if (act) {
        fb = a.f[at];
        fpb = a.fphys[at];
        if (a.kick) {
            pb += S.halfdt * fb;  // update.cpp:391-397
            a.p[at] = pb;
        }
        if (p_out) p_out[(long long)b * S.n_dof + col] = pb;
        Xq[b * C + c] = qb;
        Xp[b * C + c] = pb + S.halfdt * fb;
        if (cf) Xf[b * C + c] = fpb;
    }
    __syncthreads();
    // mean centroid force of constrained PIMD: (1/P) sum_b F_b, accumulated per step
    if (cf && b == 0 && c < W.ncols) {
        double sf = 0.0;
        for (int j = 0; j < P; ++j) sf += Xf[j * C + c];
        a.cf_acc[S.mass_off + col] += sf / (double)P;
        if (col == 0) a.run[W.sys].cf_samples += 1.0;
    }
    // the centroid (path_integrals.cpp:10-26) and the centroid normal-mode kinetic
    // energy after the next opening kick: rows b < 8 sum beads b, b + 8, ... of each
    // column, then row 0 adds the eight partials
    double k0 = 0.0;
    if (b < 8 && c < W.ncols) {
        double sq = 0.0, sp = 0.0;
        for (int j = b; j < P; j += 8) {
            sq += Xq[j * C + c];
            sp += Xp[j * C + c];
        }
        cpart[b * C + c] = make_double2(sq, sp);
    }
    __syncthreads();
    if (b == 0 && c < W.ncols) {
        double sq = 0.0, sp = 0.0;
        for (int j = 0; j < 8 && j < P; ++j) {
            sq += cpart[j * C + c].x;
            sp += cpart[j * C + c].y;
        }
        qbar[c] = sq * S.inv_p;
        const double p0 = S.sqrt_inv_p * sp;
        k0 = 0.5 * p0 * p0 * im;
    }
    __syncthreads();
    double kin = 0.0, spring = 0.0, tq = 0.0;
    if (act) {
        kin = 0.5 * pb * pb * im;
        const double qn = Xq[((b + 1) % P) * C + c];
        const double dq = qb - qn;
        spring = m * S.half_omega_psq * dq * dq;
        const int all = a.kcv_all_beads < 0 ? (S.propagator == 1) : a.kcv_all_beads;
        if (all || (b % 2 == 0)) tq = -(qb - qbar[c]) * fpb;
    }
    // block reduction of the four sums: transposed through shared memory so that
    // warp w sums quantity w (8 values a lane, then 5 shuffle levels), a third of
    // the FP64 adds of four full warp reductions per warp
    red4[0][threadIdx.x] = kin;
    red4[1][threadIdx.x] = spring;
    red4[2][threadIdx.x] = tq;
    red4[3][threadIdx.x] = k0;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __shared__ double bsum[4];
    if (w < 4) {
        double t = 0.0;
        for (int k = lane; k < (int)blockDim.x; k += 32) t += red4[w][k];
        t = warp_sum(t);
        if (lane == 0) bsum[w] = t;
    }
    __syncthreads();
    // the blocks' sums go to the system's accumulators in slot order
    SysAcc *ac = &a.acc[W.sys];
    double *const dst[4] = {&ac->kin, &ac->spring, &ac->kcv_tq, &ac->k0};
    // the step counters as they stand while this step runs (only the block that
    // finishes the last system advances them, after every system's close below)
    const unsigned long long st0 = a.fuse_fin ? *a.fin.step : 0ull, rec0 = a.fuse_fin ? *a.fin.records : 0ull;
    const bool last = ordered_system_sum<4>(bsum, W.slot, S.cw_begin, S.cw_count, a.cw_part, a.cw_ticket + W.sys, dst);
    if (last && a.post_box) {
        for (int k = threadIdx.x; k < P; k += blockDim.x) {
            a.post_energy[k] = a.sys_energy[k];
            a.post_rebuilt[k] = a.sys_rebuilt[k];
        }
        if (threadIdx.x == 0) {  // the thread that completed the accumulators
            a.post_box->heat_out = a.run[W.sys].heat;
            a.post_box->acc = a.acc[W.sys];
            a.post_box->status = *a.status;
            a.acc[W.sys] = SysAcc{};
            *a.status = 0u;
        }
    }
    // fused close of the step: the block that completed a system's sums records it
    // and sets its next centroid factor; the last system to finish advances the
    // step and record counters, as k_finalize would after every system
    if (last && a.fuse_fin && threadIdx.x < 32) {
        __syncwarp();
        finalize_system(a.fin, W.sys, st0, rec0);
        if (threadIdx.x == 0) {
            __threadfence();
            if (atomicAdd(a.fin.ticket, 1u) == (unsigned)(a.fin.sys_end - a.fin.sys_begin - 1)) {
                if (a.fin.record) *a.fin.records = rec0 + 1;
                *a.fin.step = st0 + 1;
                *a.fin.ticket = 0u;
            }
        }
    }
}

// Centroid normal-mode kinetic energy of normal-mode momenta (row 0 of p).
__global__ void k_centroid_ke(RingArgs a) {
    const ColWork W = a.work[blockIdx.x];
    const SysDev &S = a.sys[W.sys];
    __shared__ double red[8];
    double e = 0.0;
    for (int c = threadIdx.x; c < W.ncols; c += blockDim.x) {
        const int col = W.col0 + c;
        const double pv = a.p[S.q_off + col];
        e += 0.5 * pv * pv * a.inv_mass[S.mass_off + col];
    }
    __shared__ double bsum;
    const double t = block_sum(e, red);
    if (threadIdx.x == 0) bsum = t;
    __syncthreads();
    double *const dst[1] = {&a.acc[W.sys].k0};
    ordered_system_sum<1>(&bsum, W.slot, S.cw_begin, S.cw_count, a.cw_part, a.cw_ticket + W.sys, dst);
}

// The PILE-G centroid rescale factor of one system's per-call step
// (update.cpp:271-320 with thermostat.cpp:64-100): the centroid kinetic energy
// after the opening kick, k0 = sum_dof (sqrt(1/P) sum_b (p_b + dt/2 f_b))^2 / 2m
// (the half Cayley step leaves the centroid momentum alone), and the draws R and
// g2 (caller noise, else the counter-based generator at the system's step --
// made ahead by the previous per-call ring launch when it drew for this step).
// With a mailbox (a staged per-call step) the kernel also moves p and f from the
// caller's arrays to the device ones as it reads them.
// Block 0 makes the draws while blocks 1.. sum column blocks of k0; the block
// that arrives last on the system's ticket adds the column sums in slot order,
// sets alpha = sqrt((R^2 + g2) / (2 beta_n k0)) and advances the step counter, as
// the estimator-free finalize of this step did.
__global__ void __launch_bounds__(256) k_centroid_alpha(RingArgs a, int sys) {
    const SysDev &S = a.sys[sys];
    SysRun *run = &a.run[sys];
    __shared__ double X[256];
    __shared__ double red[8];
    __shared__ int last;
    if (blockIdx.x == 0) {
        if (threadIdx.x < 32) {
            double R, g2;
            const unsigned long long st = *a.step;
            if (a.noise) {
                R = a.noise[0];
                g2 = a.noise[1];
            } else if (run->draw_step_plus1 == st + 1) {  // made ahead by an earlier ring launch
                R = run->R_draw;
                g2 = run->g2_draw;
            } else {
                centroid_draw(S, sys, st, &R, &g2, a.status);
            }
            if (threadIdx.x == 0) {
                run->R_draw = R;
                run->g2_draw = g2;
            }
        }
    } else {
        const ColWork W = a.work[blockIdx.x - 1];
        const int P = S.n_beads, C = S.cols_per_block;
        const int b = threadIdx.x / C, c = threadIdx.x - b * C;
        const bool act = (b < P) && (c < W.ncols);
        const int col = W.col0 + c;
        // staged: p and f come from the caller's arrays and are stored on the device
        __shared__ const double *src[2];
        if (threadIdx.x == 0) {
            src[0] = a.box ? a.box->p : a.p + S.q_off;
            src[1] = a.box ? a.box->f : a.f + S.q_off;
        }
        __syncthreads();
        if (act) {
            const long long at = (long long)b * S.n_dof + col;
            const double pv = src[0][at], fv = src[1][at];
            if (a.box) {
                a.p[S.q_off + at] = pv;
                const_cast<double *>(a.f)[S.q_off + at] = fv;  // the device force array (RingArgs reads it)
            }
            X[threadIdx.x] = pv + S.halfdt * fv;
        }
        __syncthreads();
        double k0 = 0.0;
        if (b == 0 && c < W.ncols) {
            double sp = 0.0;
            for (int j = 0; j < P; ++j) sp += X[j * C + c];
            const double p0 = sqrt(1.0 / P) * sp;
            k0 = 0.5 * p0 * p0 * a.inv_mass[S.mass_off + col];
        }
        const double t = block_sum(k0, red);
        if (threadIdx.x == 0) a.cw_part[(size_t)W.slot * 4] = t;
    }
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(a.cw_ticket + sys, 1u) == (unsigned)S.cw_count;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double t = 0.0;
    for (int j = threadIdx.x; j < S.cw_count; j += blockDim.x) t += __ldcg(&a.cw_part[(size_t)(S.cw_begin + j) * 4]);
    t = block_sum(t, red);
    if (threadIdx.x == 0) {
        const double R = __ldcg(&run->R_draw), g2 = __ldcg(&run->g2_draw);
        a.acc[sys].k0 = t;
        run->alpha = sqrt((R * R + g2) / (2.0 * S.beta_n * t));
        // the step counter lives in writable device memory; RingArgs hands it to
        // the ring kernels read-only
        unsigned long long *step = const_cast<unsigned long long *>(a.step);
        *step = *step + 1;
        a.cw_ticket[sys] = 0u;
    }
}

// Bussi global rescale of a system's first n_dof momenta (thermostat.cpp:12-60):
// p *= alpha, alpha = sqrt((R^2 + g2) / (beta sum p^2 / m)), R ~ N(0,1) and
// g2 ~ chi^2(n_dof - 1) (caller noise [R, g2], else the counter-based draw at the
// system's step). The heat, kinetic energy before minus after = (1 - alpha^2)
// sum p^2 / 2m, goes to the system's run state. One block.
__global__ void __launch_bounds__(1024) k_bussi(RingArgs a, int sys) {
    const SysDev &S = a.sys[sys];
    const int nd = S.n_dof;
    double *p = a.p + S.q_off;
    const double *im = a.inv_mass + S.mass_off;
    __shared__ double red[32];
    __shared__ double alpha_sh;
    double p2 = 0.0;
    for (int i = threadIdx.x; i < nd; i += blockDim.x) p2 += p[i] * p[i] * im[i];
    p2 = block_sum(p2, red);  // every lane of warp 0 holds the total
    if (threadIdx.x < 32) {
        double R, g2;
        if (a.noise) {
            R = a.noise[0];
            g2 = a.noise[1];
        } else {
            centroid_draw(S, sys, *a.step, &R, &g2, a.status);
        }
        if (threadIdx.x == 0) {
            const double al = sqrt((R * R + g2) / (S.beta * p2));
            alpha_sh = al;
            a.run[sys].heat = 0.5 * p2 * (1.0 - al * al);
        }
    }
    __syncthreads();
    const double al = alpha_sh;
    for (int i = threadIdx.x; i < nd; i += blockDim.x) p[i] *= al;
}

// One system's step close (called by a whole warp): the estimator record
// (lane 0) and the next PILE-G centroid factor, then the step accumulators
// cleared. st, rec: the step and record counters at the start of the step.
__device__ void finalize_system(const FinalizeArgs &a, int s, unsigned long long st, unsigned long long rec) {
    const int lane = threadIdx.x & 31;
    const SysDev &S = a.sys[s];
    SysAcc *ac = &a.acc[s];
    SysRun *run = &a.run[s];
    const int P = S.n_beads;
    double vsum = 0.0, veven = 0.0;
    if (a.record) {  // the beads' energies summed across the warp
        for (int b = lane; b < P; b += 32) {
            const double e = a.energy[S.job_base + b];
            vsum += e;
            if (b % 2 == 0) veven += e;
        }
        vsum = warp_sum(vsum);
        veven = warp_sum(veven);
    }
    if (a.record && lane == 0) {
        double vtot, pot, kcv;
        const double half_nd_beta = S.half_nd_beta;
        if (S.propagator == 0) {  // Suzuki-Chin (forces.cpp:724-781, path_integrals.cpp:29-48)
            vtot = (2.0 * veven + 4.0 * (vsum - veven) + ac->sc_extra) / 3.0;
            pot = 2.0 * veven * S.inv_p;
            kcv = half_nd_beta + ac->kcv_tq * S.inv_p;
        } else {
            vtot = vsum;
            pot = vsum * S.inv_p;
            kcv = half_nd_beta + ac->kcv_tq * (0.5 * S.inv_p);
        }
        const double cons = vtot + ac->kin + ac->spring + run->heat;
        double *o = a.est + ((size_t)(rec % (unsigned long long)a.max_records) * a.n_sys + s) * 8;
        o[0] = pot;
        o[1] = kcv;
        o[2] = cons;
        o[3] = run->heat;
        o[4] = ac->kin;
        o[5] = vtot;
        o[6] = ac->rebuilds;
        o[7] = (double)st;
        if (!isfinite(cons) || !isfinite(vtot)) atomicOr(a.status, (unsigned)ST_NONFINITE);
    }
    if (a.draw_alpha && (S.thermostat == 1 || a.pile_g)) {
        double R, g2;
        if (a.noise && s == 0) {
            R = a.noise[0];
            g2 = a.noise[1];
        } else if (a.pre_drawn) {
            R = run->R_draw;
            g2 = run->g2_draw;
        } else {
            centroid_draw(S, s, st, &R, &g2, a.status);
        }
        if (lane == 0) run->alpha = sqrt((R * R + g2) / (2.0 * S.beta_n * ac->k0));
    }
    __syncwarp();
    if (lane == 0) ac->kin = ac->spring = ac->kcv_tq = ac->k0 = ac->sc_extra = ac->rebuilds = 0.0;
}

// One warp per system: finalize_system for every system. One block, so the step
// counters advance after every system.
__global__ void k_finalize(FinalizeArgs a) {
    const unsigned long long st = *a.step;
    const unsigned long long rec = *a.records;
    const int nw = blockDim.x >> 5;
    for (int s = a.sys_begin + (int)(threadIdx.x >> 5); s < a.sys_end; s += nw) finalize_system(a, s, st, rec);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (a.record) *a.records = rec + 1;
        *a.step = st + 1;
    }
}

// ---- Suzuki-Chin assembly (forces.cpp:724-775) -----------------------------------
__global__ void __launch_bounds__(256) k_sc_prepare(ScArgs a) {
    const int sid = a.job_sys[blockIdx.x], b = a.job_bead[blockIdx.x];
    const SysDev &S = a.sys[sid];
    const int nd = S.n_dof, P = S.n_beads;
    const double *fp = a.fphys + S.q_off + (size_t)b * nd;
    const double *im = a.inv_mass + S.mass_off;
    __shared__ double red[8];
    __shared__ double scl_sh;
    double fsq = 0.0, dl = 0.0;
    for (int i = threadIdx.x; i < nd; i += blockDim.x) {
        const double f = fp[i];
        const double t = f * im[i];
        fsq += f * t;
        dl += t * t;
    }
    fsq = block_sum(fsq, red);
    dl = block_sum(dl, red);
    if (threadIdx.x == 0) {
        double delta = dl / (S.n_sites * P);
        delta = 1.0 / sqrt(delta);
        const double scl = S.eps_sc * delta;
        scl_sh = scl;
        a.sc_scale[S.job_base + b] = scl;
        atomicAdd(&a.acc[sid].sc_extra, fsq / (3.0 * S.omega_psq));
    }
    __syncthreads();
    const double scl = scl_sh;
    const double *qb = a.q + S.q_off + (size_t)b * nd;
    double *qp = a.qdisp + S.q_off + (size_t)b * nd;
    double *qm = a.qdisp + S.q_off + (size_t)(b - 1) * nd;
    for (int i = threadIdx.x; i < nd; i += blockDim.x) {
        const double v = fp[i] * im[i];
        const double dq = scl * v;
        qp[i] = qb[i] + dq;
        qm[i] = qb[i] - dq;
        if (a.mixed) a.dirv[S.q_off + (size_t)b * nd + i] = v;
    }
}

__global__ void __launch_bounds__(256) k_sc_finish(ScArgs a) {
    const int sid = a.job_sys[blockIdx.y], b = a.job_bead[blockIdx.y];
    const SysDev &S = a.sys[sid];
    const int nd = S.n_dof;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nd) return;
    const size_t at = S.q_off + (size_t)b * nd + i;
    const double fp = a.fphys[at];
    double f;
    if (S.propagator == 1 && !a.force_sc) {
        f = fp;  // second-order assembly: every bead weight 1
    } else if (b % 2 == 0) {
        f = 2.0 * fp / 3.0;
    } else {
        const double scl = a.sc_scale[S.job_base + b];
        const double fscale = 1.0 / (9.0 * S.omega_psq * scl);
        const size_t am = at - nd;
        double diff;
        if (a.mixed) diff = 2.0 * scl * a.fdisp[at] + (a.fsr[at] - a.fsr[am]);
        else diff = a.fdisp[at] - a.fdisp[am];
        f = 4.0 * fp / 3.0;
        f -= fscale * diff;
    }
    a.f[at] = f;
}

// Plain bead <-> normal-mode transform of an arbitrary-length array (tier-1 ftransform).
__global__ void __launch_bounds__(256) k_transform(int P, int C, const double *nm, double *x, int length,
                                                   int forwards) {
    const int k = threadIdx.x / C, c = threadIdx.x - k * C;
    const int col = blockIdx.x * C + c;
    const bool act = (k < P) && (col < length);
    extern __shared__ double sh[];
    double *Cm = sh;
    double *X = Cm + P * P;
    for (int t = threadIdx.x; t < P * P; t += blockDim.x) Cm[t] = nm[t];
    if (k < P) X[k * C + c] = act ? x[(size_t)k * length + col] : 0.0;
    __syncthreads();
    if (!act) return;
    double s = 0.0;
    if (forwards)
        for (int b = 0; b < P; ++b) s += Cm[k * P + b] * X[b * C + c];
    else
        for (int j = 0; j < P; ++j) s += Cm[j * P + k] * X[j * C + c];
    x[(size_t)k * length + col] = s;
}

__global__ void __launch_bounds__(256) k_nm_energy(const SysDev *sys, int sysi, int P, int n_dof,
                                                   const double *q, const double *p, const double *mass,
                                                   const ModeCoef *modes, double *out) {
    const SysDev &S = sys[sysi];
    __shared__ double red[8];
    double kin = 0.0, spr = 0.0;
    const size_t total = (size_t)P * n_dof;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(t / n_dof), j = (int)(t - (size_t)k * n_dof);
        const double m = mass[S.mass_off + j], pv = p[S.q_off + t], qv = q[S.q_off + t];
        kin += 0.5 * pv * pv / m;
        spr += 0.5 * modes[S.mode_off + k].w2 * m * qv * qv;
    }
    kin = block_sum(kin, red);
    spr = block_sum(spr, red);
    if (threadIdx.x == 0) {
        atomicAdd(&out[0], kin);
        atomicAdd(&out[1], spr);
    }
}

}  // namespace

void init_propagate_kernel_attributes() {
    cudaFuncSetAttribute(k_ring, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    cudaFuncSetAttribute(k_transform, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

void launch_nm_energy(const SysDev *sys, int sysi, int P, int n_dof, const double *q, const double *p,
                      const double *mass, const ModeCoef *modes, double *out, cudaStream_t s,
                      unsigned long long *n) {
    k_nm_energy<<<64, 256, 0, s>>>(sys, sysi, P, n_dof, q, p, mass, modes, out);
    if (n) ++*n;
}

void launch_ring(const RingArgs &a, cudaStream_t s, unsigned long long *n) {
    if (a.n_work <= 0) return;
    // shared memory: P^2 + 4 P C doubles, with P C <= 256
    size_t smem = (size_t)(a.max_p * a.max_p + 4 * 256) * sizeof(double);
    k_ring<<<a.n_work + a.n_draw, 256, smem, s>>>(a);
    if (n) ++*n;
}

void launch_end_step(const RingArgs &a, cudaStream_t s, unsigned long long *n) {
    if (a.n_work <= 0) return;
    launch_pdl(k_end_step, dim3(a.n_work), dim3(256), 3 * 256 * sizeof(double), s, a);
    if (n) ++*n;
}

void launch_centroid_ke(const RingArgs &a, cudaStream_t s, unsigned long long *n) {
    if (a.n_work <= 0) return;
    k_centroid_ke<<<a.n_work, 256, 0, s>>>(a);
    if (n) ++*n;
}

void launch_bussi(const RingArgs &a, int sys, cudaStream_t s, unsigned long long *n) {
    k_bussi<<<1, 1024, 0, s>>>(a, sys);
    if (n) ++*n;
}

void launch_centroid_alpha(const RingArgs &a, int sys, cudaStream_t s, unsigned long long *n) {
    if (a.n_work <= 0) return;
    k_centroid_alpha<<<a.n_work + 1, 256, 0, s>>>(a, sys);
    if (n) ++*n;
}

void launch_finalize(const FinalizeArgs &a, cudaStream_t s, unsigned long long *n) {
    k_finalize<<<1, 512, 0, s>>>(a);
    if (n) ++*n;
}

void launch_sc_prepare(const ScArgs &a, cudaStream_t s, unsigned long long *n) {
    if (a.n_jobs <= 0) return;
    k_sc_prepare<<<a.n_jobs, 256, 0, s>>>(a);
    if (n) ++*n;
}

void launch_sc_finish(const ScArgs &a, cudaStream_t s, unsigned long long *n) {
    if (a.n_jobs <= 0) return;
    k_sc_finish<<<dim3((a.max_dof + 255) / 256, a.n_jobs), 256, 0, s>>>(a);
    if (n) ++*n;
}

void launch_transform(const SysDev *, int, int P, const double *nm_sys, double *x, int length, int forwards,
                      cudaStream_t s, unsigned long long *n) {
    const int C = P >= 256 ? 1 : 256 / P;
    const size_t smem = (size_t)(P * P + P * C) * sizeof(double);
    k_transform<<<(length + C - 1) / C, 256, smem, s>>>(P, C, nm_sys, x, length, forwards);
    if (n) ++*n;
}

}  // namespace qtg
