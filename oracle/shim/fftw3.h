/* Minimal stand-in for the two FFTW3 entry points the reference's fourier.cpp uses
 * (fftw_plan_r2r_1d with FFTW_R2HC / FFTW_HC2R, and fftw_execute).
 *
 * Test infrastructure only: it lets the reference sources compile into the
 * oracle library when FFTW is not installed. Written from FFTW's documented
 * "halfcomplex" r2r convention:
 *   R2HC: out = r_0, r_1, ..., r_{n/2}, i_{(n+1)/2-1}, ..., i_1 where
 *         r_k + i*i_k = sum_j in_j * exp(-2*pi*i*j*k/n)   (unnormalised)
 *   HC2R: the inverse of R2HC up to a factor n (unnormalised), i.e.
 *         out_j = sum_k Y_k exp(+2*pi*i*j*k/n) with Y Hermitian.
 * Direct O(n^2) sums are used; the angle is reduced as (j*k mod n) before the
 * trigonometric call, so the twiddles are accurate to a few ulp.
 */
#ifndef QTIP_ORACLE_FFTW3_SHIM_H
#define QTIP_ORACLE_FFTW3_SHIM_H

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum { FFTW_R2HC = 0, FFTW_HC2R = 1 } fftw_r2r_kind;

#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

struct qtip_shim_plan {
    int n;
    double *in;
    double *out;
    fftw_r2r_kind kind;
};
typedef struct qtip_shim_plan *fftw_plan;

static inline fftw_plan fftw_plan_r2r_1d(int n, double *in, double *out,
                                         fftw_r2r_kind kind, unsigned flags) {
    (void)flags;
    fftw_plan p = (fftw_plan)malloc(sizeof(struct qtip_shim_plan));
    p->n = n;
    p->in = in;
    p->out = out;
    p->kind = kind;
    return p;
}

static inline void fftw_destroy_plan(fftw_plan p) { free(p); }

static inline void qtip_shim_twiddle(int j, int k, int n, double *c, double *s) {
    const double two_pi = 6.283185307179586476925286766559;
    long m = ((long)j * (long)k) % n;
    double ang = two_pi * (double)m / (double)n;
    *c = cos(ang);
    *s = sin(ang);
}

static inline void fftw_execute(const fftw_plan p) {
    const int n = p->n;
    double *tmp = (double *)malloc(sizeof(double) * (size_t)n);
    if (p->kind == FFTW_R2HC) {
        for (int k = 0; k <= n / 2; ++k) {
            double re = 0.0, im = 0.0;
            for (int j = 0; j < n; ++j) {
                double c, s;
                qtip_shim_twiddle(j, k, n, &c, &s);
                re += p->in[j] * c;
                im -= p->in[j] * s;
            }
            tmp[k] = re;
            if (k > 0 && 2 * k != n) tmp[n - k] = im;
        }
    } else {
        for (int j = 0; j < n; ++j) {
            double acc = p->in[0];
            for (int k = 1; 2 * k < n; ++k) {
                double c, s;
                qtip_shim_twiddle(j, k, n, &c, &s);
                acc += 2.0 * (p->in[k] * c - p->in[n - k] * s);
            }
            if (n % 2 == 0) acc += p->in[n / 2] * ((j % 2 == 0) ? 1.0 : -1.0);
            tmp[j] = acc;
        }
    }
    memcpy(p->out, tmp, sizeof(double) * (size_t)n);
    free(tmp);
}

#ifdef __cplusplus
}
#endif
#endif
