/*
 * The five FFTW 3 entry points used by the FIt-SNE reference, implemented on top of
 * this project's fft64 (TEST INFRASTRUCTURE ONLY).  A plan binds its arrays at
 * creation time and fftw_execute() transforms them, as FFTW does; no scaling is
 * applied, as in FFTW.  Only the behaviour the reference relies on is provided
 * (FFTW_ESTIMATE plans, in-place or out-of-place 1-D c2c, out-of-place 2-D r2c/c2r).
 */
#include "shim_include/fftw3.h"

#include <stdlib.h>

#include "fft64.h"

enum { KIND_C2C = 1, KIND_R2C_2D = 2, KIND_C2R_2D = 3 };

struct fftw_shim_plan_s {
    int kind;
    int n0, n1;
    void *in;
    void *out;
    fft64_plan *c2c;
};

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags) {
    (void) flags;
    fftw_plan p = (fftw_plan) calloc(1, sizeof(*p));
    p->kind = KIND_C2C;
    p->n0 = n;
    p->in = in;
    p->out = out;
    p->c2c = fft64_plan_c2c(n, sign == FFTW_FORWARD ? -1 : +1);
    return p;
}

fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out, unsigned flags) {
    (void) flags;
    fftw_plan p = (fftw_plan) calloc(1, sizeof(*p));
    p->kind = KIND_R2C_2D;
    p->n0 = n0;
    p->n1 = n1;
    p->in = in;
    p->out = out;
    return p;
}

fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out, unsigned flags) {
    (void) flags;
    fftw_plan p = (fftw_plan) calloc(1, sizeof(*p));
    p->kind = KIND_C2R_2D;
    p->n0 = n0;
    p->n1 = n1;
    p->in = in;
    p->out = out;
    return p;
}

void fftw_execute(const fftw_plan p) {
    switch (p->kind) {
        case KIND_C2C:
            fft64_exec_c2c(p->c2c, (const double *) p->in, (double *) p->out);
            break;
        case KIND_R2C_2D:
            fft64_r2c_2d(p->n0, p->n1, (const double *) p->in, (double *) p->out);
            break;
        case KIND_C2R_2D:
            fft64_c2r_2d(p->n0, p->n1, (const double *) p->in, (double *) p->out);
            break;
        default:
            break;
    }
}

void fftw_destroy_plan(fftw_plan p) {
    if (!p) return;
    fft64_destroy(p->c2c);
    free(p);
}
