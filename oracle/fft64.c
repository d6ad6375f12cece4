/*
 * fft64 -- double-precision FFT for the CPU oracle (TEST INFRASTRUCTURE ONLY).
 * See fft64.h for the contract.  Written for this project; it replaces the FFTW 3
 * calls of the FIt-SNE reference (src/nbodyfft.cpp) when the reference is compiled
 * as a checker, and it is the FFT of the C restatement in fitsne_oracle.c.
 */
#include "fft64.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    double re, im;
} cplx;

#define FFT64_MAX_DIRECT_PRIME 31

struct fft64_plan {
    int n;
    int sign;
    int nstages;
    int radix[64];
    cplx *tw; /* tw[j] = exp(sign * 2*pi*i * j / n) */
    /* Bluestein */
    int blue;
    int m;
    cplx *chirp; /* c_k = exp(sign * pi*i * k^2 / n), k < n */
    cplx *bhat;  /* FFT_m of conj(chirp) embedded circularly */
    struct fft64_plan *sub_f;
    struct fft64_plan *sub_b;
};

static const double PI = 3.14159265358979323846264338327950288;

static inline cplx cmul(cplx a, cplx b) {
    cplx r;
    r.re = a.re * b.re - a.im * b.im;
    r.im = a.re * b.im + a.im * b.re;
    return r;
}

static int factorize(int n, int *radix) {
    int ns = 0;
    while (n % 4 == 0) { radix[ns++] = 4; n /= 4; }
    while (n % 2 == 0) { radix[ns++] = 2; n /= 2; }
    for (int p = 3; p <= FFT64_MAX_DIRECT_PRIME; p += 2) {
        while (n % p == 0) { radix[ns++] = p; n /= p; }
    }
    if (n != 1) return -1; /* a prime factor too large for the direct passes */
    return ns;
}

static cplx *twiddles(int n, int sign) {
    cplx *tw = (cplx *) malloc(sizeof(cplx) * (size_t) (n > 0 ? n : 1));
    for (int j = 0; j < n; j++) {
        double a = 2.0 * PI * (double) j / (double) n;
        tw[j].re = cos(a);
        tw[j].im = sign * sin(a);
    }
    return tw;
}

fft64_plan *fft64_plan_c2c(int n, int sign) {
    fft64_plan *p = (fft64_plan *) calloc(1, sizeof(fft64_plan));
    p->n = n;
    p->sign = sign;
    if (n <= 1) return p;
    int ns = factorize(n, p->radix);
    if (ns >= 0) {
        p->nstages = ns;
        p->tw = twiddles(n, sign);
        return p;
    }
    /* Bluestein: X_s = c_s * sum_k (x_k c_k) conj(c_{s-k}) */
    p->blue = 1;
    int m = 1;
    while (m < 2 * n - 1) m <<= 1;
    p->m = m;
    p->chirp = (cplx *) malloc(sizeof(cplx) * (size_t) n);
    for (int k = 0; k < n; k++) {
        long long kk = ((long long) k * k) % (2LL * n);
        double a = PI * (double) kk / (double) n;
        p->chirp[k].re = cos(a);
        p->chirp[k].im = sign * sin(a);
    }
    p->sub_f = fft64_plan_c2c(m, -1);
    p->sub_b = fft64_plan_c2c(m, +1);
    cplx *b = (cplx *) calloc((size_t) m, sizeof(cplx));
    for (int k = 0; k < n; k++) {
        cplx c = p->chirp[k];
        c.im = -c.im;
        b[k] = c;
        if (k) b[m - k] = c;
    }
    p->bhat = (cplx *) malloc(sizeof(cplx) * (size_t) m);
    fft64_exec_c2c(p->sub_f, (const double *) b, (double *) p->bhat);
    free(b);
    return p;
}

void fft64_destroy(fft64_plan *p) {
    if (!p) return;
    free(p->tw);
    free(p->chirp);
    free(p->bhat);
    fft64_destroy(p->sub_f);
    fft64_destroy(p->sub_b);
    free(p);
}

/* One Stockham pass of radix R; p = product of the radices of earlier passes. */
static void stockham_pass(int n, int R, int p, const cplx *tw, const cplx *in, cplx *out) {
    const int T = n / R;
    const int tws = n / (p * R);
    const int rot = n / R; /* tw[rot * q] = exp(sign*2*pi*i*q/R) */
    cplx u[FFT64_MAX_DIRECT_PRIME + 1];
    cplx y[FFT64_MAX_DIRECT_PRIME + 1];
    for (int i = 0; i < T; i++) {
        const int k = i % p;
        for (int r = 0; r < R; r++) {
            u[r] = in[i + r * T];
            if (r && k) u[r] = cmul(u[r], tw[r * k * tws]);
        }
        if (R == 2) {
            y[0].re = u[0].re + u[1].re; y[0].im = u[0].im + u[1].im;
            y[1].re = u[0].re - u[1].re; y[1].im = u[0].im - u[1].im;
        } else if (R == 4) {
            /* w = tw[n/4] = exp(sign*i*pi/2) = sign*i */
            const double s = tw[rot].im; /* +-1 */
            cplx a0 = {u[0].re + u[2].re, u[0].im + u[2].im};
            cplx a1 = {u[0].re - u[2].re, u[0].im - u[2].im};
            cplx b0 = {u[1].re + u[3].re, u[1].im + u[3].im};
            cplx b1 = {u[1].re - u[3].re, u[1].im - u[3].im};
            /* b1 * (s*i) = (-s*b1.im, s*b1.re) */
            cplx jb1 = {-s * b1.im, s * b1.re};
            y[0].re = a0.re + b0.re; y[0].im = a0.im + b0.im;
            y[2].re = a0.re - b0.re; y[2].im = a0.im - b0.im;
            y[1].re = a1.re + jb1.re; y[1].im = a1.im + jb1.im;
            y[3].re = a1.re - jb1.re; y[3].im = a1.im - jb1.im;
        } else {
            for (int s = 0; s < R; s++) {
                cplx acc = u[0];
                for (int r = 1; r < R; r++) {
                    cplx t = cmul(u[r], tw[rot * ((r * s) % R)]);
                    acc.re += t.re;
                    acc.im += t.im;
                }
                y[s] = acc;
            }
        }
        const int base = (i - k) * R + k;
        for (int r = 0; r < R; r++) out[base + r * p] = y[r];
    }
}

void fft64_exec_c2c(const fft64_plan *p, const double *xd, double *yd) {
    const int n = p->n;
    const cplx *x = (const cplx *) xd;
    cplx *y = (cplx *) yd;
    if (n <= 1) {
        if (n == 1 && xd != yd) y[0] = x[0];
        return;
    }
    if (!p->blue) {
        cplx *a = (cplx *) malloc(sizeof(cplx) * (size_t) n);
        cplx *b = (cplx *) malloc(sizeof(cplx) * (size_t) n);
        memcpy(a, x, sizeof(cplx) * (size_t) n);
        int prod = 1;
        for (int s = 0; s < p->nstages; s++) {
            stockham_pass(n, p->radix[s], prod, p->tw, a, b);
            prod *= p->radix[s];
            cplx *t = a;
            a = b;
            b = t;
        }
        memcpy(y, a, sizeof(cplx) * (size_t) n);
        free(a);
        free(b);
        return;
    }
    const int m = p->m;
    cplx *a = (cplx *) calloc((size_t) m, sizeof(cplx));
    for (int k = 0; k < n; k++) a[k] = cmul(x[k], p->chirp[k]);
    fft64_exec_c2c(p->sub_f, (const double *) a, (double *) a);
    for (int k = 0; k < m; k++) a[k] = cmul(a[k], p->bhat[k]);
    fft64_exec_c2c(p->sub_b, (const double *) a, (double *) a);
    const double inv = 1.0 / (double) m;
    for (int s = 0; s < n; s++) {
        cplx t = cmul(a[s], p->chirp[s]);
        y[s].re = t.re * inv;
        y[s].im = t.im * inv;
    }
    free(a);
}

/* Rows r and r+1 (or only r when r+1 == n0) of a real n0 x n1 array -> half spectra. */
void fft64_r2c_2d(int n0, int n1, const double *in, double *outd) {
    const int h = n1 / 2 + 1;
    cplx *out = (cplx *) outd;
    fft64_plan *pr = fft64_plan_c2c(n1, -1);
    cplx *z = (cplx *) malloc(sizeof(cplx) * (size_t) n1);
    for (int r = 0; r < n0; r += 2) {
        const int two = (r + 1 < n0);
        for (int k = 0; k < n1; k++) {
            z[k].re = in[(size_t) r * n1 + k];
            z[k].im = two ? in[(size_t) (r + 1) * n1 + k] : 0.0;
        }
        fft64_exec_c2c(pr, (const double *) z, (double *) z);
        for (int k = 0; k < h; k++) {
            cplx a = z[k];
            cplx b = z[(n1 - k) % n1];
            b.im = -b.im; /* conj(Z[n-k]) */
            out[(size_t) r * h + k].re = 0.5 * (a.re + b.re);
            out[(size_t) r * h + k].im = 0.5 * (a.im + b.im);
            if (two) {
                /* (a - b) / (2i) */
                out[(size_t) (r + 1) * h + k].re = 0.5 * (a.im - b.im);
                out[(size_t) (r + 1) * h + k].im = -0.5 * (a.re - b.re);
            }
        }
    }
    free(z);
    fft64_destroy(pr);
    fft64_plan *pc = fft64_plan_c2c(n0, -1);
    cplx *col = (cplx *) malloc(sizeof(cplx) * (size_t) n0);
    for (int k = 0; k < h; k++) {
        for (int r = 0; r < n0; r++) col[r] = out[(size_t) r * h + k];
        fft64_exec_c2c(pc, (const double *) col, (double *) col);
        for (int r = 0; r < n0; r++) out[(size_t) r * h + k] = col[r];
    }
    free(col);
    fft64_destroy(pc);
}

void fft64_c2r_2d(int n0, int n1, const double *ind, double *out) {
    const int h = n1 / 2 + 1;
    const cplx *in = (const cplx *) ind;
    cplx *tmp = (cplx *) malloc(sizeof(cplx) * (size_t) n0 * h);
    fft64_plan *pc = fft64_plan_c2c(n0, +1);
    cplx *col = (cplx *) malloc(sizeof(cplx) * (size_t) n0);
    for (int k = 0; k < h; k++) {
        for (int r = 0; r < n0; r++) col[r] = in[(size_t) r * h + k];
        fft64_exec_c2c(pc, (const double *) col, (double *) col);
        for (int r = 0; r < n0; r++) tmp[(size_t) r * h + k] = col[r];
    }
    free(col);
    fft64_destroy(pc);
    fft64_plan *pr = fft64_plan_c2c(n1, +1);
    cplx *z = (cplx *) malloc(sizeof(cplx) * (size_t) n1);
    for (int r = 0; r < n0; r += 2) {
        const int two = (r + 1 < n0);
        for (int k = 0; k < n1; k++) {
            /* Hermitian extension of each half row; DC and Nyquist taken as real */
            cplx a, b = {0.0, 0.0};
            int kk = k < h ? k : n1 - k;
            a = tmp[(size_t) r * h + kk];
            if (two) b = tmp[(size_t) (r + 1) * h + kk];
            if (k >= h) {
                a.im = -a.im;
                b.im = -b.im;
            }
            if (k == 0 || (2 * k == n1)) {
                a.im = 0.0;
                b.im = 0.0;
            }
            /* z = a + i b */
            z[k].re = a.re - b.im;
            z[k].im = a.im + b.re;
        }
        fft64_exec_c2c(pr, (const double *) z, (double *) z);
        for (int k = 0; k < n1; k++) {
            out[(size_t) r * n1 + k] = z[k].re;
            if (two) out[(size_t) (r + 1) * n1 + k] = z[k].im;
        }
    }
    free(z);
    fft64_destroy(pr);
    free(tmp);
}
