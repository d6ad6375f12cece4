/*
 * fitsne_oracle.c -- C restatement of the FIt-SNE reference path (v1.2.1).
 *
 * TEST INFRASTRUCTURE ONLY.  This is the CPU checker of the GPU library and the CPU
 * baseline that bench.py times on the GPU machine's host cores; it is never part of the GPU
 * product.  It restates, in plain C with OpenMP where the reference uses PARALLEL_FOR or
 * std::thread pools, the reference's algorithm with the same order of floating-point
 * operations, so that on identical inputs it reproduces the compiled reference
 * (oracle/_ref) to the last bit or to a few ulps.  Each function cites the reference
 * lines it follows (paths relative to the FIt-SNE project).
 *
 * The FFTs use this project's fft64 (the reference uses FFTW; see fft64.h).
 */
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "fft64.h"

typedef double (*kern1d_fn)(double, double, double);
typedef double (*kern2d_fn)(double, double, double, double, double);

/* ---------------------------------------------------------------------------------
 * kernels, src/tsne.cpp:69-94 */
static double k_sq_cauchy(double x, double y, double df) {
    (void) df;
    return pow(1.0 + pow(x - y, 2), -2);
}
static double k_general(double x, double y, double df) { return pow(1.0 + ((x - y) * (x - y)) / df, -(df)); }
static double k_sq_general(double x, double y, double df) {
    return pow(1.0 + ((x - y) * (x - y)) / df, -(df + 1.0));
}
static double k_sq_cauchy_2d(double x1, double x2, double y1, double y2, double df) {
    (void) df;
    return pow(1.0 + pow(x1 - y1, 2) + pow(x2 - y2, 2), -2);
}
static double k_general_2d(double x1, double x2, double y1, double y2, double df) {
    return pow(1.0 + ((x1 - y1) * (x1 - y1) + (x2 - y2) * (x2 - y2)) / df, -(df));
}
static double k_sq_general_2d(double x1, double x2, double y1, double y2, double df) {
    return pow(1.0 + ((x1 - y1) * (x1 - y1) + (x2 - y2) * (x2 - y2)) / df, -(df + 1.0));
}

static int nthreads_or_1(unsigned int n) { return n > 1 ? (int) n : 1; }

/* ---------------------------------------------------------------------------------
 * Lagrange basis at the in-box coordinates, src/nbodyfft.cpp:310-336.
 * out[j*N + i] = prod_{k != j} (t_i - s_k) / prod_{k != j} (s_j - s_k) */
static void lagrange_values(int p, int N, const double *t, const double *s, double *out) {
    double den[64];
    for (int j = 0; j < p; j++) {
        den[j] = 1;
        for (int k = 0; k < p; k++)
            if (k != j) den[j] *= s[j] - s[k];
    }
    for (int i = 0; i < N; i++)
        for (int j = 0; j < p; j++) {
            double v = 1;
            for (int k = 0; k < p; k++)
                if (j != k) v *= t[i] - s[k];
            out[(size_t) j * N + i] = v / den[j];
        }
}

/* node offsets inside one box: s_0 = h/2, s_k = s_{k-1} + h, h = 1/p */
static void box_nodes(int p, double *s) {
    double h = 1 / (double) p;
    s[0] = h / 2;
    for (int i = 1; i < p; i++) s[i] = s[i - 1] + h;
}

/* ---------------------------------------------------------------------------------
 * 2-D grid set-up and kernel spectrum, src/nbodyfft.cpp:9-70 */
static void setup_2d(double lo, double hi, int nb, int p, kern2d_fn kern, double df, double *lower, double *upper,
                     double *s, double *spec /* complex, (2M) x (M+1) */) {
    const int nbox = nb * nb;
    const double w = (hi - lo) / (double) nb;
    for (int i = 0; i < nb; i++)
        for (int j = 0; j < nb; j++) {
            lower[i * nb + j] = j * w + lo;
            upper[i * nb + j] = (j + 1) * w + lo;
            lower[nbox + i * nb + j] = i * w + lo;
            upper[nbox + i * nb + j] = (i + 1) * w + lo;
        }
    box_nodes(p, s);
    const int M = p * nb, n2 = 2 * M;
    double h = (1 / (double) p) * w;
    double *xt = (double *) malloc(sizeof(double) * M), *yt = (double *) malloc(sizeof(double) * M);
    xt[0] = lo + h / 2;
    yt[0] = lo + h / 2;
    for (int i = 1; i < M; i++) {
        xt[i] = xt[i - 1] + h;
        yt[i] = yt[i - 1] + h;
    }
    double *emb = (double *) calloc((size_t) n2 * n2, sizeof(double));
    for (int i = 0; i < M; i++)
        for (int j = 0; j < M; j++) {
            double v = kern(yt[0], xt[0], yt[i], xt[j], df);
            emb[(size_t) (M + i) * n2 + (M + j)] = v;
            emb[(size_t) (M - i) * n2 + (M + j)] = v;
            emb[(size_t) (M + i) * n2 + (M - j)] = v;
            emb[(size_t) (M - i) * n2 + (M - j)] = v;
        }
    fft64_r2c_2d(n2, n2, emb, spec);
    free(emb);
    free(xt);
    free(yt);
}

/* 2-D interpolation sums, src/nbodyfft.cpp:73-248 */
static void nbody_2d(int N, int T, const double *xs, const double *ys, const double *charges, int nb, int p,
                     const double *lower, const double *upper, const double *s, const double *kspec, double *pot,
                     int nthreads) {
    const int nbox = nb * nb;
    const int M = p * nb, n2 = 2 * M, H = n2 / 2 + 1;
    const size_t G = (size_t) nbox * p * p;
    const double lo = lower[0];
    const double w = upper[0] - lower[0];
    int *box = (int *) malloc(sizeof(int) * (size_t) N);
    for (int i = 0; i < N; i++) {
        int bx = (int) ((xs[i] - lo) / w);
        int by = (int) ((ys[i] - lo) / w);
        if (bx >= nb) bx = nb - 1;
        else if (bx < 0) bx = 0;
        if (by >= nb) by = nb - 1;
        else if (by < 0) by = 0;
        box[i] = by * nb + bx;
    }
    double *tx = (double *) malloc(sizeof(double) * N), *ty = (double *) malloc(sizeof(double) * N);
    for (int i = 0; i < N; i++) {
        tx[i] = (xs[i] - lower[box[i]]) / w;
        ty[i] = (ys[i] - lower[nbox + box[i]]) / w;
    }
    double *lx = (double *) malloc(sizeof(double) * (size_t) N * p);
    double *ly = (double *) malloc(sizeof(double) * (size_t) N * p);
    lagrange_values(p, N, tx, s, lx);
    lagrange_values(p, N, ty, s, ly);
    /* step 1: spread (serial, as in the reference) */
    double *wc = (double *) calloc(G * T, sizeof(double));
    for (int i = 0; i < N; i++) {
        const int bj = box[i] / nb, bi = box[i] % nb;
        for (int a = 0; a < p; a++)
            for (int b = 0; b < p; b++) {
                const size_t idx = (size_t) (bi * p + a) * M + (bj * p) + b;
                for (int d = 0; d < T; d++)
                    wc[idx * T + d] += ly[(size_t) b * N + i] * lx[(size_t) a * N + i] * charges[(size_t) i * T + d];
            }
    }
    /* step 2: per term, embed, r2c, multiply by the kernel spectrum, c2r, crop, scale */
    double *vals = (double *) calloc(G * T, sizeof(double));
    double *in = (double *) calloc((size_t) n2 * n2, sizeof(double));
    double *sp = (double *) malloc(sizeof(double) * 2 * (size_t) n2 * H);
    double *outr = (double *) malloc(sizeof(double) * (size_t) n2 * n2);
    for (int d = 0; d < T; d++) {
        for (int i = 0; i < M; i++)
            for (int j = 0; j < M; j++) in[(size_t) i * n2 + j] = wc[((size_t) i * M + j) * T + d];
        fft64_r2c_2d(n2, n2, in, sp);
        for (size_t k = 0; k < (size_t) n2 * H; k++) {
            const double xr = sp[2 * k], xi = sp[2 * k + 1], ur = kspec[2 * k], ui = kspec[2 * k + 1];
            sp[2 * k] = xr * ur - xi * ui;
            sp[2 * k + 1] = xr * ui + xi * ur;
        }
        fft64_c2r_2d(n2, n2, sp, outr);
        for (int i = 0; i < M; i++)
            for (int j = 0; j < M; j++)
                vals[((size_t) i * M + j) * T + d] = outr[(size_t) (M + i) * n2 + (M + j)] / (double) (n2 * n2);
    }
    free(in);
    free(sp);
    free(outr);
    /* step 3: gather (PARALLEL_FOR in the reference) */
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int i = 0; i < N; i++) {
        const int bi = box[i] % nb, bj = box[i] / nb;
        for (int a = 0; a < p; a++)
            for (int b = 0; b < p; b++)
                for (int d = 0; d < T; d++) {
                    const size_t idx = (size_t) (bi * p + a) * M + (bj * p) + b;
                    pot[(size_t) i * T + d] += lx[(size_t) a * N + i] * ly[(size_t) b * N + i] * vals[idx * T + d];
                }
    }
    free(box);
    free(tx);
    free(ty);
    free(lx);
    free(ly);
    free(wc);
    free(vals);
}

/* ---------------------------------------------------------------------------------
 * 1-D grid set-up, src/nbodyfft.cpp:251-307 */
static void setup_1d(double lo, double hi, int nb, int p, kern1d_fn kern, double df, double *lower, double *upper,
                     double *s, double *spec /* complex 2M */) {
    const double w = (hi - lo) / (double) nb;
    for (int b = 0; b < nb; b++) {
        lower[b] = b * w + lo;
        upper[b] = (b + 1) * w + lo;
    }
    box_nodes(p, s);
    const int M = p * nb;
    double h = (1 / (double) p) * w;
    double *yt = (double *) malloc(sizeof(double) * M);
    yt[0] = lo + h / 2;
    for (int i = 1; i < M; i++) yt[i] = yt[i - 1] + h;
    double *v = (double *) calloc(4 * (size_t) M, sizeof(double));
    for (int i = 0; i < M; i++) v[2 * (M + i)] = kern(yt[0], yt[i], df);
    for (int i = 1; i < M; i++) v[2 * i] = v[2 * (2 * M - i)];
    fft64_plan *pl = fft64_plan_c2c(2 * M, -1);
    fft64_exec_c2c(pl, v, spec);
    fft64_destroy(pl);
    free(v);
    free(yt);
}

/* 1-D interpolation sums, src/nbodyfft.cpp:339-455 (serial in the reference) */
static void nbody_1d(int N, int T, const double *Y, const double *charges, int nb, int p, const double *lower,
                     const double *upper, const double *s, const double *kspec, double *pot) {
    const int M = p * nb;
    const double lo = lower[0];
    const double w = upper[0] - lower[0];
    int *box = (int *) malloc(sizeof(int) * (size_t) N);
    for (int i = 0; i < N; i++) {
        int b = (int) ((Y[i] - lo) / w);
        if (b >= nb) b = nb - 1;
        box[i] = b;
    }
    double *t = (double *) malloc(sizeof(double) * N);
    for (int i = 0; i < N; i++) t[i] = (Y[i] - lower[box[i]]) / w;
    double *l = (double *) malloc(sizeof(double) * (size_t) N * p);
    lagrange_values(p, N, t, s, l);
    double *wc = (double *) calloc((size_t) M * T, sizeof(double));
    for (int i = 0; i < N; i++) {
        const int b0 = box[i] * p;
        for (int a = 0; a < p; a++)
            for (int d = 0; d < T; d++) wc[(size_t) (b0 + a) * T + d] += l[(size_t) a * N + i] * charges[(size_t) i * T + d];
    }
    double *emb = (double *) calloc(2 * (size_t) M * T, sizeof(double));
    for (int i = 0; i < M; i++)
        for (int d = 0; d < T; d++) emb[(size_t) (M + i) * T + d] = wc[(size_t) i * T + d];
    double *z = (double *) malloc(sizeof(double) * 4 * (size_t) M);
    double *vals = (double *) calloc((size_t) M * T, sizeof(double));
    fft64_plan *pf = fft64_plan_c2c(2 * M, -1), *pb = fft64_plan_c2c(2 * M, +1);
    for (int d = 0; d < T; d++) {
        for (int i = 0; i < 2 * M; i++) {
            z[2 * i] = emb[(size_t) i * T + d];
            z[2 * i + 1] = 0.0;
        }
        fft64_exec_c2c(pf, z, z);
        for (int i = 0; i < 2 * M; i++) {
            const double xr = z[2 * i], xi = z[2 * i + 1], ur = kspec[2 * i], ui = kspec[2 * i + 1];
            z[2 * i] = xr * ur - xi * ui;
            z[2 * i + 1] = xr * ui + xi * ur;
        }
        fft64_exec_c2c(pb, z, z);
        for (int i = 0; i < M; i++) vals[(size_t) i * T + d] = z[2 * i] / (M * 2.0);
    }
    fft64_destroy(pf);
    fft64_destroy(pb);
    for (int i = 0; i < N; i++) {
        const int b0 = box[i] * p;
        for (int a = 0; a < p; a++)
            for (int d = 0; d < T; d++)
                pot[(size_t) i * T + d] += l[(size_t) a * N + i] * vals[(size_t) (b0 + a) * T + d];
    }
    free(box);
    free(t);
    free(l);
    free(wc);
    free(emb);
    free(z);
    free(vals);
}

/* ---------------------------------------------------------------------------------
 * box counts: src/tsne.cpp:1065-1077 (2-D, rounded) and 663 / 774 (1-D) */
static int boxes_2d(double lo, double hi, double ipi, int min_int) {
    static const int allowed[20] = {25, 36, 50, 55, 60, 65, 70, 75, 80, 85, 90, 96, 100, 110, 120, 130, 140, 150, 175, 200};
    int nb = (int) fmax(min_int, (hi - lo) / ipi);
    if (nb < allowed[19]) {
        int i = 0;
        while (allowed[i] < nb) i++;
        nb = allowed[i];
    }
    return nb;
}

/* attraction over CSR rows (PARALLEL_FOR in the reference) */
static void attraction(const unsigned *row, const unsigned *col, const double *val, const double *Y, int N, int D,
                       double df, int df_is_one, double *pos, int nthreads) {
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int i = 0; i < N; i++) {
        double a0 = 0, a1 = 0;
        for (unsigned e = row[i]; e < row[i + 1]; e++) {
            const unsigned j = col[e];
            if (D == 2) {
                const double dx = Y[2 * i] - Y[2 * j], dy = Y[2 * i + 1] - Y[2 * j + 1];
                const double d2 = dx * dx + dy * dy;
                const double q = df_is_one ? 1 / (1 + d2) : 1 / (1 + d2 / df);
                a0 += val[e] * q * dx;
                a1 += val[e] * q * dy;
            } else {
                const double d = Y[i] - Y[j];
                const double q = df_is_one ? 1 / (1 + d * d) : 1 / (1 + (d * d) / df);
                a0 += val[e] * q * d;
            }
        }
        pos[(size_t) i * D] = a0;
        if (D == 2) pos[(size_t) i * D + 1] = a1;
    }
}

/* computeFftGradient (2-D, df = 1), src/tsne.cpp:1027-1169 */
static double grad_2d_df1(const unsigned *row, const unsigned *col, const double *val, const double *Y, int N,
                          double *dC, int p, double ipi, int min_int, int nthreads) {
    double *xs = (double *) malloc(sizeof(double) * N), *ys = (double *) malloc(sizeof(double) * N);
    double lo = INFINITY, hi = -INFINITY;
    for (int i = 0; i < N; i++) {
        xs[i] = Y[2 * i];
        ys[i] = Y[2 * i + 1];
        if (xs[i] > hi) hi = xs[i];
        else if (xs[i] < lo) lo = xs[i];
        if (ys[i] > hi) hi = ys[i];
        else if (ys[i] < lo) lo = ys[i];
    }
    const int T = 4;
    double *ch = (double *) malloc(sizeof(double) * (size_t) N * T);
    double *pot = (double *) calloc((size_t) N * T, sizeof(double));
    for (int j = 0; j < N; j++) {
        ch[j * T + 0] = 1;
        ch[j * T + 1] = xs[j];
        ch[j * T + 2] = ys[j];
        ch[j * T + 3] = xs[j] * xs[j] + ys[j] * ys[j];
    }
    const int nb = boxes_2d(lo, hi, ipi, min_int);
    const int M = p * nb, n2 = 2 * M;
    double *lower = (double *) malloc(sizeof(double) * 2 * nb * nb), *upper = (double *) malloc(sizeof(double) * 2 * nb * nb);
    double s[64];
    double *spec = (double *) malloc(sizeof(double) * 2 * (size_t) n2 * (n2 / 2 + 1));
    setup_2d(lo, hi, nb, p, k_sq_cauchy_2d, 1.0, lower, upper, s, spec);
    nbody_2d(N, T, xs, ys, ch, nb, p, lower, upper, s, spec, pot, nthreads);
    double Z = 0;
    for (int i = 0; i < N; i++) {
        const double p1 = pot[i * T], p2 = pot[i * T + 1], p3 = pot[i * T + 2], p4 = pot[i * T + 3];
        Z += (1 + xs[i] * xs[i] + ys[i] * ys[i]) * p1 - 2 * (xs[i] * p2 + ys[i] * p3) + p4;
    }
    Z -= N;
    double *pos = (double *) malloc(sizeof(double) * 2 * (size_t) N);
    attraction(row, col, val, Y, N, 2, 1.0, 1, pos, nthreads);
    for (int i = 0; i < N; i++) {
        const double n0 = (xs[i] * pot[i * T] - pot[i * T + 1]) / Z;
        const double n1 = (ys[i] * pot[i * T] - pot[i * T + 2]) / Z;
        dC[2 * i] = pos[2 * i] - n0;
        dC[2 * i + 1] = pos[2 * i + 1] - n1;
    }
    free(xs);
    free(ys);
    free(ch);
    free(pot);
    free(lower);
    free(upper);
    free(spec);
    free(pos);
    return Z;
}

/* computeFftGradientVariableDf (2-D), src/tsne.cpp:860-1024 */
static double grad_2d_vardf(const unsigned *row, const unsigned *col, const double *val, const double *Y, int N,
                            double *dC, int p, double ipi, int min_int, int nthreads, double df) {
    double *xs = (double *) malloc(sizeof(double) * N), *ys = (double *) malloc(sizeof(double) * N);
    double lo = INFINITY, hi = -INFINITY;
    for (int i = 0; i < N; i++) {
        xs[i] = Y[2 * i];
        ys[i] = Y[2 * i + 1];
        if (xs[i] > hi) hi = xs[i];
        else if (xs[i] < lo) lo = xs[i];
        if (ys[i] > hi) hi = ys[i];
        else if (ys[i] < lo) lo = ys[i];
    }
    const int nb = boxes_2d(lo, hi, ipi, min_int);
    const int M = p * nb, n2 = 2 * M;
    double *ch3 = (double *) malloc(sizeof(double) * (size_t) N * 3);
    double *pot3 = (double *) calloc((size_t) N * 3, sizeof(double));
    for (int j = 0; j < N; j++) {
        ch3[j * 3 + 0] = xs[j];
        ch3[j * 3 + 1] = ys[j];
        ch3[j * 3 + 2] = 1;
    }
    double *lower = (double *) malloc(sizeof(double) * 2 * nb * nb), *upper = (double *) malloc(sizeof(double) * 2 * nb * nb);
    double s[64];
    double *spec = (double *) malloc(sizeof(double) * 2 * (size_t) n2 * (n2 / 2 + 1));
    setup_2d(lo, hi, nb, p, k_sq_general_2d, df, lower, upper, s, spec);
    nbody_2d(N, 3, xs, ys, ch3, nb, p, lower, upper, s, spec, pot3, nthreads);
    double *ch1 = (double *) malloc(sizeof(double) * (size_t) N);
    double *pot1 = (double *) calloc((size_t) N, sizeof(double));
    for (int j = 0; j < N; j++) ch1[j] = 1;
    setup_2d(lo, hi, nb, p, k_general_2d, df, lower, upper, s, spec);
    nbody_2d(N, 1, xs, ys, ch1, nb, p, lower, upper, s, spec, pot1, nthreads);
    double Z = 0;
    for (int i = 0; i < N; i++) Z += pot1[i];
    Z -= N;
    double *pos = (double *) malloc(sizeof(double) * 2 * (size_t) N);
    attraction(row, col, val, Y, N, 2, df, 0, pos, nthreads);
    for (int i = 0; i < N; i++) {
        const double h2 = pot3[i * 3], h3 = pot3[i * 3 + 1], h4 = pot3[i * 3 + 2];
        const double n0 = (xs[i] * h4 - h2) / Z, n1 = (ys[i] * h4 - h3) / Z;
        dC[2 * i] = pos[2 * i] - n0;
        dC[2 * i + 1] = pos[2 * i + 1] - n1;
    }
    free(xs);
    free(ys);
    free(ch3);
    free(pot3);
    free(ch1);
    free(pot1);
    free(lower);
    free(upper);
    free(spec);
    free(pos);
    return Z;
}

/* computeFftGradientOneD (src/tsne.cpp:758-856) and ...OneDVariableDf (647-754) */
static double grad_1d(const unsigned *row, const unsigned *col, const double *val, const double *Y, int N,
                      double *dC, int p, double ipi, int min_int, int nthreads, double df) {
    double lo = INFINITY, hi = -INFINITY;
    for (int i = 0; i < N; i++) {
        if (Y[i] < lo) lo = Y[i];
        if (Y[i] > hi) hi = Y[i];
    }
    const int nb = (int) fmax(min_int, (hi - lo) / ipi);
    const int M = p * nb;
    double *lower = (double *) malloc(sizeof(double) * nb), *upper = (double *) malloc(sizeof(double) * nb);
    double s[64];
    double *spec = (double *) malloc(sizeof(double) * 4 * (size_t) M);
    double Z = 0;
    double *pos = (double *) malloc(sizeof(double) * (size_t) N);
    if (df == 1.0) {
        const int T = 3;
        double *ch = (double *) malloc(sizeof(double) * (size_t) N * T);
        double *pot = (double *) calloc((size_t) N * T, sizeof(double));
        for (int j = 0; j < N; j++) {
            ch[j * T] = 1;
            ch[j * T + 1] = Y[j];
            ch[j * T + 2] = Y[j] * Y[j];
        }
        setup_1d(lo, hi, nb, p, k_sq_cauchy, 1.0, lower, upper, s, spec);
        nbody_1d(N, T, Y, ch, nb, p, lower, upper, s, spec, pot);
        for (int i = 0; i < N; i++)
            Z += (1 + Y[i] * Y[i]) * pot[i * T] - 2 * (Y[i] * pot[i * T + 1]) + pot[i * T + 2];
        Z -= N;
        attraction(row, col, val, Y, N, 1, 1.0, 1, pos, nthreads);
        for (int i = 0; i < N; i++) dC[i] = pos[i] - (Y[i] * pot[i * T] - pot[i * T + 1]) / Z;
        free(ch);
        free(pot);
    } else {
        double *ch2 = (double *) malloc(sizeof(double) * (size_t) N * 2);
        double *pot2 = (double *) calloc((size_t) N * 2, sizeof(double));
        for (int j = 0; j < N; j++) {
            ch2[j * 2] = Y[j];
            ch2[j * 2 + 1] = 1;
        }
        setup_1d(lo, hi, nb, p, k_sq_general, df, lower, upper, s, spec);
        nbody_1d(N, 2, Y, ch2, nb, p, lower, upper, s, spec, pot2);
        double *ch1 = (double *) malloc(sizeof(double) * (size_t) N);
        double *pot1 = (double *) calloc((size_t) N, sizeof(double));
        for (int j = 0; j < N; j++) ch1[j] = 1;
        setup_1d(lo, hi, nb, p, k_general, df, lower, upper, s, spec);
        nbody_1d(N, 1, Y, ch1, nb, p, lower, upper, s, spec, pot1);
        for (int i = 0; i < N; i++) Z += pot1[i];
        Z -= N;
        attraction(row, col, val, Y, N, 1, df, 0, pos, nthreads);
        for (int i = 0; i < N; i++) dC[i] = pos[i] - (Y[i] * pot2[i * 2 + 1] - pot2[i * 2]) / Z;
        free(ch2);
        free(pot2);
        free(ch1);
        free(pot1);
    }
    free(lower);
    free(upper);
    free(spec);
    free(pos);
    return Z;
}

/* dispatch of src/tsne.cpp:444-464; returns Z (current_sum_Q) */
double orc_fft_gradient(const unsigned *row, const unsigned *col, const double *val, const double *Y, int N, int D,
                        double *dC, int nterms, double ipi, int min_int, unsigned int nthreads, double df) {
    const int nt = nthreads_or_1(nthreads);
    for (size_t i = 0; i < (size_t) N * D; i++) dC[i] = 0.0;
    if (D == 1) return grad_1d(row, col, val, Y, N, dC, nterms, ipi, min_int, nt, df);
    if (df == 1.0) return grad_2d_df1(row, col, val, Y, N, dC, nterms, ipi, min_int, nt);
    return grad_2d_vardf(row, col, val, Y, N, dC, nterms, ipi, min_int, nt, df);
}

/* evaluateErrorFft, src/tsne.cpp:1329-1355 (serial sum: the threaded form races) */
double orc_evaluate_error_fft(const unsigned *row, const unsigned *col, const double *val, const double *Y, int N,
                              int D, double df, double sum_Q) {
    double C = 0.0;
    for (int i = 0; i < N; i++) {
        double t = 0;
        for (unsigned e = row[i]; e < row[i + 1]; e++) {
            double q = 0.0;
            for (int d = 0; d < D; d++) {
                const double b = Y[(size_t) i * D + d] - Y[(size_t) col[e] * D + d];
                q += b * b;
            }
            q = pow(1.0 / (1.0 + q / df), df) / sum_Q;
            t += val[e] * log((val[e] + FLT_MIN) / (q + FLT_MIN));
        }
        C += t;
    }
    return C;
}

/* ---------------------------------------------------------------------------------
 * perplexity calibration, src/tsne.cpp:1394-1469 (single) and 1474-1500 (list) */
static double calibrate_row(const double *Dd, double *P, int N, int n, double perplexity, double sigma,
                            int if_squared) {
    double sum_P = 0, beta;
    if (perplexity > 0) {
        double min_beta = -DBL_MAX, max_beta = DBL_MAX, tol = 1e-5;
        int iter = 0, found = 0;
        beta = 1.0;
        while (!found && iter < 200) {
            for (int m = 0; m < N; m++) P[m] = exp(-beta * (if_squared ? Dd[m] : Dd[m] * Dd[m]));
            if (n >= 0) P[n] = DBL_MIN;
            sum_P = DBL_MIN;
            for (int m = 0; m < N; m++) sum_P += P[m];
            double H = 0.0;
            for (int m = 0; m < N; m++) H += beta * ((if_squared ? Dd[m] : Dd[m] * Dd[m]) * P[m]);
            H = (H / sum_P) + log(sum_P);
            const double Hdiff = H - log(perplexity);
            if (Hdiff < tol && -Hdiff < tol) {
                found = 1;
            } else if (Hdiff > 0) {
                min_beta = beta;
                if (max_beta == DBL_MAX || max_beta == -DBL_MAX) beta *= 2.0;
                else beta = (beta + max_beta) / 2.0;
            } else {
                max_beta = beta;
                if (min_beta == -DBL_MAX || min_beta == DBL_MAX) beta /= 2.0;
                else beta = (beta + min_beta) / 2.0;
            }
            iter++;
        }
    } else {
        beta = 1 / (2 * sigma * sigma);
        for (int m = 0; m < N; m++) P[m] = exp(-beta * (if_squared ? Dd[m] : Dd[m] * Dd[m]));
        if (n >= 0) P[n] = DBL_MIN;
        sum_P = DBL_MIN;
        for (int m = 0; m < N; m++) sum_P += P[m];
    }
    for (int m = 0; m < N; m++) P[m] /= sum_P;
    return beta;
}

double orc_distances2similarities(const double *Dd, double *P, int N, int n, double perplexity, double sigma,
                                  int if_squared, int list_len, const double *list) {
    (void) if_squared; /* the list overload always calls the single one with ifSquared = true */
    if (perplexity != 0) return calibrate_row(Dd, P, N, n, perplexity, sigma, 1);
    double *tmp = (double *) malloc(sizeof(double) * (N > 0 ? N : 1));
    double beta = calibrate_row(Dd, P, N, n, list[0], sigma, 1);
    for (int m = 1; m < list_len; m++) {
        beta = calibrate_row(Dd, tmp, N, n, list[m], sigma, 1);
        for (int i = 0; i < N; i++) P[i] += tmp[i];
    }
    for (int i = 0; i < N; i++) P[i] /= list_len;
    free(tmp);
    return beta;
}

/* ---------------------------------------------------------------------------------
 * exact kNN.  The VP-tree of src/vptree.h:110-280 (random vantage point, median split,
 * priority-queue search on non-squared distances) is restated for the CPU baseline;
 * orc_knn is a plain brute-force check. */
typedef struct {
    int index;
    double thr;
    int left, right;
} vp_node;

typedef struct {
    const double *X;
    int D;
    int *items;
    vp_node *nodes;
    int nn;
} vp_tree;

static double vp_dist(const vp_tree *t, int a, int b) {
    const double *x = t->X + (size_t) a * t->D, *y = t->X + (size_t) b * t->D;
    double dd = 0;
    for (int d = 0; d < t->D; d++) {
        const double f = x[d] - y[d];
        dd += f * f;
    }
    return sqrt(dd);
}

/* partial sort items[lo..hi) so that items[k] holds the element of rank k by distance to v */
static void vp_select(vp_tree *t, int v, int lo, int hi, int k, double *dist_buf) {
    for (int i = lo; i < hi; i++) dist_buf[i] = vp_dist(t, v, t->items[i]);
    while (hi - lo > 1) {
        const double piv = dist_buf[lo + (hi - lo) / 2];
        int i = lo, j = hi - 1;
        while (i <= j) {
            while (dist_buf[i] < piv) i++;
            while (dist_buf[j] > piv) j--;
            if (i <= j) {
                double td = dist_buf[i];
                dist_buf[i] = dist_buf[j];
                dist_buf[j] = td;
                int ti = t->items[i];
                t->items[i] = t->items[j];
                t->items[j] = ti;
                i++;
                j--;
            }
        }
        if (k <= j) hi = j + 1;
        else if (k >= i) lo = i;
        else break;
    }
}

static int vp_build(vp_tree *t, int lo, int hi, double *buf) {
    if (hi == lo) return -1;
    const int id = t->nn++;
    t->nodes[id].index = lo;
    t->nodes[id].thr = 0;
    t->nodes[id].left = t->nodes[id].right = -1;
    if (hi - lo > 1) {
        const int r = (int) ((double) rand() / RAND_MAX * (hi - lo - 1)) + lo;
        int tmp = t->items[lo];
        t->items[lo] = t->items[r];
        t->items[r] = tmp;
        const int med = (hi + lo) / 2;
        vp_select(t, t->items[lo], lo + 1, hi, med, buf);
        t->nodes[id].thr = vp_dist(t, t->items[lo], t->items[med]);
        const int l = vp_build(t, lo + 1, med, buf);
        const int rr = vp_build(t, med, hi, buf);
        t->nodes[id].left = l;
        t->nodes[id].right = rr;
    }
    return id;
}

typedef struct {
    int *idx;
    double *dist;
    int size, cap;
} vp_heap; /* max-heap on dist */

static void heap_push(vp_heap *h, int idx, double d) {
    int i = h->size++;
    while (i > 0) {
        const int p = (i - 1) / 2;
        if (h->dist[p] >= d) break;
        h->dist[i] = h->dist[p];
        h->idx[i] = h->idx[p];
        i = p;
    }
    h->dist[i] = d;
    h->idx[i] = idx;
}
static void heap_pop(vp_heap *h) {
    const int n = --h->size;
    const double d = h->dist[n];
    const int id = h->idx[n];
    int i = 0;
    for (;;) {
        int c = 2 * i + 1;
        if (c >= n) break;
        if (c + 1 < n && h->dist[c + 1] > h->dist[c]) c++;
        if (h->dist[c] <= d) break;
        h->dist[i] = h->dist[c];
        h->idx[i] = h->idx[c];
        i = c;
    }
    h->dist[i] = d;
    h->idx[i] = id;
}

static void vp_search(const vp_tree *t, int node, int q, int k, vp_heap *h, double *tau) {
    if (node < 0) return;
    const vp_node *nd = &t->nodes[node];
    const double dist = vp_dist(t, t->items[nd->index], q);
    if (dist < *tau) {
        if (h->size == k) heap_pop(h);
        heap_push(h, nd->index, dist);
        if (h->size == k) *tau = h->dist[0];
    }
    if (nd->left < 0 && nd->right < 0) return;
    if (dist < nd->thr) {
        if (dist - *tau <= nd->thr) vp_search(t, nd->left, q, k, h, tau);
        if (dist + *tau >= nd->thr) vp_search(t, nd->right, q, k, h, tau);
    } else {
        if (dist + *tau >= nd->thr) vp_search(t, nd->right, q, k, h, tau);
        if (dist - *tau <= nd->thr) vp_search(t, nd->left, q, k, h, tau);
    }
}

/* kNN + calibration into fixed-K CSR rows, src/tsne.cpp:1643-1726 */
void orc_gaussian_perplexity_vptree(const double *X, int N, int D, unsigned **row_P, unsigned **col_P, double **val_P,
                                    double perplexity, int K, double sigma, unsigned int nthreads, int list_len,
                                    const double *list) {
    unsigned *row = (unsigned *) malloc(sizeof(unsigned) * (N + 1));
    unsigned *col = (unsigned *) calloc((size_t) N * K, sizeof(unsigned));
    double *val = (double *) calloc((size_t) N * K, sizeof(double));
    row[0] = 0;
    for (int n = 0; n < N; n++) row[n + 1] = row[n] + (unsigned) K;
    vp_tree t;
    t.X = X;
    t.D = D;
    t.items = (int *) malloc(sizeof(int) * N);
    for (int i = 0; i < N; i++) t.items[i] = i;
    t.nodes = (vp_node *) malloc(sizeof(vp_node) * (N > 0 ? N : 1));
    t.nn = 0;
    double *buf = (double *) malloc(sizeof(double) * (N > 0 ? N : 1));
    const int root = vp_build(&t, 0, N, buf);
    free(buf);
    const int nt = nthreads_or_1(nthreads);
#pragma omp parallel num_threads(nt)
    {
        vp_heap h;
        h.idx = (int *) malloc(sizeof(int) * (K + 1));
        h.dist = (double *) malloc(sizeof(double) * (K + 1));
        h.cap = K + 1;
        int *oi = (int *) malloc(sizeof(int) * (K + 1));
        double *od = (double *) malloc(sizeof(double) * (K + 1));
        double *cur = (double *) malloc(sizeof(double) * K);
#pragma omp for schedule(static)
        for (int n = 0; n < N; n++) {
            h.size = 0;
            double tau = DBL_MAX;
            vp_search(&t, root, n, K + 1, &h, &tau);
            /* pop in decreasing distance, store increasing */
            int cnt = h.size;
            for (int r = cnt - 1; r >= 0; r--) {
                oi[r] = t.items[h.idx[0]];
                od[r] = h.dist[0];
                heap_pop(&h);
            }
            orc_distances2similarities(&od[1], cur, K, -1, perplexity, sigma, 0, list_len, list);
            for (int m = 0; m < K; m++) {
                col[row[n] + m] = (unsigned) oi[m + 1];
                val[row[n] + m] = cur[m];
            }
        }
        free(h.idx);
        free(h.dist);
        free(oi);
        free(od);
        free(cur);
    }
    free(t.items);
    free(t.nodes);
    *row_P = row;
    *col_P = col;
    *val_P = val;
}

/* brute-force exact kNN in FP64 (self included), for tests */
void orc_knn(const double *X, int N, int D, int K, unsigned *idx, double *dist, int nthreads) {
    const int nt = nthreads_or_1((unsigned) nthreads);
#pragma omp parallel num_threads(nt)
    {
        vp_heap h;
        h.idx = (int *) malloc(sizeof(int) * (K + 1));
        h.dist = (double *) malloc(sizeof(double) * (K + 1));
#pragma omp for schedule(dynamic, 16)
        for (int i = 0; i < N; i++) {
            h.size = 0;
            for (int j = 0; j < N; j++) {
                double dd = 0;
                for (int d = 0; d < D; d++) {
                    const double f = X[(size_t) i * D + d] - X[(size_t) j * D + d];
                    dd += f * f;
                }
                dd = sqrt(dd);
                if (h.size < K) heap_push(&h, j, dd);
                else if (dd < h.dist[0]) {
                    heap_pop(&h);
                    heap_push(&h, j, dd);
                }
            }
            for (int r = h.size - 1; r >= 0; r--) {
                idx[(size_t) i * K + r] = (unsigned) h.idx[0];
                dist[(size_t) i * K + r] = h.dist[0];
                heap_pop(&h);
            }
        }
        free(h.idx);
        free(h.dist);
    }
}

/* ---------------------------------------------------------------------------------
 * (P + P^T) / 2 on the union pattern, src/tsne.cpp:1730-1828 */
void orc_symmetrize(unsigned **row_P, unsigned **col_P, double **val_P, int N) {
    unsigned *row = *row_P, *col = *col_P;
    double *val = *val_P;
    int *cnt = (int *) calloc(N > 0 ? N : 1, sizeof(int));
    for (int n = 0; n < N; n++)
        for (unsigned i = row[n]; i < row[n + 1]; i++) {
            int present = 0;
            for (unsigned m = row[col[i]]; m < row[col[i] + 1]; m++)
                if (col[m] == (unsigned) n) present = 1;
            if (present) cnt[n]++;
            else {
                cnt[n]++;
                cnt[col[i]]++;
            }
        }
    size_t total = 0;
    for (int n = 0; n < N; n++) total += cnt[n];
    unsigned *srow = (unsigned *) malloc(sizeof(unsigned) * (N + 1));
    unsigned *scol = (unsigned *) malloc(sizeof(unsigned) * (total ? total : 1));
    double *sval = (double *) malloc(sizeof(double) * (total ? total : 1));
    srow[0] = 0;
    for (int n = 0; n < N; n++) srow[n + 1] = srow[n] + (unsigned) cnt[n];
    int *off = (int *) calloc(N > 0 ? N : 1, sizeof(int));
    for (int n = 0; n < N; n++)
        for (unsigned i = row[n]; i < row[n + 1]; i++) {
            const unsigned c = col[i];
            int present = 0;
            for (unsigned m = row[c]; m < row[c + 1]; m++)
                if (col[m] == (unsigned) n) {
                    present = 1;
                    if ((unsigned) n <= c) {
                        scol[srow[n] + off[n]] = c;
                        scol[srow[c] + off[c]] = (unsigned) n;
                        sval[srow[n] + off[n]] = val[i] + val[m];
                        sval[srow[c] + off[c]] = val[i] + val[m];
                    }
                }
            if (!present) {
                scol[srow[n] + off[n]] = c;
                scol[srow[c] + off[c]] = (unsigned) n;
                sval[srow[n] + off[n]] = val[i];
                sval[srow[c] + off[c]] = val[i];
            }
            if (!present || ((unsigned) n <= c)) {
                off[n]++;
                if (c != (unsigned) n) off[c]++;
            }
        }
    for (size_t i = 0; i < total; i++) sval[i] /= 2.0;
    free(*row_P);
    free(*col_P);
    free(*val_P);
    *row_P = srow;
    *col_P = scol;
    *val_P = sval;
    free(off);
    free(cnt);
}

/* ---------------------------------------------------------------------------------
 * the optimiser step, src/tsne.cpp:479-531, and zeroMean, 1851-1876 */
static double sgn(double x) { return (x == .0 ? .0 : (x < .0 ? -1.0 : 1.0)); }

static void zero_mean(double *X, int N, int D) {
    double *mean = (double *) calloc(D, sizeof(double));
    size_t nD = 0;
    for (int n = 0; n < N; n++) {
        for (int d = 0; d < D; d++) mean[d] += X[nD + d];
        nD += D;
    }
    for (int d = 0; d < D; d++) mean[d] /= (double) N;
    nD = 0;
    for (int n = 0; n < N; n++) {
        for (int d = 0; d < D; d++) X[nD + d] -= mean[d];
        nD += D;
    }
    free(mean);
}

static void update(double *Y, double *uY, double *gains, const double *dY, int N, int D, int use_gains,
                   int plain_descent, double momentum, double lr, double max_step_norm) {
    const size_t n = (size_t) N * D;
    if (plain_descent) {
        for (size_t i = 0; i < n; i++) Y[i] = Y[i] - dY[i];
        return;
    }
    (void) use_gains;
    for (size_t i = 0; i < n; i++) gains[i] = (sgn(dY[i]) != sgn(uY[i])) ? (gains[i] + .2) : (gains[i] * .8);
    for (size_t i = 0; i < n; i++)
        if (gains[i] < .01) gains[i] = .01;
    for (size_t i = 0; i < n; i++) uY[i] = momentum * uY[i] - lr * gains[i] * dY[i];
    if (max_step_norm > 0) {
        for (int i = 0; i < N; i++) {
            double step = 0;
            for (int j = 0; j < D; j++) step += uY[(size_t) i * D + j] * uY[(size_t) i * D + j];
            step = sqrt(step);
            if (step > max_step_norm)
                for (int j = 0; j < D; j++) uY[(size_t) i * D + j] *= (max_step_norm / step);
        }
    }
    for (size_t i = 0; i < n; i++) Y[i] = Y[i] + uY[i];
}

/* One iteration: gradient with P scaled by exag, step, zero-mean.  The exaggeration is
 * applied to a scaled copy of val (the reference scales val_P in place). */
int orc_gradient_step(const unsigned *row, const unsigned *col, const double *val, double *Y, double *uY,
                      double *gains, int N, int D, int nterms, int min_int, double ipi, int nthreads, int unused,
                      double df, double exag, double momentum, double lr, int use_gains, double max_step_norm) {
    (void) unused;
    const size_t nnz = row[N];
    double *v = (double *) malloc(sizeof(double) * (nnz ? nnz : 1));
    for (size_t i = 0; i < nnz; i++) v[i] = val[i] * exag;
    double *dY = (double *) malloc(sizeof(double) * (size_t) N * D);
    orc_fft_gradient(row, col, v, Y, N, D, dY, nterms, ipi, min_int, (unsigned) nthreads, df);
    update(Y, uY, gains, dY, N, D, use_gains, !use_gains, momentum, lr, max_step_norm);
    zero_mean(Y, N, D);
    free(v);
    free(dY);
    return 0;
}

/* random normal of TSNE::randn, src/tsne.cpp:1880-1890 */
static double randn_polar(void) {
    double x, y, radius;
    do {
        x = 2 * (rand() / ((double) RAND_MAX + 1)) - 1;
        y = 2 * (rand() / ((double) RAND_MAX + 1)) - 1;
        radius = (x * x) + (y * y);
    } while ((radius >= 1.0) || (radius == 0.0));
    radius = sqrt(-2 * log(radius) / radius);
    x *= radius;
    return x;
}

/* The optimisation loop of TSNE::run (src/tsne.cpp:389-577): auto early exaggeration,
 * val scaled in place by the exaggeration, the update, zero-mean, the schedule switches
 * after each iteration's update, KL every 50 iterations with the stale Z (quirk Q6). */
static void optimise(unsigned *row, unsigned *col, double *val, int N, double *Y, int no_dims, int max_iter,
                     int stop_lying_iter, int mom_switch_iter, double momentum, double final_momentum,
                     double learning_rate, double early_exag_coeff, double *costs, int no_momentum_during_exag,
                     int start_late_exag_iter, double late_exag_coeff, int nterms, double ipi, int min_int,
                     unsigned int nthreads, double df, double max_step_norm, double *dY, double *uY, double *gains) {
    if (early_exag_coeff == 0) {
        double mxs = 0;
        for (int n = 0; n < N; n++) {
            double s = 0;
            for (unsigned i = row[n]; i < row[n + 1]; i++) s += val[i];
            if (s > mxs) mxs = s;
        }
        early_exag_coeff = (1.0 / (learning_rate * mxs));
    }
    for (unsigned i = 0; i < row[N]; i++) val[i] *= early_exag_coeff;
    for (int iter = 0; iter < max_iter; iter++) {
        /* Z of this iteration's gradient is the current_sum_Q the cost uses */
        const double zq = orc_fft_gradient(row, col, val, Y, N, no_dims, dY, nterms, ipi, min_int, nthreads, df);
        if (no_momentum_during_exag) {
            if (iter > stop_lying_iter) update(Y, uY, gains, dY, N, no_dims, 1, 0, momentum, learning_rate, -1.0);
            else update(Y, uY, gains, dY, N, no_dims, 0, 1, momentum, learning_rate, -1.0);
        } else {
            update(Y, uY, gains, dY, N, no_dims, 1, 0, momentum, learning_rate, max_step_norm);
        }
        zero_mean(Y, N, no_dims);
        if (iter == stop_lying_iter)
            for (unsigned i = 0; i < row[N]; i++) val[i] /= early_exag_coeff;
        if (iter == start_late_exag_iter)
            for (unsigned i = 0; i < row[N]; i++) val[i] *= late_exag_coeff;
        if (iter == mom_switch_iter) momentum = final_momentum;
        if ((iter + 1) % 50 == 0 || iter == max_iter - 1) {
            double C = orc_evaluate_error_fft(row, col, val, Y, N, no_dims, df, zq);
            if (iter < stop_lying_iter && stop_lying_iter != -1)
                C = C / early_exag_coeff - log(early_exag_coeff);
            if (iter >= start_late_exag_iter && start_late_exag_iter != -1)
                C = C / late_exag_coeff - log(late_exag_coeff);
            costs[iter] = C;
        }
    }
}

/* ---------------------------------------------------------------------------------
 * TSNE::run restricted to the FFT path (src/tsne.cpp:118-592): theta != 0, nbody 2,
 * exact kNN (knn_algo 1 is served by the same VP-tree), no P-file I/O. */
int orc_run(double *X, int N, int D, double *Y, int no_dims, double perplexity, double theta, int rand_seed,
            int skip_random_init, int max_iter, int stop_lying_iter, int mom_switch_iter, double momentum,
            double final_momentum, double learning_rate, int K, double sigma, int nbody_algorithm, int knn_algo,
            double early_exag_coeff, double *costs, int no_momentum_during_exag, int start_late_exag_iter,
            double late_exag_coeff, int n_trees, int search_k, int nterms, double ipi, int min_int,
            unsigned int nthreads, int load_affinities, int list_len, double *list, double df,
            double max_step_norm) {
    (void) theta;
    (void) nbody_algorithm;
    (void) knn_algo;
    (void) n_trees;
    (void) search_k;
    (void) load_affinities;
    if (N - 1 < 3 * perplexity) return -3;
    const size_t nd = (size_t) N * no_dims;
    double *dY = (double *) malloc(sizeof(double) * nd), *uY = (double *) calloc(nd, sizeof(double));
    double *gains = (double *) malloc(sizeof(double) * nd);
    for (size_t i = 0; i < nd; i++) gains[i] = 1.0;
    zero_mean(X, N, D);
    if (perplexity > 0 || list_len > 0) {
        double mx = .0;
        for (size_t i = 0; i < (size_t) N * D; i++)
            if (fabs(X[i]) > mx) mx = fabs(X[i]);
        for (size_t i = 0; i < (size_t) N * D; i++) X[i] /= mx;
    }
    int Kuse;
    double sig;
    if (perplexity < 0) {
        Kuse = K;
        sig = sigma;
    } else {
        if (perplexity > 0) Kuse = (int) 3 * perplexity;
        else {
            Kuse = (int) 3 * list[0];
            for (int pp = 1; pp < list_len; pp++)
                if ((int) 3 * list[pp] > Kuse) Kuse = (int) 3 * list[pp];
        }
        sig = -1;
    }
    unsigned *row, *col;
    double *val;
    orc_gaussian_perplexity_vptree(X, N, D, &row, &col, &val, perplexity, Kuse, sig, nthreads, list_len, list);
    orc_symmetrize(&row, &col, &val, N);
    double sum_P = .0;
    for (unsigned i = 0; i < row[N]; i++) sum_P += val[i];
    for (unsigned i = 0; i < row[N]; i++) val[i] /= sum_P;
    if (!skip_random_init) {
        srand(rand_seed >= 0 ? (unsigned) rand_seed : (unsigned) time(NULL));
        for (size_t i = 0; i < nd; i++) Y[i] = randn_polar() * .0001;
    }
    optimise(row, col, val, N, Y, no_dims, max_iter, stop_lying_iter, mom_switch_iter, momentum, final_momentum,
             learning_rate, early_exag_coeff, costs, no_momentum_during_exag, start_late_exag_iter, late_exag_coeff,
             nterms, ipi, min_int, nthreads, df, max_step_norm, dY, uY, gains);
    free(dY);
    free(uY);
    free(gains);
    free(row);
    free(col);
    free(val);
    return 0;
}

/* TSNE::run with load_affinities = 1 (src/tsne.cpp:236-281): the loop on a given P (the
 * symmetrised, normalised matrix the reference saves with load_affinities = 2) from the
 * given Y.  val is copied: the loop scales its P in place. */
int orc_run_from_P(const unsigned *row, const unsigned *col, const double *val, int N, double *Y, int no_dims,
                   int max_iter, int stop_lying_iter, int mom_switch_iter, double momentum, double final_momentum,
                   double learning_rate, double early_exag_coeff, double *costs, int no_momentum_during_exag,
                   int start_late_exag_iter, double late_exag_coeff, int nterms, double ipi, int min_int,
                   unsigned int nthreads, double df, double max_step_norm) {
    const size_t nd = (size_t) N * no_dims, nnz = row[N];
    unsigned *r = (unsigned *) malloc(sizeof(unsigned) * (N + 1));
    unsigned *c = (unsigned *) malloc(sizeof(unsigned) * (nnz ? nnz : 1));
    double *v = (double *) malloc(sizeof(double) * (nnz ? nnz : 1));
    memcpy(r, row, sizeof(unsigned) * (N + 1));
    memcpy(c, col, sizeof(unsigned) * nnz);
    memcpy(v, val, sizeof(double) * nnz);
    double *dY = (double *) malloc(sizeof(double) * nd), *uY = (double *) calloc(nd, sizeof(double));
    double *gains = (double *) malloc(sizeof(double) * nd);
    for (size_t i = 0; i < nd; i++) gains[i] = 1.0;
    optimise(r, c, v, N, Y, no_dims, max_iter, stop_lying_iter, mom_switch_iter, momentum, final_momentum,
             learning_rate, early_exag_coeff, costs, no_momentum_during_exag, start_late_exag_iter, late_exag_coeff,
             nterms, ipi, min_int, nthreads, df, max_step_norm, dY, uY, gains);
    free(dY);
    free(uY);
    free(gains);
    free(r);
    free(c);
    free(v);
    return 0;
}

void orc_free(void *p) { free(p); }
