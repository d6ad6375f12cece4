/*
 * fft64 -- a small double-precision FFT written for this project's test oracle.
 *
 * TEST INFRASTRUCTURE ONLY: this code is part of the CPU oracle (the checker),
 * never of the GPU product path.
 *
 * It provides what the FIt-SNE reference asks of FFTW 3 (src/nbodyfft.cpp:64-68,
 * 164-212, 301-304, 400-433): unnormalised complex 1-D transforms of any length and
 * real<->half-complex 2-D transforms, in the FFTW sign convention
 * (forward = exp(-2*pi*i*j*k/n), backward = exp(+2*pi*i*j*k/n), no scaling).
 *
 * Algorithm: iterative mixed-radix Stockham (radices 4, 2, 3, 5 and any other small
 * prime through a direct DFT), Bluestein's chirp-z method for lengths with a prime
 * factor above 31.  Twiddles are evaluated directly with cos/sin for every index.
 */
#ifndef FITSNE_ORACLE_FFT64_H
#define FITSNE_ORACLE_FFT64_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fft64_plan fft64_plan;

/* complex 1-D transform of length n; sign = -1 forward, +1 backward */
fft64_plan *fft64_plan_c2c(int n, int sign);
/* x (interleaved re,im; length n) -> y; x == y allowed */
void fft64_exec_c2c(const fft64_plan *p, const double *x, double *y);
void fft64_destroy(fft64_plan *p);

/* 2-D real -> half complex: in[n0*n1] -> out[n0*(n1/2+1)] complex (FFTW layout) */
void fft64_r2c_2d(int n0, int n1, const double *in, double *out);
/* 2-D half complex -> real (unnormalised inverse): in[n0*(n1/2+1)] -> out[n0*n1] */
void fft64_c2r_2d(int n0, int n1, const double *in, double *out);

#ifdef __cplusplus
}
#endif
#endif
