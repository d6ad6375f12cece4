/*
 * Project-written declarations of the five FFTW 3 entry points that the FIt-SNE
 * reference calls (src/nbodyfft.cpp:64-68, 164-212, 301-304, 400-433).  This is NOT
 * FFTW's header: it declares only what the reference uses, with the same names and
 * argument meaning, so that the unmodified reference sources compile against
 * oracle/fftw_shim.c (which is backed by oracle/fft64.c).
 *
 * TEST INFRASTRUCTURE ONLY: used to build the reference as a checker under
 * oracle/_ref/; nothing of the GPU product includes it.
 */
#ifndef FITSNE_ORACLE_FFTW_SHIM_H
#define FITSNE_ORACLE_FFTW_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct fftw_shim_plan_s *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out, unsigned flags);
void fftw_execute(const fftw_plan plan);
void fftw_destroy_plan(fftw_plan plan);

#ifdef __cplusplus
}
#endif
#endif
