// FFT convolution of the interpolation grid with the t-SNE kernels.
//
// Replaces the FFTW-based step 2 of n_body_fft_2d / nbodyfft and the kernel
// precomputation of precompute_2d / precompute (src/nbodyfft.cpp:9-70, 154-209,
// 251-307, 397-430 of the reference).
//
// The reference embeds the M x M Toeplitz kernel in a (2M)^2 circulant.  Any circulant
// length L >= 2M-1 gives the same cropped result exactly, so L is chosen here as the
// smallest even 5-smooth number >= 2M (radix 2/3/4/5 passes only).  The kernel is laid
// out with signed node offsets d in (-M, M) at index d mod L, and the output is read
// back from the same [0, M)^2 window the charges were written to.
//
// Four kernels are convolved (see grad.cu for why):
//   K(d)  = kernel value at node offset d
//   Gx(d) = K(d) * dx * h,   Gy(d) = K(d) * dy * h     (odd kernels: imaginary spectra)
//   H(d)  = K(d) * |d h|^2   (df = 1)   or   Kgen(d)  (variable df, the Z kernel)
#pragma once

#include "common.cuh"

namespace fitsne {

struct FftPlan {
    int L;        // transform length
    int nst;      // number of passes
    int radix[24];
};

// Builds the pass list for a 5-smooth L; returns false if L has another prime factor.
bool make_fft_plan(int L, FftPlan *plan);
// Smallest even 5-smooth integer >= n.
int smooth_even_at_least(int n);

// Largest transform length the shared-memory passes accept for each precision.
constexpr int kMaxL32 = 5760;
constexpr int kMaxL64 = 2880;
template <typename T>
constexpr int max_fft_len() { return sizeof(T) == 4 ? kMaxL32 : kMaxL64; }

// Compact kernel spectrum entry: Re K, Im Gx, Im Gy, Re H (already scaled by 1/L^dims).
template <typename T>
struct KSpec {
    T k, gx, gy, h;
};

// 4-field grid cell.
template <typename T>
struct alignas(4 * sizeof(T)) Cell4 {
    T a, b, c, d;
};

enum KernelMode { KERNEL_DF1 = 0, KERNEL_VARDF = 1 };

// 2-D: twiddles tw[j] = exp(-2 pi i j / L), j < L.
// scratch sizes (complex elements): rows = 4 * L * (L/2+1) each for krows/d1/d2,
// kspec = L * (L/2+1) entries.
template <typename T>
cudaError_t conv2d_launch(const Cell4<T> *grid_in, Cell4<T> *grid_out, int M, const FftPlan &plan,
                          const typename Cx<T>::t *tw, typename Cx<T>::t *work_a, typename Cx<T>::t *work_b,
                          KSpec<T> *kspec, double h, double df, int mode, cudaStream_t st);

// 1-D: grid_in/out hold 4 fields per node (only the first 3 are used); work holds 6*L
// complex values.
template <typename T>
cudaError_t conv1d_launch(const Cell4<T> *grid_in, Cell4<T> *grid_out, int M, const FftPlan &plan,
                          const typename Cx<T>::t *tw, typename Cx<T>::t *work, double h, double df, int mode,
                          cudaStream_t st);

}  // namespace fitsne
