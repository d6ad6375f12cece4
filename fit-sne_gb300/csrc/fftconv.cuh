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
FITSNE_HD bool make_fft_plan(int L, FftPlan *p) {
    p->L = L;
    p->nst = 0;
    int n = L;
    while (n % 4 == 0 && p->nst < 24) { p->radix[p->nst++] = 4; n /= 4; }
    while (n % 2 == 0 && p->nst < 24) { p->radix[p->nst++] = 2; n /= 2; }
    while (n % 3 == 0 && p->nst < 24) { p->radix[p->nst++] = 3; n /= 3; }
    while (n % 5 == 0 && p->nst < 24) { p->radix[p->nst++] = 5; n /= 5; }
    return n == 1 && L >= 2;
}

// Smallest even 5-smooth integer >= n.
FITSNE_HD int smooth_even_at_least(int n) {
    for (int m = n < 2 ? 2 : n;; ++m) {
        if (m & 1) continue;
        int k = m;
        while (k % 2 == 0) k /= 2;
        while (k % 3 == 0) k /= 3;
        while (k % 5 == 0) k /= 5;
        if (k == 1) return m;
    }
}

// Convolution geometry kept in device memory, written each iteration by the kernel that
// sizes the interpolation grid, so that an iteration needs no host decision (and can be
// captured in a CUDA graph).  Kernels launched for a capacity (M_cap, L_cap) read it and
// idle the blocks beyond the current M and L.
struct ConvGeom {
    int M;         // nodes per dimension
    double h;      // node spacing of the kernel samples
    FftPlan plan;  // passes of the current L (plan.L)
};

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
                          KSpec<T> *kspec, double h, double df, int mode, cudaStream_t st, int threads = 256);

// As conv2d_launch with the geometry read from device memory (cg); grids and shared
// memory sized for M_cap and L_cap (cg->M <= M_cap, cg->plan.L <= L_cap; tw holds the
// twiddles of cg->plan.L).
template <typename T>
cudaError_t conv2d_launch_dev(const Cell4<T> *grid_in, Cell4<T> *grid_out, int M_cap, int L_cap, const ConvGeom *cg,
                              const typename Cx<T>::t *tw, typename Cx<T>::t *work_a, typename Cx<T>::t *work_b,
                              KSpec<T> *kspec, double df, int mode, cudaStream_t st, int threads = 256);
// Threads per block the 2-D passes accept (any multiple of 32 up to 1024); the launch shapes
// the autotuner picks from.
constexpr int kFftThreadChoices[3] = {128, 256, 512};
template <typename T>
cudaError_t conv1d_launch_dev(const Cell4<T> *grid_in, Cell4<T> *grid_out, int L_cap, const ConvGeom *cg,
                              const typename Cx<T>::t *tw, typename Cx<T>::t *work, double df, int mode,
                              cudaStream_t st);
// tw[j] = exp(-2 pi i j / L) for the L of cg (FP64 sincospi, rounded to T).
template <typename T>
cudaError_t twiddles_dev(const ConvGeom *cg, typename Cx<T>::t *tw, cudaStream_t st);

// 1-D: grid_in/out hold 4 fields per node (only the first 3 are used); work holds 6*L
// complex values.
template <typename T>
cudaError_t conv1d_launch(const Cell4<T> *grid_in, Cell4<T> *grid_out, int M, const FftPlan &plan,
                          const typename Cx<T>::t *tw, typename Cx<T>::t *work, double h, double df, int mode,
                          cudaStream_t st);

// Batched 2-D convolution (many embeddings, one launch per pass).  Job j's current geometry
// is *jobs[j].cg (device), its grids / work buffers / spectra / twiddles start at the given
// offsets of the concatenated arrays, sized for its capacity.  The blocks of each pass are
// split among the jobs by a map (job of each block, first block of each job): kernel rows
// (M_cap blocks per job), columns (L_cap / 2 + 1) and data rows (M_cap); blocks beyond
// the job's current size return at once.  L_max: the largest capacity (shared memory).
struct FftBatchJob {
    const ConvGeom *cg;
    size_t cell0, work0, kspec0, tw0;
};
struct FftBatchMap {
    const int *job;
    const int *first;
};
template <typename T>
cudaError_t conv2d_launch_batch(const Cell4<T> *grid_in, Cell4<T> *grid_out, const FftBatchJob *jobs,
                                FftBatchMap krow, int nkrow, FftBatchMap cols, int ncols, FftBatchMap rows, int nrows,
                                int L_max, const typename Cx<T>::t *tw, typename Cx<T>::t *work_a,
                                typename Cx<T>::t *work_b, KSpec<T> *kspec, double df, int mode, cudaStream_t st);
// The twiddles of each job's current length (jobs[j].cg->plan.L) at tw + jobs[j].tw0.
template <typename T>
cudaError_t twiddles_batch(const FftBatchJob *jobs, int J, typename Cx<T>::t *tw, cudaStream_t st);

}  // namespace fitsne
