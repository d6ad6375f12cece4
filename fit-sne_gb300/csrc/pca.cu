// PCA initialisation on the GPU (replaces the scikit-learn step of fast_tsne.py:186-197,
// which runs before the reference's path): centre X, the Gram matrix X_c^T X_c (k_gram_tiles
// + k_gram_reduce, FP64) and the projection X_c V (k_project), the D x D eigenproblem on the
// host by cyclic Jacobi rotations (D <= 2048; 50 in the configurations).  Signs follow
// scikit-learn's svd_flip(u_based_decision=False): the largest-magnitude entry of each
// component is positive.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/fitsne_gb300.h"
#include "capi_internal.h"

namespace fitsne {
namespace {

__global__ void k_col_mean(const double *__restrict__ X, int N, int D, double *__restrict__ mean) {
    // one block per column, sums in a fixed order (per-thread strides, then a tree)
    __shared__ double sh[256];
    const int d = blockIdx.x;
    double s = 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) s += X[(size_t) i * D + d];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o; o >>= 1) {
        if ((int) threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) mean[d] = sh[0] / (double) N;
}

__global__ void k_centre(double *__restrict__ X, size_t n, int D, const double *__restrict__ mean) {
    for (size_t e = blockIdx.x * (size_t) blockDim.x + threadIdx.x; e < n; e += (size_t) gridDim.x * blockDim.x)
        X[e] -= mean[e % D];
}

// Gram matrix of the centred rows, upper triangle by 32 x 32 tiles: block (t, c) adds up
// tile t over row chunk c (rows [c rows_per, (c + 1) rows_per)), staging 32 rows of the
// tile's two column ranges in shared memory; partial tiles go to part[c][t][32 x 32].
// Every entry's sum has a fixed order (chunk by chunk, then k_gram_reduce), so the result is
// repeatable.
constexpr int kGT = 32;

__global__ void __launch_bounds__(256) k_gram_tiles(const double *__restrict__ X, int N, int D, int ntd,
                                                    int rows_per, double *__restrict__ part) {
    __shared__ double sa[kGT][kGT + 1], sb[kGT][kGT + 1];
    // tile t -> (ti, tj), ti <= tj, in row-major order of the upper triangle of ntd x ntd tiles
    int t = blockIdx.x, ti = 0;
    while (t >= ntd - ti) {
        t -= ntd - ti;
        ++ti;
    }
    const int tj = ti + t;
    const int c0 = ti * kGT, c1 = tj * kGT;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 8 row groups of the tile
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const int r0 = blockIdx.y * rows_per, r1 = min(N, r0 + rows_per);
    for (int rb = r0; rb < r1; rb += kGT) {
        for (int e = threadIdx.x; e < kGT * kGT; e += blockDim.x) {
            const int rr = e / kGT, cc = e % kGT, r = rb + rr;
            sa[rr][cc] = (r < r1 && c0 + cc < D) ? X[(size_t) r * D + c0 + cc] : 0.0;
            sb[rr][cc] = (r < r1 && c1 + cc < D) ? X[(size_t) r * D + c1 + cc] : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int rr = 0; rr < kGT; ++rr) {
            const double b = sb[rr][tx];
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[q] = fma(sa[rr][ty + 8 * q], b, acc[q]);
        }
        __syncthreads();
    }
    const int ntiles = gridDim.x;
    double *out = part + ((size_t) blockIdx.y * ntiles + blockIdx.x) * kGT * kGT;
#pragma unroll
    for (int q = 0; q < 4; ++q) out[(ty + 8 * q) * kGT + tx] = acc[q];
}

// C[i][j] (both triangles) = sum over the chunks of the partial tiles, chunk by chunk
__global__ void k_gram_reduce(const double *__restrict__ part, int ntd, int nchunks, int D, double *__restrict__ C) {
    const int ntiles = ntd * (ntd + 1) / 2;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ntiles * kGT * kGT; e += gridDim.x * blockDim.x) {
        const int tile = e / (kGT * kGT), w = e % (kGT * kGT);
        int t = tile, ti = 0;
        while (t >= ntd - ti) {
            t -= ntd - ti;
            ++ti;
        }
        const int i = ti * kGT + w / kGT, j = (ti + t) * kGT + w % kGT;
        if (i >= D || j >= D || i > j) continue;
        double s = 0.0;
        for (int c = 0; c < nchunks; ++c) s += part[((size_t) c * ntiles + tile) * kGT * kGT + w];
        C[(size_t) i * D + j] = s;
        C[(size_t) j * D + i] = s;
    }
}

// Y[r][c] = sum_d X_c[r][d] V[d][c] for the components c in [c0, c0 + kc) (V: D x k
// row-major; that slice in shared memory): a warp per row, lanes over d (coalesced), one
// shuffle reduction per component
__global__ void __launch_bounds__(256) k_project(const double *__restrict__ X, int N, int D,
                                                 const double *__restrict__ V, int k, int c0, int kc,
                                                 double *__restrict__ Y) {
    extern __shared__ double sv[];
    for (int e = threadIdx.x; e < D * kc; e += blockDim.x) sv[e] = V[(size_t) (e / kc) * k + c0 + e % kc];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int r = wg; r < N; r += nw) {
        const double *x = X + (size_t) r * D;
        for (int c = 0; c < kc; ++c) {
            double s = 0.0;
            for (int d = lane; d < D; d += 32) s = fma(x[d], sv[d * kc + c], s);
            for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) Y[(size_t) r * k + c0 + c] = s;
        }
    }
}

// Cyclic Jacobi on the symmetric D x D matrix A (row-major, destroyed): eigenvalues w,
// eigenvectors in the columns of V.
void jacobi_eigen(std::vector<double> &A, int D, std::vector<double> &w, std::vector<double> &V) {
    V.assign((size_t) D * D, 0.0);
    for (int i = 0; i < D; ++i) V[(size_t) i * D + i] = 1.0;
    auto a = [&](int i, int j) -> double & { return A[(size_t) i * D + j]; };
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < D; ++i)
            for (int j = 0; j < D; ++j) {
                tot += a(i, j) * a(i, j);
                if (i != j) off += a(i, j) * a(i, j);
            }
        if (off <= 1e-30 * tot || off == 0.0) break;
        for (int p = 0; p < D - 1; ++p)
            for (int q = p + 1; q < D; ++q) {
                const double apq = a(p, q);
                if (apq == 0.0) continue;
                const double theta = (a(q, q) - a(p, p)) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < D; ++k) {  // A <- A J (columns p, q)
                    const double akp = a(k, p), akq = a(k, q);
                    a(k, p) = c * akp - s * akq;
                    a(k, q) = s * akp + c * akq;
                }
                for (int k = 0; k < D; ++k) {  // A <- J^T A (rows p, q)
                    const double apk = a(p, k), aqk = a(q, k);
                    a(p, k) = c * apk - s * aqk;
                    a(q, k) = s * apk + c * aqk;
                }
                for (int k = 0; k < D; ++k) {
                    const double vkp = V[(size_t) k * D + p], vkq = V[(size_t) k * D + q];
                    V[(size_t) k * D + p] = c * vkp - s * vkq;
                    V[(size_t) k * D + q] = s * vkp + c * vkq;
                }
            }
    }
    w.resize(D);
    for (int i = 0; i < D; ++i) w[i] = a(i, i);
}

}  // namespace
}  // namespace fitsne

using namespace fitsne;

extern "C" int fitsne_pca(const double *X, int N, int D, int n_components, double *Y) {
    if (!X || !Y || N < 2 || D < 1 || n_components < 1 || n_components > D || n_components > N)
        return set_error(FITSNE_E_ARG, "invalid PCA arguments");
    if (D > 2048) return set_error(FITSNE_E_ARG, "PCA: at most 2048 input dimensions");
    int rc = check_cuda_device();
    if (rc) return rc;
    const int k = n_components;
    const int ntd = (D + kGT - 1) / kGT, ntiles = ntd * (ntd + 1) / 2;
    // row chunks: about two blocks per SM in all, at least 32 rows each
    int nsm = 152, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    int nchunks = std::max(1, std::min((N + kGT - 1) / kGT, (2 * nsm + ntiles - 1) / ntiles));
    const int rows_per = ((N + nchunks - 1) / nchunks + kGT - 1) / kGT * kGT;
    nchunks = (N + rows_per - 1) / rows_per;
    double *dX = nullptr, *dmean = nullptr, *dC = nullptr, *dV = nullptr, *dY = nullptr, *dpart = nullptr;
    auto cleanup = [&]() {
        cudaFree(dX);
        cudaFree(dmean);
        cudaFree(dC);
        cudaFree(dV);
        cudaFree(dY);
        cudaFree(dpart);
    };
    const size_t n = (size_t) N * D;
    if (cudaMalloc(&dX, sizeof(double) * n) != cudaSuccess || cudaMalloc(&dmean, sizeof(double) * D) != cudaSuccess ||
        cudaMalloc(&dC, sizeof(double) * (size_t) D * D) != cudaSuccess ||
        cudaMalloc(&dV, sizeof(double) * (size_t) D * k) != cudaSuccess ||
        cudaMalloc(&dY, sizeof(double) * (size_t) N * k) != cudaSuccess ||
        cudaMalloc(&dpart, sizeof(double) * (size_t) nchunks * ntiles * kGT * kGT) != cudaSuccess) {
        cleanup();
        return set_error(FITSNE_E_NOMEM, "PCA: device allocation failed");
    }
    cudaMemcpy(dX, X, sizeof(double) * n, cudaMemcpyHostToDevice);
    k_col_mean<<<D, 256>>>(dX, N, D, dmean);
    k_centre<<<2048, 256>>>(dX, n, D, dmean);
    k_gram_tiles<<<dim3(ntiles, nchunks), 256>>>(dX, N, D, ntd, rows_per, dpart);
    k_gram_reduce<<<std::min(4096, (ntiles * kGT * kGT + 255) / 256), 256>>>(dpart, ntd, nchunks, D, dC);
    std::vector<double> C((size_t) D * D);
    cudaError_t e = cudaMemcpy(C.data(), dC, sizeof(double) * C.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        cleanup();
        return set_error(FITSNE_E_CUDA, std::string("PCA: ") + cudaGetErrorString(e));
    }
    std::vector<double> w, V;
    jacobi_eigen(C, D, w, V);
    std::vector<int> order(D);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return w[a] > w[b]; });
    // components as the columns of V_k (D x k, row-major), signs per svd_flip on V^T rows
    std::vector<double> Vk((size_t) D * k);
    for (int c = 0; c < k; ++c) {
        const int ev = order[c];
        int am = 0;
        for (int d = 1; d < D; ++d)
            if (std::fabs(V[(size_t) d * D + ev]) > std::fabs(V[(size_t) am * D + ev])) am = d;
        const double sg = V[(size_t) am * D + ev] < 0 ? -1.0 : 1.0;
        for (int d = 0; d < D; ++d) Vk[(size_t) d * k + c] = sg * V[(size_t) d * D + ev];
    }
    cudaMemcpy(dV, Vk.data(), sizeof(double) * Vk.size(), cudaMemcpyHostToDevice);
    // components in slices whose columns of V fit in 96 KB of shared memory
    const int kc_max = std::max(1, (int) (96 * 1024 / (sizeof(double) * (size_t) D)));
    cudaFuncSetAttribute(k_project, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
    for (int c0 = 0; c0 < k; c0 += kc_max) {
        const int kc = std::min(kc_max, k - c0);
        k_project<<<std::min(4096, (N + 7) / 8), 256, sizeof(double) * (size_t) D * kc>>>(dX, N, D, dV, k, c0, kc,
                                                                                          dY);
    }
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(Y, dY, sizeof(double) * (size_t) N * k, cudaMemcpyDeviceToHost);
    cleanup();
    if (e != cudaSuccess) return set_error(FITSNE_E_CUDA, std::string("PCA: ") + cudaGetErrorString(e));
    return 0;
}
