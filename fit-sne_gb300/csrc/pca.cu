// PCA initialisation on the GPU (replaces the scikit-learn step of fast_tsne.py:186-197,
// which runs before the reference's path): centre X, covariance X_c^T X_c and the
// projection X_c V with cuBLAS (plain FP64 GEMMs), the D x D eigenproblem on the host by
// cyclic Jacobi rotations.  Signs follow scikit-learn's svd_flip(u_based_decision=False):
// the largest-magnitude entry of each component is positive.
#include <cublas_v2.h>

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
    double *dX = nullptr, *dmean = nullptr, *dC = nullptr, *dV = nullptr, *dY = nullptr;
    cublasHandle_t h = nullptr;
    std::string err;
    auto cleanup = [&]() {
        cudaFree(dX);
        cudaFree(dmean);
        cudaFree(dC);
        cudaFree(dV);
        cudaFree(dY);
        if (h) cublasDestroy(h);
    };
    const size_t n = (size_t) N * D;
    if (cudaMalloc(&dX, sizeof(double) * n) != cudaSuccess || cudaMalloc(&dmean, sizeof(double) * D) != cudaSuccess ||
        cudaMalloc(&dC, sizeof(double) * (size_t) D * D) != cudaSuccess ||
        cudaMalloc(&dV, sizeof(double) * (size_t) D * k) != cudaSuccess ||
        cudaMalloc(&dY, sizeof(double) * (size_t) N * k) != cudaSuccess) {
        cleanup();
        return set_error(FITSNE_E_NOMEM, "PCA: device allocation failed");
    }
    if (cublasCreate(&h) != CUBLAS_STATUS_SUCCESS) {
        cleanup();
        return set_error(FITSNE_E_CUDA, "PCA: cublasCreate failed");
    }
    cudaMemcpy(dX, X, sizeof(double) * n, cudaMemcpyHostToDevice);
    k_col_mean<<<D, 256>>>(dX, N, D, dmean);
    k_centre<<<2048, 256>>>(dX, n, D, dmean);
    // X_c is row-major N x D = column-major D x N (lda D): C = X_c^T X_c = A A^T (D x D)
    const double one = 1.0, zero = 0.0;
    if (cublasDgemm(h, CUBLAS_OP_N, CUBLAS_OP_T, D, D, N, &one, dX, D, dX, D, &zero, dC, D) !=
        CUBLAS_STATUS_SUCCESS) {
        cleanup();
        return set_error(FITSNE_E_CUDA, "PCA: covariance GEMM failed");
    }
    std::vector<double> C((size_t) D * D);
    if (cudaMemcpy(C.data(), dC, sizeof(double) * C.size(), cudaMemcpyDeviceToHost) != cudaSuccess) {
        cleanup();
        return set_error(FITSNE_E_CUDA, "PCA: copy failed");
    }
    for (int i = 0; i < D; ++i)  // symmetrise the rounding
        for (int j = i + 1; j < D; ++j) C[(size_t) i * D + j] = C[(size_t) j * D + i] =
                                            0.5 * (C[(size_t) i * D + j] + C[(size_t) j * D + i]);
    std::vector<double> w, V;
    jacobi_eigen(C, D, w, V);
    std::vector<int> order(D);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return w[a] > w[b]; });
    // components as columns of a D x k column-major matrix, signs per svd_flip on V^T rows
    std::vector<double> Vk((size_t) D * k);
    for (int c = 0; c < k; ++c) {
        const int e = order[c];
        int am = 0;
        for (int d = 1; d < D; ++d)
            if (std::fabs(V[(size_t) d * D + e]) > std::fabs(V[(size_t) am * D + e])) am = d;
        const double sg = V[(size_t) am * D + e] < 0 ? -1.0 : 1.0;
        for (int d = 0; d < D; ++d) Vk[(size_t) c * D + d] = sg * V[(size_t) d * D + e];
    }
    cudaMemcpy(dV, Vk.data(), sizeof(double) * Vk.size(), cudaMemcpyHostToDevice);
    // Y^T (k x N, column-major = Y row-major N x k) = V_k^T X_c
    if (cublasDgemm(h, CUBLAS_OP_T, CUBLAS_OP_N, k, N, D, &one, dV, D, dX, D, &zero, dY, k) !=
        CUBLAS_STATUS_SUCCESS) {
        cleanup();
        return set_error(FITSNE_E_CUDA, "PCA: projection GEMM failed");
    }
    cudaError_t e = cudaMemcpy(Y, dY, sizeof(double) * (size_t) N * k, cudaMemcpyDeviceToHost);
    cleanup();
    if (e != cudaSuccess) return set_error(FITSNE_E_CUDA, cudaGetErrorString(e));
    return 0;
}
