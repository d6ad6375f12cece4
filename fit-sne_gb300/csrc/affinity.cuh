// Input-similarity stage on the GPU: data preparation, perplexity calibration,
// symmetrisation and normalisation of P.
//
// Reference functions replaced (src/tsne.cpp of FIt-SNE v1.2.1):
//   zeroMean + max-abs scaling of X        153-164, 1851-1876
//   distances2similarities (+ list)        1394-1469, 1474-1500
//   computeGaussianPerplexity (VP tree)    1643-1726  (kNN in knn.cu)
//   symmetrizeMatrix                       1730-1828
//   normalisation by sum(P)                327-330
//   automatic early exaggeration           392-402
#pragma once

#include <cstdint>
#include <cstdlib>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace fitsne {

// FITSNE_TIMING=1 in the environment prints the similarity-stage phase times to stderr.
inline bool timing_requested() {
    const char *e = std::getenv("FITSNE_TIMING");
    return e && std::atoi(e) != 0;
}

// CSR on the device; free with free_csr.
struct DevCSR {
    int N = 0;
    size_t nnz = 0;
    uint32_t *row = nullptr;
    uint32_t *col = nullptr;
    double *val = nullptr;
};
void free_csr(DevCSR &P);

// Uploads X (host, N x D) and applies zeroMean and, when normalize, X /= max|X|.
int prepare_X(const double *X_host, int N, int D, bool normalize, double **Xd, cudaStream_t st, std::string &err);

// Row-wise calibration of K distances per row (row r at dist + r*stride + offset).
// P receives nrows x K similarities, beta (may be null) the precisions, iters (may be null)
// the number of entropy evaluations of each row (the first perplexity of a list).
int calibrate_rows(const double *dist, int stride, int offset, double *P, int nrows, int K, double perplexity,
                   double sigma, int list_len, const double *list_host, double *beta, cudaStream_t st,
                   std::string &err, std::vector<int> *iters = nullptr);

// kNN + calibration into fixed-length rows (row n = n*K).  Xd on the device.
// order_out / order_written (may be null): the kNN's locality order, when it used one
// (knn_candidates_tc, knn_tc.cuh).
int gaussian_perplexity_device(const double *Xd, int N, int D, int K, double perplexity, double sigma, int list_len,
                               const double *list_host, DevCSR *out, cudaStream_t st, std::string &err,
                               int *knn_rescanned = nullptr, uint32_t *order_out = nullptr,
                               bool *order_written = nullptr);

// (P + P^T)/2 in the reference's entry order.  in is left untouched.
int symmetrize_device(const DevCSR &in, DevCSR *out, cudaStream_t st, std::string &err);

// val /= sum(val); returns the sum through *sum.
int normalize_device(DevCSR &P, double *sum, cudaStream_t st, std::string &err);

// max over rows of the row sums of val.
int max_row_sum_device(const DevCSR &P, double *out, cudaStream_t st, std::string &err);

// host <-> device copies of a CSR
int csr_to_device(const uint32_t *row, const uint32_t *col, const double *val, int N, DevCSR *out, cudaStream_t st,
                  std::string &err);
int csr_to_host(const DevCSR &P, uint32_t *row, uint32_t *col, double *val, cudaStream_t st, std::string &err);

}  // namespace fitsne
