// Tensor-core (tcgen05) candidate search for the exact kNN; see knn_tc.cu.
#pragma once

#include <cstdint>
#include <string>

#include <cuda_runtime.h>

namespace fitsne {

// Longest candidate list the shared-memory heaps of the tensor-core kernel hold.
constexpr int kMaxTcCandidates = 120;

// True when the device is a Blackwell (cc 10.x) part, the driver exposes the tensor-map
// encoder, D <= 64 and C <= kMaxTcCandidates.
bool knn_tc_supported(int D, int C);

// For every row of X (N x D, FP64 on the device) the C smallest approximate squared
// distances to all rows, ascending, into cand_d / cand_i (N x C).  Approximation: BF16
// hi/lo split products with FP32 accumulation; |error| <= 8e-5 |x||y| + 4e-7 (|x|^2 + |y|^2)
// + 1.5 (D + 4) 2^-24 d^2 (the bound the verification in knn.cu uses).
int knn_candidates_tc(const double *Xd, int N, int D, int C, float *cand_d, uint32_t *cand_i, cudaStream_t st,
                      std::string &err);

}  // namespace fitsne
