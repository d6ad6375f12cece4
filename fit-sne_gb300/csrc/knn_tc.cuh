// Tensor-core (tcgen05) candidate search for the exact kNN; see knn_tc.cu.
#pragma once

#include <cstdint>
#include <string>

#include <cuda_runtime.h>

namespace fitsne {

// Longest candidate list the shared-memory heaps of the tensor-core kernel hold.
constexpr int kMaxTcCandidates = 120;

// True when the device is a Blackwell (cc 10.x) part, the driver exposes the tensor-map
// encoder, D <= 62 (two spare columns of the 64-wide operand rows) and C <= kMaxTcCandidates.
bool knn_tc_supported(int D, int C);

// For every row of X (N x D, FP64 on the device) the C smallest approximate squared
// distances to all rows, ascending, into cand_d / cand_i (N x C).  Approximation: BF16
// hi/lo split products and a 3-piece -|y|^2 / 2 with FP32 accumulation, d2 = |x|^2 - 2 acc;
// |error| <= 3e-5 |x||y| + 4e-6 (|x|^2 + |y|^2) + 1.5 (D + 4) 2^-24 d^2, the bound the
// verification in knn.cu uses.  The split drops lo.lo and the BF16 rounding of lo, at most
// 3 * 2^-18 |x||y| in the product (2.3e-5 |x||y| in d2); the accumulation adds at most
// sixteen FP32 roundings (truncating or not) of partial sums below |x||y| + |y|^2 / 2
// (< 2e-6 (|x||y| + |y|^2)).
int knn_candidates_tc(const double *Xd, int N, int D, int C, float *cand_d, uint32_t *cand_i, cudaStream_t st,
                      std::string &err);

}  // namespace fitsne
