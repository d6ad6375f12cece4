// Tensor-core (tcgen05) candidate search for the exact kNN; see knn_tc.cu.
#pragma once

#include <cstdint>
#include <string>

#include <cuda_runtime.h>

namespace fitsne {

// Longest candidate list the shared-memory heaps of the tensor-core kernel hold.
constexpr int kMaxTcCandidates = 120;

struct KnnTcStats {
    double tiles_kept = 1.0;         // fraction of (query tile, reference tile) pairs computed
    double cols_per_query = 0;       // columns that passed a query's threshold test, per query
    double inserts_per_query = 0;    // heap insertions (fills and replacements) per query
    double s_order = 0;              // host-clock seconds of the locality order
    // shares of the kernel's time (each role's own clock): the TMA producer waiting for a free
    // stage, the MMA issuer waiting for operands / for a free accumulator, the epilogue warps
    // waiting for a full accumulator / walking their kept columns into the heaps
    double producer_stage_wait = 0, mma_data_wait = 0, mma_acc_wait = 0;
    double epilogue_acc_wait = 0, epilogue_inserts = 0;
    double insert_iters_per_tile = 0, cycles_per_insert_iter = 0;  // epilogue warp level
};

// The locality order of the data that the tensor-core kNN also sorts its rows by: the points in
// the cells of ~N/1024 pivots (evenly spaced rows of X; each point in the cell of its nearest),
// the cells grouped by the nearest of 32 super-pivots.  order[r] = the point at row r.  Rows
// close in this order are close in the data space, so their neighbour lists overlap.  It looks
// at the first kDataOrderMaxD coordinates, which is all of them where it is used.
constexpr int kDataOrderMaxD = 64;
int data_locality_order(const double *Xd, int N, int D, uint32_t *order, cudaStream_t st, std::string &err);

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
//
// Reference tiles (64 points) that cannot hold a candidate of any query of a query tile (128
// points) are skipped: their bounding spheres bound d^2 from below, and a tile is skipped when
// that bound, less the error bound above (maxnorm = the largest |x|), exceeds the largest
// current C-th distance of the tile's queries.  Superblocks of tiles are visited nearest
// first, so the thresholds fall early and the walk stops at the first superblock too far
// away.  The points are first put in a locality order (cells of the nearest of ~N/1024
// sampled pivots, cells grouped by 32 super-pivots; FITSNE_KNN_ORDER=input keeps the
// caller's order): the lists do not depend on the order, the skipping does.  stats may be
// null.
//
// Exactness: a skipped point would not have entered the list had its tile been computed (its
// approximate d^2 is above the threshold then in force, and thresholds only fall), so the
// lists are the ones the full scan keeps, up to the order of equal approximate distances.
// order_out (may be null, device, N entries): receives the locality order when the search used
// one, and *order_written is then set (data_locality_order gives the same order).
int knn_candidates_tc(const double *Xd, int N, int D, int C, double maxnorm, float *cand_d, uint32_t *cand_i,
                      cudaStream_t st, KnnTcStats *stats, std::string &err, uint32_t *order_out = nullptr,
                      bool *order_written = nullptr);

// 1: locality order before the candidate search (default), 0: the caller's order
// (FITSNE_KNN_ORDER=input).
int knn_order_mode();

}  // namespace fitsne
