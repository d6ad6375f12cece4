// Exact k-nearest neighbours on the GPU (replaces the VP-tree search of the reference,
// src/vptree.h:110-280 driven by src/tsne.cpp:1643-1726).
//
// Two stages:
//  1. candidates: every query scans all points in FP32 (direct differences) and keeps the
//     C = K + slack smallest approximate squared distances (shared-memory lists per query);
//  2. re-rank: the C candidates get their exact FP64 distance, summed over dimensions in
//     the reference's order (sqrt of sum of squared differences, vptree.h:97-107), are
//     sorted, and the first K are kept.  A row is accepted only if no point outside the
//     candidate list can beat its K-th distance given the FP32 error bound; rejected rows
//     are rescanned with a larger C.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "knn_tc.cuh"

namespace fitsne {

struct KnnStats {
    int rows_rescanned = 0;    // rows that failed verification in the first pass
    int rows_unverified = 0;   // rows still unverified after the rescans (exact ties)
    bool tensor_cores = false; // first pass ran on the tcgen05 kernel (knn_tc.cu)
    double s_candidates = 0;   // host-clock seconds: first-pass candidates (tensor-core path)
    double s_first_pass = 0;   // first pass including the re-rank
    double s_rescans = 0;      // rescans of the unverified rows
    KnnTcStats tc;             // tensor-core pass: tiles computed, inserts, ordering time
};

// One line of the timing report (FITSNE_TIMING): "[fitsne] kNN (K=..., path): ..."; total_s < 0
// leaves the total out.
void print_knn_stats(int K, const KnnStats &ks, double total_s);

// Xd: N x D FP64 (device).  Writes idx[N*K] and dist[N*K] (device, FP64 non-squared,
// ascending).  K includes the point itself (the reference asks for K + 1 neighbours).
// Returns 0 or a negative error code; err receives a message.
// order_out / order_written (may be null): see knn_candidates_tc (knn_tc.cuh).
int knn_exact(const double *Xd, int N, int D, int K, uint32_t *idx, double *dist, cudaStream_t st, KnnStats *stats,
              const char **err, uint32_t *order_out = nullptr, bool *order_written = nullptr);

}  // namespace fitsne
