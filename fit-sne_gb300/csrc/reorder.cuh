// Locality renumbering of the points of an embedding.
//
// The attraction pass gathers Y at the column indices of P and the spread / gather passes
// scatter to and read from grid cells near each point.  Numbering the points along a
// Z-order (Morton) curve of the current embedding puts the neighbours of a point (which
// the optimisation has pulled close in the embedding) at nearby indices, so those gathers
// and atomics hit the same cache lines.  The permutation is internal: results are returned
// in the caller's order.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace fitsne {

// keys[i] = Morton code of point i quantised on [lo, hi]^D (16 bits per axis in 2-D,
// 32 bits in 1-D); ids[i] = i.  Y holds the hi parts at stride `stride` floats/doubles.
template <typename T>
cudaError_t launch_morton_keys(const T *Y, int N, int D, int stride, double lo, double hi, uint32_t *keys,
                               uint32_t *ids, cudaStream_t st);
// inv[order[k]] = k
cudaError_t launch_invert(const uint32_t *order, uint32_t *inv, int N, cudaStream_t st);
// dst[k] = src[order[k]] for records of `width` elements of T
template <typename T>
cudaError_t launch_gather_rows(const T *src, T *dst, const uint32_t *order, int N, int width, cudaStream_t st);
// new CSR: row k of the result is row order[k] of the input, columns mapped through inv
cudaError_t launch_perm_lengths(const uint32_t *row, const uint32_t *order, int N, uint32_t *len, cudaStream_t st);
template <typename T>
cudaError_t launch_perm_csr(const uint32_t *row, const uint32_t *col, const T *val, const uint32_t *order,
                            const uint32_t *inv, const uint32_t *row_new, int N, uint32_t *col_new, T *val_new,
                            cudaStream_t st);
// dst[perm[k]] = src[k] for records of `width` elements of T (back to the caller's order)
template <typename T>
cudaError_t launch_scatter_rows(const T *src, T *dst, const uint32_t *perm, int N, int width, cudaStream_t st);
// perm[k] = k
cudaError_t launch_iota(uint32_t *perm, int N, cudaStream_t st);
// perm_new[k] = perm_old[order[k]]
cudaError_t launch_compose(const uint32_t *perm_old, const uint32_t *order, uint32_t *perm_new, int N,
                           cudaStream_t st);

}  // namespace fitsne
