// Stable LSD radix sort of (u32 key, u32 value) pairs and an exclusive prefix sum.
//
// Used by the symmetrisation (grouping kNN edges by target row while keeping the source
// order, which the reference's entry order needs) and by the locality renumbering of the
// points.  8-bit digits, one histogram / scan / scatter round per digit; the scatter ranks
// items warp by warp in input order (match_any), so equal keys keep their input order.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace fitsne {

// Bytes of device scratch radix_sort_pairs needs for n items.
size_t radix_sort_scratch_bytes(size_t n);

// Sorts keys[0..n) (only the low key_bits bits are looked at) carrying vals along.
// keys_alt / vals_alt are ping-pong buffers of n items; on return the sorted data is in
// keys / vals.  scratch must hold radix_sort_scratch_bytes(n) bytes.
cudaError_t radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *keys_alt, uint32_t *vals_alt, size_t n,
                             int key_bits, void *scratch, cudaStream_t st);

// Bytes of device scratch exclusive_scan_u32 needs for n items.
size_t scan_scratch_bytes(size_t n);
// out[i] = sum_{k<i} in[i]; also writes the total to out[n] (out has n+1 slots).
cudaError_t exclusive_scan_u32(const uint32_t *in, uint32_t *out, size_t n, void *scratch, cudaStream_t st);

}  // namespace fitsne
