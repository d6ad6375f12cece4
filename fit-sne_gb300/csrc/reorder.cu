// Locality renumbering kernels (see reorder.cuh).
#include "reorder.cuh"

namespace fitsne {
namespace {

__device__ __forceinline__ uint32_t spread_bits16(uint32_t x) {
    x &= 0xffffu;
    x = (x | (x << 8)) & 0x00ff00ffu;
    x = (x | (x << 4)) & 0x0f0f0f0fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
}

template <typename T>
__global__ void k_morton(const T *__restrict__ Y, int N, int D, int stride, double lo, double scale,
                         uint32_t *__restrict__ keys, uint32_t *__restrict__ ids) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        uint32_t key;
        if (D == 2) {
            double fx = ((double) Y[(size_t) i * stride] - lo) * scale;
            double fy = ((double) Y[(size_t) i * stride + 1] - lo) * scale;
            fx = fmin(fmax(fx, 0.0), 65535.0);
            fy = fmin(fmax(fy, 0.0), 65535.0);
            key = spread_bits16((uint32_t) fx) | (spread_bits16((uint32_t) fy) << 1);
        } else {
            double f = ((double) Y[(size_t) i * stride] - lo) * scale;
            f = fmin(fmax(f, 0.0), 4294967295.0);
            key = (uint32_t) f;
        }
        keys[i] = key;
        ids[i] = (uint32_t) i;
    }
}

__global__ void k_invert(const uint32_t *__restrict__ order, uint32_t *__restrict__ inv, int N) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x) inv[order[k]] = (uint32_t) k;
}

template <typename T>
__global__ void k_gather_rows(const T *__restrict__ src, T *__restrict__ dst, const uint32_t *__restrict__ order,
                              int N, int width) {
    const size_t n = (size_t) N * width;
    for (size_t e = blockIdx.x * (size_t) blockDim.x + threadIdx.x; e < n; e += (size_t) gridDim.x * blockDim.x) {
        const size_t k = e / width;
        const int w = (int) (e % width);
        dst[e] = src[(size_t) order[k] * width + w];
    }
}

__global__ void k_perm_len(const uint32_t *__restrict__ row, const uint32_t *__restrict__ order, int N,
                           uint32_t *__restrict__ len) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x) {
        const uint32_t c = order[k];
        len[k] = row[c + 1] - row[c];
    }
}

// Rows up to kSortRow entries are also sorted by (new) column index, so that the
// attraction pass gathers neighbours in index order (adjacent lanes, adjacent lines).
constexpr int kSortRow = 256;

template <typename T>
__global__ void __launch_bounds__(256) k_perm_csr(const uint32_t *__restrict__ row, const uint32_t *__restrict__ col,
                                                  const T *__restrict__ val, const uint32_t *__restrict__ order,
                                                  const uint32_t *__restrict__ inv,
                                                  const uint32_t *__restrict__ row_new, int N,
                                                  uint32_t *__restrict__ col_new, T *__restrict__ val_new) {
    __shared__ uint32_t sc[8][kSortRow];
    __shared__ T sv[8][kSortRow];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int k = gw; k < N; k += nw) {
        const uint32_t c = order[k];
        const uint32_t a = row[c], b = row[c + 1], o = row_new[k];
        const int len = (int) (b - a);
        if (len > 1 && len <= kSortRow) {
            int p2 = 2;
            while (p2 < len) p2 <<= 1;
            for (int i = lane; i < p2; i += 32) {
                if (i < len) {
                    sc[w][i] = inv[col[a + i]];
                    sv[w][i] = val[a + i];
                } else {
                    sc[w][i] = 0xffffffffu;
                    sv[w][i] = T(0);
                }
            }
            __syncwarp();
            for (int kk = 2; kk <= p2; kk <<= 1)
                for (int j = kk >> 1; j > 0; j >>= 1) {
                    for (int i = lane; i < p2; i += 32) {
                        const int q = i ^ j;
                        if (q > i) {
                            const bool up = (i & kk) == 0;
                            const uint32_t x = sc[w][i], y = sc[w][q];
                            if ((x > y) == up) {
                                sc[w][i] = y;
                                sc[w][q] = x;
                                const T t = sv[w][i];
                                sv[w][i] = sv[w][q];
                                sv[w][q] = t;
                            }
                        }
                    }
                    __syncwarp();
                }
            for (int i = lane; i < len; i += 32) {
                col_new[o + i] = sc[w][i];
                val_new[o + i] = sv[w][i];
            }
            __syncwarp();
        } else {
            for (uint32_t e = a + lane; e < b; e += 32) {
                col_new[o + (e - a)] = inv[col[e]];
                val_new[o + (e - a)] = val[e];
            }
        }
    }
}

template <typename T>
__global__ void k_scatter_rows(const T *__restrict__ src, T *__restrict__ dst, const uint32_t *__restrict__ perm,
                               int N, int width) {
    const size_t n = (size_t) N * width;
    for (size_t e = blockIdx.x * (size_t) blockDim.x + threadIdx.x; e < n; e += (size_t) gridDim.x * blockDim.x) {
        const size_t k = e / width;
        const int w = (int) (e % width);
        dst[(size_t) perm[k] * width + w] = src[e];
    }
}

__global__ void k_iota32(uint32_t *__restrict__ p, int N) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x) p[k] = (uint32_t) k;
}

__global__ void k_compose(const uint32_t *__restrict__ perm_old, const uint32_t *__restrict__ order,
                          uint32_t *__restrict__ perm_new, int N) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x)
        perm_new[k] = perm_old[order[k]];
}

int blocks_for(size_t n) {
    size_t b = (n + 255) / 256;
    return (int) (b < 1 ? 1 : (b > 8192 ? 8192 : b));
}

}  // namespace

template <typename T>
cudaError_t launch_morton_keys(const T *Y, int N, int D, int stride, double lo, double hi, uint32_t *keys,
                               uint32_t *ids, cudaStream_t st) {
    const double span = hi > lo ? hi - lo : 1.0;
    const double scale = (D == 2 ? 65535.0 : 4294967295.0) / span;
    k_morton<T><<<blocks_for(N), 256, 0, st>>>(Y, N, D, stride, lo, scale, keys, ids);
    return cudaGetLastError();
}

cudaError_t launch_invert(const uint32_t *order, uint32_t *inv, int N, cudaStream_t st) {
    k_invert<<<blocks_for(N), 256, 0, st>>>(order, inv, N);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_gather_rows(const T *src, T *dst, const uint32_t *order, int N, int width, cudaStream_t st) {
    k_gather_rows<T><<<blocks_for((size_t) N * width), 256, 0, st>>>(src, dst, order, N, width);
    return cudaGetLastError();
}

cudaError_t launch_perm_lengths(const uint32_t *row, const uint32_t *order, int N, uint32_t *len, cudaStream_t st) {
    k_perm_len<<<blocks_for(N), 256, 0, st>>>(row, order, N, len);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_perm_csr(const uint32_t *row, const uint32_t *col, const T *val, const uint32_t *order,
                            const uint32_t *inv, const uint32_t *row_new, int N, uint32_t *col_new, T *val_new,
                            cudaStream_t st) {
    k_perm_csr<T><<<blocks_for((size_t) N * 32), 256, 0, st>>>(row, col, val, order, inv, row_new, N, col_new,
                                                               val_new);
    return cudaGetLastError();
}

cudaError_t launch_compose(const uint32_t *perm_old, const uint32_t *order, uint32_t *perm_new, int N,
                           cudaStream_t st) {
    k_compose<<<blocks_for(N), 256, 0, st>>>(perm_old, order, perm_new, N);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_scatter_rows(const T *src, T *dst, const uint32_t *perm, int N, int width, cudaStream_t st) {
    k_scatter_rows<T><<<blocks_for((size_t) N * width), 256, 0, st>>>(src, dst, perm, N, width);
    return cudaGetLastError();
}

cudaError_t launch_iota(uint32_t *perm, int N, cudaStream_t st) {
    k_iota32<<<blocks_for(N), 256, 0, st>>>(perm, N);
    return cudaGetLastError();
}

template cudaError_t launch_scatter_rows<float>(const float *, float *, const uint32_t *, int, int, cudaStream_t);
template cudaError_t launch_scatter_rows<double>(const double *, double *, const uint32_t *, int, int, cudaStream_t);

template cudaError_t launch_morton_keys<float>(const float *, int, int, int, double, double, uint32_t *, uint32_t *,
                                               cudaStream_t);
template cudaError_t launch_morton_keys<double>(const double *, int, int, int, double, double, uint32_t *,
                                                uint32_t *, cudaStream_t);
template cudaError_t launch_gather_rows<float>(const float *, float *, const uint32_t *, int, int, cudaStream_t);
template cudaError_t launch_gather_rows<double>(const double *, double *, const uint32_t *, int, int, cudaStream_t);
template cudaError_t launch_perm_csr<float>(const uint32_t *, const uint32_t *, const float *, const uint32_t *,
                                            const uint32_t *, const uint32_t *, int, uint32_t *, float *,
                                            cudaStream_t);
template cudaError_t launch_perm_csr<double>(const uint32_t *, const uint32_t *, const double *, const uint32_t *,
                                             const uint32_t *, const uint32_t *, int, uint32_t *, double *,
                                             cudaStream_t);

}  // namespace fitsne
