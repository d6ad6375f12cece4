// Stable LSD radix sort and exclusive scan (see sort.cuh).
#include "sort.cuh"

namespace fitsne {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanBlock = kScanThreads * kScanItems;

constexpr int kRsThreads = 256;
constexpr int kRsItems = 8;
constexpr int kRsTile = kRsThreads * kRsItems;
constexpr int kRsWarps = kRsThreads / 32;

size_t cdiv(size_t a, size_t b) { return (a + b - 1) / b; }

__global__ void __launch_bounds__(kScanThreads) k_scan_block(const uint32_t *__restrict__ in,
                                                             uint32_t *__restrict__ out, size_t n,
                                                             uint32_t *__restrict__ bsum) {
    __shared__ uint32_t wsum[kScanThreads / 32];
    const size_t base = (size_t) blockIdx.x * kScanBlock + (size_t) threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t tot = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = (base + k < n) ? in[base + k] : 0u;
        tot += v[k];
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t w = lane < kScanThreads / 32 ? wsum[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kScanThreads / 32) wsum[lane] = w;
    }
    __syncthreads();
    uint32_t run = x - tot + (wid ? wsum[wid - 1] : 0u);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == kScanThreads - 1) bsum[blockIdx.x] = run;
}

__global__ void k_scan_add(uint32_t *__restrict__ out, size_t n, const uint32_t *__restrict__ boff) {
    const size_t base = (size_t) blockIdx.x * kScanBlock;
    const uint32_t add = boff[blockIdx.x];
    for (int k = threadIdx.x; k < kScanBlock; k += blockDim.x)
        if (base + k < n) out[base + k] += add;
}

__global__ void k_scan_total(const uint32_t *__restrict__ in, uint32_t *__restrict__ out, size_t n) {
    out[n] = n ? out[n - 1] + in[n - 1] : 0u;
}

// recursive exclusive scan; scratch is consumed as [bsum (nb) | bscan (nb + 1) | deeper]
cudaError_t scan_rec(const uint32_t *in, uint32_t *out, size_t n, uint32_t *scratch, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const size_t nb = cdiv(n, kScanBlock);
    uint32_t *bsum = scratch;
    uint32_t *bscan = scratch + nb;
    k_scan_block<<<(unsigned) nb, kScanThreads, 0, st>>>(in, out, n, bsum);
    if (nb > 1) {
        cudaError_t e = scan_rec(bsum, bscan, nb, scratch + 2 * nb + 1, st);
        if (e != cudaSuccess) return e;
        k_scan_add<<<(unsigned) nb, kScanThreads, 0, st>>>(out, n, bscan);
    }
    return cudaGetLastError();
}

__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const uint32_t *__restrict__ keys, size_t n, int shift,
                                                        uint32_t *__restrict__ hist, unsigned nblk) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0u;
    __syncthreads();
    const size_t base = (size_t) blockIdx.x * kRsTile;
    for (int k = threadIdx.x; k < kRsTile; k += kRsThreads)
        if (base + k < n) atomicAdd(&h[(keys[base + k] >> shift) & 255u], 1u);
    __syncthreads();
    hist[(size_t) threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const uint32_t *__restrict__ kin,
                                                           const uint32_t *__restrict__ vin,
                                                           uint32_t *__restrict__ kout, uint32_t *__restrict__ vout,
                                                           size_t n, int shift, const uint32_t *__restrict__ off,
                                                           unsigned nblk) {
    __shared__ uint32_t cnt[kRsWarps][256];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int d = lane; d < 256; d += 32) cnt[w][d] = 0u;
    __syncwarp();
    const uint32_t lt = (1u << lane) - 1u;
    const size_t base = (size_t) blockIdx.x * kRsTile + (size_t) w * (32 * kRsItems);
    uint32_t key[kRsItems], val[kRsItems], rank[kRsItems];
    int dig[kRsItems];
#pragma unroll
    for (int j = 0; j < kRsItems; ++j) {
        const size_t idx = base + (size_t) j * 32 + lane;
        const bool valid = idx < n;
        key[j] = valid ? kin[idx] : 0u;
        val[j] = valid ? vin[idx] : 0u;
        const int d = valid ? (int) ((key[j] >> shift) & 255u) : 256;
        dig[j] = d;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int leader = __ffs(peers) - 1;
        const uint32_t c0 = valid ? cnt[w][d] : 0u;
        __syncwarp();
        if (valid && lane == leader) cnt[w][d] = c0 + (uint32_t) __popc(peers);
        __syncwarp();
        rank[j] = c0 + (uint32_t) __popc(peers & lt);
    }
    __syncthreads();
    {
        // exclusive prefix over warps for digit threadIdx.x
        uint32_t run = 0u;
        const int d = threadIdx.x;
#pragma unroll
        for (int ww = 0; ww < kRsWarps; ++ww) {
            const uint32_t c = cnt[ww][d];
            cnt[ww][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kRsItems; ++j) {
        if (dig[j] < 256) {
            const uint32_t pos = off[(size_t) dig[j] * nblk + blockIdx.x] + cnt[w][dig[j]] + rank[j];
            kout[pos] = key[j];
            vout[pos] = val[j];
        }
    }
}

}  // namespace

size_t scan_scratch_bytes(size_t n) {
    size_t total = 0;
    while (n > 1) {
        const size_t nb = cdiv(n, kScanBlock);
        total += 2 * nb + 1;
        n = nb;
    }
    return (total + 64) * sizeof(uint32_t);
}

cudaError_t exclusive_scan_u32(const uint32_t *in, uint32_t *out, size_t n, void *scratch, cudaStream_t st) {
    cudaError_t e = scan_rec(in, out, n, static_cast<uint32_t *>(scratch), st);
    if (e != cudaSuccess) return e;
    k_scan_total<<<1, 1, 0, st>>>(in, out, n);
    return cudaGetLastError();
}

size_t radix_sort_scratch_bytes(size_t n) {
    const size_t nblk = cdiv(n ? n : 1, kRsTile);
    const size_t h = 256 * nblk;
    return (2 * h + 2) * sizeof(uint32_t) + scan_scratch_bytes(h) + 256;
}

cudaError_t radix_sort_pairs(uint32_t *keys, uint32_t *vals, uint32_t *keys_alt, uint32_t *vals_alt, size_t n,
                             int key_bits, void *scratch, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const unsigned nblk = (unsigned) cdiv(n, kRsTile);
    const size_t h = 256 * (size_t) nblk;
    uint32_t *hist = static_cast<uint32_t *>(scratch);
    uint32_t *off = hist + h + 1;
    void *sscr = off + h + 1;
    uint32_t *kin = keys, *vin = vals, *kout = keys_alt, *vout = vals_alt;
    int passes = 0;
    for (int shift = 0; shift < key_bits; shift += 8) {
        k_rs_hist<<<nblk, kRsThreads, 0, st>>>(kin, n, shift, hist, nblk);
        cudaError_t e = exclusive_scan_u32(hist, off, h, sscr, st);
        if (e != cudaSuccess) return e;
        k_rs_scatter<<<nblk, kRsThreads, 0, st>>>(kin, vin, kout, vout, n, shift, off, nblk);
        uint32_t *t = kin;
        kin = kout;
        kout = t;
        t = vin;
        vin = vout;
        vout = t;
        ++passes;
    }
    if (passes & 1) {
        cudaMemcpyAsync(keys, kin, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(vals, vin, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
    }
    return cudaGetLastError();
}

}  // namespace fitsne
