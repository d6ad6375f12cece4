// Exact kNN: FP32 candidate scan + FP64 re-rank with verification (see knn.cuh).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <chrono>
#include <string>
#include <vector>

#include "knn.cuh"
#include "knn_tc.cuh"

namespace fitsne {
namespace {

constexpr int kThreads = 256;
constexpr int kRefTile = 64;
constexpr int kDChunk = 64;
constexpr int kStride = kDChunk + 4;  // 17 float4 units per row: conflict-free 16-byte loads
constexpr int kSlack = 16;
constexpr int kTcSlack = 29;  // longer lists for the coarser tensor-core distances

__device__ __forceinline__ bool pair_gt(float a, uint32_t ia, float b, uint32_t ib) {
    return a > b || (a == b && ia > ib);
}
__device__ __forceinline__ bool pair_gt(double a, uint32_t ia, double b, uint32_t ib) {
    return a > b || (a == b && ia > ib);
}
// non-negative doubles by their bit patterns (the same order; integer compares instead of the
// FP64 pipe, whose warp instructions cost GB300 many cycles)
__device__ __forceinline__ bool pair_gt(unsigned long long a, uint32_t ia, unsigned long long b, uint32_t ib) {
    return a > b || (a == b && ia > ib);
}

// ascending bitonic sort of n (power of two) (key, index) pairs in shared memory by one warp
template <typename KT>
__device__ void warp_bitonic(KT *d, uint32_t *ix, int n) {
    const int lane = threadIdx.x & 31;
    for (int k = 2; k <= n; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < n; i += 32) {
                const int p = i ^ j;
                if (p > i) {
                    const bool up = (i & k) == 0;
                    const KT a = d[i], b = d[p];
                    const uint32_t ia = ix[i], ib = ix[p];
                    if (pair_gt(a, ia, b, ib) == up) {
                        d[i] = b;
                        d[p] = a;
                        ix[i] = ib;
                        ix[p] = ia;
                    }
                }
            }
            __syncwarp();
        }
}

// Candidate scan.  Block = QPC queries; the points stream through shared memory in tiles of
// 64; each query keeps up to CAP candidates (sorted and cut to C when the list fills).  With
// gridDim.y = S > 1 the points are cut into S segments of whole tiles, block (x, s) scans
// segment s and writes its C best at slot * S + s (k_cand_merge then keeps the C best of the
// S lists): a re-scan of a few rows then runs on S blocks instead of one.
template <int QPC, int CAP>
__global__ void __launch_bounds__(kThreads) k_knn_cand(const float *__restrict__ Xf, int N, int Dp, int C,
                                                       const int *__restrict__ qlist, int nq,
                                                       float *__restrict__ out_d, uint32_t *__restrict__ out_i) {
    constexpr int QPW = QPC / 8;  // queries per warp
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *qs = reinterpret_cast<float *>(smem_raw);      // [QPC][kStride]
    float *rs = qs + QPC * kStride;                        // [kRefTile][kStride]
    float *dt = rs + kRefTile * kStride;                   // [QPC][kRefTile + 1]
    float *cd = dt + QPC * (kRefTile + 1);                 // [QPC][CAP]
    uint32_t *ci = reinterpret_cast<uint32_t *>(cd + QPC * CAP);  // [QPC][CAP]
    __shared__ int cnt[QPC];
    __shared__ float thr[QPC];
    __shared__ int qid[QPC];

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid < QPC) {
        const int slot = blockIdx.x * QPC + tid;
        qid[tid] = slot < nq ? (qlist ? qlist[slot] : slot) : -1;
        cnt[tid] = 0;
        thr[tid] = FLT_MAX;
    }
    __syncthreads();
    const int nchunk = (Dp + kDChunk - 1) / kDChunk;
    const int qv = kDChunk / 4;  // float4 per chunk row

    auto load_queries = [&](int c0) {
        for (int e = tid; e < QPC * qv; e += kThreads) {
            const int q = e / qv, v = e % qv;
            const int dcol = c0 + 4 * v;
            float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
            if (qid[q] >= 0 && dcol < Dp) x = *reinterpret_cast<const float4 *>(Xf + (size_t) qid[q] * Dp + dcol);
            *reinterpret_cast<float4 *>(qs + q * kStride + 4 * v) = x;
        }
    };
    if (nchunk == 1) load_queries(0);
    const int S = (int) gridDim.y, seg = (int) blockIdx.y;
    const int rbeg = (int) ((long long) N * seg / S / kRefTile * kRefTile);
    const int rend = seg + 1 == S ? N : (int) ((long long) N * (seg + 1) / S / kRefTile * kRefTile);

    for (int r0 = rbeg; r0 < rend; r0 += kRefTile) {
        float acc[QPW][2];
#pragma unroll
        for (int a = 0; a < QPW; ++a) acc[a][0] = acc[a][1] = 0.f;
        for (int ch = 0; ch < nchunk; ++ch) {
            const int c0 = ch * kDChunk;
            if (nchunk > 1) load_queries(c0);
            for (int e = tid; e < kRefTile * qv; e += kThreads) {
                const int r = e / qv, v = e % qv;
                const int dcol = c0 + 4 * v;
                float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
                if (r0 + r < N && dcol < Dp) x = *reinterpret_cast<const float4 *>(Xf + (size_t) (r0 + r) * Dp + dcol);
                *reinterpret_cast<float4 *>(rs + r * kStride + 4 * v) = x;
            }
            __syncthreads();
            const int nv = min(qv, (Dp - c0 + 3) / 4);
            for (int v = 0; v < nv; ++v) {
                const float4 r0v = *reinterpret_cast<const float4 *>(rs + (2 * lane) * kStride + 4 * v);
                const float4 r1v = *reinterpret_cast<const float4 *>(rs + (2 * lane + 1) * kStride + 4 * v);
#pragma unroll
                for (int a = 0; a < QPW; ++a) {
                    const float4 q = *reinterpret_cast<const float4 *>(qs + (w * QPW + a) * kStride + 4 * v);
                    float t;
                    t = q.x - r0v.x; acc[a][0] = fmaf(t, t, acc[a][0]);
                    t = q.y - r0v.y; acc[a][0] = fmaf(t, t, acc[a][0]);
                    t = q.z - r0v.z; acc[a][0] = fmaf(t, t, acc[a][0]);
                    t = q.w - r0v.w; acc[a][0] = fmaf(t, t, acc[a][0]);
                    t = q.x - r1v.x; acc[a][1] = fmaf(t, t, acc[a][1]);
                    t = q.y - r1v.y; acc[a][1] = fmaf(t, t, acc[a][1]);
                    t = q.z - r1v.z; acc[a][1] = fmaf(t, t, acc[a][1]);
                    t = q.w - r1v.w; acc[a][1] = fmaf(t, t, acc[a][1]);
                }
            }
            __syncthreads();
        }
#pragma unroll
        for (int a = 0; a < QPW; ++a) {
            const int q = w * QPW + a;
            dt[q * (kRefTile + 1) + 2 * lane] = (r0 + 2 * lane < N) ? acc[a][0] : FLT_MAX;
            dt[q * (kRefTile + 1) + 2 * lane + 1] = (r0 + 2 * lane + 1 < N) ? acc[a][1] : FLT_MAX;
        }
        __syncwarp();
        // selection: the warp owns its QPW queries' lists
        const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
        for (int a = 0; a < QPW; ++a) {
            const int q = w * QPW + a;
            if (qid[q] < 0) continue;
            int n = cnt[q];
            const float th = thr[q];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int r = lane + 32 * h;
                const float d = dt[q * (kRefTile + 1) + r];
                const bool pass = (r0 + r < N) && (d < th);
                const unsigned m = __ballot_sync(0xffffffffu, pass);
                if (pass) {
                    const int pos = n + __popc(m & lt);
                    cd[q * CAP + pos] = d;
                    ci[q * CAP + pos] = (uint32_t) (r0 + r);
                }
                n += __popc(m);
            }
            __syncwarp();
            if (n > CAP - kRefTile) {
                for (int i = n + lane; i < CAP; i += 32) {
                    cd[q * CAP + i] = FLT_MAX;
                    ci[q * CAP + i] = 0xffffffffu;
                }
                __syncwarp();
                warp_bitonic<float>(cd + q * CAP, ci + q * CAP, CAP);
                if (n >= C) {
                    n = C;
                    if (lane == 0) thr[q] = cd[q * CAP + C - 1];
                }
            }
            if (lane == 0) cnt[q] = n;
            __syncwarp();
        }
        __syncthreads();
    }
    // final sort and write-out of the C best
#pragma unroll
    for (int a = 0; a < QPW; ++a) {
        const int q = w * QPW + a;
        if (qid[q] < 0) continue;
        const int n = cnt[q];
        for (int i = n + lane; i < CAP; i += 32) {
            cd[q * CAP + i] = FLT_MAX;
            ci[q * CAP + i] = 0xffffffffu;
        }
        __syncwarp();
        warp_bitonic<float>(cd + q * CAP, ci + q * CAP, CAP);
        const size_t slot = (size_t) (blockIdx.x * QPC + q) * S + seg;
        for (int i = lane; i < C; i += 32) {
            out_d[slot * C + i] = cd[q * CAP + i];
            out_i[slot * C + i] = ci[q * CAP + i];
        }
        __syncwarp();
    }
}

// The C best of a query's S segment lists (k_knn_cand with S segments): one block per query,
// the S x C (distance, index) pairs sorted in shared memory (P2 = the next power of two).
__global__ void __launch_bounds__(512) k_cand_merge(const float *__restrict__ seg_d,
                                                    const uint32_t *__restrict__ seg_i, int S, int C, int P2,
                                                    float *__restrict__ out_d, uint32_t *__restrict__ out_i) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *d = reinterpret_cast<float *>(smem_raw);
    uint32_t *ix = reinterpret_cast<uint32_t *>(d + P2);
    const size_t q = blockIdx.x;
    const int n = S * C;
    for (int e = threadIdx.x; e < P2; e += blockDim.x) {
        d[e] = e < n ? seg_d[q * n + e] : FLT_MAX;
        ix[e] = e < n ? seg_i[q * n + e] : 0xffffffffu;
    }
    __syncthreads();
    for (int k = 2; k <= P2; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P2; i += blockDim.x) {
                const int p = i ^ j;
                if (p > i) {
                    const bool up = (i & k) == 0;
                    const float a = d[i], b = d[p];
                    const uint32_t ia = ix[i], ib = ix[p];
                    if (pair_gt(a, ia, b, ib) == up) {
                        d[i] = b;
                        d[p] = a;
                        ix[i] = ib;
                        ix[p] = ia;
                    }
                }
            }
            __syncthreads();
        }
    for (int e = threadIdx.x; e < C; e += blockDim.x) {
        out_d[q * C + e] = d[e];
        out_i[q * C + e] = ix[e];
    }
}

// FP64 re-rank of the candidates of each query (one warp per query) + verification.
//
// The FP64 distances are the reference's (sequential sum of rounded squared differences, then
// the square root).  GB300's FP64 pipe charges each warp instruction whatever the lanes
// active, so the work goes by chunks of 32 candidates: a chunk whose candidates are all
// farther (by their approximate squared distances) than the K-th one plus twice the error
// bound of the approximation cannot hold one of the K nearest, and is not evaluated (its
// entries sort last).  The sort compares the non-negative distances as integers.
template <int CP>
__global__ void __launch_bounds__(128) k_knn_rerank(const double *__restrict__ Xd, int N, int D, int K, int C,
                                                    const int *__restrict__ qlist, int nq,
                                                    const float *__restrict__ cand_d,
                                                    const uint32_t *__restrict__ cand_i,
                                                    const double *__restrict__ norms, double maxnorm, int tc,
                                                    uint32_t *__restrict__ idx, double *__restrict__ dist,
                                                    int *__restrict__ flag) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double *ed = reinterpret_cast<double *>(smem_raw) + w * CP;
    uint32_t *ei = reinterpret_cast<uint32_t *>(reinterpret_cast<double *>(smem_raw) + 4 * CP) + w * CP;
    const int slot = blockIdx.x * 4 + w;
    if (slot >= nq) return;
    const int q = qlist ? qlist[slot] : slot;
    const double *xq = Xd + (size_t) q * D;
    // bound on |approximate - exact| squared distance of every candidate (all are at most the
    // C-th approximate one): the verification's below
    const double u = 5.9604644775390625e-08;  // 2^-24
    const double xn = norms[q];
    const double sC = (double) cand_d[(size_t) slot * C + C - 1];
    const double eps = tc ? 1.5 * (D + 4) * u * sC + 3e-5 * xn * maxnorm + 4e-6 * (xn * xn + maxnorm * maxnorm) + 1e-30
                          : 1.5 * ((D + 4) * u * sC + 4.0 * u * sqrt(sC) * (xn + maxnorm)) + 1e-30;
    const double cut = (double) cand_d[(size_t) slot * C + (K < C ? K : C) - 1] + 2.0 * eps;
    for (int c = lane; c < CP; c += 32) {
        double e = DBL_MAX;
        uint32_t j = 0xffffffffu;
        // the chunk is evaluated when one of its candidates may be among the K nearest
        const bool may = c < C && (c < K || (double) cand_d[(size_t) slot * C + c] <= cut);
        if (__any_sync(0xffffffffu, may) && c < C) {
            j = cand_i[(size_t) slot * C + c];
            if (j != 0xffffffffu) {
                const double *xj = Xd + (size_t) j * D;
                double dd = 0.0;
                for (int d = 0; d < D; ++d) {
                    const double f = __dsub_rn(xq[d], xj[d]);
                    dd = __dadd_rn(dd, __dmul_rn(f, f));
                }
                e = __dsqrt_rn(dd);
            }
        }
        ed[c] = e;
        ei[c] = j;
    }
    __syncwarp();
    warp_bitonic<unsigned long long>(reinterpret_cast<unsigned long long *>(ed), ei, CP);
    for (int k = lane; k < K; k += 32) {
        idx[(size_t) q * K + k] = ei[k];
        dist[(size_t) q * K + k] = ed[k];
    }
    if (lane == 0) {
        int ok = 1;
        if (C < N) {
            // every point outside the list has an approximate squared distance >= the C-th
            // one, sC; eps bounds the approximation: FP32 direct differences (SIMT scan) or
            // BF16 hi/lo tensor-core products (knn_tc.cuh)
            const double sK = ed[K - 1] * ed[K - 1];
            ok = (sK < sC - eps) ? 1 : 0;
        }
        flag[slot] = ok ? 0 : 1;
    }
}

__global__ void k_to_f32(const double *__restrict__ Xd, float *__restrict__ Xf, int N, int D, int Dp) {
    const size_t n = (size_t) N * Dp;
    for (size_t e = blockIdx.x * (size_t) blockDim.x + threadIdx.x; e < n; e += (size_t) gridDim.x * blockDim.x) {
        const size_t i = e / Dp;
        const int d = (int) (e % Dp);
        Xf[e] = d < D ? (float) Xd[i * D + d] : 0.f;
    }
}

__global__ void k_norms(const double *__restrict__ Xd, int N, int D, double *__restrict__ norms) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int d = 0; d < D; ++d) s += Xd[(size_t) i * D + d] * Xd[(size_t) i * D + d];
        norms[i] = sqrt(s);
    }
}

int cap_for(int C) {
    int cap = 128;
    while (cap < C + kRefTile) cap <<= 1;
    return cap;
}

size_t cand_smem(int qpc, int cap) {
    return sizeof(float) * ((size_t) qpc * kStride + kRefTile * kStride + qpc * (kRefTile + 1)) +
           (sizeof(float) + sizeof(uint32_t)) * (size_t) qpc * cap;
}

template <int QPC, int CAP>
cudaError_t launch_cand(const float *Xf, int N, int Dp, int C, const int *qlist, int nq, float *od, uint32_t *oi,
                        cudaStream_t st, int S) {
    const size_t sm = cand_smem(QPC, CAP);
    cudaError_t e = cudaFuncSetAttribute(k_knn_cand<QPC, CAP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sm);
    if (e != cudaSuccess) return e;
    const int blocks = (nq + QPC - 1) / QPC;
    k_knn_cand<QPC, CAP><<<dim3(blocks, S), kThreads, sm, st>>>(Xf, N, Dp, C, qlist, nq, od, oi);
    return cudaGetLastError();
}

// S > 1: S segment lists per query slot (od / oi hold nq x S x C entries)
cudaError_t dispatch_cand(int cap, const float *Xf, int N, int Dp, int C, const int *qlist, int nq, float *od,
                          uint32_t *oi, cudaStream_t st, int S = 1) {
    switch (cap) {
        case 128: return launch_cand<32, 128>(Xf, N, Dp, C, qlist, nq, od, oi, st, S);
        case 256: return launch_cand<32, 256>(Xf, N, Dp, C, qlist, nq, od, oi, st, S);
        case 512: return launch_cand<32, 512>(Xf, N, Dp, C, qlist, nq, od, oi, st, S);
        case 1024: return launch_cand<8, 1024>(Xf, N, Dp, C, qlist, nq, od, oi, st, S);
        case 2048: return launch_cand<8, 2048>(Xf, N, Dp, C, qlist, nq, od, oi, st, S);
        default: return cudaErrorInvalidValue;
    }
}

// segment count of a re-scan: 1 when the rows already fill the GPU's SMs; otherwise enough
// segments for two blocks per SM, at most 16, and S x C within the merge's shared memory (8,192
// pairs).  N = 1M: 3 rows re-scanned in 0.041 s instead of 0.131 s.
int rescan_segments(int cap, int C, int nq) {
    int dev = 0, nsm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int qpc = cap >= 1024 ? 8 : 32;
    const int blocks = (nq + qpc - 1) / qpc;
    if (blocks >= nsm) return 1;
    int S = (2 * nsm + blocks - 1) / blocks;
    S = std::min(S, 16);
    S = std::min(S, 8192 / std::max(C, 1));
    return std::max(S, 1);
}

cudaError_t launch_merge(const float *seg_d, const uint32_t *seg_i, int nq, int S, int C, float *od, uint32_t *oi,
                         cudaStream_t st) {
    int P2 = 1;
    while (P2 < S * C) P2 <<= 1;
    const size_t sm = (size_t) P2 * (sizeof(float) + sizeof(uint32_t));
    cudaError_t e = cudaFuncSetAttribute(k_cand_merge, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sm);
    if (e != cudaSuccess) return e;
    k_cand_merge<<<nq, 512, sm, st>>>(seg_d, seg_i, S, C, P2, od, oi);
    return cudaGetLastError();
}

template <int CP>
cudaError_t launch_rerank(const double *Xd, int N, int D, int K, int C, const int *qlist, int nq, const float *cd,
                          const uint32_t *ci, const double *norms, double maxnorm, int tc, uint32_t *idx,
                          double *dist, int *flag, cudaStream_t st) {
    const size_t sm = 4 * (size_t) CP * (sizeof(double) + sizeof(uint32_t));
    cudaError_t e = cudaFuncSetAttribute(k_knn_rerank<CP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sm);
    if (e != cudaSuccess) return e;
    k_knn_rerank<CP><<<(nq + 3) / 4, 128, sm, st>>>(Xd, N, D, K, C, qlist, nq, cd, ci, norms, maxnorm, tc, idx,
                                                     dist, flag);
    return cudaGetLastError();
}

cudaError_t dispatch_rerank(int cp, const double *Xd, int N, int D, int K, int C, const int *qlist, int nq,
                            const float *cd, const uint32_t *ci, const double *norms, double maxnorm, int tc,
                            uint32_t *idx, double *dist, int *flag, cudaStream_t st) {
    switch (cp) {
        case 128: return launch_rerank<128>(Xd, N, D, K, C, qlist, nq, cd, ci, norms, maxnorm, tc, idx, dist, flag, st);
        case 256: return launch_rerank<256>(Xd, N, D, K, C, qlist, nq, cd, ci, norms, maxnorm, tc, idx, dist, flag, st);
        case 512: return launch_rerank<512>(Xd, N, D, K, C, qlist, nq, cd, ci, norms, maxnorm, tc, idx, dist, flag, st);
        case 1024:
            return launch_rerank<1024>(Xd, N, D, K, C, qlist, nq, cd, ci, norms, maxnorm, tc, idx, dist, flag, st);
        case 2048:
            return launch_rerank<2048>(Xd, N, D, K, C, qlist, nq, cd, ci, norms, maxnorm, tc, idx, dist, flag, st);
        default: return cudaErrorInvalidValue;
    }
}

int pow2_at_least(int n) {
    int p = 128;
    while (p < n) p <<= 1;
    return p;
}

}  // namespace

void print_knn_stats(int K, const KnnStats &ks, double total_s) {
    char tot[32] = "";
    if (total_s >= 0) std::snprintf(tot, sizeof tot, "%.3f s, ", total_s);
    std::fprintf(stderr,
                 "[fitsne] kNN (K=%d, %s): %scandidates %.3f s, first pass %.3f s, rescans %.3f s, rows rescanned %d, "
                 "unverified %d",
                 K, ks.tensor_cores ? "tcgen05 candidates" : "FP32 candidates", tot, ks.s_candidates, ks.s_first_pass,
                 ks.s_rescans, ks.rows_rescanned, ks.rows_unverified);
    if (ks.tensor_cores)
        std::fprintf(stderr, ", locality order %.3f s, tile pairs computed %.1f%%, per query %.0f columns kept, %.0f inserts",
                     ks.tc.s_order, 100.0 * ks.tc.tiles_kept, ks.tc.cols_per_query, ks.tc.inserts_per_query);
    std::fprintf(stderr, "\n");
    if (ks.tensor_cores)
        std::fprintf(stderr,
                     "[fitsne] kNN tcgen05 pipeline (shares of each role's time): producer waiting for a stage "
                     "%.1f%%, MMA waiting for operands %.1f%% / for an accumulator %.1f%%, epilogue waiting for an "
                     "accumulator %.1f%%, in threshold stash and inserts %.1f%% (%.2f insert-loop iterations a tile, "
                     "%.0f cycles each)\n",
                     100.0 * ks.tc.producer_stage_wait, 100.0 * ks.tc.mma_data_wait, 100.0 * ks.tc.mma_acc_wait,
                     100.0 * ks.tc.epilogue_acc_wait, 100.0 * ks.tc.epilogue_inserts, ks.tc.insert_iters_per_tile,
                     ks.tc.cycles_per_insert_iter);
}

int knn_exact(const double *Xd, int N, int D, int K, uint32_t *idx, double *dist, cudaStream_t st, KnnStats *stats,
              const char **err, uint32_t *order_out, bool *order_written) {
    static thread_local std::string msg;
    auto fail = [&](const char *what, cudaError_t e) {
        msg = std::string(what) + ": " + cudaGetErrorString(e);
        if (err) *err = msg.c_str();
        return -10;
    };
    if (K < 1 || K > N) {
        msg = "K must be in [1, N]";
        if (err) *err = msg.c_str();
        return -3;
    }
    const int Dp = (D + 3) / 4 * 4;
    int C = K + kSlack;
    if (C > N) C = N;
    int cap = cap_for(C);
    if (cap > 2048) {
        msg = "too many neighbours requested for the on-chip candidate lists (K <= 1968)";
        if (err) *err = msg.c_str();
        return -3;
    }
    float *Xf = nullptr, *cd = nullptr;
    uint32_t *ci = nullptr;
    double *norms = nullptr;
    int *flag = nullptr, *qlist = nullptr;
    cudaError_t e;
#define KCK(x)                              \
    do {                                    \
        e = (x);                            \
        if (e != cudaSuccess) {             \
            cudaFree(Xf);                   \
            cudaFree(cd);                   \
            cudaFree(ci);                   \
            cudaFree(norms);                \
            cudaFree(flag);                 \
            cudaFree(qlist);                \
            return fail(#x, e);             \
        }                                   \
    } while (0)
    KCK(cudaMalloc(&Xf, sizeof(float) * (size_t) N * Dp));
    KCK(cudaMalloc(&norms, sizeof(double) * N));
    KCK(cudaMalloc(&flag, sizeof(int) * N));
    KCK(cudaMalloc(&qlist, sizeof(int) * N));
    k_to_f32<<<4096, 256, 0, st>>>(Xd, Xf, N, D, Dp);
    k_norms<<<(N + 255) / 256, 256, 0, st>>>(Xd, N, D, norms);
    std::vector<double> hn(N);
    KCK(cudaMemcpyAsync(hn.data(), norms, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
    KCK(cudaStreamSynchronize(st));
    double maxnorm = 0.0;
    for (double v : hn) maxnorm = v > maxnorm ? v : maxnorm;

    // first pass over all rows: tensor-core candidates where the device and the shape allow,
    // else the FP32 scan; both are verified by the FP64 re-rank
    const auto clk0 = std::chrono::steady_clock::now();
    auto secs = [&clk0]() { return std::chrono::duration<double>(std::chrono::steady_clock::now() - clk0).count(); };
    const char *mode = std::getenv("FITSNE_KNN");
    const bool force_simt = mode && std::string(mode) == "simt";
    int slack = kTcSlack;  // FITSNE_KNN_SLACK overrides it
    if (const char *es = std::getenv("FITSNE_KNN_SLACK")) slack = std::max(0, std::atoi(es));
    const int Ctc = K + slack < N ? K + slack : N;
    const bool use_tc = !force_simt && N >= 256 && knn_tc_supported(D, Ctc);
    if (use_tc) {
        C = Ctc;
        cap = cap_for(C);
        KCK(cudaMalloc(&cd, sizeof(float) * (size_t) N * C));
        KCK(cudaMalloc(&ci, sizeof(uint32_t) * (size_t) N * C));
        std::string terr;
        if (knn_candidates_tc(Xd, N, D, C, maxnorm, cd, ci, st, stats ? &stats->tc : nullptr, terr, order_out,
                              order_written) != 0) {
            msg = terr;
            if (err) *err = msg.c_str();
            cudaFree(Xf);
            cudaFree(cd);
            cudaFree(ci);
            cudaFree(norms);
            cudaFree(flag);
            cudaFree(qlist);
            return -10;
        }
        if (stats) stats->s_candidates = secs();
        KCK(dispatch_rerank(pow2_at_least(C), Xd, N, D, K, C, nullptr, N, cd, ci, norms, maxnorm, 1, idx, dist, flag,
                            st));
    } else {
        KCK(cudaMalloc(&cd, sizeof(float) * (size_t) N * C));
        KCK(cudaMalloc(&ci, sizeof(uint32_t) * (size_t) N * C));
        KCK(dispatch_cand(cap, Xf, N, Dp, C, nullptr, N, cd, ci, st));
        KCK(dispatch_rerank(pow2_at_least(C), Xd, N, D, K, C, nullptr, N, cd, ci, norms, maxnorm, 0, idx, dist, flag,
                            st));
    }
    if (stats) stats->tensor_cores = use_tc;
    std::vector<int> hf(N);
    KCK(cudaMemcpyAsync(hf.data(), flag, sizeof(int) * N, cudaMemcpyDeviceToHost, st));
    KCK(cudaStreamSynchronize(st));
    std::vector<int> bad;
    for (int i = 0; i < N; ++i)
        if (hf[i]) bad.push_back(i);
    if (stats) stats->rows_rescanned = (int) bad.size();
    const double s_first = secs();
    if (stats) stats->s_first_pass = s_first;
    // rescans of the unverified rows with longer lists
    while (!bad.empty() && C < N && cap < 2048) {
        C = C * 4 < N ? C * 4 : N;
        if (cap_for(C) > 2048) C = 2048 - kRefTile < N ? 2048 - kRefTile : N;
        cap = cap_for(C);
        const int nq = (int) bad.size();
        cudaFree(cd);
        cudaFree(ci);
        cd = nullptr;
        ci = nullptr;
        KCK(cudaMalloc(&cd, sizeof(float) * (size_t) nq * C));
        KCK(cudaMalloc(&ci, sizeof(uint32_t) * (size_t) nq * C));
        KCK(cudaMemcpyAsync(qlist, bad.data(), sizeof(int) * nq, cudaMemcpyHostToDevice, st));
        // few rows: the points in segments over several blocks, then the lists merged
        const int S = rescan_segments(cap, C, nq);
        if (S > 1) {
            float *sd = nullptr;
            uint32_t *si = nullptr;
            KCK(cudaMalloc(&sd, sizeof(float) * (size_t) nq * S * C));
            cudaError_t e2 = cudaMalloc(&si, sizeof(uint32_t) * (size_t) nq * S * C);
            if (e2 == cudaSuccess) e2 = dispatch_cand(cap, Xf, N, Dp, C, qlist, nq, sd, si, st, S);
            if (e2 == cudaSuccess) e2 = launch_merge(sd, si, nq, S, C, cd, ci, st);
            if (e2 == cudaSuccess) e2 = cudaStreamSynchronize(st);
            cudaFree(sd);
            cudaFree(si);
            KCK(e2);
        } else {
            KCK(dispatch_cand(cap, Xf, N, Dp, C, qlist, nq, cd, ci, st));
        }
        KCK(dispatch_rerank(pow2_at_least(C), Xd, N, D, K, C, qlist, nq, cd, ci, norms, maxnorm, 0, idx, dist, flag,
                            st));
        std::vector<int> f2(nq);
        KCK(cudaMemcpyAsync(f2.data(), flag, sizeof(int) * nq, cudaMemcpyDeviceToHost, st));
        KCK(cudaStreamSynchronize(st));
        std::vector<int> still;
        for (int k = 0; k < nq; ++k)
            if (f2[k]) still.push_back(bad[k]);
        bad.swap(still);
    }
    if (stats) {
        stats->rows_unverified = (int) bad.size();
        stats->s_rescans = secs() - s_first;
    }
#undef KCK
    cudaFree(Xf);
    cudaFree(cd);
    cudaFree(ci);
    cudaFree(norms);
    cudaFree(flag);
    cudaFree(qlist);
    return 0;
}

}  // namespace fitsne
