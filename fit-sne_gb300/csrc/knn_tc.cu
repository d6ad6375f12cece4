// Tensor-core candidate search for the exact kNN (tcgen05 / TMEM / TMA, sm_103a).
//
// Squared distance d2(q, r) = |q|^2 - 2 acc(q, r) with acc = q.r - |r|^2 / 2 from the
// 5th-generation tensor cores.  X is split into two BF16 planes, hi = bf16(x) and
// lo = bf16(x - hi), and q.r ~ q_hi.r_hi + q_hi.r_lo + q_lo.r_hi (three BF16 products into
// one FP32 accumulator, relative error about 3 * 2^-18 of |q||r|).  The reference-side term
// -|r|^2 / 2 rides in two spare K columns (D and D + 1): the query planes hold 1 there, the
// reference planes three BF16 pieces of -|r|^2 / 2 (about 24 bits), so that the epilogue
// needs one FMA and one compare per candidate.  The candidates are then re-ranked in FP64
// and verified by knn.cu, exactly as the FP32 candidates of the SIMT scan are.
//
// One persistent CTA per SM, 6 warps:
//   warp 0      TMA producer: query tile (128 x 64, hi + lo) once per query tile, then the
//               reference tiles (64 x 64, hi + lo) through a 3-stage shared-memory ring;
//               128-byte swizzled tiles, completion through mbarrier transaction counts.
//               Tiles go superblock by superblock (SBT tiles each), nearest superblock first
//               by the lower bound of their bounding spheres (the query tile's own first), so
//               that the C-th distances, and with them the thresholds, drop early.  The lanes
//               test 32 tiles at a time against those thresholds (published by the epilogue)
//               and skip the tiles that cannot hold a candidate; the walk ends at the first
//               superblock too far away, and an end-marker stage (tile index -1) closes the
//               query tile
//   warp 1      allocates 256 TMEM columns (a ring of four 128 x 64 FP32 accumulators, so
//               that the MMAs run up to four tiles ahead of the epilogue) and issues the
//               tcgen05.mma (M = 128, N = 64, K = 16) from one thread; tcgen05.commit
//               releases the shared-memory stage and hands the accumulator to the epilogue
//   warps 2..5  epilogue: one tcgen05.ld of the whole 64-column tile for their 32 TMEM lanes
//               (= 32 queries), after which the accumulator is handed back to the MMA warp;
//               threshold test into per-thread bit masks (four independent chains per 32
//               columns); when a lane of the warp keeps a column, that 32-column half of the
//               tile goes to a shared-memory stash and every lane walks its own mask: the
//               columns below its threshold go to its row's queue, and the queues go into the
//               per-query 4-ary max-heaps of the C best (shared memory, knn_heap.cuh)
//               together, when one of them would overflow, so the lanes' heap updates run
//               side by side and overlap the next MMAs
// Every mbarrier wait gives up after about a second, sets an error flag, and the CTA
// drains its own in-flight work, frees TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include <cfloat>
#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <string>

#include "knn_heap.cuh"
#include "knn_tc.cuh"
#include "sort.cuh"

namespace fitsne {
namespace {

constexpr int BM = 128;      // queries per tile (MMA M)
constexpr int BN = 64;       // reference points per tile (MMA N)
constexpr int KD = 64;       // padded dimension (4 MMA K-steps of 16), D + 2 <= KD
constexpr int kThreads = 192;
constexpr int kBoxRows = 64;                       // rows per TMA box (both operands)
constexpr int kBoxBytes = kBoxRows * KD * 2;       // 8 KB
constexpr int kATileBytes = BM * KD * 2;           // 16 KB per plane
constexpr int kBTileBytes = BN * KD * 2;           // 8 KB per plane
constexpr int kStages = 3;
constexpr int kMaxSB = 1024;                       // superblocks per query tile's ordering
constexpr uint32_t kSbMask = kMaxSB - 1;
constexpr int kAccs = 4;                           // TMEM accumulators in the MMA -> epilogue ring
constexpr int kTmemCols = kAccs * BN;
constexpr int kStashOff = 2 * kATileBytes + kStages * 2 * kBTileBytes;  // 80 KB
constexpr int kStashCols = 32;  // columns of a tile stashed at a time: one half
constexpr int kHeapOff = kStashOff + kStashCols * BM * 4;               // + 16 KB stash
// candidates queued per query row between heap flushes (13 with 16-column stashes measured
// slower: a flush comes when any lane's queue fills, so longer queues save few flush rounds)
constexpr int kQueue = 5;
constexpr int kQueueOff = kHeapOff + kMaxTcCandidates * BM * 8;          // + 120 KB heaps
constexpr size_t kSmemBytes = (size_t) kQueueOff + (size_t) kQueue * BM * 8 + 1024;  // + 5 KB queues
constexpr long long kWaitCycles = 2000000000LL;  // about one second
// counters: kept tiles, columns past the threshold test, heap inserts, producer cycles waiting
// for a free stage, producer cycles, MMA cycles waiting for data, MMA cycles waiting for an
// accumulator, epilogue cycles waiting for an accumulator, epilogue cycles in the threshold
// stash and inserts, epilogue cycles, insert-loop iterations (warp level), tiles (per warp)
constexpr int kNumCounters = 12;
// with the kernel's 4.5 KB of static shared memory, within the 227 KB a block may use
static_assert(kSmemBytes + 4608 <= 232448, "shared memory budget");
static_assert(kMaxTcCandidates <= 341, "Heap4::replace_top covers four levels of children");

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t) __cvta_generic_to_shared(p); }

// ascending bitonic sort of n (a power of two, >= 32) keys in shared memory by one warp
__device__ void warp_sort_u32(uint32_t *k, int n) {
    const int lane = threadIdx.x & 31;
    for (int size = 2; size <= n; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = lane; i < n; i += 32) {
                const int p = i ^ stride;
                if (p > i) {
                    const uint32_t a = k[i], b = k[p];
                    if ((a > b) == ((i & size) == 0)) {
                        k[i] = b;
                        k[p] = a;
                    }
                }
            }
            __syncwarp();
        }
}

// K-major operand tile with 128-byte swizzle: rows 128 B apart, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t) ((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t) 1 << 16;
    d |= (uint64_t) ((1024u >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t) 1 << 46;
    d |= (uint64_t) 2 << 61;
    return d;
}

// kind::f16 instruction descriptor: FP32 accumulate, BF16 A and B, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t) (N >> 3) << 17) | ((uint32_t) (M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t addr, uint32_t parity) {
    uint32_t done;
    asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                 : "=r"(done) : "r"(addr), "r"(parity) : "memory");
    return done != 0;
}

// bounded wait; returns false (and raises the CTA abort flag) after ~1 s
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag) {
    const uint32_t addr = smem_u32(bar);
    const long long t0 = clock64();
    while (true) {
        if (mbar_try(addr, parity)) return true;
        if (*abort_flag) return false;
        if (clock64() - t0 > kWaitCycles) {
            *abort_flag = 1;
            return false;
        }
    }
}

// bounded wait that ignores the abort flag (used to drain in-flight work before exit); the
// phase waited for always completes, so running out of time marks a protocol fault
__device__ __forceinline__ void mbar_drain(uint64_t *bar, uint32_t parity, volatile int *abort) {
    const uint32_t addr = smem_u32(bar);
    const long long t0 = clock64();
    while (!mbar_try(addr, parity)) {
        if (clock64() - t0 > kWaitCycles) {
            *abort = 1;
            return;
        }
    }
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"((uint64_t) map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
    asm volatile("{ .reg .pred p; setp.ne.u32 p, %4, 0; tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p; }"
                 ::"r"(tmem_d), "l"(da), "l"(db), "r"(idesc), "r"(acc) : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 64 consecutive columns of this warp's 32 lanes; the wait is part of the statement
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, uint32_t (&r)[64]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
        "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,"
        "%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]),
          "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]),
          "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]),
          "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]),
          "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
        : "r"(taddr)
        : "memory");
}

__global__ void __launch_bounds__(kThreads, 1)
    k_knn_tc(const __grid_constant__ CUtensorMap map_qhi, const __grid_constant__ CUtensorMap map_qlo,
             const __grid_constant__ CUtensorMap map_rhi, const __grid_constant__ CUtensorMap map_rlo,
             const float *__restrict__ qnorm2, int N, int Npad, int D, int C, int SBT,
             const uint32_t *__restrict__ perm, const float *__restrict__ rcentT,
             const float *__restrict__ rrad, const float *__restrict__ sbcentT, const float *__restrict__ sbrad,
             const float *__restrict__ qcentT, const float *__restrict__ qrad, float errm, float *__restrict__ out_d, uint32_t *__restrict__ out_i, int *__restrict__ err,
             unsigned long long *__restrict__ counters) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t bar_a_full, bar_a_empty, bar_done;
    __shared__ __align__(8) uint64_t bar_b_full[kStages], bar_b_empty[kStages];
    __shared__ __align__(8) uint64_t bar_acc_full[kAccs], bar_acc_empty[kAccs];
    __shared__ uint32_t tmem_base;
    __shared__ volatile int abort_flag;
    // reference tile of each stage / accumulator (-1: end of the query tile)
    __shared__ volatile int stage_tile[kStages];
    __shared__ volatile int acc_tile[kAccs];
    // per epilogue warp: (query-tile sequence number << 32) | bits of its largest threshold
    __shared__ volatile unsigned long long warp_thr[4];
    __shared__ float qc_s[KD];  // producer: centre of the current query tile
    __shared__ uint32_t sb_key[kMaxSB];  // producer: the superblocks, nearest first

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t raw = smem_u32(smem_raw);
    uint8_t *base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    uint8_t *sA_hi = base;
    uint8_t *sA_lo = base + kATileBytes;
    uint8_t *sB = base + 2 * kATileBytes;  // stage s: hi at s*2*kBTileBytes, lo after it
    float *stash = reinterpret_cast<float *>(base + kStashOff);  // [kStashCols columns][BM rows]
    HeapEntry *heaps = reinterpret_cast<HeapEntry *>(base + kHeapOff);  // entry e of row r at e*BM + r
    HeapEntry *queues = reinterpret_cast<HeapEntry *>(base + kQueueOff);  // entry k of row r at k*BM + r

    const int nQT = Npad / BM;
    const int nRT = Npad / BN;
    const int nSB = (nRT + SBT - 1) / SBT;

    if (tid == 0) {
        abort_flag = 0;
        mbar_init(&bar_a_full, 1);
        mbar_init(&bar_a_empty, 1);
        mbar_init(&bar_done, 1);
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&bar_b_full[s], 1);
            mbar_init(&bar_b_empty[s], 1);
        }
        for (int b = 0; b < kAccs; ++b) {
            mbar_init(&bar_acc_full[b], 2);  // the MMA commit + the issuer's release of acc_tile
            mbar_init(&bar_acc_empty[b], 4);
        }
        for (int w = 0; w < 4; ++w) warp_thr[w] = ~0ull;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;

    if (warp == 0) {
        // ---------------- producer (whole warp: lanes share the tile-bound arithmetic) ----------
        int j = 0;
        bool ok = true;
        int last_a = -1;
        long long g = 0;  // stages filled so far (tiles and end markers)
        long long last_g[kStages];
        for (int s = 0; s < kStages; ++s) last_g[s] = -1;
        unsigned long long kept = 0, t_stage_wait = 0;
        const long long t_begin = clock64();
        for (int qt = blockIdx.x; qt < nQT && ok; qt += gridDim.x, ++j) {
            if (lane == 0) {
                ok = mbar_wait(&bar_a_empty, (j & 1) ^ 1, &abort_flag);
                if (ok) {
                    mbar_expect_tx(&bar_a_full, 2 * kATileBytes);
                    for (int h = 0; h < BM / kBoxRows; ++h) {
                        tma_load_2d(sA_hi + h * kBoxBytes, &map_qhi, 0, qt * BM + h * kBoxRows, &bar_a_full);
                        tma_load_2d(sA_lo + h * kBoxBytes, &map_qlo, 0, qt * BM + h * kBoxRows, &bar_a_full);
                    }
                    last_a = j;
                }
            }
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) break;
            // bounding sphere of this query tile (centre in shared memory for the lanes' loops)
            __syncwarp();
            qc_s[lane] = qcentT[(size_t) lane * nQT + qt];
            qc_s[lane + 32] = qcentT[(size_t) (lane + 32) * nQT + qt];
            __syncwarp();
            const float rq = qrad[qt];
            // lower bound on d^2 between the query tile's sphere and a sphere (centre t of
            // centT, radius rr), less nothing: the callers subtract the error bound of the split
            // distances
            auto lower_bound2 = [&](const float *__restrict__ centT, int ntiles, int t, float rr) {
                float dd = 0.f;
#pragma unroll 8
                for (int d = 0; d < D; ++d) {
                    const float e = qc_s[d] - centT[(size_t) d * ntiles + t];
                    dd = fmaf(e, e, dd);
                }
                const float lb = fmaxf(0.f, sqrtf(dd) * (1.f - 1e-5f) - rq - rr);
                return lb * lb * (1.f - 1e-5f);
            };
            // the largest current threshold of the tile's 128 queries (published by the epilogue
            // warps, tagged with this query tile); FLT_MAX until every list holds C candidates
            auto threshold = [&]() {
                float thr = FLT_MAX;
                if (lane == 0) {
                    for (int w = 0; w < 4; ++w) {
                        const unsigned long long v = warp_thr[w];
                        const float tv = (int) (v >> 32) == j ? __uint_as_float((uint32_t) v) : FLT_MAX;
                        thr = w == 0 ? tv : fmaxf(thr, tv);
                    }
                }
                return __shfl_sync(0xffffffffu, thr, 0);
            };
            auto issue = [&](int rt) {  // rt = -1: the end marker of this query tile
                const int s = (int) (g % kStages);
                const uint32_t ph = (uint32_t) ((g / kStages) & 1);
                if (lane == 0) {
                    const long long tw = clock64();
                    ok = mbar_wait(&bar_b_empty[s], ph ^ 1, &abort_flag);
                    t_stage_wait += (unsigned long long) (clock64() - tw);
                    if (ok) {
                        stage_tile[s] = rt;
                        // the stage's latest phase (a copy or a marker): the final drain waits on
                        // its parity, which a later phase of the same barrier would invert
                        last_g[s] = g;
                        if (rt >= 0) {
                            mbar_expect_tx(&bar_b_full[s], 2 * kBTileBytes);
                            uint8_t *dst = sB + (size_t) s * 2 * kBTileBytes;
                            tma_load_2d(dst, &map_rhi, 0, rt * BN, &bar_b_full[s]);
                            tma_load_2d(dst + kBTileBytes, &map_rlo, 0, rt * BN, &bar_b_full[s]);
                        } else {
                            mbar_arrive(&bar_b_full[s]);  // end marker: no data
                        }
                    }
                }
                ok = __shfl_sync(0xffffffffu, ok, 0);
                ++g;
            };
            // superblocks (SBT tiles each) nearest first: key = the truncated lower bound (low
            // log2(kMaxSB) bits cleared, so never above the bound) | index distance from the
            // query tile's own superblock, which comes first with bound 0
            const int t0 = qt * (BM / BN);
            const int sbq = t0 / SBT, rot = t0 - sbq * SBT;
            int nsp = 32;
            while (nsp < nSB) nsp <<= 1;
            __syncwarp();
            for (int i = lane; i < nsp; i += 32) {
                uint32_t key = 0xffffffffu;
                if (i < nSB) {
                    const int sb = sbq + i < nSB ? sbq + i : sbq + i - nSB;
                    const float sr = sbrad[sb];
                    if (sr >= 0.f) key = (__float_as_uint(lower_bound2(sbcentT, nSB, sb, sr)) & ~kSbMask) | (uint32_t) i;
                }
                sb_key[i] = key;
            }
            __syncwarp();
            warp_sort_u32(sb_key, nsp);
            for (int k = 0; k < nSB && ok; ++k) {
                const uint32_t key = sb_key[k];
                if (key == 0xffffffffu) break;  // empty superblocks sort last
                // a superblock is skipped when no point of it can enter any query's list; the
                // thresholds only fall, so every later (farther) superblock is skipped as well
                const float thr = threshold();
                if (thr < FLT_MAX && __uint_as_float(key & ~kSbMask) - errm > thr) break;
                const int i = (int) (key & kSbMask);
                const int sbk = sbq + i < nSB ? sbq + i : sbq + i - nSB;
                const int r = sbk == sbq ? rot : 0;  // own superblock: the query tile's rows first
                for (int c = 0; c < SBT && ok; c += 32) {
                    const int rt = sbk * SBT + ((c + lane + r) & (SBT - 1));
                    const int rtc = rt < nRT ? rt : nRT - 1;
                    const float rr = rt < nRT ? rrad[rtc] : -1.f;
                    const float thr_t = threshold();
                    const bool keep =
                        rr >= 0.f && !(thr_t < FLT_MAX && lower_bound2(rcentT, nRT, rtc, rr) - errm > thr_t);
                    uint32_t tmask = __ballot_sync(0xffffffffu, keep);
                    while (tmask && ok) {
                        const int tl = __ffs(tmask) - 1;
                        tmask &= tmask - 1;
                        ++kept;
                        issue(sbk * SBT + ((c + tl + r) & (SBT - 1)));
                    }
                }
            }
            if (ok) issue(-1);
        }
        // every copy this warp issued has landed before the CTA may exit
        if (lane == 0) {
            if (last_a >= 0) mbar_drain(&bar_a_full, (uint32_t) (last_a & 1), &abort_flag);
            for (int s = 0; s < kStages; ++s)
                if (last_g[s] >= 0) mbar_drain(&bar_b_full[s], (uint32_t) ((last_g[s] / kStages) & 1), &abort_flag);
            atomicAdd(&counters[0], kept);
            atomicAdd(&counters[3], t_stage_wait);
            atomicAdd(&counters[4], (unsigned long long) (clock64() - t_begin));
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---------------- MMA issuer ----------------
            const uint32_t idesc = idesc_bf16(BM, BN);
            int j = 0;
            bool ok = true;
            long long g = 0, a = 0;  // stages consumed, accumulators handed over
            unsigned long long t_data = 0, t_acc = 0;
            for (int qt = blockIdx.x; qt < nQT && ok; qt += gridDim.x, ++j) {
                if (!(ok = mbar_wait(&bar_a_full, j & 1, &abort_flag))) break;
                while (true) {
                    const int s = (int) (g % kStages);
                    const uint32_t ph = (uint32_t) ((g / kStages) & 1);
                    const int b = (int) (a % kAccs);
                    const uint32_t phb = (uint32_t) ((a / kAccs) & 1);
                    const long long t0 = clock64();
                    if (!(ok = mbar_wait(&bar_b_full[s], ph, &abort_flag))) break;
                    const long long t1 = clock64();
                    if (!(ok = mbar_wait(&bar_acc_empty[b], phb ^ 1, &abort_flag))) break;
                    t_data += (unsigned long long) (t1 - t0);
                    t_acc += (unsigned long long) (clock64() - t1);
                    const int rt = stage_tile[s];
                    acc_tile[b] = rt;
                    if (rt >= 0) {
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        const uint32_t acc = tmem + (uint32_t) (b * BN);
                        const uint32_t a_hi = smem_u32(sA_hi), a_lo = smem_u32(sA_lo);
                        const uint32_t b_hi = smem_u32(sB + (size_t) s * 2 * kBTileBytes), b_lo = b_hi + kBTileBytes;
                        // hi.hi + hi.lo + lo.hi
                        const uint32_t As[3] = {a_hi, a_hi, a_lo};
                        const uint32_t Bs[3] = {b_hi, b_lo, b_hi};
#pragma unroll
                        for (int p = 0; p < 3; ++p)
#pragma unroll
                            for (int ks = 0; ks < KD / 16; ++ks)
                                mma_bf16(acc, desc_sw128(As[p] + ks * 32), desc_sw128(Bs[p] + ks * 32), idesc,
                                         (p | ks) ? 1u : 0u);
                        mma_commit(&bar_b_empty[s]);
                    } else {
                        mbar_arrive(&bar_b_empty[s]);
                    }
                    mma_commit(&bar_acc_full[b]);
                    mbar_arrive(&bar_acc_full[b]);  // releases acc_tile[b]
                    ++g;
                    ++a;
                    if (rt < 0) break;
                }
                if (ok) mma_commit(&bar_a_empty);
            }
            atomicAdd(&counters[5], t_data);
            atomicAdd(&counters[6], t_acc);
            // all issued MMAs retire before TMEM is released
            mma_commit(&bar_done);
            mbar_drain(&bar_done, 0u, &abort_flag);
        }
    } else {
        // ---------------- epilogue: warps 2..5 ----------------
        const int quarter = warp & 3;  // TMEM lanes this warp may read
        const int row = quarter * 32 + lane;
        const Heap4<BM> hp{heaps + row};
        float *my_stash = stash + row;
        HeapEntry *my_queue = queues + row;
        int j = 0;
        bool ok = true;
        long long a = 0;  // accumulators received
        unsigned ncols = 0, nins = 0;  // columns through the threshold test, heap insertions
        unsigned long long t_wait = 0, t_ins = 0, n_iter = 0, n_tiles = 0;
        const long long t_begin = clock64();
        for (int qt = blockIdx.x; qt < nQT && ok; qt += gridDim.x, ++j) {
            const int q = qt * BM + row;
            const bool qvalid = q < N;
            const float nq = qvalid ? qnorm2[q] : 0.f;
            int n = 0;
            float thr = qvalid ? FLT_MAX : -FLT_MAX;  // rows past N keep nothing
            int qn = 0;  // queued candidates of this row
            // one candidate into the row's heap (thr: the heap's top once it holds C)
            auto insert = [&](float d2, uint32_t col) {
                if (d2 < thr) {
                    ++nins;
                    if (n < C) {
                        hp.push(n, d2, col);
                        if (n == C) thr = hp.top();
                    } else {
                        hp.replace_top(n, d2, col);
                        thr = hp.top();
                    }
                }
            };
            // every row's queued candidates into its heap, the warp's lanes side by side
            auto flush = [&]() {
                const int m = (int) __reduce_max_sync(0xffffffffu, (unsigned) qn);
                n_iter += (unsigned long long) m;
                for (int k = 0; k < m; ++k)
                    if (k < qn) {
                        const HeapEntry e = my_queue[k * BM];
                        insert(e.d, e.i);
                    }
                qn = 0;
            };
            while (true) {
                const int b = (int) (a % kAccs);
                const uint32_t phb = (uint32_t) ((a / kAccs) & 1);
                ++a;
                // warp-uniform outcome: the TMEM loads below need all 32 lanes
                const long long tacc = clock64();
                if (!(ok = __all_sync(0xffffffffu, mbar_wait(&bar_acc_full[b], phb, &abort_flag)))) break;
                t_wait += (unsigned long long) (clock64() - tacc);
                const int rt = acc_tile[b];
                if (rt < 0) {  // end of this query tile
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&bar_acc_empty[b]);
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t tbase = tmem + ((uint32_t) (quarter * 32) << 16) + (uint32_t) (b * BN);
                // the whole 64-column tile in one load; the accumulator goes back to the MMA
                // warp at once, so the next MMAs overlap this tile's threshold test and inserts
                uint32_t v[BN];
                tmem_ld64(tbase, v);
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(&bar_acc_empty[b]);
                const int tilebase = rt * BN;
                const int nvalid = N - tilebase;
                // the test d2 = nq - 2 acc < thr in accumulator form, acc > (nq - thr) / 2, with
                // the bound lowered by a margin above both roundings: the masks keep every
                // column the exact test at the insert keeps (rows past N: none; lists not yet
                // full: all)
                float vt;
                if (!qvalid) {
                    vt = __int_as_float(0x7f800000);
                } else if (thr >= FLT_MAX) {
                    vt = -__int_as_float(0x7f800000);
                } else {
                    vt = 0.5f * (nq - thr) - (fabsf(nq) + fabsf(thr)) * 2.384185791015625e-07f;
                }
                // kept-candidate masks, built in four independent chains per 32 columns
                uint32_t mk[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    uint32_t q0 = 0, q1 = 0, q2 = 0, q3 = 0;
#pragma unroll
                    for (int jj = 0; jj < 32; jj += 4) {
                        q0 |= (__uint_as_float(v[32 * h + jj]) > vt) ? (1u << jj) : 0u;
                        q1 |= (__uint_as_float(v[32 * h + jj + 1]) > vt) ? (2u << jj) : 0u;
                        q2 |= (__uint_as_float(v[32 * h + jj + 2]) > vt) ? (4u << jj) : 0u;
                        q3 |= (__uint_as_float(v[32 * h + jj + 3]) > vt) ? (8u << jj) : 0u;
                    }
                    const int nv = nvalid - 32 * h;
                    const uint32_t lim = nv >= 32 ? 0xffffffffu : (nv <= 0 ? 0u : ((1u << nv) - 1u));
                    mk[h] = ((q0 | q1) | (q2 | q3)) & lim;
                }
                const long long ti = clock64();
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    uint32_t mask = mk[h];
                    if (__any_sync(0xffffffffu, mask != 0u)) {
                        // stash the columns (entry jj of row r at jj*BM + r: conflict-free), then each
                        // lane walks its own kept columns
#pragma unroll
                        for (int jj = 0; jj < kStashCols; ++jj)
                            my_stash[jj * BM] = __uint_as_float(v[kStashCols * h + jj]);
                        const int colbase = tilebase + kStashCols * h;
                        const int pc = __popc(mask);
                        // a heap insert is a chain of dependent shared-memory round trips that the
                        // warp runs once per kept column of its busiest lane; so the candidates that
                        // pass the threshold are queued per row, and the queues go into the heaps
                        // together when one of them would overflow (the threshold lags until then,
                        // which only queues more candidates: each is tested again at the flush)
                        if (__any_sync(0xffffffffu, qn + pc > kQueue)) flush();
                        if (__any_sync(0xffffffffu, pc > kQueue)) {
                            // more kept columns than a queue holds (lists still filling): straight in
                            n_iter += (unsigned long long) __reduce_max_sync(0xffffffffu, (unsigned) pc);
                            while (mask) {
                                const int jj = __ffs(mask) - 1;
                                mask &= mask - 1;
                                ++ncols;
                                insert(fmaf(-2.f, my_stash[jj * BM], nq), (uint32_t) (colbase + jj));
                            }
                        } else {
                            while (mask) {
                                const int jj = __ffs(mask) - 1;
                                mask &= mask - 1;
                                ++ncols;
                                const float d2 = fmaf(-2.f, my_stash[jj * BM], nq);
                                if (d2 < thr) {
                                    my_queue[qn * BM] = HeapEntry{d2, (uint32_t) (colbase + jj)};
                                    ++qn;
                                }
                            }
                        }
                        __syncwarp();
                    }
                }
                t_ins += (unsigned long long) (clock64() - ti);
                ++n_tiles;
                // publish this warp's largest threshold for the producer's tile skipping
                const uint32_t tw = __reduce_max_sync(0xffffffffu, __float_as_uint(fmaxf(thr, 0.f)));
                if (lane == 0) warp_thr[quarter] = ((unsigned long long) (uint32_t) j << 32) | tw;
            }
            if (!ok) break;
            flush();
            if (qvalid) {
                hp.sort_ascending(n);
                // rows and indices back to the caller's numbering
                const size_t orow = (size_t) (perm ? perm[q] : (uint32_t) q) * C;
                for (int e = 0; e < C; ++e) {
                    const HeapEntry en = hp.at(e);
                    out_d[orow + e] = e < n ? en.d : FLT_MAX;
                    out_i[orow + e] = e < n ? (perm ? perm[en.i] : en.i) : 0xffffffffu;
                }
            }
        }
        const unsigned cs = __reduce_add_sync(0xffffffffu, ncols), is = __reduce_add_sync(0xffffffffu, nins);
        if (lane == 0) {
            atomicAdd(&counters[1], (unsigned long long) cs);
            atomicAdd(&counters[2], (unsigned long long) is);
            atomicAdd(&counters[7], t_wait);
            atomicAdd(&counters[8], t_ins);
            atomicAdd(&counters[9], (unsigned long long) (clock64() - t_begin));
            atomicAdd(&counters[10], n_iter);
            atomicAdd(&counters[11], n_tiles);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
    if (tid == 0 && abort_flag) atomicExch(err, 1);
}

// Query planes (hi, lo; 1 in columns D and D + 1 of hi), reference planes (hi, lo; three
// BF16 pieces of -|x|^2 / 2 in columns D and D + 1) and FP32 |x|^2.  One warp per row; row i
// is point perm[i] (i without perm); rows N .. Npad-1 are zero.
__global__ void k_tc_prep(const double *__restrict__ X, const uint32_t *__restrict__ perm, int N, int D, int Npad,
                          __nv_bfloat16 *__restrict__ qhi,
                          __nv_bfloat16 *__restrict__ qlo, __nv_bfloat16 *__restrict__ rhi,
                          __nv_bfloat16 *__restrict__ rlo, float *__restrict__ qnorm2) {
    const int lane = threadIdx.x & 31;
    const int gw = (int) ((blockIdx.x * (size_t) blockDim.x + threadIdx.x) >> 5);
    const int nw = (int) ((gridDim.x * (size_t) blockDim.x) >> 5);
    const __nv_bfloat16 zero = __float2bfloat16(0.f), one = __float2bfloat16(1.f);
    for (int i = gw; i < Npad; i += nw) {
        double x[KD / 32];
        double s = 0.0;
#pragma unroll
        for (int h = 0; h < KD / 32; ++h) {
            const int d = lane + 32 * h;
            x[h] = (i < N && d < D) ? X[(size_t) (perm ? perm[i] : (uint32_t) i) * D + d] : 0.0;
            s += x[h] * x[h];
        }
        for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        const double v = -0.5 * s;
        const __nv_bfloat16 p1 = __double2bfloat16(v);
        const double r1 = v - (double) __bfloat162float(p1);
        const __nv_bfloat16 p2 = __double2bfloat16(r1);
        const __nv_bfloat16 p3 = __double2bfloat16(r1 - (double) __bfloat162float(p2));
        const bool live = i < N;
#pragma unroll
        for (int h = 0; h < KD / 32; ++h) {
            const int d = lane + 32 * h;
            const size_t e = (size_t) i * KD + d;
            __nv_bfloat16 a_hi = __double2bfloat16(x[h]);
            __nv_bfloat16 a_lo = __double2bfloat16(x[h] - (double) __bfloat162float(a_hi));
            __nv_bfloat16 b_hi = a_hi, b_lo = a_lo;
            if (d == D) {
                a_hi = live ? one : zero;
                a_lo = zero;
                b_hi = live ? p1 : zero;
                b_lo = live ? p2 : zero;
            } else if (d == D + 1) {
                a_hi = live ? one : zero;
                a_lo = zero;
                b_hi = live ? p3 : zero;
                b_lo = zero;
            }
            qhi[e] = a_hi;
            qlo[e] = a_lo;
            rhi[e] = b_hi;
            rlo[e] = b_lo;
        }
        if (lane == 0) qnorm2[i] = (float) s;
    }
}

// Bounding sphere of each tile of `rows` consecutive rows (row r = point perm[r]): centre (FP64 mean, stored as
// FP32, transposed: dimension d of tile t at centT[d * ntiles + t], so that lanes testing
// consecutive tiles load consecutive words) and radius about that stored centre (FP64,
// rounded up to FP32); radius -1 for a tile without any of the N points.  256 threads:
// 4 row groups x 64 dimensions for the mean.
__global__ void __launch_bounds__(256) k_tile_bounds(const double *__restrict__ X, const uint32_t *__restrict__ perm,
                                                     int N, int D, int rows, int ntiles,
                                                     float *__restrict__ centT, float *__restrict__ rad) {
    __shared__ double part[4][KD];
    __shared__ float cs[KD];
    __shared__ double red[256];
    const int t = blockIdx.x;
    if (t >= ntiles) return;
    const int r0 = t * rows, r1 = min(N, r0 + rows);
    const int grp = threadIdx.x / KD, d = threadIdx.x % KD;
    double sum = 0.0;
    if (d < D)
        for (int r = r0 + grp; r < r1; r += 4) sum += X[(size_t) (perm ? perm[r] : (uint32_t) r) * D + d];
    part[grp][d] = sum;
    __syncthreads();
    if (threadIdx.x < KD) {
        const double tot = (part[0][d] + part[1][d]) + (part[2][d] + part[3][d]);
        const float c = (r1 > r0 && d < D) ? (float) (tot / (r1 - r0)) : 0.f;
        cs[d] = c;
        centT[(size_t) d * ntiles + t] = c;
    }
    __syncthreads();
    double m = 0.0;
    for (int r = r0 + (int) threadIdx.x; r < r1; r += blockDim.x) {
        const double *x = X + (size_t) (perm ? perm[r] : (uint32_t) r) * D;
        double s2 = 0.0;
        for (int e = 0; e < D; ++e) {
            const double f = x[e] - (double) cs[e];
            s2 += f * f;
        }
        m = fmax(m, s2);
    }
    red[threadIdx.x] = m;
    __syncthreads();
    for (int o = blockDim.x / 2; o; o >>= 1) {
        if ((int) threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) rad[t] = r1 > r0 ? __double2float_ru(sqrt(red[0]) * (1.0 + 1e-6) + 1e-12) : -1.f;
}

// Locality order of the points for the tile skipping: P pivots (evenly spaced rows of X),
// each point in the cell of its nearest pivot (FP32 scores |c|^2 - 2 x.c), cells grouped by
// the nearest of kSuperPivots super-pivots (evenly spaced pivots), then a stable sort by
// (group, cell).  Any order gives the same lists; this one makes consecutive rows close.
constexpr int kSuperPivots = 32;
constexpr int kOrderMinN = 16384;  // below this the order is left as it is
constexpr int kPivChunk = 32;

__global__ void k_pivot_rows(const double *__restrict__ X, int N, int D, int P, float *__restrict__ piv,
                             float *__restrict__ pn) {
    const int p = blockIdx.x;
    if (p >= P) return;
    const size_t row = (size_t) ((long long) p * N / P);
    float s = 0.f;
    for (int d = threadIdx.x; d < KD; d += blockDim.x) {
        const float c = d < D ? (float) X[row * D + d] : 0.f;
        piv[(size_t) p * KD + d] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int d = 0; d < D; ++d) s = fmaf(piv[(size_t) p * KD + d], piv[(size_t) p * KD + d], s);
        pn[p] = s;
    }
}

// nearest of P pivots (rows of piv, KD floats, zero-padded) for n points (row i at pts + i*ld)
template <typename T>
__global__ void __launch_bounds__(256) k_nearest_pivot(const T *__restrict__ pts, int ld, int n, int D,
                                                       const float *__restrict__ piv, const float *__restrict__ pn,
                                                       int P, uint32_t *__restrict__ out) {
    __shared__ float cs[kPivChunk][KD];
    __shared__ float cn[kPivChunk];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float x[KD];
#pragma unroll
    for (int d = 0; d < KD; ++d) x[d] = (i < n && d < D) ? (float) pts[(size_t) i * ld + d] : 0.f;
    float best = FLT_MAX;
    uint32_t arg = 0;
    for (int p0 = 0; p0 < P; p0 += kPivChunk) {
        __syncthreads();
        for (int e = threadIdx.x; e < kPivChunk * KD; e += blockDim.x) {
            const int pp = p0 + e / KD;
            cs[e / KD][e % KD] = pp < P ? piv[(size_t) pp * KD + e % KD] : 0.f;
        }
        if (threadIdx.x < kPivChunk) cn[threadIdx.x] = p0 + (int) threadIdx.x < P ? pn[p0 + threadIdx.x] : FLT_MAX;
        __syncthreads();
        for (int pp = 0; pp < kPivChunk; ++pp) {
            float dot = 0.f;
#pragma unroll
            for (int d = 0; d < KD; ++d) dot = fmaf(x[d], cs[pp][d], dot);
            const float sc = fmaf(-2.f, dot, cn[pp]);
            if (sc < best) {
                best = sc;
                arg = (uint32_t) (p0 + pp);
            }
        }
    }
    if (i < n) out[i] = arg;
}

__global__ void k_cell_keys(const uint32_t *__restrict__ cell, const uint32_t *__restrict__ group, int N, int P,
                            uint32_t *__restrict__ keys, uint32_t *__restrict__ ids) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const uint32_t c = cell[i];
        keys[i] = group[c] * (uint32_t) P + c;
        ids[i] = (uint32_t) i;
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

// rows of KD BF16 values (128 B), boxes of kBoxRows rows, 128-byte swizzle
bool make_map(CUtensorMap *map, void *ptr, int Npad) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {(cuuint64_t) KD, (cuuint64_t) Npad};
    const cuuint64_t strides[1] = {(cuuint64_t) KD * 2};
    const cuuint32_t box[2] = {(cuuint32_t) KD, (cuuint32_t) kBoxRows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, ptr, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

bool knn_tc_supported(int D, int C) {
    static int avail = -1;
    if (avail < 0) {
        int dev = 0, major = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
        avail = (major == 10 && encode_fn() != nullptr) ? 1 : 0;
    }
    return avail == 1 && D >= 1 && D + 2 <= KD && C >= 1 && C <= kMaxTcCandidates;
}

int knn_order_mode() {
    const char *e = std::getenv("FITSNE_KNN_ORDER");
    return (e && std::string(e) == "input") ? 0 : 1;
}

namespace {

// perm[r] = the point at row r of the locality order (see k_nearest_pivot)
int locality_order(const double *Xd, int N, int D, uint32_t *perm, cudaStream_t st, std::string &err) {
    int P = 16;
    while (P < 2048 && P * 1024 < N) P <<= 1;
    const int S = kSuperPivots;
    int bits = 1;
    while ((1LL << bits) < (long long) S * P) ++bits;
    float *fbuf = nullptr;
    uint32_t *ubuf = nullptr;
    void *scratch = nullptr;
    auto cleanup = [&]() {
        cudaFree(fbuf);
        cudaFree(ubuf);
        cudaFree(scratch);
    };
    cudaError_t e;
    const size_t scr = radix_sort_scratch_bytes((size_t) N);
    if ((e = cudaMalloc(&fbuf, sizeof(float) * (size_t) (P + S) * (KD + 1))) != cudaSuccess ||
        (e = cudaMalloc(&ubuf, sizeof(uint32_t) * ((size_t) 4 * N + P))) != cudaSuccess ||
        (e = cudaMalloc(&scratch, scr)) != cudaSuccess) {
        err = std::string("knn order allocation: ") + cudaGetErrorString(e);
        cleanup();
        return -10;
    }
    float *piv = fbuf, *spiv = piv + (size_t) P * KD, *pn = spiv + (size_t) S * KD, *spn = pn + P;
    uint32_t *cell = ubuf, *keys = cell + N, *kalt = keys + N, *valt = kalt + N, *group = valt + N;
    k_pivot_rows<<<P, 64, 0, st>>>(Xd, N, D, P, piv, pn);
    k_pivot_rows<<<S, 64, 0, st>>>(Xd, N, D, S, spiv, spn);
    k_nearest_pivot<float><<<(P + 255) / 256, 256, 0, st>>>(piv, KD, P, D, spiv, spn, S, group);
    k_nearest_pivot<double><<<(N + 255) / 256, 256, 0, st>>>(Xd, D, N, D, piv, pn, P, cell);
    k_cell_keys<<<1024, 256, 0, st>>>(cell, group, N, P, keys, perm);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = radix_sort_pairs(keys, perm, kalt, valt, (size_t) N, bits, scratch, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the buffers are freed below
    cleanup();
    if (e != cudaSuccess) {
        err = std::string("knn order: ") + cudaGetErrorString(e);
        return -10;
    }
    return 0;
}

}  // namespace

int data_locality_order(const double *Xd, int N, int D, uint32_t *order, cudaStream_t st, std::string &err) {
    static_assert(kDataOrderMaxD == KD, "the pivot kernels read KD coordinates");
    return locality_order(Xd, N, D, order, st, err);
}

int knn_candidates_tc(const double *Xd, int N, int D, int C, double maxnorm, float *cand_d, uint32_t *cand_i,
                      cudaStream_t st, KnnTcStats *stats, std::string &err, uint32_t *order_out,
                      bool *order_written) {
    const int Npad = (N + BM - 1) / BM * BM;
    const size_t plane = (size_t) Npad * KD;
    const int nQT = Npad / BM, nRT = Npad / BN;
    __nv_bfloat16 *planes = nullptr;
    float *qn = nullptr, *bounds = nullptr;
    int *derr = nullptr;
    unsigned long long *dcount = nullptr;  // tiles computed, columns kept, heap insertions
    uint32_t *perm = nullptr;
    auto cleanup = [&]() {
        cudaFree(planes);
        cudaFree(qn);
        cudaFree(bounds);
        cudaFree(derr);
        cudaFree(dcount);
        cudaFree(perm);
    };
    cudaError_t e;
    // superblocks of SBT tiles (a power of two >= 32): at most kMaxSB of them
    int SBT = 32;
    while ((nRT + SBT - 1) / SBT > kMaxSB) SBT <<= 1;
    const int nSB = (nRT + SBT - 1) / SBT;
    if (knn_order_mode() == 1 && N >= kOrderMinN) {
        if ((e = cudaMalloc(&perm, sizeof(uint32_t) * N)) != cudaSuccess) {
            err = std::string("knn tc allocation: ") + cudaGetErrorString(e);
            return -10;
        }
        const auto t0 = std::chrono::steady_clock::now();
        const int rc = locality_order(Xd, N, D, perm, st, err);
        if (stats) stats->s_order = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (rc) {
            cleanup();
            return rc;
        }
        if (order_out) {
            if ((e = cudaMemcpyAsync(order_out, perm, sizeof(uint32_t) * N, cudaMemcpyDeviceToDevice, st)) !=
                cudaSuccess) {
                err = std::string("knn order copy: ") + cudaGetErrorString(e);
                cleanup();
                return -10;
            }
            if (order_written) *order_written = true;
        }
    }
    const size_t nb = (size_t) (nQT + nRT + nSB) * (KD + 1);
    if ((e = cudaMalloc(&planes, sizeof(__nv_bfloat16) * plane * 4)) != cudaSuccess ||
        (e = cudaMalloc(&qn, sizeof(float) * Npad)) != cudaSuccess ||
        (e = cudaMalloc(&bounds, sizeof(float) * nb)) != cudaSuccess ||
        (e = cudaMalloc(&derr, sizeof(int))) != cudaSuccess ||
        (e = cudaMalloc(&dcount, kNumCounters * sizeof(unsigned long long))) != cudaSuccess) {
        err = std::string("knn tc allocation: ") + cudaGetErrorString(e);
        cleanup();
        return -10;
    }
    __nv_bfloat16 *qhi = planes, *qlo = planes + plane, *rhi = planes + 2 * plane, *rlo = planes + 3 * plane;
    float *rcent = bounds, *qcent = rcent + (size_t) nRT * KD, *sbcent = qcent + (size_t) nQT * KD;
    float *rrad = sbcent + (size_t) nSB * KD, *qrad = rrad + nRT, *sbrad = qrad + nQT;
    cudaMemsetAsync(derr, 0, sizeof(int), st);
    cudaMemsetAsync(dcount, 0, kNumCounters * sizeof(unsigned long long), st);
    k_tc_prep<<<2048, 256, 0, st>>>(Xd, perm, N, D, Npad, qhi, qlo, rhi, rlo, qn);
    k_tile_bounds<<<nRT, 256, 0, st>>>(Xd, perm, N, D, BN, nRT, rcent, rrad);
    k_tile_bounds<<<nQT, 256, 0, st>>>(Xd, perm, N, D, BM, nQT, qcent, qrad);
    k_tile_bounds<<<nSB, 256, 0, st>>>(Xd, perm, N, D, BN * SBT, nSB, sbcent, sbrad);
    // approximate and exact squared distances differ by at most 3e-5 |x||y| + 4e-6 (|x|^2 + |y|^2)
    // + 1.5 (D + 4) 2^-24 d^2 (the verification's bound); the first terms are below 4e-5 M^2
    const float errm = (float) (4e-5 * maxnorm * maxnorm) + 1e-30f;
    CUtensorMap m_qhi, m_qlo, m_rhi, m_rlo;
    if (!make_map(&m_qhi, qhi, Npad) || !make_map(&m_qlo, qlo, Npad) || !make_map(&m_rhi, rhi, Npad) ||
        !make_map(&m_rlo, rlo, Npad)) {
        err = "cuTensorMapEncodeTiled failed";
        cleanup();
        return -10;
    }
    if ((e = cudaFuncSetAttribute(k_knn_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) kSmemBytes)) !=
        cudaSuccess) {
        err = std::string("knn tc smem: ") + cudaGetErrorString(e);
        cleanup();
        return -10;
    }
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int grid = nQT < nsm ? nQT : nsm;
    k_knn_tc<<<grid, kThreads, kSmemBytes, st>>>(m_qhi, m_qlo, m_rhi, m_rlo, qn, N, Npad, D, C, SBT, perm, rcent, rrad, sbcent, sbrad,
                                                 qcent, qrad, errm, cand_d, cand_i, derr, dcount);
    int herr = 0;
    unsigned long long hc[kNumCounters] = {};
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hc, dcount, sizeof(hc), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (stats) {
        stats->tiles_kept = (double) hc[0] / ((double) nQT * nRT);
        stats->cols_per_query = (double) hc[1] / N;
        stats->inserts_per_query = (double) hc[2] / N;
        // shares of each role's own clock: the producer's (one warp per CTA), the MMA
        // issuer's (one thread), the epilogue's (four warps)
        const double tp = hc[4] > 0 ? (double) hc[4] : 1.0, te = hc[9] > 0 ? (double) hc[9] : 1.0;
        stats->producer_stage_wait = (double) hc[3] / tp;
        stats->mma_data_wait = (double) hc[5] / tp;
        stats->mma_acc_wait = (double) hc[6] / tp;
        stats->epilogue_acc_wait = (double) hc[7] / te;
        stats->epilogue_inserts = (double) hc[8] / te;
        stats->insert_iters_per_tile = hc[11] > 0 ? (double) hc[10] / (double) hc[11] : 0.0;
        stats->cycles_per_insert_iter = hc[10] > 0 ? (double) hc[8] / (double) hc[10] : 0.0;
    }
    cleanup();
    if (e != cudaSuccess) {
        err = std::string("knn tc kernel: ") + cudaGetErrorString(e);
        return -10;
    }
    if (herr) {
        err = "knn tc kernel: a pipeline wait timed out";
        return -10;
    }
    return 0;
}

}  // namespace fitsne
