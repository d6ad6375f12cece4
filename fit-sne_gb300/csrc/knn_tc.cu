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
//               reference tiles (64 x 64, hi + lo) through a 3-stage shared-memory ring,
//               starting at the query tile's own rows (index neighbours first: on data with
//               any locality in its order the C-th distance, and with it the threshold,
//               drops within the first tiles); 128-byte swizzled tiles, completion through
//               mbarrier transaction counts
//   warp 1      allocates 128 TMEM columns (two 128 x 64 FP32 accumulators) and issues
//               the tcgen05.mma (M = 128, N = 64, K = 16) from one thread; tcgen05.commit
//               releases the shared-memory stage and hands the accumulator to the epilogue
//   warps 2..5  epilogue: one tcgen05.ld of the whole 64-column tile for their 32 TMEM lanes
//               (= 32 queries), after which the accumulator is handed back to the MMA warp;
//               threshold test into per-thread bit masks (four independent chains per 32
//               columns); when a lane of the warp keeps a column, the 32-column half goes to
//               a shared-memory stash and every lane walks its own mask into its per-query
//               max-heap of the C best (shared memory), so the lanes' heap updates run side by
//               side and overlap the next MMAs
// Every mbarrier wait gives up after about a second, sets an error flag, and the CTA
// drains its own in-flight work, frees TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>

#include <cfloat>
#include <cstdint>
#include <string>

#include "knn_tc.cuh"

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
constexpr int kTmemCols = 2 * BN;                  // two accumulators
constexpr int kStashOff = 2 * kATileBytes + kStages * 2 * kBTileBytes;  // 80 KB
constexpr int kHeapOff = kStashOff + 32 * BM * 4;                       // + 16 KB stash
constexpr size_t kSmemBytes = (size_t) kHeapOff + (size_t) kMaxTcCandidates * BM * 8 + 1024;
constexpr long long kWaitCycles = 2000000000LL;  // about one second
static_assert(kSmemBytes <= 232448, "shared memory budget");

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t) __cvta_generic_to_shared(p); }

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

// bounded wait that ignores the abort flag (used to drain in-flight work before exit)
__device__ __forceinline__ void mbar_drain(uint64_t *bar, uint32_t parity) {
    const uint32_t addr = smem_u32(bar);
    const long long t0 = clock64();
    while (!mbar_try(addr, parity) && clock64() - t0 <= kWaitCycles) {
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

// per-thread max-heap of (distance, index) in shared memory, entry e of row `r` at e*BM + r
struct Heap {
    float *d;
    uint32_t *ix;
    int r;
    __device__ __forceinline__ float &D(int e) { return d[e * BM + r]; }
    __device__ __forceinline__ uint32_t &I(int e) { return ix[e * BM + r]; }
    __device__ void push(int &n, float v, uint32_t id) {
        int pos = n++;
        while (pos > 0) {
            const int par = (pos - 1) >> 1;
            if (D(par) >= v) break;
            D(pos) = D(par);
            I(pos) = I(par);
            pos = par;
        }
        D(pos) = v;
        I(pos) = id;
    }
    __device__ void sift_down(int n, int pos, float v, uint32_t id) {
        while (true) {
            const int l = 2 * pos + 1;
            if (l >= n) break;
            const int rr = l + 1;
            const int m = (rr < n && D(rr) > D(l)) ? rr : l;
            if (D(m) <= v) break;
            D(pos) = D(m);
            I(pos) = I(m);
            pos = m;
        }
        D(pos) = v;
        I(pos) = id;
    }
};

__global__ void __launch_bounds__(kThreads, 1)
    k_knn_tc(const __grid_constant__ CUtensorMap map_qhi, const __grid_constant__ CUtensorMap map_qlo,
             const __grid_constant__ CUtensorMap map_rhi, const __grid_constant__ CUtensorMap map_rlo,
             const float *__restrict__ qnorm2, int N, int Npad, int C, float *__restrict__ out_d,
             uint32_t *__restrict__ out_i, int *__restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t bar_a_full, bar_a_empty, bar_done;
    __shared__ __align__(8) uint64_t bar_b_full[kStages], bar_b_empty[kStages];
    __shared__ __align__(8) uint64_t bar_acc_full[2], bar_acc_empty[2];
    __shared__ uint32_t tmem_base;
    __shared__ volatile int abort_flag;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t raw = smem_u32(smem_raw);
    uint8_t *base = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    uint8_t *sA_hi = base;
    uint8_t *sA_lo = base + kATileBytes;
    uint8_t *sB = base + 2 * kATileBytes;  // stage s: hi at s*2*kBTileBytes, lo after it
    float *stash = reinterpret_cast<float *>(base + kStashOff);  // [32 columns][BM rows]
    float *heap_d = reinterpret_cast<float *>(base + kHeapOff);
    uint32_t *heap_i = reinterpret_cast<uint32_t *>(base + kHeapOff + (size_t) kMaxTcCandidates * BM * 4);

    const int nQT = Npad / BM;
    const int nRT = Npad / BN;

    if (tid == 0) {
        abort_flag = 0;
        mbar_init(&bar_a_full, 1);
        mbar_init(&bar_a_empty, 1);
        mbar_init(&bar_done, 1);
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&bar_b_full[s], 1);
            mbar_init(&bar_b_empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&bar_acc_full[b], 1);
            mbar_init(&bar_acc_empty[b], 4);
        }
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
        if (lane == 0) {
            // ---------------- producer ----------------
            int j = 0;
            bool ok = true;
            int last_a = -1;
            long long last_g[kStages];
            for (int s = 0; s < kStages; ++s) last_g[s] = -1;
            for (int qt = blockIdx.x; qt < nQT && ok; qt += gridDim.x, ++j) {
                if (!(ok = mbar_wait(&bar_a_empty, (j & 1) ^ 1, &abort_flag))) break;
                mbar_expect_tx(&bar_a_full, 2 * kATileBytes);
                for (int h = 0; h < BM / kBoxRows; ++h) {
                    tma_load_2d(sA_hi + h * kBoxBytes, &map_qhi, 0, qt * BM + h * kBoxRows, &bar_a_full);
                    tma_load_2d(sA_lo + h * kBoxBytes, &map_qlo, 0, qt * BM + h * kBoxRows, &bar_a_full);
                }
                last_a = j;
                const int t0 = qt * (BM / BN);
                for (int t = 0; t < nRT; ++t) {
                    const long long g = (long long) j * nRT + t;
                    const int s = (int) (g % kStages);
                    const uint32_t ph = (uint32_t) ((g / kStages) & 1);
                    const int rt = (t0 + t) % nRT;
                    if (!(ok = mbar_wait(&bar_b_empty[s], ph ^ 1, &abort_flag))) break;
                    mbar_expect_tx(&bar_b_full[s], 2 * kBTileBytes);
                    uint8_t *dst = sB + (size_t) s * 2 * kBTileBytes;
                    tma_load_2d(dst, &map_rhi, 0, rt * BN, &bar_b_full[s]);
                    tma_load_2d(dst + kBTileBytes, &map_rlo, 0, rt * BN, &bar_b_full[s]);
                    last_g[s] = g;
                }
            }
            // every copy this thread issued has landed before the CTA may exit
            if (last_a >= 0) mbar_drain(&bar_a_full, (uint32_t) (last_a & 1));
            for (int s = 0; s < kStages; ++s)
                if (last_g[s] >= 0) mbar_drain(&bar_b_full[s], (uint32_t) ((last_g[s] / kStages) & 1));
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---------------- MMA issuer ----------------
            const uint32_t idesc = idesc_bf16(BM, BN);
            int j = 0;
            bool ok = true;
            for (int qt = blockIdx.x; qt < nQT && ok; qt += gridDim.x, ++j) {
                if (!(ok = mbar_wait(&bar_a_full, j & 1, &abort_flag))) break;
                for (int t = 0; t < nRT; ++t) {
                    const long long g = (long long) j * nRT + t;
                    const int s = (int) (g % kStages);
                    const uint32_t ph = (uint32_t) ((g / kStages) & 1);
                    const int b = (int) (g & 1);
                    const uint32_t phb = (uint32_t) ((g >> 1) & 1);
                    if (!(ok = mbar_wait(&bar_b_full[s], ph, &abort_flag))) break;
                    if (!(ok = mbar_wait(&bar_acc_empty[b], phb ^ 1, &abort_flag))) break;
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
                    mma_commit(&bar_acc_full[b]);
                }
                if (ok) mma_commit(&bar_a_empty);
            }
            // all issued MMAs retire before TMEM is released
            mma_commit(&bar_done);
            mbar_drain(&bar_done, 0u);
        }
    } else {
        // ---------------- epilogue: warps 2..5 ----------------
        const int quarter = warp & 3;  // TMEM lanes this warp may read
        const int row = quarter * 32 + lane;
        Heap hp{heap_d, heap_i, row};
        float *my_stash = stash + row;
        int j = 0;
        bool ok = true;
        for (int qt = blockIdx.x; qt < nQT && ok; qt += gridDim.x, ++j) {
            const int q = qt * BM + row;
            const bool qvalid = q < N;
            const float nq = qvalid ? qnorm2[q] : 0.f;
            int n = 0;
            float thr = qvalid ? FLT_MAX : -FLT_MAX;  // rows past N keep nothing
            const int t0 = qt * (BM / BN);
            for (int t = 0; t < nRT; ++t) {
                const long long g = (long long) j * nRT + t;
                const int b = (int) (g & 1);
                const uint32_t phb = (uint32_t) ((g >> 1) & 1);
                // warp-uniform outcome: the TMEM loads below need all 32 lanes
                if (!(ok = __all_sync(0xffffffffu, mbar_wait(&bar_acc_full[b], phb, &abort_flag)))) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t tbase = tmem + ((uint32_t) (quarter * 32) << 16) + (uint32_t) (b * BN);
                // the whole 64-column tile in one load; the accumulator goes back to the MMA
                // warp at once, so the next MMAs overlap this tile's threshold test and inserts
                uint32_t v[BN];
                tmem_ld64(tbase, v);
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(&bar_acc_empty[b]);
                const int tilebase = ((t0 + t) % nRT) * BN;
                const int nvalid = N - tilebase;
                // kept-candidate masks, built in four independent chains per 32 columns
                uint32_t mk[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    uint32_t q0 = 0, q1 = 0, q2 = 0, q3 = 0;
#pragma unroll
                    for (int jj = 0; jj < 32; jj += 4) {
                        q0 |= (fmaf(-2.f, __uint_as_float(v[32 * h + jj]), nq) < thr) ? (1u << jj) : 0u;
                        q1 |= (fmaf(-2.f, __uint_as_float(v[32 * h + jj + 1]), nq) < thr) ? (2u << jj) : 0u;
                        q2 |= (fmaf(-2.f, __uint_as_float(v[32 * h + jj + 2]), nq) < thr) ? (4u << jj) : 0u;
                        q3 |= (fmaf(-2.f, __uint_as_float(v[32 * h + jj + 3]), nq) < thr) ? (8u << jj) : 0u;
                    }
                    const int nv = nvalid - 32 * h;
                    const uint32_t lim = nv >= 32 ? 0xffffffffu : (nv <= 0 ? 0u : ((1u << nv) - 1u));
                    mk[h] = ((q0 | q1) | (q2 | q3)) & lim;
                }
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    uint32_t mask = mk[h];
                    if (__any_sync(0xffffffffu, mask != 0u)) {
                        // stash the half (entry jj of row r at jj*BM + r: conflict-free), then each
                        // lane inserts its own kept columns
#pragma unroll
                        for (int jj = 0; jj < 32; ++jj) my_stash[jj * BM] = __uint_as_float(v[32 * h + jj]);
                        const int colbase = tilebase + 32 * h;
                        while (mask) {
                            const int jj = __ffs(mask) - 1;
                            mask &= mask - 1;
                            const float d2 = fmaf(-2.f, my_stash[jj * BM], nq);
                            if (d2 < thr) {
                                if (n < C) {
                                    hp.push(n, d2, (uint32_t) (colbase + jj));
                                    if (n == C) thr = hp.D(0);
                                } else {
                                    hp.sift_down(n, 0, d2, (uint32_t) (colbase + jj));
                                    thr = hp.D(0);
                                }
                            }
                        }
                        __syncwarp();
                    }
                }
            }
            if (!ok) break;
            if (qvalid) {
                // heap sort ascending and write the list
                for (int end = n - 1; end > 0; --end) {
                    const float dv = hp.D(end);
                    const uint32_t iv = hp.I(end);
                    hp.D(end) = hp.D(0);
                    hp.I(end) = hp.I(0);
                    hp.sift_down(end, 0, dv, iv);
                }
                for (int e = 0; e < C; ++e) {
                    out_d[(size_t) q * C + e] = e < n ? hp.D(e) : FLT_MAX;
                    out_i[(size_t) q * C + e] = e < n ? hp.I(e) : 0xffffffffu;
                }
            }
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
// BF16 pieces of -|x|^2 / 2 in columns D and D + 1) and FP32 |x|^2.  One warp per row;
// rows N .. Npad-1 are zero.
__global__ void k_tc_prep(const double *__restrict__ X, int N, int D, int Npad, __nv_bfloat16 *__restrict__ qhi,
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
            x[h] = (i < N && d < D) ? X[(size_t) i * D + d] : 0.0;
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

int knn_candidates_tc(const double *Xd, int N, int D, int C, float *cand_d, uint32_t *cand_i, cudaStream_t st,
                      std::string &err) {
    const int Npad = (N + BM - 1) / BM * BM;
    const size_t plane = (size_t) Npad * KD;
    __nv_bfloat16 *planes = nullptr;
    float *qn = nullptr;
    int *derr = nullptr;
    auto cleanup = [&]() {
        cudaFree(planes);
        cudaFree(qn);
        cudaFree(derr);
    };
    cudaError_t e;
    if ((e = cudaMalloc(&planes, sizeof(__nv_bfloat16) * plane * 4)) != cudaSuccess ||
        (e = cudaMalloc(&qn, sizeof(float) * Npad)) != cudaSuccess ||
        (e = cudaMalloc(&derr, sizeof(int))) != cudaSuccess) {
        err = std::string("knn tc allocation: ") + cudaGetErrorString(e);
        cleanup();
        return -10;
    }
    __nv_bfloat16 *qhi = planes, *qlo = planes + plane, *rhi = planes + 2 * plane, *rlo = planes + 3 * plane;
    cudaMemsetAsync(derr, 0, sizeof(int), st);
    k_tc_prep<<<2048, 256, 0, st>>>(Xd, N, D, Npad, qhi, qlo, rhi, rlo, qn);
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
    const int nQT = Npad / BM;
    const int grid = nQT < nsm ? nQT : nsm;
    k_knn_tc<<<grid, kThreads, kSmemBytes, st>>>(m_qhi, m_qlo, m_rhi, m_rlo, qn, N, Npad, C, cand_d, cand_i, derr);
    int herr = 0;
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
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
