// Per-point and per-edge kernels of one FIt-SNE gradient iteration (see grad.cuh).
#include <algorithm>
#include <cfloat>

#include "grad.cuh"

namespace fitsne {
namespace {

constexpr int kBlock = 256;
constexpr int kRedGrid = 1216;  // 152 SMs x 8 resident blocks of 256 threads
// Launch shapes of the attraction pass: consecutive rows per work item (<= 32) and CSR
// edges per lane per batch.  Entry 0 is the default; Embedding's autotuner times the rest.
// Shape 5: the 8 warps of a block take 8 consecutive groups at once, so that the neighbour
// gathers of an SM's warps overlap in its L1.  Shape 6: a warp loads the next row's first
// batch of CSR entries before it gathers the current row's neighbours.  Shapes 7, 8: registers
// capped for 6 resident blocks (48 warps) per SM.  Shape 9: 160-edge batches (a typical row in
// one batch).  Shape 10: 16 x 2 with registers capped for 6 resident blocks (40 per thread): the
// gathers are latency-bound, and the extra warps keep more of them in flight (FP32 form at
// N = 1M: 0.680 ms against 0.717 - 0.731 ms for shape 3 on the same box).
constexpr int kAttrShapes[kNumAttrShapes][2] = {{16, 4}, {32, 4}, {8, 4}, {16, 2}, {32, 2}, {16, 4},
                                                {16, 4}, {16, 4}, {8, 4},  {16, 5}, {16, 2}};

// ---------------------------------------------------------------------------------
// storage layouts of Y
template <typename T, int D>
struct YL;
template <>
struct YL<float, 2> {
    typedef df32 P;
    static FITSNE_D void load(const float *Y, int i, P *c) {
        const float4 v = __ldg(reinterpret_cast<const float4 *>(Y) + i);
        c[0] = {v.x, v.z};
        c[1] = {v.y, v.w};
    }
    static FITSNE_D void store(float *Y, int i, const P *c) {
        reinterpret_cast<float4 *>(Y)[i] = make_float4(c[0].hi, c[1].hi, c[0].lo, c[1].lo);
    }
};
template <>
struct YL<float, 1> {
    typedef df32 P;
    static FITSNE_D void load(const float *Y, int i, P *c) {
        const float2 v = __ldg(reinterpret_cast<const float2 *>(Y) + i);
        c[0] = {v.x, v.y};
    }
    static FITSNE_D void store(float *Y, int i, const P *c) {
        reinterpret_cast<float2 *>(Y)[i] = make_float2(c[0].hi, c[0].lo);
    }
};
template <>
struct YL<double, 2> {
    typedef double P;
    static FITSNE_D void load(const double *Y, int i, P *c) {
        const double2 v = __ldg(reinterpret_cast<const double2 *>(Y) + i);
        c[0] = v.x;
        c[1] = v.y;
    }
    static FITSNE_D void store(double *Y, int i, const P *c) {
        reinterpret_cast<double2 *>(Y)[i] = make_double2(c[0], c[1]);
    }
};
template <>
struct YL<double, 1> {
    typedef double P;
    static FITSNE_D void load(const double *Y, int i, P *c) { c[0] = __ldg(Y + i); }
    static FITSNE_D void store(double *Y, int i, const P *c) { Y[i] = c[0]; }
};

// 1 / x correctly rounded: the same value as the IEEE division 1.f / x, in fewer
// instructions (the attraction evaluates it once per non-zero of P)
FITSNE_D float recip(float x) { return __frcp_rn(x); }
FITSNE_D double recip(double x) { return 1.0 / x; }

FITSNE_D float pdiff(df32 a, df32 b) { return df_diff(a, b); }
FITSNE_D double pdiff(double a, double b) { return a - b; }
FITSNE_D df32 padd(df32 a, float u) { return df_add_f(a, u); }
FITSNE_D double padd(double a, double u) { return a + u; }
FITSNE_D df32 pshift(df32 a, df32 negm) { return df_add(a, negm); }
FITSNE_D double pshift(double a, double negm) { return a + negm; }
FITSNE_D double ptod(df32 a) { return (double) a.hi + (double) a.lo; }
FITSNE_D double ptod(double a) { return a; }

// ---------------------------------------------------------------------------------
// box geometry in the precision of T
template <typename T>
struct BoxP;
template <>
struct BoxP<float> {
    df32 neg_mn, bw;
    float inv_bw, bwT;
    double mn64, bw64;  // the FP64 geometry, for points on a box edge
    int nb, nterms, M;
    float s[kMaxInterp], inv_den[kMaxInterp];
};
template <>
struct BoxP<double> {
    double mn, bw, bwT;
    int nb, nterms, M;
    double s[kMaxInterp], inv_den[kMaxInterp];
};

__host__ __device__ BoxP<float> make_box(const GridGeom &g, float *) {
    BoxP<float> b;  // the FP32 values as grid_geom made them (df_from_double, 1 / bw)
    b.neg_mn = {g.neg_mn32[0], g.neg_mn32[1]};
    b.bw = {g.bw32[0], g.bw32[1]};
    b.inv_bw = g.inv_bw32;
    b.bwT = g.bw32[0];
    b.mn64 = g.mn;
    b.bw64 = g.bw;
    b.nb = g.nb;
    b.nterms = g.nterms;
    b.M = g.M;
    for (int k = 0; k < kMaxInterp; ++k) {
        b.s[k] = g.s32[k];
        b.inv_den[k] = g.inv_den32[k];
    }
    return b;
}
__host__ __device__ BoxP<double> make_box(const GridGeom &g, double *) {
    BoxP<double> b;
    b.mn = g.mn;
    b.bw = g.bw;
    b.bwT = g.bw;
    b.nb = g.nb;
    b.nterms = g.nterms;
    b.M = g.M;
    for (int k = 0; k < kMaxInterp; ++k) {
        b.s[k] = g.s64[k];
        b.inv_den[k] = g.inv_den64[k];
    }
    return b;
}

// box index (truncated and clamped as in n_body_fft_2d, nbodyfft.cpp:82-114) and the
// in-box coordinate t = (x - lower) / width.
// The float quotient q carries a relative error below 3 * 2^-24.  When that error could
// move q across an integer, the index is taken from the FP64 quotient (x - min) / width
// that the reference computes, so that both forms interpolate every point from the same
// box: a point on an edge interpolated from the neighbouring box changes its own and its
// neighbours' repulsion by the interpolation error (about 1e-2 of a near-field term),
// far above FP32 rounding.
FITSNE_D void box_coord(df32 c, const BoxP<float> &b, int &k, float &t) {
    const df32 d = df_add(c, b.neg_mn);
    const float q = (d.hi + d.lo) * b.inv_bw;
    k = (int) q;
    const float fr = q - (float) k;
    const float tol = 4e-7f * fabsf(q);
    if (fr < tol || fr > 1.f - tol)  // (every q < 0 takes this branch too)
        k = (int) ((((double) c.hi + (double) c.lo) - b.mn64) / b.bw64);
    if (k >= b.nb) k = b.nb - 1;
    else if (k < 0) k = 0;
    df32 p = two_prod((float) k, b.bw.hi);
    p.lo += (float) k * b.bw.lo;
    const df32 r = df_add(d, df_neg(p));
    t = (r.hi + r.lo) * b.inv_bw;
}
FITSNE_D void box_coord(double c, const BoxP<double> &b, int &k, double &t) {
    k = (int) ((c - b.mn) / b.bw);
    if (k >= b.nb) k = b.nb - 1;
    else if (k < 0) k = 0;
    t = (c - (k * b.bw + b.mn)) / b.bw;
}

// Lagrange basis on the nodes s_k = (k + 1/2) / nterms (interpolate, nbodyfft.cpp:310-336)
template <typename T, int NT>
FITSNE_D void lagrange(T t, const BoxP<T> &b, T *w) {
    const int n = NT > 0 ? NT : b.nterms;
#pragma unroll
    for (int j = 0; j < (NT > 0 ? NT : kMaxInterp); ++j) {
        if (j < n) {
            T num = T(1);
#pragma unroll
            for (int k = 0; k < (NT > 0 ? NT : kMaxInterp); ++k)
                if (k < n && k != j) num *= (t - b.s[k]);
            w[j] = num * b.inv_den[j];
        }
    }
}

FITSNE_D void atomic_add4(Cell4<float> *p, const Cell4<float> &v) {
    atomicAdd(reinterpret_cast<float4 *>(p), make_float4(v.a, v.b, v.c, v.d));
}
FITSNE_D void atomic_add4(Cell4<double> *p, const Cell4<double> &v) {
    atomicAdd(&p->a, v.a);
    atomicAdd(&p->b, v.b);
    atomicAdd(&p->c, v.c);
    atomicAdd(&p->d, v.d);
}

// ---------------------------------------------------------------------------------
// block reductions with a deterministic "last block finishes" step
template <int NV>
FITSNE_D void block_sum(double (&v)[NV], double *sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double x = v[k];
        for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) sh[wid * NV + k] = x;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double x = 0.0;
            for (int w = 0; w < nw; ++w) x += sh[w * NV + k];
            v[k] = x;
        }
    }
    __syncthreads();
}

// Second half of grid_sum: thread 0 holds the block's sums in v.
template <int NV>
FITSNE_D bool grid_sum_finish(double (&v)[NV], double *part, unsigned int *count, double *sh, int blk, int nblk) {
    __shared__ bool last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) part[blk * NV + k] = v[k];
        __threadfence();
        const unsigned int prev = atomicAdd(count, 1u);
        last = (prev == (unsigned int) nblk - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x)
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] += ((volatile double *) part)[b * NV + k];
    block_sum<NV>(acc, sh);
    if (threadIdx.x == 0) {
        *count = 0u;
#pragma unroll
        for (int k = 0; k < NV; ++k) v[k] = acc[k];
        return true;
    }
    return false;
}

// Writes this block's partials; returns true in thread 0 of the last block to finish,
// with v replaced by the total over all blocks.
template <int NV>
FITSNE_D bool grid_sum(double (&v)[NV], double *part, unsigned int *count, double *sh, int blk, int nblk) {
    block_sum<NV>(v, sh);
    return grid_sum_finish<NV>(v, part, count, sh, blk, nblk);
}

// The block's sums of double-float values in double-float arithmetic (FP32 pipe), into out
// (FP64) in thread 0: one conversion a block instead of FP64 shuffles and adds in every warp
// (the FP64 pipe takes ~16 cycles a warp instruction; the attraction's warps all reach their
// mean reduction at the end of the launch).  sh holds NV doubles per warp.
template <int NV>
FITSNE_D void block_sum_df(df32 (&v)[NV], double (&out)[NV], double *sh) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    float *shf = reinterpret_cast<float *>(sh);
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        df32 x = v[k];
        for (int o = 16; o; o >>= 1) x = df_add(x, df32{__shfl_xor_sync(full, x.hi, o), __shfl_xor_sync(full, x.lo, o)});
        if (lane == 0) {
            shf[2 * (wid * NV + k)] = x.hi;
            shf[2 * (wid * NV + k) + 1] = x.lo;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            df32 x{0.f, 0.f};
            for (int w = 0; w < nw; ++w) x = df_add(x, df32{shf[2 * (w * NV + k)], shf[2 * (w * NV + k) + 1]});
            out[k] = df_to_double(x);
        }
    }
    __syncthreads();
}

// grid min / max, second half: thread 0 holds the block's (mn, mx); the last block to finish
// combines the blocks' values and returns true in its thread 0
FITSNE_D bool grid_minmax_finish(double &mn, double &mx, double *part, unsigned int *count, double *sh, int blk,
                                 int nblk) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __shared__ bool last;
    if (threadIdx.x == 0) {
        part[2 * blk] = mn;
        part[2 * blk + 1] = mx;
        __threadfence();
        const unsigned int prev = atomicAdd(count, 1u);
        last = (prev == (unsigned int) nblk - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double a = HUGE_VAL, b = -HUGE_VAL;
    for (int k = threadIdx.x; k < nblk; k += blockDim.x) {
        a = fmin(a, ((volatile double *) part)[2 * k]);
        b = fmax(b, ((volatile double *) part)[2 * k + 1]);
    }
    for (int o = 16; o; o >>= 1) {
        a = fmin(a, __shfl_xor_sync(0xffffffffu, a, o));
        b = fmax(b, __shfl_xor_sync(0xffffffffu, b, o));
    }
    __syncthreads();
    if (lane == 0) {
        sh[2 * wid] = a;
        sh[2 * wid + 1] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < nw; ++w) {
            a = fmin(a, sh[2 * w]);
            b = fmax(b, sh[2 * w + 1]);
        }
        mn = a;
        mx = b;
        *count = 0u;
        return true;
    }
    return false;
}

// min / max with the same rule as the reference (FP64 values per thread)
FITSNE_D bool grid_minmax(double &mn, double &mx, double *part, unsigned int *count, double *sh, int blk, int nblk) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o; o >>= 1) {
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if (lane == 0) {
        sh[2 * wid] = mn;
        sh[2 * wid + 1] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < nw; ++w) {
            mn = fmin(mn, sh[2 * w]);
            mx = fmax(mx, sh[2 * w + 1]);
        }
    }
    __syncthreads();  // sh is reused by the finish
    return grid_minmax_finish(mn, mx, part, count, sh, blk, nblk);
}

// FP32 form: the same over double-float values ordered by their (hi, lo) pairs, reduced within
// the block in FP32 (shuffles and compares) and converted to FP64 once per block; the FP64
// pipe takes ~16 cycles a warp instruction, which the per-warp FP64 reductions of 1,216
// blocks paid in every iteration.  (double) hi + (double) lo is exact, so the result is the
// FP64 reduction's.
FITSNE_D void pair_min(float &h, float &l, float h2, float l2) {
    if (h2 < h || (h2 == h && l2 < l)) {
        h = h2;
        l = l2;
    }
}
FITSNE_D void pair_max(float &h, float &l, float h2, float l2) {
    if (h2 > h || (h2 == h && l2 > l)) {
        h = h2;
        l = l2;
    }
}
FITSNE_D bool grid_minmax_pairs(float nh, float nl, float xh, float xl, double &mn, double &mx, double *part,
                                unsigned int *count, double *sh, int blk, int nblk) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int o = 16; o; o >>= 1) {
        pair_min(nh, nl, __shfl_xor_sync(full, nh, o), __shfl_xor_sync(full, nl, o));
        pair_max(xh, xl, __shfl_xor_sync(full, xh, o), __shfl_xor_sync(full, xl, o));
    }
    float *shf = reinterpret_cast<float *>(sh);  // 4 floats per warp (sh holds 2 doubles a warp)
    if (lane == 0) {
        shf[4 * wid] = nh;
        shf[4 * wid + 1] = nl;
        shf[4 * wid + 2] = xh;
        shf[4 * wid + 3] = xl;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < nw; ++w) {
            pair_min(nh, nl, shf[4 * w], shf[4 * w + 1]);
            pair_max(xh, xl, shf[4 * w + 2], shf[4 * w + 3]);
        }
        mn = (double) nh + (double) nl;
        mx = (double) xh + (double) xl;
    }
    __syncthreads();  // sh is reused by the finish
    return grid_minmax_finish(mn, mx, part, count, sh, blk, nblk);
}

// ---------------------------------------------------------------------------------
// center (subtract the pending mean) + min/max (tsne.cpp:531, 1039-1049, 769-773)
template <typename T, int D>
FITSNE_D void center_minmax_body(T *Y, int N, int apply_mean, int excl, RedScratch r, double *sh, int blk, int nblk) {
    typedef typename YL<T, D>::P P;
    // -mean in the positions' form, made by thread 0 (FP64 conversions, ~16 cycles a warp
    // instruction on GB300's FP64 pipe, once per block instead of once per warp)
    __shared__ P s_negm[D];
    if (threadIdx.x == 0) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
            const double m = apply_mean ? r.mean[d] : 0.0;
            if constexpr (sizeof(T) == 4)
                s_negm[d] = df_from_double(-m);
            else
                s_negm[d] = -m;
        }
    }
    __syncthreads();
    P negm[D];
#pragma unroll
    for (int d = 0; d < D; ++d) negm[d] = s_negm[d];
    double mn = HUGE_VAL, mx = -HUGE_VAL;
    // FP32 form: the double-float values compared by their (hi, lo) pairs, whose order is the
    // values' order for normalised pairs (hi = fl(hi + lo)), so the thread's min / max cost one
    // conversion to double at the end instead of FP64 operations per coordinate
    float nh = INFINITY, nl = 0.f, xh = -INFINITY, xl = 0.f;
    for (int i = blk * blockDim.x + threadIdx.x; i < N; i += nblk * blockDim.x) {
        P c[D];
        YL<T, D>::load(Y, i, c);
        if (apply_mean) {
#pragma unroll
            for (int d = 0; d < D; ++d) c[d] = pshift(c[d], negm[d]);
            YL<T, D>::store(Y, i, c);
        }
#pragma unroll
        for (int d = 0; d < D; ++d) {
            // 2-D: the first coordinate of the first point never reaches the min
            // (if / else-if pair of tsne.cpp:1045-1048)
            const bool in_min = !(D == 2 && i == excl && d == 0);
            if constexpr (sizeof(T) == 4) {
                const df32 v = c[d];
                if (v.hi > xh || (v.hi == xh && v.lo > xl)) {
                    xh = v.hi;
                    xl = v.lo;
                }
                if (in_min && (v.hi < nh || (v.hi == nh && v.lo < nl))) {
                    nh = v.hi;
                    nl = v.lo;
                }
            } else {
                const double v = ptod(c[d]);
                mx = fmax(mx, v);
                if (in_min) mn = fmin(mn, v);
            }
        }
    }
    bool done;
    if constexpr (sizeof(T) == 4)
        done = grid_minmax_pairs(nh, nl, xh, xl, mn, mx, r.part, r.count + 0, sh, blk, nblk);
    else
        done = grid_minmax(mn, mx, r.part, r.count + 0, sh, blk, nblk);
    if (done) {
        r.mnmx[0] = mn;
        r.mnmx[1] = mx;
    }
}

template <typename T, int D>
__global__ void __launch_bounds__(kBlock) k_center_minmax(T *Y, int N, int apply_mean, int excl, RedScratch r) {
    __shared__ double sh[2 * 32];
    center_minmax_body<T, D>(Y, N, apply_mean, excl, r, sh, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------------
// spread (step 1 of n_body_fft_2d / nbodyfft) in box-local charges
template <typename T, int D, int NT>
__global__ void __launch_bounds__(kBlock) k_spread(const T *__restrict__ Y, int N, BoxP<T> b,
                                                   Cell4<T> *__restrict__ grid, const DevGeom *__restrict__ dg) {
    typedef typename YL<T, D>::P P;
    if (dg) b = make_box(dg->g, (T *) nullptr);
    const int n = NT > 0 ? NT : b.nterms;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        P c[D];
        YL<T, D>::load(Y, i, c);
        int bx[D];
        T t[D];
        T w[D][NT > 0 ? NT : kMaxInterp];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            box_coord(c[d], b, bx[d], t[d]);
            lagrange<T, NT>(t[d], b, w[d]);
        }
        if constexpr (D == 2) {
            for (int ia = 0; ia < n; ++ia) {
                const T ux = (t[0] - b.s[ia]) * b.bwT;
                const size_t rowbase = (size_t) (bx[0] * n + ia) * b.M + bx[1] * n;
                for (int ib = 0; ib < n; ++ib) {
                    const T uy = (t[1] - b.s[ib]) * b.bwT;
                    const T ww = w[0][ia] * w[1][ib];
                    Cell4<T> v;
                    v.a = ww;
                    v.b = ww * ux;
                    v.c = ww * uy;
                    v.d = ww * (ux * ux + uy * uy);
                    atomic_add4(grid + rowbase + ib, v);
                }
            }
        } else {
            for (int ia = 0; ia < n; ++ia) {
                const T u = (t[0] - b.s[ia]) * b.bwT;
                const T ww = w[0][ia];
                T *cell = reinterpret_cast<T *>(grid + bx[0] * n + ia);
                atomicAdd(cell + 0, ww);
                atomicAdd(cell + 1, ww * u);
                atomicAdd(cell + 2, ww * u * u);
            }
        }
    }
}

// FP32 spread with nterms = 3, aggregated per warp before the atomics.  After the locality
// renumbering consecutive points mostly share a box, and every point of a box charges the
// same 9 (2-D) or 3 (1-D) nodes, so a warp sums its 32 points' charges over runs of equal box
// index and issues one atomic per run and node.  2-D: the 36 values per point go through a
// per-warp shared-memory table (9 stores per lane, then 32 loads by each of 9 node lanes)
// instead of a segmented shuffle scan (180 shuffles per warp).  1-D (9 values): a segmented
// inclusive scan (head flags where the box changes, five shuffle steps per value) leaves each
// run's sums in its last lane.  Identical charges to k_spread; only the order of the FP32
// additions differs.
struct SpreadWarpTable {
    float4 v[9][33];      // [node][point]; 33 columns so that the node lanes' loads spread over banks
    long long cell[32];   // first grid cell of each point's box (-1: no point)
};
constexpr int kSpreadWarps = kBlock / 32;

// order (may be null): slot k of the walk takes point order[k] (a 2-D locality order of the
// points when they are numbered by another one), so that a warp's points share boxes.
template <int D>
FITSNE_D void spread_runs_body(const float *__restrict__ Y, int N, const BoxP<float> &b,
                               Cell4<float> *__restrict__ grid, int blk, int nblk,
                               const uint32_t *__restrict__ order = nullptr) {
    SpreadWarpTable *wb = nullptr;
    if constexpr (D == 2) {
        __shared__ SpreadWarpTable tables[kSpreadWarps];
        wb = &tables[threadIdx.x >> 5];
    }
    constexpr int NT = 3;
    constexpr int NV = (D == 2) ? NT * NT : NT;  // nodes per point
    constexpr int NC = (D == 2) ? 4 : 3;         // charge values per node
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int warp0 = (blk * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (nblk * blockDim.x) >> 5;
    for (int base = warp0 * 32; base < N; base += nwarps * 32) {
        const int i = base + lane;
        const bool valid = i < N;
        int bx[D];
        float t[D];
        float w[D][NT];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            bx[d] = 0;
            t[d] = 0.5f;
#pragma unroll
            for (int k = 0; k < NT; ++k) w[d][k] = 0.f;
        }
        if (valid) {
            df32 c[D];
            YL<float, D>::load(Y, order ? (int) order[i] : i, c);
#pragma unroll
            for (int d = 0; d < D; ++d) {
                box_coord(c[d], b, bx[d], t[d]);
                lagrange<float, NT>(t[d], b, w[d]);
            }
        }
        const int key = valid ? (D == 2 ? bx[0] * b.nb + bx[1] : bx[0]) : -1 - lane;
        float v[NV][NC];
        if constexpr (D == 2) {
#pragma unroll
            for (int ia = 0; ia < NT; ++ia) {
                const float ux = (t[0] - b.s[ia]) * b.bwT;
#pragma unroll
                for (int ib = 0; ib < NT; ++ib) {
                    const float uy = (t[1] - b.s[ib]) * b.bwT;
                    const float ww = w[0][ia] * w[1][ib];
                    float *o = v[ia * NT + ib];
                    o[0] = ww;
                    o[1] = ww * ux;
                    o[2] = ww * uy;
                    o[3] = ww * (ux * ux + uy * uy);
                }
            }
        } else {
#pragma unroll
            for (int ia = 0; ia < NT; ++ia) {
                const float u = (t[0] - b.s[ia]) * b.bwT;
                const float ww = w[0][ia];
                v[ia][0] = ww;
                v[ia][1] = ww * u;
                v[ia][2] = ww * u * u;
            }
        }
        if constexpr (D == 2) {
            // run sums through the warp's table: lane l stores its 9 node charges in column l.
            // Then 27 lanes add up the table, lane (q, j) = (lane % 9, lane / 9) node q over
            // the points of range j ([0, 11), [11, 22), [22, 32)) in order: a run that ends
            // inside the range and began there is issued at once (one float4 atomic for the
            // run's box); the first run end of a range also closes the run carried in from the
            // ranges before, whose pieces (the earlier ranges' tails) come by shuffles.  A warp's
            // run ends (`ends`, lane 31 always) are the same for every lane.
            const int next = __shfl_down_sync(full, key, 1);
            const unsigned ends = __ballot_sync(full, lane == 31 || next != key);
#pragma unroll
            for (int q = 0; q < NV; ++q) wb->v[q][lane] = make_float4(v[q][0], v[q][1], v[q][2], v[q][3]);
            wb->cell[lane] = valid ? (long long) bx[0] * NT * b.M + (long long) bx[1] * NT : -1ll;
            __syncwarp();
            const int q = lane % NV, j = lane / NV;  // lanes 27 - 31: j = 3, no range
            const int lo = 11 * j, n = j < 2 ? 11 : (j == 2 ? 10 : 0);
            const long long off = (long long) (q / NT) * b.M + q % NT;
            float4 acc = make_float4(0.f, 0.f, 0.f, 0.f), head = acc;
            int first_end = -1;
#pragma unroll
            for (int k = 0; k < 11; ++k) {
                if (k < n) {
                    const int pt = lo + k;
                    const float4 x = wb->v[q][pt];
                    acc.x += x.x;
                    acc.y += x.y;
                    acc.z += x.z;
                    acc.w += x.w;
                    if ((ends >> pt) & 1u) {
                        if (first_end < 0) {
                            first_end = pt;  // closes the run carried in: issued after the join
                            head = acc;
                        } else {
                            const long long c = wb->cell[pt];
                            if (c >= 0) atomicAdd(reinterpret_cast<float4 *>(grid + c + off), acc);
                        }
                        acc = make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                }
            }
            // acc is now this range's tail (the part of a run that goes on past the range).
            // The run closed at range j's first end began in range j, or earlier: its earlier
            // pieces are range j - 1's tail and, when range j - 1 has no run end, range j - 2's.
            const int s1 = lane >= NV ? lane - NV : lane, s2 = lane >= 2 * NV ? lane - 2 * NV : lane;
            const float4 t1 = make_float4(__shfl_sync(full, acc.x, s1), __shfl_sync(full, acc.y, s1),
                                          __shfl_sync(full, acc.z, s1), __shfl_sync(full, acc.w, s1));
            const float4 t2 = make_float4(__shfl_sync(full, acc.x, s2), __shfl_sync(full, acc.y, s2),
                                          __shfl_sync(full, acc.z, s2), __shfl_sync(full, acc.w, s2));
            if (first_end >= 0) {
                float4 carry = make_float4(0.f, 0.f, 0.f, 0.f);
                if (j >= 1) carry = t1;
                if (j == 2 && (ends & (0x7ffu << 11)) == 0u) {  // range 1 has no run end
                    carry.x += t2.x;
                    carry.y += t2.y;
                    carry.z += t2.z;
                    carry.w += t2.w;
                }
                const float4 run = make_float4(carry.x + head.x, carry.y + head.y, carry.z + head.z,
                                               carry.w + head.w);
                const long long c = wb->cell[first_end];
                if (c >= 0) atomicAdd(reinterpret_cast<float4 *>(grid + c + off), run);
            }
            __syncwarp();  // the table is rewritten by the next 32 points
        } else {
            // segmented inclusive scan: after the step with offset `off`, lane l holds the sum
            // over [max(head(l), l - 2 off + 1), l]
            const int prev = __shfl_up_sync(full, key, 1);
            const unsigned heads = __ballot_sync(full, lane == 0 || prev != key);
            const int my_head = 31 - __clz(heads & (full >> (31 - lane)));
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const bool take = lane - off >= my_head;
#pragma unroll
                for (int q = 0; q < NV; ++q)
#pragma unroll
                    for (int r = 0; r < NC; ++r) {
                        const float y = __shfl_up_sync(full, v[q][r], off);
                        if (take) v[q][r] += y;
                    }
            }
            const int next = __shfl_down_sync(full, key, 1);
            if (valid && (lane == 31 || next != key)) {
#pragma unroll
                for (int ia = 0; ia < NT; ++ia) {
                    float *cell = reinterpret_cast<float *>(grid + bx[0] * NT + ia);
                    atomicAdd(cell + 0, v[ia][0]);
                    atomicAdd(cell + 1, v[ia][1]);
                    atomicAdd(cell + 2, v[ia][2]);
                }
            }
        }
    }
}

template <int D>
__global__ void __launch_bounds__(kBlock) k_spread_runs(const float *__restrict__ Y, int N, BoxP<float> b,
                                                        Cell4<float> *__restrict__ grid,
                                                        const DevGeom *__restrict__ dg,
                                                        const uint32_t *__restrict__ order) {
    if (dg) b = make_box(dg->g, (float *) nullptr);
    spread_runs_body<D>(Y, N, b, grid, blockIdx.x, gridDim.x, order);
}

// ---------------------------------------------------------------------------------
// gather (step 3) + the repulsion numerators + Z
template <typename T, int D, int NT>
FITSNE_D void gather_body(const T *__restrict__ Y, int N, const BoxP<T> &b, const Cell4<T> *__restrict__ pot,
                          int mode, T *__restrict__ rep, RedScratch r, float *__restrict__ yh, double *sh, int blk,
                          int nblk) {
    typedef typename YL<T, D>::P P;
    const int n = NT > 0 ? NT : b.nterms;
    double zacc[1] = {0.0};
    for (int i = blk * blockDim.x + threadIdx.x; i < N; i += nblk * blockDim.x) {
        P c[D];
        YL<T, D>::load(Y, i, c);
        if constexpr (sizeof(T) == 4) {
            // the FP32 positions (high words) that the attraction gathers as neighbours
            if (yh) {
                if constexpr (D == 2)
                    reinterpret_cast<float2 *>(yh)[i] = make_float2(c[0].hi, c[1].hi);
                else
                    yh[i] = c[0].hi;
            }
        }
        int bx[D];
        T t[D];
        T w[D][NT > 0 ? NT : kMaxInterp];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            box_coord(c[d], b, bx[d], t[d]);
            lagrange<T, NT>(t[d], b, w[d]);
        }
        T zi = T(0);
        if constexpr (D == 2) {
            T rx = T(0), ry = T(0);
            for (int ia = 0; ia < n; ++ia) {
                const T ux = (t[0] - b.s[ia]) * b.bwT;
                const size_t rowbase = (size_t) (bx[0] * n + ia) * b.M + bx[1] * n;
                for (int ib = 0; ib < n; ++ib) {
                    const T uy = (t[1] - b.s[ib]) * b.bwT;
                    const T ww = w[0][ia] * w[1][ib];
                    const Cell4<T> p = pot[rowbase + ib];
                    rx += ww * (ux * p.a + p.b);
                    ry += ww * (uy * p.a + p.c);
                    if (mode == KERNEL_DF1)
                        zi += ww * ((T(1) + ux * ux + uy * uy) * p.a + T(2) * (ux * p.b + uy * p.c) + p.d);
                    else
                        zi += ww * p.d;
                }
            }
            rep[2 * (size_t) i] = rx;
            rep[2 * (size_t) i + 1] = ry;
        } else {
            T rx = T(0);
            for (int ia = 0; ia < n; ++ia) {
                const T u = (t[0] - b.s[ia]) * b.bwT;
                const Cell4<T> p = pot[bx[0] * n + ia];
                rx += w[0][ia] * (u * p.a + p.b);
                if (mode == KERNEL_DF1)
                    zi += w[0][ia] * ((T(1) + u * u) * p.a + T(2) * u * p.b + p.c);
                else
                    zi += w[0][ia] * p.c;
            }
            rep[i] = rx;
        }
        zacc[0] += (double) zi;
    }
    if (grid_sum<1>(zacc, r.part, r.count + 1, sh, blk, nblk)) *r.z = zacc[0] - (double) N;
}

template <typename T, int D, int NT>
__global__ void __launch_bounds__(kBlock) k_gather(const T *__restrict__ Y, int N, BoxP<T> b,
                                                   const Cell4<T> *__restrict__ pot, int mode,
                                                   T *__restrict__ rep, RedScratch r,
                                                   const DevGeom *__restrict__ dg, float *__restrict__ yh) {
    __shared__ double sh[32];
    if (dg) b = make_box(dg->g, (T *) nullptr);
    gather_body<T, D, NT>(Y, N, b, pot, mode, rep, r, yh, sh, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------------
// Row `my` of the attraction kernels: the gradient (exaggeration x attraction amy, minus the
// repulsion over Z; tsne.cpp:1121-1155) and, in mode 1, the reference's update (gains,
// momentum, step clipping; tsne.cpp:479-531) into Yout, the new position added to msum; in
// mode 0 the gradient into dC only.
template <typename T, int D>
FITSNE_D void attr_row_update(int my, const T (&amy)[D], const typename YL<T, D>::P (&cmy)[D], const UpdateParams &p,
                              T zinv, T exag, const T *__restrict__ rep, T *__restrict__ dC, T *__restrict__ gains,
                              T *__restrict__ uY, T *__restrict__ Yout, typename YL<T, D>::P (&msum)[D]) {
    typedef typename YL<T, D>::P P;
    T gr[D];
#pragma unroll
    for (int d = 0; d < D; ++d) gr[d] = exag * amy[d] - rep[(size_t) my * D + d] * zinv;
    if (p.mode == 0) {
#pragma unroll
        for (int d = 0; d < D; ++d) dC[(size_t) my * D + d] = gr[d];
        return;
    }
    P cn[D];
    if (p.use_gains) {
        T u[D];
        T nrm2 = T(0);
#pragma unroll
        for (int d = 0; d < D; ++d) {
            T gn = gains[(size_t) my * D + d];
            const T uo = uY[(size_t) my * D + d];
            gn = (sgn(gr[d]) != sgn(uo)) ? (gn + T(0.2)) : (gn * T(0.8));
            if (gn < T(0.01)) gn = T(0.01);
            gains[(size_t) my * D + d] = gn;
            u[d] = T(p.momentum) * uo - T(p.learning_rate) * gn * gr[d];
            nrm2 += u[d] * u[d];
        }
        if (p.max_step_norm > 0) {
            const T step = sqrt(nrm2);
            if (step > T(p.max_step_norm)) {
                const T sc = T(p.max_step_norm) / step;
#pragma unroll
                for (int d = 0; d < D; ++d) u[d] *= sc;
            }
        }
#pragma unroll
        for (int d = 0; d < D; ++d) {
            uY[(size_t) my * D + d] = u[d];
            cn[d] = padd(cmy[d], u[d]);
        }
    } else {
#pragma unroll
        for (int d = 0; d < D; ++d) cn[d] = padd(cmy[d], -gr[d]);
    }
    YL<T, D>::store(Yout, my, cn);
#pragma unroll
    for (int d = 0; d < D; ++d) {
        if constexpr (sizeof(T) == 4)
            msum[d] = df_add(msum[d], cn[d]);
        else
            msum[d] += cn[d];
    }
}

// End of an attraction kernel: the last warp out resets the work counter for the next launch
// (every warp's last counter increment is ordered before its exit increment by the fence);
// in mode 1 the grid sum of the new positions gives the mean that the next centring removes.
template <typename T, int D>
FITSNE_D void attr_finish(int lane, unsigned int nwarps, int N, const UpdateParams &p, RedScratch r,
                          const typename YL<T, D>::P (&msum)[D], double *sh, int blk, int nblk) {
    if (lane == 0) {
        __threadfence();
        const unsigned int out = atomicAdd(r.count + 5, 1u);
        if (out == nwarps - 1) {
            atomicExch(r.count + 4, 0u);
            atomicExch(r.count + 5, 0u);
        }
    }
    if (p.mode != 0) {
        double m[2] = {0.0, 0.0};
        bool done;
        if constexpr (sizeof(T) == 4) {
            df32 v[2] = {msum[0], D == 2 ? msum[D - 1] : df32{0.f, 0.f}};
            block_sum_df<2>(v, m, sh);
            done = grid_sum_finish<2>(m, r.part, r.count + 2, sh, blk, nblk);
        } else {
#pragma unroll
            for (int d = 0; d < D; ++d) m[d] = ptod(msum[d]);
            done = grid_sum<2>(m, r.part, r.count + 2, sh, blk, nblk);
        }
        if (done) {
            r.mean[0] = m[0] / (double) N;
            r.mean[1] = m[1] / (double) N;
        }
    }
}

// ---------------------------------------------------------------------------------
// CSR attraction fused with the optimiser step (tsne.cpp:1121-1155 and 479-531).
//
// Warps take groups of kAttrGroup consecutive rows from a work counter (so that the grid sweeps
// one window of consecutive rows, whose neighbours share L1/L2 lines after the locality
// renumbering, and every warp stays busy whatever the row lengths).  Lane j of a group
// loads row j's pointers and Y with coalesced loads and, at the end, applies row j's update
// (gains, momentum, clipping, double-float Y) — so per row only two memory round trips
// remain: the CSR entries (prefetched into L2 while the previous row is processed) and the
// neighbour Y gathers (L2-resident).  Within a row, lanes take kAttrUnroll edges each per
// batch: all index / value loads first, then all gathers.
// Rows [row0, row0 + N) of the CSR (column indices and Y are global); blk / nblk: this
// block's index among the nblk blocks that share the rows (and r's counters).
// kKL: the same traversal evaluates the KL divergence instead (evaluateErrorFft,
// tsne.cpp:1329-1355): per edge val * exag * log((val * exag + FLT_MIN) / (Q + FLT_MIN)) with
// Q = q^df / Z (p.exag the multiplier, *r.z the Z of the last gradient, full positions: yh
// null), a lane's terms of a row summed in FP32 and added to its FP64 sum once per row, the
// grid sum into *r.kl; no update.
template <typename T, int D, int kAttrGroup, int kAttrUnroll, bool kBlockGroups, bool kPipe, bool kKL = false>
FITSNE_D void attr_body(const uint32_t *__restrict__ row, const uint32_t *__restrict__ col,
                        const T *__restrict__ val, const T *__restrict__ Yin, T *__restrict__ Yout,
                        T *__restrict__ uY, T *__restrict__ gains, T *__restrict__ dC, const T *__restrict__ rep,
                        int row0, int N, const UpdateParams &p, RedScratch r, const float *__restrict__ yh,
                        double *sh, int *block_item, int blk, int nblk) {
    typedef typename YL<T, D>::P P;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int ngroups = (N + kAttrGroup - 1) / kAttrGroup;
    const unsigned int nwarps = (nblk * blockDim.x) >> 5;
    const double Zd = *r.z;
    const T zinv = T(1.0 / Zd);
    const T df = T(p.df);
    const bool df1 = (p.df == 1.0);
    const T exag = T(p.exag);
    P msum[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
        if constexpr (sizeof(T) == 4)
            msum[d] = {0.f, 0.f};
        else
            msum[d] = 0.0;
    }
    double klsum[1] = {0.0};  // kKL: this lane's terms
    while (true) {
        int g = 0;
        if constexpr (kBlockGroups) {
            __syncthreads();  // every warp has read the previous item
            if (threadIdx.x == 0) *block_item = (int) atomicAdd(r.count + 4, 1u);
            __syncthreads();
            const int wpb = blockDim.x >> 5;
            if (*block_item * wpb >= ngroups) break;  // uniform over the block
            g = *block_item * wpb + (threadIdx.x >> 5);
            if (g >= ngroups) continue;
        } else {
            if (lane == 0) g = (int) atomicAdd(r.count + 4, 1u);
            g = __shfl_sync(full, g, 0);
            if (g >= ngroups) break;
        }
        const int i0 = row0 + g * kAttrGroup;
        const int nr = min(kAttrGroup, row0 + N - i0);
        const int my = i0 + lane;
        const bool live = lane < nr;
        const uint32_t rb = live ? row[my] : 0u;
        const uint32_t re = live ? row[my + 1] : 0u;
        P cmy[D];
        if (live) {
            YL<T, D>::load(Yin, my, cmy);
        } else {
#pragma unroll
            for (int d = 0; d < D; ++d) cmy[d] = P{};
        }
        T amy[D];
#pragma unroll
        for (int d = 0; d < D; ++d) amy[d] = T(0);
        // one batch of kAttrUnroll edges per lane: CSR index and value, or (self, 0) past e1
        auto load_batch = [&](uint32_t base, uint32_t e1, int self, uint32_t (&jj)[kAttrUnroll],
                              T (&vv)[kAttrUnroll]) {
#pragma unroll
            for (int u = 0; u < kAttrUnroll; ++u) {
                const uint32_t e = base + lane + 32 * u;
                const bool ok = e < e1;
                jj[u] = ok ? __ldcs(col + e) : (uint32_t) self;
                vv[u] = ok ? __ldcs(val + e) : T(0);
            }
        };
        // pipelined shape: the next row's first batch is loaded while this row gathers
        uint32_t jn[kAttrUnroll];
        T vn[kAttrUnroll];
        if constexpr (kPipe) load_batch(__shfl_sync(full, rb, 0), __shfl_sync(full, re, 0), i0, jn, vn);
        for (int k = 0; k < nr; ++k) {
            const uint32_t e0 = __shfl_sync(full, rb, k), e1 = __shfl_sync(full, re, k);
            uint32_t jc[kAttrUnroll];
            T vc[kAttrUnroll];
            if constexpr (kPipe) {
#pragma unroll
                for (int u = 0; u < kAttrUnroll; ++u) {
                    jc[u] = jn[u];
                    vc[u] = vn[u];
                }
                if (k + 1 < nr)
                    load_batch(__shfl_sync(full, rb, k + 1), __shfl_sync(full, re, k + 1), i0 + k + 1, jn, vn);
            }
            if (k + 1 < nr) {
                // the next row's CSR lines into L2 (lanes 0-15 columns, 16-31 values)
                const uint32_t f0 = __shfl_sync(full, rb, k + 1), f1 = __shfl_sync(full, re, k + 1);
                if (f1 > f0) {
                    const char *lo = lane < 16 ? reinterpret_cast<const char *>(col + f0)
                                               : reinterpret_cast<const char *>(val + f0);
                    const char *hi = lane < 16 ? reinterpret_cast<const char *>(col + f1)
                                               : reinterpret_cast<const char *>(val + f1);
                    const uintptr_t l0 = reinterpret_cast<uintptr_t>(lo) & ~(uintptr_t) 127;
                    for (uintptr_t a = l0 + (uintptr_t) (lane & 15) * 128; a < reinterpret_cast<uintptr_t>(hi);
                         a += 16 * 128)
                        asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
                }
            }
            const int i = i0 + k;
            P ci[D];
#pragma unroll
            for (int d = 0; d < D; ++d) {
                if constexpr (sizeof(T) == 4)
                    ci[d] = {__shfl_sync(full, cmy[d].hi, k), __shfl_sync(full, cmy[d].lo, k)};
                else
                    ci[d] = __shfl_sync(full, cmy[d], k);
            }
            T a[D];
#pragma unroll
            for (int d = 0; d < D; ++d) a[d] = T(0);
            for (uint32_t base = e0; base < e1; base += 32 * kAttrUnroll) {
                uint32_t j[kAttrUnroll];
                T v[kAttrUnroll];
                if (kPipe && base == e0) {
#pragma unroll
                    for (int u = 0; u < kAttrUnroll; ++u) {
                        j[u] = jc[u];
                        v[u] = vc[u];
                    }
                } else {
                    load_batch(base, e1, i, j, v);
                }
                P cj[kAttrUnroll][D];
#pragma unroll
                for (int u = 0; u < kAttrUnroll; ++u) {
                    if constexpr (sizeof(T) == 4) {
                        if (yh) {  // FP32 neighbour positions (high words only): 8 instead of 16 bytes
                            if constexpr (D == 2) {
                                const float2 h = __ldg(reinterpret_cast<const float2 *>(yh) + j[u]);
                                cj[u][0] = {h.x, 0.f};
                                cj[u][1] = {h.y, 0.f};
                            } else {
                                cj[u][0] = {__ldg(yh + j[u]), 0.f};
                            }
                            continue;
                        }
                    }
                    YL<T, D>::load(Yin, (int) j[u], cj[u]);
                }
#pragma unroll
                for (int u = 0; u < kAttrUnroll; ++u) {
                    T dx[D];
                    T d2 = T(0);
#pragma unroll
                    for (int d = 0; d < D; ++d) {
                        dx[d] = pdiff(ci[d], cj[u][d]);
                        d2 += dx[d] * dx[d];
                    }
                    const T q = recip(df1 ? T(1) + d2 : T(1) + d2 / df);
                    if constexpr (kKL) {
                        const T Q = (df1 ? q : pow(q, df)) * zinv;
                        const T pv = v[u] * exag;
                        a[0] += pv * log((pv + T(FLT_MIN)) / (Q + T(FLT_MIN)));  // 0 past the row
                    } else {
                        const T vq = v[u] * q;
#pragma unroll
                        for (int d = 0; d < D; ++d) a[d] += vq * dx[d];
                    }
                }
            }
            if constexpr (kKL) {
                klsum[0] += (double) a[0];  // FP32 form: the row's terms of this lane, once
                continue;
            }
#pragma unroll
            for (int d = 0; d < D; ++d) {
                for (int o = 16; o; o >>= 1) a[d] += __shfl_xor_sync(full, a[d], o);
                if (lane == k) amy[d] = a[d];
            }
        }
        if (kKL || !live) continue;
        attr_row_update<T, D>(my, amy, cmy, p, zinv, exag, rep, dC, gains, uY, Yout, msum);
    }
    if constexpr (kKL) {
        if (lane == 0) {  // the work counter's reset, as attr_finish does it
            __threadfence();
            const unsigned int out = atomicAdd(r.count + 5, 1u);
            if (out == nwarps - 1) {
                atomicExch(r.count + 4, 0u);
                atomicExch(r.count + 5, 0u);
            }
        }
        if (grid_sum<1>(klsum, r.part, r.count + 3, sh, blk, nblk)) *r.kl = klsum[0];
        return;
    }
    attr_finish<T, D>(lane, nwarps, N, p, r, msum, sh, blk, nblk);
}

template <typename T, int D, int kAttrGroup, int kAttrUnroll, bool kBlockGroups = false, bool kPipe = false,
          int kMinBlocks = 1>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_attr(const uint32_t *__restrict__ row, const uint32_t *__restrict__ col,
                                                 const T *__restrict__ val, const T *__restrict__ Yin,
                                                 T *__restrict__ Yout, T *__restrict__ uY, T *__restrict__ gains,
                                                 T *__restrict__ dC, const T *__restrict__ rep, int N,
                                                 UpdateParams p, RedScratch r, const float *__restrict__ yh) {
    __shared__ double sh[2 * 32];
    __shared__ int block_item;
    attr_body<T, D, kAttrGroup, kAttrUnroll, kBlockGroups, kPipe>(row, col, val, Yin, Yout, uY, gains, dC, rep, 0, N,
                                                                  p, r, yh, sh, &block_item, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------------
// Tiled attraction over the half-stored symmetric P (FP32 form).
//
// After symmetrizeMatrix P is symmetric: the edge {i, j} is stored in row i and in row j with
// the same value, and the reference computes p q (y_i - y_j) from both ends, each end
// gathering the other's position.  That gather (one random L2 sector per non-zero) binds the
// full-CSR attraction: about one L1 wavefront per non-zero.
//
// Here the points (in the embedding's locality order) are cut into blocks of kTileRows; each
// undirected edge {i, j}, i < j, falls in the tile (A, B) = (block of i, block of j), A <= B,
// and is stored once as an 8-byte record (i mod kTileRows | (j mod kTileRows) << 16, p), the
// records sorted by tile and, within a tile, by row.  A CTA takes an equal share of the
// records and walks its tiles in order, keeping the double-float positions of blocks A and B
// and an FP32 force accumulator for each in shared memory: every edge reads both positions
// from shared memory, adds its force to row i (a segmented sum over the warp's lanes of equal
// i, then one shared-memory atomic) and subtracts it from row j (a shared-memory atomic).  An
// accumulator goes to the global one (red.global.add, non-zero entries only) when its block
// changes, so global reductions come per block switch, not per edge.  In the embedding's
// locality order the edges concentrate in few tiles (measured on a 100,000-point t-SNE
// embedding: 114 of the 325 tiles of 4,096-point blocks hold all of them, 65,000 edges per
// tile on average), so a CTA meets few block switches.  k_sym_update then applies the update
// and clears the accumulator.  Both ends use double-float positions, so y_i - y_j is as
// accurate as in the full-CSR form; the summation order differs (FP32 atomics).

// 64-bit mix of (row, column, value bits) for the symmetry check
FITSNE_D unsigned long long edge_hash(uint32_t a, uint32_t b, uint32_t v) {
    unsigned long long z = ((unsigned long long) a << 32 | b) ^ ((unsigned long long) v * 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// h[0] = sum of hash(i, j, p_ij), h[1] = sum of hash(j, i, p_ij) over the entries: equal
// (up to a 2^-64 chance) exactly when the multiset of entries equals its transpose.
__global__ void k_sym_hash(const uint32_t *__restrict__ row, const uint32_t *__restrict__ col,
                           const float *__restrict__ val, int N, unsigned long long *__restrict__ h) {
    const int lane = threadIdx.x & 31;
    unsigned long long a = 0, b = 0;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < N; i += (gridDim.x * blockDim.x) >> 5) {
        const uint32_t e1 = row[i + 1];
        for (uint32_t e = row[i] + lane; e < e1; e += 32) {
            const uint32_t j = col[e], v = __float_as_uint(val[e]);
            a += edge_hash((uint32_t) i, j, v);
            b += edge_hash(j, (uint32_t) i, v);
        }
    }
    for (int o = 16; o; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (lane == 0) {
        atomicAdd(h, a);
        atomicAdd(h + 1, b);
    }
}

// ulen[i] = number of entries of row i above the diagonal
__global__ void k_upper_count(const uint32_t *__restrict__ row, const uint32_t *__restrict__ col, int N,
                              uint32_t *__restrict__ ulen) {
    const int lane = threadIdx.x & 31;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < N; i += (gridDim.x * blockDim.x) >> 5) {
        uint32_t c = 0;
        const uint32_t e1 = row[i + 1];
        for (uint32_t e = row[i] + lane; e < e1; e += 32) c += (col[e] > (uint32_t) i) ? 1u : 0u;
        for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if (lane == 0) ulen[i] = c;
    }
}

FITSNE_D void red_add(float *a, const float (&v)[1]) { atomicAdd(a, v[0]); }
FITSNE_D void red_add(float *a, const float (&v)[2]) {
    atomicAdd(reinterpret_cast<float2 *>(a), make_float2(v[0], v[1]));
}

// The update of every point from its accumulated attraction (attr_row_update: gradient,
// gains, momentum, clipping, double-float Y), the accumulator cleared for the next
// iteration, and in mode 1 the grid sum of the new positions for the next centring.
template <int D>
__global__ void __launch_bounds__(kBlock)
    k_sym_update(float *__restrict__ acc, const float *__restrict__ Yin, float *__restrict__ Yout,
                 float *__restrict__ uY, float *__restrict__ gains, float *__restrict__ dC,
                 const float *__restrict__ rep, int N, UpdateParams p, RedScratch r) {
    __shared__ double sh[2 * 32];
    typedef df32 P;
    const float zinv = (float) (1.0 / *r.z);
    const float exag = (float) p.exag;
    P msum[D];
#pragma unroll
    for (int d = 0; d < D; ++d) msum[d] = {0.f, 0.f};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        float amy[D];
        if constexpr (D == 2) {
            const float2 v = reinterpret_cast<const float2 *>(acc)[i];
            amy[0] = v.x;
            amy[1] = v.y;
            reinterpret_cast<float2 *>(acc)[i] = make_float2(0.f, 0.f);
        } else {
            amy[0] = acc[i];
            acc[i] = 0.f;
        }
        P cmy[D];
        YL<float, D>::load(Yin, i, cmy);
        attr_row_update<float, D>(i, amy, cmy, p, zinv, exag, rep, dC, gains, uY, Yout, msum);
    }
    if (p.mode != 0) {
        double m[2] = {0.0, 0.0};
        df32 v[2] = {msum[0], D == 2 ? msum[D - 1] : df32{0.f, 0.f}};
        block_sum_df<2>(v, m, sh);
        if (grid_sum_finish<2>(m, r.part, r.count + 2, sh, blockIdx.x, gridDim.x)) {
            r.mean[0] = m[0] / (double) N;
            r.mean[1] = m[1] / (double) N;
        }
    }
}

constexpr int kTileShift = 12;
constexpr int kTileRows = 1 << kTileShift;
constexpr int kTileThreads = 1024;

// per upper entry (a warp per row, ballot compaction, row order): its tile key A * nblk + B,
// its index, and its record; tile sizes counted into tcount
__global__ void k_tile_keys(const uint32_t *__restrict__ row, const uint32_t *__restrict__ col,
                            const float *__restrict__ val, int N, int nblk, const uint32_t *__restrict__ urow,
                            uint32_t *__restrict__ keys, uint32_t *__restrict__ ids, uint2 *__restrict__ rec,
                            uint32_t *__restrict__ tcount) {
    const int lane = threadIdx.x & 31;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < N; i += (gridDim.x * blockDim.x) >> 5) {
        uint32_t out = urow[i];
        const uint32_t e0 = row[i], e1 = row[i + 1];
        const uint32_t A = (uint32_t) i >> kTileShift;
        for (uint32_t base = e0; base < e1; base += 32) {
            const uint32_t e = base + lane;
            const bool ok = e < e1;
            const uint32_t j = ok ? col[e] : 0u;
            const bool up = ok && j > (uint32_t) i;
            const unsigned m = __ballot_sync(0xffffffffu, up);
            if (up) {
                const uint32_t k = out + __popc(m & ((1u << lane) - 1u));
                const uint32_t key = A * (uint32_t) nblk + (j >> kTileShift);
                keys[k] = key;
                ids[k] = k;
                rec[k] = make_uint2(((uint32_t) i & (kTileRows - 1)) | ((j & (kTileRows - 1)) << 16),
                                    __float_as_uint(val[e]));
                atomicAdd(tcount + key, 1u);
            }
            out += __popc(m);
        }
    }
}

__global__ void k_tile_gather(const uint2 *__restrict__ rec, const uint32_t *__restrict__ ids, size_t n,
                              uint2 *__restrict__ trec) {
    for (size_t k = blockIdx.x * (size_t) blockDim.x + threadIdx.x; k < n; k += (size_t) gridDim.x * blockDim.x)
        trec[k] = rec[ids[k]];
}

template <int D>
struct TileYL;
template <>
struct TileYL<2> {
    typedef float4 V;  // {x_hi, y_hi, x_lo, y_lo}
    static FITSNE_D void split(const V &v, df32 (&c)[2]) {
        c[0] = {v.x, v.z};
        c[1] = {v.y, v.w};
    }
};
template <>
struct TileYL<1> {
    typedef float2 V;  // {hi, lo}
    static FITSNE_D void split(const V &v, df32 (&c)[1]) { c[0] = {v.x, v.y}; }
};

template <int D>
FITSNE_D void tile_load(typename TileYL<D>::V *ys, float *as, const float *__restrict__ Yin, int blk, int N) {
    typedef typename TileYL<D>::V V;
    const V *src = reinterpret_cast<const V *>(Yin);
    for (int k = threadIdx.x; k < kTileRows; k += blockDim.x) {
        const int g = blk * kTileRows + k;
        V v{};
        if (g < N) v = src[g];
        ys[k] = v;
#pragma unroll
        for (int d = 0; d < D; ++d) as[k * D + d] = 0.f;
    }
}

template <int D>
FITSNE_D void tile_flush(const float *as, float *__restrict__ acc, int blk, int N) {
    for (int k = threadIdx.x; k < kTileRows; k += blockDim.x) {
        const int g = blk * kTileRows + k;
        if (g >= N) break;
        float v[D];
        bool nz = false;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            v[d] = as[k * D + d];
            nz |= (v[d] != 0.f);
        }
        if (nz) red_add(acc + (size_t) g * D, v);
    }
}

template <int D, int kUnroll>
__global__ void __launch_bounds__(kTileThreads, 1)
    k_attr_tiles(const uint2 *__restrict__ trec, const uint32_t *__restrict__ tstart, int nkeys, int nblk,
                 const float *__restrict__ Yin, float *__restrict__ acc, int N, float df, int df1) {
    typedef typename TileYL<D>::V V;
    typedef df32 P;
    extern __shared__ __align__(16) unsigned char tsm[];
    V *yA = reinterpret_cast<V *>(tsm);
    V *yB = yA + kTileRows;
    float *aA = reinterpret_cast<float *>(yB + kTileRows);
    float *aB = aA + kTileRows * D;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const long long nrec = tstart[nkeys];
    const long long e0 = nrec * blockIdx.x / gridDim.x, e1 = nrec * (blockIdx.x + 1) / gridDim.x;
    if (e0 >= e1) return;  // uniform over the block
    // the tile holding e0: the last key whose start is <= e0
    int lo = 0, hi = nkeys;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if ((long long) tstart[mid] <= e0)
            lo = mid;
        else
            hi = mid;
    }
    int key = lo;
    int curA = -1, curB = -1;
    bool bdirty = false;
    long long e = e0;
    while (e < e1) {
        while ((long long) tstart[key + 1] <= e) ++key;  // empty tiles
        const int A = key / nblk, B = key % nblk;
        const long long te = min((long long) tstart[key + 1], e1);
        if (A != curA || (B != A && B != curB)) {
            __syncthreads();  // the previous tile's accumulations are complete
            if (A != curA) {
                if (curA >= 0) tile_flush<D>(aA, acc, curA, N);
                if (curB == A) {  // the new row block was the column block: flush it first
                    if (bdirty) tile_flush<D>(aB, acc, curB, N);
                    bdirty = false;
                    curB = -1;
                }
                tile_load<D>(yA, aA, Yin, A, N);
                curA = A;
            }
            if (B != A && B != curB) {
                if (curB >= 0 && bdirty) tile_flush<D>(aB, acc, curB, N);
                tile_load<D>(yB, aB, Yin, B, N);
                curB = B;
                bdirty = false;
            }
            __syncthreads();
        }
        const bool diag = (A == B);
        if (!diag) bdirty = true;
        const V *yJ = diag ? yA : yB;
        float *aJ = diag ? aA : aB;
        for (long long base = e + (long long) warp * 32 * kUnroll; base < te; base += (long long) nw * 32 * kUnroll) {
            uint2 r[kUnroll];
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) {
                const long long k = base + 32 * u + lane;
                r[u] = k < te ? __ldcs(trec + k) : make_uint2(0xffffffffu, 0u);
            }
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) {
                const bool ok = r[u].x != 0xffffffffu;
                const int li = (int) (r[u].x & 0xffffu), lj = (int) (r[u].x >> 16);
                float f[D];
#pragma unroll
                for (int d = 0; d < D; ++d) f[d] = 0.f;
                if (ok) {
                    P ci[D], cj[D];
                    TileYL<D>::split(yA[li], ci);
                    TileYL<D>::split(yJ[lj], cj);
                    float dx[D];
                    float d2 = 0.f;
#pragma unroll
                    for (int d = 0; d < D; ++d) {
                        dx[d] = pdiff(ci[d], cj[d]);
                        d2 += dx[d] * dx[d];
                    }
                    const float vq = __uint_as_float(r[u].y) * recip(df1 ? 1.f + d2 : 1.f + d2 / df);
#pragma unroll
                    for (int d = 0; d < D; ++d) {
                        f[d] = vq * dx[d];
                        atomicAdd(aJ + lj * D + d, -f[d]);
                    }
                }
                // row i: lanes of equal i are consecutive (records in row order within a tile)
                const int seg = ok ? li : (0x10000 + lane);
                const int prev = __shfl_up_sync(full, seg, 1);
                const unsigned heads = __ballot_sync(full, lane == 0 || prev != seg);
                const int my_head = 31 - __clz(heads & (full >> (31 - lane)));
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
#pragma unroll
                    for (int d = 0; d < D; ++d) {
                        const float y = __shfl_up_sync(full, f[d], off);
                        if (lane - off >= my_head) f[d] += y;
                    }
                }
                const int next = __shfl_down_sync(full, seg, 1);
                if (ok && (lane == 31 || next != seg)) {
#pragma unroll
                    for (int d = 0; d < D; ++d) atomicAdd(aA + li * D + d, f[d]);
                }
            }
        }
        e = te;
    }
    __syncthreads();
    if (curA >= 0) tile_flush<D>(aA, acc, curA, N);
    if (curB >= 0 && bdirty) tile_flush<D>(aB, acc, curB, N);
}

// ---------------------------------------------------------------------------------
// KL divergence over the CSR edges (evaluateErrorFft, tsne.cpp:1329-1355)
template <typename T, int D>
FITSNE_D void kl_body(const uint32_t *__restrict__ row, const uint32_t *__restrict__ col, const T *__restrict__ val,
                      const T *__restrict__ Y, int row0, int N, double exag, double dfd, RedScratch r, double *sh,
                      int blk, int nblk) {
    typedef typename YL<T, D>::P P;
    const int lane = threadIdx.x & 31;
    const int gw = (blk * blockDim.x + threadIdx.x) >> 5;
    const int nw = (nblk * blockDim.x) >> 5;
    const T zinv = T(1.0 / *r.z);
    const T df = T(dfd);
    const T ex = T(exag);
    const bool df1 = dfd == 1.0;
    double acc[1] = {0.0};
    for (int i = row0 + gw; i < row0 + N; i += nw) {
        P ci[D];
        YL<T, D>::load(Y, i, ci);
        const uint32_t e1 = row[i + 1];
        // FP32 form: a lane's terms of the row (about five) add up in FP32, then once into
        // the FP64 sum (one conversion and FP64 add per row and lane instead of per edge; the
        // FP64 pipe runs at a small fraction of the FP32 rate)
        T racc = T(0);
        for (uint32_t e = row[i] + lane; e < e1; e += 32) {
            P cj[D];
            YL<T, D>::load(Y, (int) col[e], cj);
            T d2 = T(0);
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const T dx = pdiff(ci[d], cj[d]);
                d2 += dx * dx;
            }
            // 1 / (1 + d2 / df), the same value in fewer instructions for df = 1
            const T base = df1 ? recip(T(1) + d2) : T(1) / (T(1) + d2 / df);
            const T Q = (df1 ? base : pow(base, df)) * zinv;
            const T pv = val[e] * ex;
            const T term = pv * log((pv + T(FLT_MIN)) / (Q + T(FLT_MIN)));
            if constexpr (sizeof(T) == 4)
                racc += term;
            else
                acc[0] += (double) term;
        }
        if constexpr (sizeof(T) == 4) acc[0] += (double) racc;
    }
    if (grid_sum<1>(acc, r.part, r.count + 3, sh, blk, nblk)) *r.kl = acc[0];
}

// KL over the CSR in the attraction's traversal (groups of 16 rows from the work counter, two
// edges per lane per batch, the next row's CSR lines prefetched): 1.15 ms at N = 1M with a warp
// per row and lanes striding its edges.  p: exag and df.
template <typename T, int D>
__global__ void __launch_bounds__(kBlock, 4) k_kl_rows(const uint32_t *__restrict__ row,
                                                       const uint32_t *__restrict__ col, const T *__restrict__ val,
                                                       const T *__restrict__ Y, int N, UpdateParams p, RedScratch r) {
    __shared__ double sh[2 * 32];
    __shared__ int block_item;
    attr_body<T, D, 16, 2, false, false, true>(row, col, val, Y, nullptr, nullptr, nullptr, nullptr, nullptr, 0, N, p,
                                               r, nullptr, sh, &block_item, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------------------------
template <typename T, int D>
__global__ void k_y_from_double(const double *__restrict__ src, T *__restrict__ Y, int N) {
    typedef typename YL<T, D>::P P;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        P c[D];
#pragma unroll
        for (int d = 0; d < D; ++d) {
            if constexpr (sizeof(T) == 4)
                c[d] = df_from_double(src[(size_t) i * D + d]);
            else
                c[d] = src[(size_t) i * D + d];
        }
        YL<T, D>::store(Y, i, c);
    }
}
template <typename T, int D>
__global__ void k_y_to_double(const T *__restrict__ Y, double *__restrict__ dst, int N) {
    typedef typename YL<T, D>::P P;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        P c[D];
        YL<T, D>::load(Y, i, c);
#pragma unroll
        for (int d = 0; d < D; ++d) dst[(size_t) i * D + d] = ptod(c[d]);
    }
}
template <typename T>
__global__ void k_cast(const double *__restrict__ src, T *__restrict__ dst, size_t n) {
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n; i += (size_t) gridDim.x * blockDim.x)
        dst[i] = (T) src[i];
}

inline int grid_for(long long n, int per_block, int cap) {
    long long g = (n + per_block - 1) / per_block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int) g;
}

}  // namespace

template <typename T>
cudaError_t launch_center_minmax(T *Y, int N, int D, int apply_mean, int excl, RedScratch r, cudaStream_t st) {
    const int g = grid_for(N, kBlock, kRedGrid);
    if (D == 2)
        k_center_minmax<T, 2><<<g, kBlock, 0, st>>>(Y, N, apply_mean, excl, r);
    else
        k_center_minmax<T, 1><<<g, kBlock, 0, st>>>(Y, N, apply_mean, excl, r);
    return cudaGetLastError();
}

template <typename T>
cudaError_t spread_impl(const T *Y, int N, int D, int nterms, const BoxP<T> &b, Cell4<T> *grid, const DevGeom *dg,
                        cudaStream_t st, const uint32_t *order = nullptr) {
    const int g = grid_for(N, kBlock, 1 << 20);
    if constexpr (sizeof(T) == 4) {
        if (nterms == 3) {
            if (D == 2)
                k_spread_runs<2><<<g, kBlock, 0, st>>>(Y, N, b, grid, dg, order);
            else
                k_spread_runs<1><<<g, kBlock, 0, st>>>(Y, N, b, grid, dg, order);
            return cudaGetLastError();
        }
    }
    if (D == 2) {
        if (nterms == 3)
            k_spread<T, 2, 3><<<g, kBlock, 0, st>>>(Y, N, b, grid, dg);
        else
            k_spread<T, 2, 0><<<g, kBlock, 0, st>>>(Y, N, b, grid, dg);
    } else {
        if (nterms == 3)
            k_spread<T, 1, 3><<<g, kBlock, 0, st>>>(Y, N, b, grid, dg);
        else
            k_spread<T, 1, 0><<<g, kBlock, 0, st>>>(Y, N, b, grid, dg);
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_spread(const T *Y, int N, int D, const GridGeom &gg, Cell4<T> *grid, cudaStream_t st,
                          const uint32_t *order) {
    return spread_impl<T>(Y, N, D, gg.nterms, make_box(gg, (T *) nullptr), grid, nullptr, st, order);
}

template <typename T>
cudaError_t launch_spread_dev(const T *Y, int N, int D, int nterms, const DevGeom *dg, Cell4<T> *grid,
                              cudaStream_t st, const uint32_t *order) {
    BoxP<T> b{};
    b.nterms = nterms;
    return spread_impl<T>(Y, N, D, nterms, b, grid, dg, st, order);
}

template <typename T>
cudaError_t gather_impl(const T *Y, int N, int D, int nterms, const BoxP<T> &b, const Cell4<T> *pot, int mode, T *rep,
                        RedScratch r, const DevGeom *dg, float *yh, cudaStream_t st) {
    const int g = grid_for(N, kBlock, kRedGrid);
    if (D == 2) {
        if (nterms == 3)
            k_gather<T, 2, 3><<<g, kBlock, 0, st>>>(Y, N, b, pot, mode, rep, r, dg, yh);
        else
            k_gather<T, 2, 0><<<g, kBlock, 0, st>>>(Y, N, b, pot, mode, rep, r, dg, yh);
    } else {
        if (nterms == 3)
            k_gather<T, 1, 3><<<g, kBlock, 0, st>>>(Y, N, b, pot, mode, rep, r, dg, yh);
        else
            k_gather<T, 1, 0><<<g, kBlock, 0, st>>>(Y, N, b, pot, mode, rep, r, dg, yh);
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_gather(const T *Y, int N, int D, const GridGeom &gg, const Cell4<T> *pot, int mode, T *rep,
                          RedScratch r, cudaStream_t st, float *yh) {
    return gather_impl<T>(Y, N, D, gg.nterms, make_box(gg, (T *) nullptr), pot, mode, rep, r, nullptr, yh, st);
}

template <typename T>
cudaError_t launch_gather_dev(const T *Y, int N, int D, int nterms, const DevGeom *dg, const Cell4<T> *pot, int mode,
                              T *rep, RedScratch r, cudaStream_t st, float *yh) {
    BoxP<T> b{};
    b.nterms = nterms;
    return gather_impl<T>(Y, N, D, nterms, b, pot, mode, rep, r, dg, yh, st);
}

namespace {
// Sizes the grid of this iteration from the min / max that k_center_minmax left in r.mnmx
// (the host rule of make_grid_geom, in the same FP64 operations) and ORs its status into
// *status_acc.  A grid above the capacity is clamped to it so that every kernel stays in
// its buffers; the iteration is then void and the caller repeats it with a larger one.
FITSNE_D void geometry_one(const RedScratch &r, int D, int nterms, double ipi, int min_num, int nb_cap, int L_cap,
                          DevGeom *__restrict__ dg, int *__restrict__ status_acc) {
    double mn = r.mnmx[0], mx = r.mnmx[1];
    int status = 0;
    if (!isfinite(mn) || !isfinite(mx)) {
        status = 2;
        mn = 0.0;
        mx = 1.0;
    }
    int clamped = 0;
    GridGeom g = grid_geom(mn, mx, D, nterms, ipi, min_num, nb_cap, &clamped);
    int L = smooth_even_at_least(2 * g.M);
    if (clamped || L > L_cap) {
        status = status ? status : 1;
        while (L > L_cap && g.nb > 1) {  // shrink until it fits (results void anyway)
            g = grid_geom(mn, mx, D, nterms, ipi, min_num, g.nb - 1, &clamped);
            L = smooth_even_at_least(2 * g.M);
        }
    }
    dg->g = g;
    dg->conv.M = g.M;
    dg->conv.h = g.hk;
    make_fft_plan(L, &dg->conv.plan);
    dg->status = status;
    if (status) atomicOr(status_acc, status == 2 ? 2 : 1);
}

__global__ void k_geometry(RedScratch r, int D, int nterms, double ipi, int min_num, int nb_cap, int L_cap,
                           DevGeom *__restrict__ dg, int *__restrict__ status_acc) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    geometry_one(r, D, nterms, ipi, min_num, nb_cap, L_cap, dg, status_acc);
}
}  // namespace

cudaError_t launch_geometry(RedScratch r, int D, int nterms, double ipi, int min_num, int nb_cap, int L_cap,
                            DevGeom *dg, int *status_acc, cudaStream_t st) {
    k_geometry<<<1, 32, 0, st>>>(r, D, nterms, ipi, min_num, nb_cap, L_cap, dg, status_acc);
    return cudaGetLastError();
}

template <typename T, int D, int G, int U, bool B = false, bool PP = false, int MB = 1>
cudaError_t attr_launch(const uint32_t *row, const uint32_t *col, const T *val, const T *Yin, T *Yout, T *uY,
                        T *gains, T *dC, const T *rep, int N, const UpdateParams &p, RedScratch r, cudaStream_t st,
                        const float *yh) {
    // one resident wave: the warps take row groups from a counter
    static int wave = 0;
    if (wave == 0) {
        int dev = 0, nsm = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        cudaError_t e =
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_attr<T, D, G, U, B, PP, MB>, kBlock, 0);
        if (e != cudaSuccess) return e;
        wave = std::min(kMaxRedBlocks, nsm * (per_sm > 0 ? per_sm : 1));
    }
    const int g = grid_for(((long long) N + 31) / 32 * 32, kBlock, wave);
    k_attr<T, D, G, U, B, PP, MB><<<g, kBlock, 0, st>>>(row, col, val, Yin, Yout, uY, gains, dC, rep, N, p, r, yh);
    return cudaGetLastError();
}

template <typename T, int D>
cudaError_t attr_dispatch(int shape, const uint32_t *row, const uint32_t *col, const T *val, const T *Yin, T *Yout,
                          T *uY, T *gains, T *dC, const T *rep, int N, const UpdateParams &p, RedScratch r,
                          cudaStream_t st, const float *yh) {
    switch (shape) {
        case 1: return attr_launch<T, D, 32, 4>(row, col, val, Yin, Yout, uY, gains, dC, rep, N, p, r, st, yh);
        case 2: return attr_launch<T, D, 8, 4>(row, col, val, Yin, Yout, uY, gains, dC, rep, N, p, r, st, yh);
        case 3: return attr_launch<T, D, 16, 2>(row, col, val, Yin, Yout, uY, gains, dC, rep, N, p, r, st, yh);
        case 4: return attr_launch<T, D, 32, 2>(row, col, val, Yin, Yout, uY, gains, dC, rep, N, p, r, st, yh);
        case 5: return attr_launch<T, D, 16, 4, true>(row, col, val, Yin, Yout, uY, gains, dC, rep, N, p, r, st, yh);
        case 6:
            return attr_launch<T, D, 16, 4, false, true>(row, col, val, Yin, Yout, uY, gains, dC, rep, N, p, r, st, yh);
        case 7:
            return attr_launch<T, D, 16, 4, false, false, 6>(row, col, val, Yin, Yout, uY, gains, dC, rep, N, p, r,
                                                            st, yh);
        case 8:
            return attr_launch<T, D, 8, 4, false, false, 6>(row, col, val, Yin, Yout, uY, gains, dC, rep, N, p, r,
                                                           st, yh);
        case 9: return attr_launch<T, D, 16, 5>(row, col, val, Yin, Yout, uY, gains, dC, rep, N, p, r, st, yh);
        case 10:
            return attr_launch<T, D, 16, 2, false, false, 6>(row, col, val, Yin, Yout, uY, gains, dC, rep, N, p, r,
                                                            st, yh);

        default: return attr_launch<T, D, 16, 4>(row, col, val, Yin, Yout, uY, gains, dC, rep, N, p, r, st, yh);
    }
}

template <typename T>
cudaError_t launch_attr_update(const uint32_t *row, const uint32_t *col, const T *val, const T *Yin, T *Yout,
                               T *uY, T *gains, T *dC, const T *rep, int N, int D, const UpdateParams &p,
                               RedScratch r, cudaStream_t st, int shape, const float *yh) {
    if (D == 2) return attr_dispatch<T, 2>(shape, row, col, val, Yin, Yout, uY, gains, dC, rep, N, p, r, st, yh);
    return attr_dispatch<T, 1>(shape, row, col, val, Yin, Yout, uY, gains, dC, rep, N, p, r, st, yh);
}

int attr_shape_info(int shape, int *group, int *unroll) {
    if (shape < 0 || shape >= kNumAttrShapes) return -1;
    *group = kAttrShapes[shape][0];
    *unroll = kAttrShapes[shape][1];
    return 0;
}

cudaError_t launch_sym_hash(const uint32_t *row, const uint32_t *col, const float *val, int N,
                            unsigned long long *h, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(h, 0, 2 * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    k_sym_hash<<<grid_for((long long) N * 32, kBlock, 4096), kBlock, 0, st>>>(row, col, val, N, h);
    return cudaGetLastError();
}

cudaError_t launch_upper_count(const uint32_t *row, const uint32_t *col, int N, uint32_t *ulen, cudaStream_t st) {
    k_upper_count<<<grid_for((long long) N * 32, kBlock, 4096), kBlock, 0, st>>>(row, col, N, ulen);
    return cudaGetLastError();
}

size_t tile_smem_bytes(int D) {
    return (size_t) kTileRows * ((D == 2 ? sizeof(float4) : sizeof(float2)) * 2 + sizeof(float) * D * 2);
}

int tile_blocks(int N) { return (N + kTileRows - 1) / kTileRows; }

cudaError_t launch_tile_keys(const uint32_t *row, const uint32_t *col, const float *val, int N, const uint32_t *urow,
                             uint32_t *keys, uint32_t *ids, uint2 *rec, uint32_t *tcount, cudaStream_t st) {
    k_tile_keys<<<grid_for((long long) N * 32, kBlock, 4096), kBlock, 0, st>>>(row, col, val, N, tile_blocks(N), urow,
                                                                              keys, ids, rec, tcount);
    return cudaGetLastError();
}

cudaError_t launch_tile_gather(const uint2 *rec, const uint32_t *ids, size_t n, uint2 *trec, cudaStream_t st) {
    k_tile_gather<<<4096, kBlock, 0, st>>>(rec, ids, n, trec);
    return cudaGetLastError();
}

template <int D, int U>
cudaError_t attr_tiles_launch(const uint2 *trec, const uint32_t *tstart, int N, const float *Yin, float *acc,
                              double df, cudaStream_t st) {
    static int nsm = 0;
    const size_t smem = tile_smem_bytes(D);
    if (nsm == 0) {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        cudaError_t e = cudaFuncSetAttribute(k_attr_tiles<D, U>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int) smem);
        if (e != cudaSuccess) return e;
        nsm = n;
    }
    const int nblk = tile_blocks(N);
    k_attr_tiles<D, U><<<nsm, kTileThreads, smem, st>>>(trec, tstart, nblk * nblk, nblk, Yin, acc, N, (float) df,
                                                         df == 1.0 ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_attr_tiles_update(const uint2 *trec, const uint32_t *tstart, float *acc, const float *Yin,
                                     float *Yout, float *uY, float *gains, float *dC, const float *rep, int N, int D,
                                     const UpdateParams &p, RedScratch r, cudaStream_t st) {
    cudaError_t e = (D == 2) ? attr_tiles_launch<2, 4>(trec, tstart, N, Yin, acc, p.df, st)
                             : attr_tiles_launch<1, 4>(trec, tstart, N, Yin, acc, p.df, st);
    if (e != cudaSuccess) return e;
    const int g = grid_for(N, kBlock, kRedGrid);
    if (D == 2)
        k_sym_update<2><<<g, kBlock, 0, st>>>(acc, Yin, Yout, uY, gains, dC, rep, N, p, r);
    else
        k_sym_update<1><<<g, kBlock, 0, st>>>(acc, Yin, Yout, uY, gains, dC, rep, N, p, r);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_kl(const uint32_t *row, const uint32_t *col, const T *val, const T *Y, int N, int D, double exag,
                      double df, RedScratch r, cudaStream_t st) {
    UpdateParams p{};
    p.exag = exag;
    p.df = df;
    // one resident wave: the warps take row groups from the work counter
    static int wave[2] = {0, 0};
    int &w = wave[D == 2 ? 1 : 0];
    if (w == 0) {
        int dev = 0, nsm = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        const cudaError_t e = D == 2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_kl_rows<T, 2>, kBlock, 0)
                                     : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_kl_rows<T, 1>, kBlock, 0);
        if (e != cudaSuccess) return e;
        w = std::min(kMaxRedBlocks, nsm * (per_sm > 0 ? per_sm : 1));
    }
    const int g = grid_for(((long long) N + 31) / 32 * 32, kBlock, w);
    if (D == 2)
        k_kl_rows<T, 2><<<g, kBlock, 0, st>>>(row, col, val, Y, N, p, r);
    else
        k_kl_rows<T, 1><<<g, kBlock, 0, st>>>(row, col, val, Y, N, p, r);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_y_from_double(const double *src, T *Y, int N, int D, cudaStream_t st) {
    const int g = grid_for(N, kBlock, 4096);
    if (D == 2)
        k_y_from_double<T, 2><<<g, kBlock, 0, st>>>(src, Y, N);
    else
        k_y_from_double<T, 1><<<g, kBlock, 0, st>>>(src, Y, N);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_y_to_double(const T *Y, double *dst, int N, int D, cudaStream_t st) {
    const int g = grid_for(N, kBlock, 4096);
    if (D == 2)
        k_y_to_double<T, 2><<<g, kBlock, 0, st>>>(Y, dst, N);
    else
        k_y_to_double<T, 1><<<g, kBlock, 0, st>>>(Y, dst, N);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_cast_from_double(const double *src, T *dst, size_t n, cudaStream_t st) {
    const int g = grid_for((long long) n, kBlock, 8192);
    k_cast<T><<<g, kBlock, 0, st>>>(src, dst, n);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------------
// Batched stages: a thin wrapper per stage finds the block's job and runs the single-job body
// on that job's slice of the concatenated arrays, with the job's own geometry and reduction
// scratch, over the job's share of the launch's blocks.
namespace {
constexpr int kBatchGroup = 16;   // attraction: rows per work item
constexpr int kBatchUnroll = 2;   //             edges per lane per batch

template <int D>
__global__ void __launch_bounds__(kBlock) k_bcenter(float *Y, BatchMap m, const BatchJobDev *__restrict__ jobs,
                                                    const RedScratch *__restrict__ rs, int apply_mean) {
    __shared__ double sh[2 * 32];
    const int j = m.job[blockIdx.x];
    const BatchJobDev jb = jobs[j];
    // excl = 0: the job's first point (the batched form keeps the caller's numbering)
    center_minmax_body<float, D>(Y + (size_t) jb.p0 * (2 * D), jb.n, apply_mean, 0, rs[j], sh,
                                 (int) blockIdx.x - m.first[j], m.count[j]);
}

__global__ void k_bgeometry(const RedScratch *__restrict__ rs, const BatchJobDev *__restrict__ jobs, int J, int D,
                            int nterms, double ipi, int min_num, DevGeom *__restrict__ dg, int *__restrict__ status) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= J) return;
    geometry_one(rs[j], D, nterms, ipi, min_num, jobs[j].nb_cap, jobs[j].L_cap, &dg[j], &status[j]);
}

template <int D>
__global__ void __launch_bounds__(kBlock) k_bspread(const float *__restrict__ Y, BatchMap m,
                                                    const BatchJobDev *__restrict__ jobs,
                                                    const DevGeom *__restrict__ dg, Cell4<float> *__restrict__ grid) {
    const int j = m.job[blockIdx.x];
    const BatchJobDev jb = jobs[j];
    const BoxP<float> b = make_box(dg[j].g, (float *) nullptr);
    spread_runs_body<D>(Y + (size_t) jb.p0 * (2 * D), jb.n, b, grid + jb.cell0, (int) blockIdx.x - m.first[j],
                        m.count[j]);
}

template <int D>
__global__ void __launch_bounds__(kBlock) k_bgather(const float *__restrict__ Y, BatchMap m,
                                                    const BatchJobDev *__restrict__ jobs,
                                                    const DevGeom *__restrict__ dg,
                                                    const Cell4<float> *__restrict__ pot, float *__restrict__ rep,
                                                    const RedScratch *__restrict__ rs, float *__restrict__ yh) {
    __shared__ double sh[32];
    const int j = m.job[blockIdx.x];
    const BatchJobDev jb = jobs[j];
    const BoxP<float> b = make_box(dg[j].g, (float *) nullptr);
    gather_body<float, D, 3>(Y + (size_t) jb.p0 * (2 * D), jb.n, b, pot + jb.cell0, KERNEL_DF1,
                             rep + (size_t) jb.p0 * D, rs[j], yh + (size_t) jb.p0 * D, sh,
                             (int) blockIdx.x - m.first[j], m.count[j]);
}

template <int D>
__global__ void __launch_bounds__(kBlock, 6) k_battr(const uint32_t *__restrict__ row, const uint32_t *__restrict__ col,
                                                  const float *__restrict__ val, const float *__restrict__ Yin,
                                                  float *__restrict__ Yout, float *__restrict__ uY,
                                                  float *__restrict__ gains, const float *__restrict__ rep,
                                                  BatchMap m, const BatchJobDev *__restrict__ jobs,
                                                  const RedScratch *__restrict__ rs, UpdateParams p,
                                                  const float *__restrict__ yh) {
    __shared__ double sh[2 * 32];
    __shared__ int block_item;
    const int j = m.job[blockIdx.x];
    const BatchJobDev jb = jobs[j];
    p.learning_rate = jb.lr;
    attr_body<float, D, kBatchGroup, kBatchUnroll, false, false>(row, col, val, Yin, Yout, uY, gains, nullptr, rep,
                                                                 jb.p0, jb.n, p, rs[j], yh, sh, &block_item,
                                                                 (int) blockIdx.x - m.first[j], m.count[j]);
}

template <int D>
__global__ void __launch_bounds__(kBlock) k_bkl(const uint32_t *__restrict__ row, const uint32_t *__restrict__ col,
                                                const float *__restrict__ val, const float *__restrict__ Y,
                                                BatchMap m, const BatchJobDev *__restrict__ jobs, double exag,
                                                const RedScratch *__restrict__ rs) {
    __shared__ double sh[32];
    const int j = m.job[blockIdx.x];
    const BatchJobDev jb = jobs[j];
    kl_body<float, D>(row, col, val, Y, jb.p0, jb.n, exag, 1.0, rs[j], sh, (int) blockIdx.x - m.first[j],
                      m.count[j]);
}
}  // namespace

cudaError_t launch_batch_center(float *Y, int D, BatchMap m, int nblocks, const BatchJobDev *jobs,
                                const RedScratch *rs, int apply_mean, cudaStream_t st) {
    if (D == 2)
        k_bcenter<2><<<nblocks, kBlock, 0, st>>>(Y, m, jobs, rs, apply_mean);
    else
        k_bcenter<1><<<nblocks, kBlock, 0, st>>>(Y, m, jobs, rs, apply_mean);
    return cudaGetLastError();
}

cudaError_t launch_batch_geometry(const RedScratch *rs, const BatchJobDev *jobs, int J, int D, int nterms,
                                  double ipi, int min_num, DevGeom *dg, int *status, cudaStream_t st) {
    k_bgeometry<<<(J + 31) / 32, 32, 0, st>>>(rs, jobs, J, D, nterms, ipi, min_num, dg, status);
    return cudaGetLastError();
}

cudaError_t launch_batch_spread(const float *Y, int D, BatchMap m, int nblocks, const BatchJobDev *jobs,
                                const DevGeom *dg, Cell4<float> *grid, cudaStream_t st) {
    if (D == 2)
        k_bspread<2><<<nblocks, kBlock, 0, st>>>(Y, m, jobs, dg, grid);
    else
        k_bspread<1><<<nblocks, kBlock, 0, st>>>(Y, m, jobs, dg, grid);
    return cudaGetLastError();
}

cudaError_t launch_batch_gather(const float *Y, int D, BatchMap m, int nblocks, const BatchJobDev *jobs,
                                const DevGeom *dg, const Cell4<float> *pot, float *rep, const RedScratch *rs,
                                float *yh, cudaStream_t st) {
    if (D == 2)
        k_bgather<2><<<nblocks, kBlock, 0, st>>>(Y, m, jobs, dg, pot, rep, rs, yh);
    else
        k_bgather<1><<<nblocks, kBlock, 0, st>>>(Y, m, jobs, dg, pot, rep, rs, yh);
    return cudaGetLastError();
}

cudaError_t launch_batch_attr(const uint32_t *row, const uint32_t *col, const float *val, const float *Yin,
                              float *Yout, float *uY, float *gains, const float *rep, int D, BatchMap m,
                              int nblocks, const BatchJobDev *jobs, const RedScratch *rs, const UpdateParams &p,
                              const float *yh, cudaStream_t st) {
    if (D == 2)
        k_battr<2><<<nblocks, kBlock, 0, st>>>(row, col, val, Yin, Yout, uY, gains, rep, m, jobs, rs, p, yh);
    else
        k_battr<1><<<nblocks, kBlock, 0, st>>>(row, col, val, Yin, Yout, uY, gains, rep, m, jobs, rs, p, yh);
    return cudaGetLastError();
}

cudaError_t launch_batch_kl(const uint32_t *row, const uint32_t *col, const float *val, const float *Y, int D,
                            BatchMap m, int nblocks, const BatchJobDev *jobs, double exag, const RedScratch *rs,
                            cudaStream_t st) {
    if (D == 2)
        k_bkl<2><<<nblocks, kBlock, 0, st>>>(row, col, val, Y, m, jobs, exag, rs);
    else
        k_bkl<1><<<nblocks, kBlock, 0, st>>>(row, col, val, Y, m, jobs, exag, rs);
    return cudaGetLastError();
}

int batch_attr_blocks_per_sm() {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_battr<2>, kBlock, 0) != cudaSuccess) return 1;
    return per_sm > 0 ? per_sm : 1;
}

#define FITSNE_INST(T)                                                                                           \
    template cudaError_t launch_center_minmax<T>(T *, int, int, int, int, RedScratch, cudaStream_t);                \
    template cudaError_t launch_spread<T>(const T *, int, int, const GridGeom &, Cell4<T> *, cudaStream_t,      \
                                          const uint32_t *);                                                    \
    template cudaError_t launch_gather<T>(const T *, int, int, const GridGeom &, const Cell4<T> *, int, T *,     \
                                          RedScratch, cudaStream_t, float *);                                   \
    template cudaError_t launch_gather_dev<T>(const T *, int, int, int, const DevGeom *, const Cell4<T> *, int,  \
                                              T *, RedScratch, cudaStream_t, float *);                          \
    template cudaError_t launch_spread_dev<T>(const T *, int, int, int, const DevGeom *, Cell4<T> *,            \
                                              cudaStream_t, const uint32_t *);                                  \
    template cudaError_t launch_attr_update<T>(const uint32_t *, const uint32_t *, const T *, const T *, T *,    \
                                               T *, T *, T *, const T *, int, int, const UpdateParams &,         \
                                               RedScratch, cudaStream_t, int, const float *);                   \
    template cudaError_t launch_kl<T>(const uint32_t *, const uint32_t *, const T *, const T *, int, int, double, \
                                      double, RedScratch, cudaStream_t);                                        \
    template cudaError_t launch_y_from_double<T>(const double *, T *, int, int, cudaStream_t);                  \
    template cudaError_t launch_y_to_double<T>(const T *, double *, int, int, cudaStream_t);                    \
    template cudaError_t launch_cast_from_double<T>(const double *, T *, size_t, cudaStream_t);
FITSNE_INST(float)
FITSNE_INST(double)
#undef FITSNE_INST

}  // namespace fitsne
