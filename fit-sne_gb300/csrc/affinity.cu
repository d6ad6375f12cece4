// Input-similarity kernels (see affinity.cuh).
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "affinity.cuh"
#include "screen.cuh"
#include "calib_mlp.cuh"
#include "knn.cuh"
#include "sort.cuh"

namespace fitsne {
namespace {

#define ACK(x)                                                          \
    do {                                                                \
        cudaError_t e__ = (x);                                          \
        if (e__ != cudaSuccess) {                                       \
            err = std::string(#x) + ": " + cudaGetErrorString(e__);     \
            return -10;                                                 \
        }                                                               \
    } while (0)

// ---------------------------------------------------------------------------------
// X preparation
__global__ void k_col_partial(const double *__restrict__ X, int N, int D, int rows_per_block,
                              double *__restrict__ part) {
    // part[block * D + d] = sum over this block's rows of X[:, d]
    const int r0 = blockIdx.x * rows_per_block;
    const int r1 = min(N, r0 + rows_per_block);
    for (int d = threadIdx.x; d < D; d += blockDim.x) {
        double s = 0.0;
        for (int r = r0; r < r1; ++r) s += X[(size_t) r * D + d];
        part[(size_t) blockIdx.x * D + d] = s;
    }
}

__global__ void k_col_finish(const double *__restrict__ part, int nblk, int D, int N, double *__restrict__ mean) {
    for (int d = threadIdx.x; d < D; d += blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < nblk; ++b) s += part[(size_t) b * D + d];
        mean[d] = s / (double) N;
    }
}

__global__ void k_center_absmax(double *__restrict__ X, size_t n, int D, const double *__restrict__ mean,
                                unsigned long long *__restrict__ amax) {
    double m = 0.0;
    for (size_t e = blockIdx.x * (size_t) blockDim.x + threadIdx.x; e < n; e += (size_t) gridDim.x * blockDim.x) {
        const double v = X[e] - mean[e % D];
        X[e] = v;
        m = fmax(m, fabs(v));
    }
    for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    // non-negative doubles order like their bit patterns
    if ((threadIdx.x & 31) == 0) atomicMax(amax, (unsigned long long) __double_as_longlong(m));
}

__global__ void k_scale(double *__restrict__ X, size_t n, const unsigned long long *__restrict__ amax) {
    const double s = __longlong_as_double((long long) *amax);
    for (size_t e = blockIdx.x * (size_t) blockDim.x + threadIdx.x; e < n; e += (size_t) gridDim.x * blockDim.x)
        X[e] /= s;
}

// ---------------------------------------------------------------------------------
// perplexity calibration, one thread per row, sums in the reference's order
// (distances2similarities, src/tsne.cpp:1394-1469).
//
// The bisection is bound by the FP64 pipe (GB300 runs FP64 at a small fraction of its FP32
// rate): every step evaluates K exponentials.  But a step's outcome is only which way the
// bracket moves, and the sequence of betas is fixed by those outcomes.  So each step is
// first evaluated in FP32 on the row's distances shifted by their minimum, with a bound on
// that value's error; when the FP32 value decides the outcome for certain (|H - log U| is
// farther from tol than the bound), the step takes it; otherwise the step is evaluated in
// FP64 exactly as the reference does.  The betas visited, the number of steps and P (the
// FP64 row of the last evaluation, which is always an FP64 one when the bisection
// converges) are therefore the reference's, bit for bit.
//
// The FP64 pipe issues a warp instruction at the same cost however many of its lanes are
// active, and a row needs its FP64 steps (1.5 on average, at most about 3) near the end of
// its bisection, at a step index that differs from row to row.  Taken where they fall, a
// warp's FP64 steps would run one after another with a lane or two active each.  So the
// warp's rows advance in rounds: each row takes FP32 steps until its next step needs FP64,
// then every row that needs one takes it together.  Each row's sequence of steps is
// unchanged, only the interleaving between rows differs.

// One bisection step in FP32 (screen_value): +1 when H(beta) - logU > tol for certain, -1
// when it is below -tol for certain, 0 when the FP32 value cannot decide.  The shifted form
// is the reference's value only while exp(-beta d0) is far from FP64 underflow, where the
// reference's DBL_MIN seed of sum_P matters: beyond beta d0 = 600 the step goes to FP64 (and
// beta must stay within FP32's range).
__device__ __forceinline__ int screen_step(const float *__restrict__ s, int sstride, int K, double beta, double d0,
                                           double logU, double tol) {
    if (!(beta > 1e-30 && beta < 1e30) || beta * d0 > 600.0) return 0;
    double E;
    const float h = screen_value(s, sstride, K, beta, &E);
    const double Hd = (double) h - logU;
    if (!(E < 1e-2)) return 0;
    if (Hd > tol + E) return 1;
    if (Hd < -(tol + E)) return -1;
    return 0;
}

// Calibrates one row.  s (may be null: FP64 steps only) is the row's FP32 shifted copy for
// screen_step; d0 the row's smallest distance.  Writes the normalised row p and returns the
// beta the reference's loop returns.  Called by every lane of the warp together (the FP64
// rounds are warp-wide); a lane without a row passes active = false and touches no memory.
__device__ double calibrate_row(const double *__restrict__ d, double *__restrict__ p, int K, double perplexity,
                                double sigma, bool active, int *evals = nullptr, const float *__restrict__ s = nullptr,
                                int sstride = 0, double d0 = 0.0) {
    if (perplexity > 0) {
        double min_beta = -DBL_MAX, max_beta = DBL_MAX;
        const double tol = 1e-5;
        const double logU = log(perplexity);
        bool found = !active;
        int iter = 0;
        double beta = 1.0;
        double beta_eval = beta;
        bool last_fp64 = false;  // p holds exp(-beta_eval d) and last_sum their sum
        double last_sum = DBL_MIN;
        // the bracket moves up (dir > 0: H too large) or down
        auto move = [&](int dir) {
            if (dir > 0) {
                min_beta = beta;
                if (max_beta == DBL_MAX || max_beta == -DBL_MAX)
                    beta *= 2.0;
                else
                    beta = (beta + max_beta) / 2.0;
            } else {
                max_beta = beta;
                if (min_beta == -DBL_MAX || min_beta == DBL_MAX)
                    beta /= 2.0;
                else
                    beta = (beta + min_beta) / 2.0;
            }
        };
        while (true) {
            // FP32 steps while they decide; stop at the first step that needs FP64
            bool need64 = false;
            while (!found && iter < 200) {
                beta_eval = beta;
                const int dir = s ? screen_step(s, sstride, K, beta, d0, logU, tol) : 0;
                if (dir == 0) {
                    need64 = true;
                    break;
                }
                last_fp64 = false;
                move(dir);
                iter++;
            }
            // one round: the FP64 step of every row of the warp that needs one
            if (!__any_sync(0xffffffffu, need64)) break;
            if (need64) {
                double sum_P = DBL_MIN, H = 0.0;
                for (int m = 0; m < K; ++m) {
                    const double e = exp(-beta * d[m]);
                    p[m] = e;
                    sum_P += e;
                    H += beta * (d[m] * e);
                }
                H = (H / sum_P) + log(sum_P);
                last_sum = sum_P;
                last_fp64 = true;
                const double Hdiff = H - logU;
                if (Hdiff < tol && -Hdiff < tol)
                    found = true;
                else
                    move(Hdiff > 0 ? 1 : -1);
                iter++;
            }
            // the next round's FP32 steps start with the whole warp together
            __syncwarp();
        }
        if (!active) return beta;
        if (evals) *evals = iter;
        // P of the reference is the row evaluated at beta_eval; the returned beta is the
        // updated one when the loop ran out of iterations (as in the reference)
        if (!last_fp64) {
            last_sum = DBL_MIN;
            for (int m = 0; m < K; ++m) {
                p[m] = exp(-beta_eval * d[m]);
                last_sum += p[m];
            }
        }
        for (int m = 0; m < K; ++m) p[m] /= last_sum;
        return beta;
    }
    const double beta_eval = 1 / (2 * sigma * sigma);
    if (!active) return beta_eval;
    double sum_P = DBL_MIN;
    for (int m = 0; m < K; ++m) {
        p[m] = exp(-beta_eval * d[m]);
        sum_P += p[m];
    }
    for (int m = 0; m < K; ++m) p[m] /= sum_P;
    return beta_eval;
}

// Rows of the block in shared memory as FP32 shifted distances, one column per thread
// ([m][thread]: the lanes of a warp read consecutive words), when the launch provides the
// space (stage = 1); the FP64 distances stay in global memory (read only by FP64 steps).
// The block size is a multiple of 32, and lanes past the last row stay in their warp.
__global__ void k_calibrate(const double *__restrict__ dist, int stride, int offset, double *__restrict__ P,
                            double *__restrict__ tmp, int nrows, int K, double perplexity, double sigma,
                            const double *__restrict__ list, int list_len, double *__restrict__ beta_out,
                            int *__restrict__ evals_out, int stage) {
    extern __shared__ float s_shift[];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = r < nrows;
    const int rr = active ? r : 0;
    const double *d = dist + (size_t) rr * stride + offset;
    double *p = P + (size_t) rr * K;
    const float *s = nullptr;
    double d0 = 0.0;
    if (stage && perplexity >= 0) {
        float *w = s_shift + threadIdx.x;
        if (active) {
            d0 = d[0];
            for (int m = 1; m < K; ++m) d0 = fmin(d0, d[m]);
            for (int m = 0; m < K; ++m) w[(size_t) m * blockDim.x] = (float) (d[m] - d0);
        }
        s = w;
    }
    double beta;
    int evals = 0;
    if (perplexity != 0) {
        beta = calibrate_row(d, p, K, perplexity, sigma, active, &evals, s, blockDim.x, d0);
    } else {
        double *t = tmp + (size_t) rr * K;
        beta = calibrate_row(d, p, K, list[0], sigma, active, &evals, s, blockDim.x, d0);
        for (int m = 1; m < list_len; ++m) {
            beta = calibrate_row(d, t, K, list[m], sigma, active, nullptr, s, blockDim.x, d0);
            if (active)
                for (int i = 0; i < K; ++i) p[i] += t[i];
        }
        if (active)
            for (int i = 0; i < K; ++i) p[i] /= list_len;
    }
    if (!active) return;
    if (beta_out) beta_out[r] = beta;
    if (evals_out) evals_out[r] = evals;
}

__global__ void k_knn_to_csr(const uint32_t *__restrict__ idx, int N, int K, uint32_t *__restrict__ row,
                             uint32_t *__restrict__ col) {
    const size_t n = (size_t) N * K;
    for (size_t e = blockIdx.x * (size_t) blockDim.x + threadIdx.x; e < n; e += (size_t) gridDim.x * blockDim.x) {
        const size_t r = e / K, m = e % K;
        col[e] = idx[r * (K + 1) + m + 1];
    }
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r <= N; r += gridDim.x * blockDim.x) row[r] = (uint32_t) r * K;
}

// ---------------------------------------------------------------------------------
// symmetrisation helpers
__global__ void k_row_src(const uint32_t *__restrict__ row, int N, uint32_t *__restrict__ src) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < N; r += gridDim.x * blockDim.x)
        for (uint32_t e = row[r]; e < row[r + 1]; ++e) src[e] = (uint32_t) r;
}

// per-row copy of (col, position) sorted by col (insertion sort; rows are short)
// Rows longer than kWarpRow entries (k_row_sorted_warp below sorts the others).
constexpr int kWarpRow = 256;

__global__ void k_row_sorted(const uint32_t *__restrict__ row, const uint32_t *__restrict__ col, int N,
                             uint32_t *__restrict__ scol, uint32_t *__restrict__ spos) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < N; r += gridDim.x * blockDim.x) {
        const uint32_t a = row[r], b = row[r + 1];
        if (b - a <= (uint32_t) kWarpRow) continue;
        for (uint32_t e = a; e < b; ++e) {
            const uint32_t c = col[e];
            uint32_t k = e;
            while (k > a && scol[k - 1] > c) {
                scol[k] = scol[k - 1];
                spos[k] = spos[k - 1];
                --k;
            }
            scol[k] = c;
            spos[k] = e;
        }
    }
}

// position of c in row a (sorted copy), or 0xffffffff
__device__ __forceinline__ uint32_t find_in_row(const uint32_t *__restrict__ row, const uint32_t *__restrict__ scol,
                                                const uint32_t *__restrict__ spos, uint32_t a, uint32_t c) {
    uint32_t lo = row[a], hi = row[a + 1];
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        const uint32_t v = scol[mid];
        if (v < c)
            lo = mid + 1;
        else if (v > c)
            hi = mid;
        else
            return spos[mid];
    }
    return 0xffffffffu;
}

__global__ void k_iota(uint32_t *__restrict__ v, size_t n) {
    for (size_t e = blockIdx.x * (size_t) blockDim.x + threadIdx.x; e < n; e += (size_t) gridDim.x * blockDim.x)
        v[e] = (uint32_t) e;
}

__global__ void k_count_in(const uint32_t *__restrict__ col, size_t nnz, uint32_t *__restrict__ indeg) {
    for (size_t e = blockIdx.x * (size_t) blockDim.x + threadIdx.x; e < nnz; e += (size_t) gridDim.x * blockDim.x)
        atomicAdd(&indeg[col[e]], 1u);
}

// ---------------------------------------------------------------------------------
// Warp per row.  k_row_sorted_warp sorts rows of at most kWarpRow entries (the kNN rows: K per
// row; longer rows: k_row_sorted above, a thread each); the sort is by column (columns of a
// row are distinct).  k_sym_rows_warp writes every output row (tsne.cpp:1772-1811): incoming
// n < r (ascending), r's own entries in list order except those mirrored earlier, incoming
// n > r that r does not list (ascending).  It streams a row's entries and incoming edges in
// chunks of 32 and compacts each group in its own order with warp ballots, so a hub row (many
// incoming edges) costs its warp (incoming / 32) rounds.

__global__ void __launch_bounds__(128) k_row_sorted_warp(const uint32_t *__restrict__ row,
                                                         const uint32_t *__restrict__ col, int N,
                                                         uint32_t *__restrict__ scol, uint32_t *__restrict__ spos,
                                                         int *__restrict__ long_rows) {
    __shared__ unsigned long long buf[4][kWarpRow];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned long long *b = buf[w];
    for (int r = blockIdx.x * 4 + w; r < N; r += gridDim.x * 4) {
        const uint32_t a = row[r], len = row[r + 1] - a;
        if (len > (uint32_t) kWarpRow) {  // left to the thread-per-row kernel
            if (lane == 0) atomicOr(long_rows, 1);
            continue;
        }
        int n = 32;
        while (n < (int) len) n <<= 1;
        for (int i = lane; i < n; i += 32)
            b[i] = i < (int) len ? ((unsigned long long) col[a + i] << 32) | (unsigned long long) (a + i) : ~0ull;
        __syncwarp();
        for (int k = 2; k <= n; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int i = lane; i < n; i += 32) {
                    const int q = i ^ j;
                    if (q > i) {
                        const unsigned long long x = b[i], y = b[q];
                        if ((x > y) == ((i & k) == 0)) {
                            b[i] = y;
                            b[q] = x;
                        }
                    }
                }
                __syncwarp();
            }
        for (int i = lane; i < (int) len; i += 32) {
            scol[a + i] = (uint32_t) (b[i] >> 32);
            spos[a + i] = (uint32_t) b[i];
        }
        __syncwarp();
    }
}

// One warp per output row, every row (see above).
template <bool FILL>
__global__ void __launch_bounds__(128) k_sym_rows_warp(const uint32_t *__restrict__ row,
                                                       const uint32_t *__restrict__ col,
                                                       const double *__restrict__ val,
                                                       const uint32_t *__restrict__ scol,
                                                       const uint32_t *__restrict__ spos,
                                                       const uint32_t *__restrict__ toff,
                                                       const uint32_t *__restrict__ tedge,
                                                       const uint32_t *__restrict__ src, int N,
                                                       uint32_t *__restrict__ count, const uint32_t *__restrict__ srow,
                                                       uint32_t *__restrict__ ocol, double *__restrict__ oval) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int r = gw; r < N; r += nw) {
        const uint32_t ur = (uint32_t) r;
        const uint32_t r0 = row[r], r1 = row[r + 1], t0 = toff[r], t1 = toff[r + 1];
        uint32_t o = FILL ? srow[r] : 0u;
        uint32_t c0 = 0;
        const uint32_t lanemask = (1u << lane) - 1u;
        // first group: incoming n < r, in incoming order (ascending n)
        for (uint32_t base = t0; base < t1; base += 32) {
            const uint32_t t = base + lane;
            bool keep = false;
            uint32_t n = 0, e = 0;
            if (t < t1) {
                e = tedge[t];
                n = src[e];
                keep = n < ur;
            }
            const unsigned m = __ballot_sync(full, keep);
            if (FILL && keep) {
                const uint32_t at = o + __popc(m & lanemask);
                const uint32_t mm = find_in_row(row, scol, spos, ur, n);
                ocol[at] = n;
                oval[at] = (mm != 0xffffffffu) ? (val[e] + val[mm]) / 2.0 : val[e] / 2.0;
            }
            o += __popc(m);
            c0 += __popc(m);
        }
        // middle: own entries in list order, except those mirrored earlier
        for (uint32_t base = r0; base < r1; base += 32) {
            const uint32_t e = base + lane;
            bool keep = false;
            uint32_t c = 0, mm = 0xffffffffu;
            if (e < r1) {
                c = col[e];
                mm = find_in_row(row, scol, spos, c, ur);
                keep = !(mm != 0xffffffffu && c < ur);
            }
            const unsigned m = __ballot_sync(full, keep);
            if (FILL && keep) {
                const uint32_t at = o + __popc(m & lanemask);
                ocol[at] = c;
                oval[at] = (mm != 0xffffffffu) ? (val[e] + val[mm]) / 2.0 : val[e] / 2.0;
            }
            o += __popc(m);
            c0 += __popc(m);
        }
        // last group: incoming n > r that r does not list, in incoming order
        for (uint32_t base = t0; base < t1; base += 32) {
            const uint32_t t = base + lane;
            bool keep = false;
            uint32_t n = 0, e = 0;
            if (t < t1) {
                e = tedge[t];
                n = src[e];
                keep = n > ur && find_in_row(row, scol, spos, ur, n) == 0xffffffffu;
            }
            const unsigned m = __ballot_sync(full, keep);
            if (FILL && keep) {
                const uint32_t at = o + __popc(m & lanemask);
                ocol[at] = n;
                oval[at] = val[e] / 2.0;
            }
            o += __popc(m);
            c0 += __popc(m);
        }
        if (!FILL && lane == 0) count[r] = c0;
    }
}

// ---------------------------------------------------------------------------------
__global__ void k_sum_part(const double *__restrict__ v, size_t n, double *__restrict__ part) {
    __shared__ double sh[32];
    double s = 0.0;
    for (size_t e = blockIdx.x * (size_t) blockDim.x + threadIdx.x; e < n; e += (size_t) gridDim.x * blockDim.x)
        s += v[e];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int) (blockDim.x >> 5); ++w) t += sh[w];
        part[blockIdx.x] = t;
    }
}

__global__ void k_div(double *__restrict__ v, size_t n, const double *__restrict__ part, int nb) {
    __shared__ double total;
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int b = 0; b < nb; ++b) t += part[b];
        total = t;
    }
    __syncthreads();
    const double s = total;
    for (size_t e = blockIdx.x * (size_t) blockDim.x + threadIdx.x; e < n; e += (size_t) gridDim.x * blockDim.x)
        v[e] /= s;
}

__global__ void k_row_sums_max(const uint32_t *__restrict__ row, const double *__restrict__ val, int N,
                               unsigned long long *__restrict__ mx) {
    double m = 0.0;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < N; r += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (uint32_t e = row[r]; e < row[r + 1]; ++e) s += val[e];
        m = fmax(m, s);
    }
    for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(mx, (unsigned long long) __double_as_longlong(m));
}

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int key_bits_for(int N) {
    int b = 1;
    while (b < 32 && (1u << b) < (unsigned) N) ++b;
    return b;
}

}  // namespace

void free_csr(DevCSR &P) {
    cudaFree(P.row);
    cudaFree(P.col);
    cudaFree(P.val);
    P.row = P.col = nullptr;
    P.val = nullptr;
    P.nnz = 0;
}

int prepare_X(const double *X_host, int N, int D, bool normalize, double **Xd_out, cudaStream_t st,
              std::string &err) {
    double *Xd = nullptr, *part = nullptr, *mean = nullptr;
    unsigned long long *amax = nullptr;
    const size_t n = (size_t) N * D;
    ACK(cudaMalloc(&Xd, sizeof(double) * (n ? n : 1)));
    ACK(cudaMemcpyAsync(Xd, X_host, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    const int rpb = 256;
    const int nblk = (N + rpb - 1) / rpb;
    ACK(cudaMalloc(&part, sizeof(double) * (size_t) nblk * D + 8));
    ACK(cudaMalloc(&mean, sizeof(double) * D + 8));
    ACK(cudaMalloc(&amax, sizeof(unsigned long long)));
    ACK(cudaMemsetAsync(amax, 0, sizeof(unsigned long long), st));
    k_col_partial<<<nblk, 64, 0, st>>>(Xd, N, D, rpb, part);
    k_col_finish<<<1, 256, 0, st>>>(part, nblk, D, N, mean);
    k_center_absmax<<<2048, 256, 0, st>>>(Xd, n, D, mean, amax);
    if (normalize) k_scale<<<2048, 256, 0, st>>>(Xd, n, amax);
    ACK(cudaGetLastError());
    ACK(cudaStreamSynchronize(st));
    cudaFree(part);
    cudaFree(mean);
    cudaFree(amax);
    *Xd_out = Xd;
    return 0;
}

int calibrate_rows(const double *dist, int stride, int offset, double *P, int nrows, int K, double perplexity,
                   double sigma, int list_len, const double *list_host, double *beta, cudaStream_t st,
                   std::string &err, std::vector<int> *iters) {
    double *list = nullptr, *tmp = nullptr;
    int *evals = nullptr;
    if (iters) ACK(cudaMalloc(&evals, sizeof(int) * (size_t) (nrows > 0 ? nrows : 1)));
    if (perplexity == 0) {
        if (list_len < 1 || !list_host) {
            err = "perplexity 0 needs a perplexity list";
            return -3;
        }
        ACK(cudaMalloc(&list, sizeof(double) * list_len));
        ACK(cudaMemcpyAsync(list, list_host, sizeof(double) * list_len, cudaMemcpyHostToDevice, st));
        ACK(cudaMalloc(&tmp, sizeof(double) * (size_t) nrows * K));
    }
    // FP32 shifted rows in shared memory: 128 rows per block up to K = 320, fewer rows for
    // longer ones, none (FP64 steps only) beyond K = 1280
    int bd = 128;
    while (bd > 32 && (size_t) bd * K * sizeof(float) > 160 * 1024) bd /= 2;
    const size_t smem = (size_t) bd * K * sizeof(float);
    const int stage = smem <= 160 * 1024 ? 1 : 0;
    if (stage) ACK(cudaFuncSetAttribute(k_calibrate, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem));
    k_calibrate<<<(nrows + bd - 1) / bd, bd, stage ? smem : 0, st>>>(dist, stride, offset, P, tmp, nrows, K,
                                                                      perplexity, sigma, list, list_len, beta, evals,
                                                                      stage);
    ACK(cudaGetLastError());
    if (iters) {
        iters->resize(nrows);
        ACK(cudaMemcpyAsync(iters->data(), evals, sizeof(int) * (size_t) nrows, cudaMemcpyDeviceToHost, st));
    }
    ACK(cudaStreamSynchronize(st));
    cudaFree(list);
    cudaFree(tmp);
    cudaFree(evals);
    return 0;
}

int gaussian_perplexity_device(const double *Xd, int N, int D, int K, double perplexity, double sigma, int list_len,
                               const double *list_host, DevCSR *out, cudaStream_t st, std::string &err,
                               int *knn_rescanned, uint32_t *order_out, bool *order_written) {
    if (K < 1 || K + 1 > N) {
        err = "K + 1 must not exceed the number of points";
        return -3;
    }
    uint32_t *idx = nullptr;
    double *dist = nullptr;
    ACK(cudaMalloc(&idx, sizeof(uint32_t) * (size_t) N * (K + 1)));
    ACK(cudaMalloc(&dist, sizeof(double) * (size_t) N * (K + 1)));
    KnnStats ks;
    const char *kerr = nullptr;
    const bool tm = timing_requested();
    const double t0 = now_s();
    int rc = knn_exact(Xd, N, D, K + 1, idx, dist, st, &ks, &kerr, order_out, order_written);
    if (tm) print_knn_stats(K + 1, ks, now_s() - t0);
    if (rc) {
        err = kerr ? kerr : "kNN failed";
        cudaFree(idx);
        cudaFree(dist);
        return rc;
    }
    if (knn_rescanned) *knn_rescanned = ks.rows_rescanned;
    DevCSR P;
    P.N = N;
    P.nnz = (size_t) N * K;
    ACK(cudaMalloc(&P.row, sizeof(uint32_t) * (N + 1)));
    ACK(cudaMalloc(&P.col, sizeof(uint32_t) * P.nnz));
    ACK(cudaMalloc(&P.val, sizeof(double) * P.nnz));
    k_knn_to_csr<<<4096, 256, 0, st>>>(idx, N, K, P.row, P.col);
    ACK(cudaGetLastError());
    const double t1 = now_s();
    if (calibration_mode() == 1 && perplexity > 0 && list_len == 0) {
        MlpStats ms;
        rc = calibrate_rows_learned(dist, K + 1, 1, P.val, N, K, perplexity, st, &ms, err);
        if (!rc) store_calibration_stats(ms);
        if (tm && !rc)
            std::fprintf(stderr,
                         "[fitsne] calibration (learned warm start): %.3f s; %d harvested rows, %.1f evaluations "
                         "per row; %d training steps, loss %.3g -> %.3g; %d predicted rows, %.2f evaluations per "
                         "row, %d with bisection steps; ms harvest %.1f, train %.1f, infer %.1f, search %.1f\n",
                         now_s() - t1, ms.rows_harvest, ms.iters_plain, ms.train_steps, ms.loss_first, ms.loss_last,
                         ms.rows - ms.rows_harvest, ms.iters_warm, ms.rows_fallback, ms.ms_harvest, ms.ms_train,
                         ms.ms_infer, ms.ms_warm);
    } else {
        std::vector<int> evals;
        rc = calibrate_rows(dist, K + 1, 1, P.val, N, K, perplexity, sigma, list_len, list_host, nullptr, st, err,
                            &evals);
        if (!rc) {
            MlpStats ms;
            ms.rows = ms.rows_harvest = N;
            ms.ms_harvest = (now_s() - t1) * 1e3;  // every row takes the bisection
            double s = 0;
            for (int v : evals) s += v;
            ms.iters_plain = N ? s / N : 0;
            store_calibration_stats(ms);
        }
        if (tm) std::fprintf(stderr, "[fitsne] calibration: %.3f s\n", now_s() - t1);
    }
    cudaFree(idx);
    cudaFree(dist);
    if (rc) {
        free_csr(P);
        return rc;
    }
    *out = P;
    return 0;
}

int symmetrize_device(const DevCSR &in, DevCSR *out, cudaStream_t st, std::string &err) {
    const int N = in.N;
    const size_t nnz = in.nnz;
    uint32_t *src = nullptr, *scol = nullptr, *spos = nullptr, *keys = nullptr, *tedge = nullptr, *kalt = nullptr,
             *valt = nullptr, *indeg = nullptr, *toff = nullptr, *cnt = nullptr;
    int *long_rows = nullptr;
    void *scratch = nullptr;
    const size_t nz = nnz ? nnz : 1;
    ACK(cudaMalloc(&src, sizeof(uint32_t) * nz));
    ACK(cudaMalloc(&scol, sizeof(uint32_t) * nz));
    ACK(cudaMalloc(&spos, sizeof(uint32_t) * nz));
    ACK(cudaMalloc(&keys, sizeof(uint32_t) * nz));
    ACK(cudaMalloc(&tedge, sizeof(uint32_t) * nz));
    ACK(cudaMalloc(&kalt, sizeof(uint32_t) * nz));
    ACK(cudaMalloc(&valt, sizeof(uint32_t) * nz));
    ACK(cudaMalloc(&indeg, sizeof(uint32_t) * (N + 1)));
    ACK(cudaMalloc(&toff, sizeof(uint32_t) * (N + 2)));
    ACK(cudaMalloc(&cnt, sizeof(uint32_t) * (N + 1)));
    ACK(cudaMalloc(&long_rows, sizeof(int) * 2));
    const size_t scr = radix_sort_scratch_bytes(nz) + scan_scratch_bytes((size_t) N + 1);
    ACK(cudaMalloc(&scratch, scr));
    const int g = 2048;
    k_row_src<<<(N + 255) / 256, 256, 0, st>>>(in.row, N, src);
    // rows sorted by a warp each; rows too long for it by a thread each
    ACK(cudaMemsetAsync(long_rows, 0, sizeof(int) * 2, st));
    k_row_sorted_warp<<<std::min((N + 3) / 4, 8192), 128, 0, st>>>(in.row, in.col, N, scol, spos, long_rows);
    int hlong[2] = {0, 0};
    ACK(cudaMemcpyAsync(hlong, long_rows, sizeof(int), cudaMemcpyDeviceToHost, st));
    ACK(cudaStreamSynchronize(st));
    if (hlong[0]) k_row_sorted<<<(N + 127) / 128, 128, 0, st>>>(in.row, in.col, N, scol, spos);
    // transpose: group edge ids by column, stable in edge order
    ACK(cudaMemcpyAsync(keys, in.col, sizeof(uint32_t) * nnz, cudaMemcpyDeviceToDevice, st));
    k_iota<<<g, 256, 0, st>>>(tedge, nnz);
    ACK(radix_sort_pairs(keys, tedge, kalt, valt, nnz, key_bits_for(N), scratch, st));
    ACK(cudaMemsetAsync(indeg, 0, sizeof(uint32_t) * (N + 1), st));
    k_count_in<<<g, 256, 0, st>>>(in.col, nnz, indeg);
    ACK(exclusive_scan_u32(indeg, toff, (size_t) N, scratch, st));
    const int gw = std::min((N + 3) / 4, 8192);
    k_sym_rows_warp<false><<<gw, 128, 0, st>>>(in.row, in.col, in.val, scol, spos, toff, tedge, src, N, cnt, nullptr,
                                               nullptr, nullptr);
    DevCSR P;
    P.N = N;
    ACK(cudaMalloc(&P.row, sizeof(uint32_t) * (N + 1)));
    ACK(exclusive_scan_u32(cnt, P.row, (size_t) N, scratch, st));
    uint32_t total = 0;
    ACK(cudaMemcpyAsync(&total, P.row + N, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    ACK(cudaStreamSynchronize(st));
    P.nnz = total;
    ACK(cudaMalloc(&P.col, sizeof(uint32_t) * (total ? total : 1)));
    ACK(cudaMalloc(&P.val, sizeof(double) * (total ? total : 1)));
    k_sym_rows_warp<true><<<gw, 128, 0, st>>>(in.row, in.col, in.val, scol, spos, toff, tedge, src, N, nullptr,
                                              P.row, P.col, P.val);
    ACK(cudaGetLastError());
    ACK(cudaStreamSynchronize(st));
    cudaFree(src);
    cudaFree(scol);
    cudaFree(spos);
    cudaFree(keys);
    cudaFree(tedge);
    cudaFree(kalt);
    cudaFree(valt);
    cudaFree(indeg);
    cudaFree(toff);
    cudaFree(cnt);
    cudaFree(long_rows);
    cudaFree(scratch);
    *out = P;
    return 0;
}

int normalize_device(DevCSR &P, double *sum, cudaStream_t st, std::string &err) {
    const int nb = 1024;
    double *part = nullptr;
    ACK(cudaMalloc(&part, sizeof(double) * nb));
    k_sum_part<<<nb, 256, 0, st>>>(P.val, P.nnz, part);
    k_div<<<2048, 256, 0, st>>>(P.val, P.nnz, part, nb);
    if (sum) {
        std::vector<double> h(nb);
        ACK(cudaMemcpyAsync(h.data(), part, sizeof(double) * nb, cudaMemcpyDeviceToHost, st));
        ACK(cudaStreamSynchronize(st));
        double t = 0.0;
        for (double v : h) t += v;
        *sum = t;
    }
    ACK(cudaStreamSynchronize(st));
    cudaFree(part);
    return 0;
}

int max_row_sum_device(const DevCSR &P, double *out, cudaStream_t st, std::string &err) {
    unsigned long long *mx = nullptr;
    ACK(cudaMalloc(&mx, sizeof(unsigned long long)));
    ACK(cudaMemsetAsync(mx, 0, sizeof(unsigned long long), st));
    k_row_sums_max<<<(P.N + 255) / 256, 256, 0, st>>>(P.row, P.val, P.N, mx);
    unsigned long long h = 0;
    ACK(cudaMemcpyAsync(&h, mx, sizeof(h), cudaMemcpyDeviceToHost, st));
    ACK(cudaStreamSynchronize(st));
    cudaFree(mx);
    double d;
    static_assert(sizeof(d) == sizeof(h), "size");
    std::memcpy(&d, &h, sizeof(d));
    *out = d;
    return 0;
}

int csr_to_device(const uint32_t *row, const uint32_t *col, const double *val, int N, DevCSR *out, cudaStream_t st,
                  std::string &err) {
    DevCSR P;
    P.N = N;
    P.nnz = row[N];
    ACK(cudaMalloc(&P.row, sizeof(uint32_t) * (N + 1)));
    ACK(cudaMalloc(&P.col, sizeof(uint32_t) * (P.nnz ? P.nnz : 1)));
    ACK(cudaMalloc(&P.val, sizeof(double) * (P.nnz ? P.nnz : 1)));
    ACK(cudaMemcpyAsync(P.row, row, sizeof(uint32_t) * (N + 1), cudaMemcpyHostToDevice, st));
    if (P.nnz) {
        ACK(cudaMemcpyAsync(P.col, col, sizeof(uint32_t) * P.nnz, cudaMemcpyHostToDevice, st));
        ACK(cudaMemcpyAsync(P.val, val, sizeof(double) * P.nnz, cudaMemcpyHostToDevice, st));
    }
    ACK(cudaStreamSynchronize(st));
    *out = P;
    return 0;
}

int csr_to_host(const DevCSR &P, uint32_t *row, uint32_t *col, double *val, cudaStream_t st, std::string &err) {
    ACK(cudaMemcpyAsync(row, P.row, sizeof(uint32_t) * (P.N + 1), cudaMemcpyDeviceToHost, st));
    if (P.nnz) {
        ACK(cudaMemcpyAsync(col, P.col, sizeof(uint32_t) * P.nnz, cudaMemcpyDeviceToHost, st));
        ACK(cudaMemcpyAsync(val, P.val, sizeof(double) * P.nnz, cudaMemcpyDeviceToHost, st));
    }
    ACK(cudaStreamSynchronize(st));
    return 0;
}

}  // namespace fitsne
