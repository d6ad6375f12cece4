// Learned warm start of the perplexity calibration (see calib_mlp.cuh).
#include <cuda_bf16.h>

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "affinity.cuh"
#include "calib_mlp.cuh"
#include "screen.cuh"

namespace fitsne {
namespace {

constexpr int H = kMlpHidden;
constexpr int kSPB = 16;         // samples per block in the gradient kernel (all carried at once)
constexpr int kBatch = 512;      // minibatch (FITSNE_MLP_BATCH overrides)
constexpr int kGraphSteps = 25;  // optimiser steps per captured graph
constexpr float kLr = 3e-3f;     // Adam step size (FITSNE_MLP_LR overrides)
constexpr int kH2 = H + 1;       // padded row stride of W2 in shared memory

struct Offs {
    int w1, b1, w2, b2, w3, b3, n;
};
__host__ __device__ inline Offs offs(int K) {
    Offs o;
    o.w1 = 0;
    o.b1 = H * K;
    o.w2 = o.b1 + H;
    o.b2 = o.w2 + H * H;
    o.w3 = o.b2 + H;
    o.b3 = o.w3 + H;
    o.n = o.b3 + 1;
    return o;
}

__host__ __device__ inline int odd_stride(int K) { return K | 1; }  // conflict-free row reads

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ---- features: x = d / mean(d), scale = mean(d); target = log(beta * mean(d)) --------------
__global__ void k_features(const double *__restrict__ dist, int stride, int offset, int nrows, int K,
                           const double *__restrict__ beta, float *__restrict__ x, float *__restrict__ scale,
                           float *__restrict__ target) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x) {
        const double *d = dist + (size_t) r * stride + offset;
        double s = 0.0;
        for (int j = 0; j < K; ++j) s += d[j];
        s /= K;
        const bool ok = s > 0.0 && isfinite(s);
        const double inv = ok ? 1.0 / s : 0.0;
        for (int j = 0; j < K; ++j) x[(size_t) r * K + j] = (float) (d[j] * inv);
        scale[r] = ok ? (float) s : 0.f;
        if (target) target[r] = (ok && beta[r] > 0.0) ? (float) log(beta[r] * s) : 0.f;
    }
}

__device__ __forceinline__ unsigned mix32(unsigned a, unsigned b) {
    unsigned h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u) * 0x85EBCA77u;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return h;
}

// ---- forward + backward of one minibatch ----------------------------------------------------
// 64 threads (one per hidden unit) per block and kSPB samples per block, all carried at once
// by every thread (kSPB independent accumulation chains; every weight read once for the
// block's samples).  Each weight's gradient over the block's samples is complete after one
// pass, so it goes straight to the block's partial gradient gpart[block][n] (no atomics: the
// partials are summed in block order by k_adam / k_grad_sum, so training is repeatable).
// In the partials the two weight matrices are stored transposed (part_index), so that the
// 64 threads of a block write consecutive words.  Standardised target (target - mu) / sd;
// loss = mean squared error over the batch.  With step == nullptr the batch is rows
// 0 .. batch-1 in order, else rows drawn by a hash of (step, position).
__host__ __device__ inline int part_index(int i, const Offs &o, int K) {
    if (i < o.b1) return o.w1 + (i % K) * H + i / K;
    if (i >= o.w2 && i < o.b2) return o.w2 + ((i - o.w2) % H) * H + (i - o.w2) / H;
    return i;
}

__global__ void __launch_bounds__(H) k_mlp_grad(const float *__restrict__ params, int K, const float *__restrict__ x,
                                                 const float *__restrict__ target, int nrows, int batch, float mu,
                                                 float inv_sd, const unsigned *__restrict__ step,
                                                 float *__restrict__ gpart, double *__restrict__ loss) {
    constexpr int S = kSPB;
    extern __shared__ float sm[];
    const int KP = odd_stride(K);
    float *W1 = sm;             // [H][KP]
    float *W2 = W1 + H * KP;    // [H][kH2]
    float *xt = W2 + H * kH2;   // samples, transposed: [K][S]
    float *tt = xt + K * S;     // targets [S]
    float *h1t = tt + S;        // [H][S]
    float *dh2t = h1t + H * S;  // [H][S]
    float *red = dh2t + H * S;  // [S][2 warps]
    const unsigned full = 0xffffffffu;
    const int u = threadIdx.x;
    const Offs o = offs(K);
    // the weights into shared memory with 16-byte loads (W1 and W2 start on 16-byte boundaries:
    // offsets 0 and 64 K + 64 floats); a vector of W1 may run into the next row
    {
        const float4 *p1 = reinterpret_cast<const float4 *>(params + o.w1);
#pragma unroll 4
        for (int e = u; e < H * K / 4; e += H) {
            const float4 w = __ldg(p1 + e);
            const float wv[4] = {w.x, w.y, w.z, w.w};
            int r = (4 * e) / K, c = 4 * e - r * K;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                W1[r * KP + c] = wv[k];
                if (++c == K) {
                    c = 0;
                    ++r;
                }
            }
        }
        const float4 *p2 = reinterpret_cast<const float4 *>(params + o.w2);
#pragma unroll 4
        for (int e = u; e < H * H / 4; e += H) {
            const float4 w = __ldg(p2 + e);
            const int r = (4 * e) / H, c = (4 * e) % H;
            W2[r * kH2 + c] = w.x;
            W2[r * kH2 + c + 1] = w.y;
            W2[r * kH2 + c + 2] = w.z;
            W2[r * kH2 + c + 3] = w.w;
        }
    }
    const float b1 = params[o.b1 + u], b2 = params[o.b2 + u], w3 = params[o.w3 + u], b3 = params[o.b3];
    const unsigned stp = step ? *step : 0u;
    // the block's samples and targets in one round of loads; samples past the batch are zero
#pragma unroll
    for (int q = 0; q < S; ++q) {
        const int pos = blockIdx.x * S + q;
        const bool valid = pos < batch;
        const int row = !valid ? 0 : (step ? (int) (mix32(stp, (unsigned) pos) % (unsigned) nrows) : pos);
        for (int j = u; j < K; j += H) xt[j * S + q] = valid ? x[(size_t) row * K + j] : 0.f;
        if (u == 0) tt[q] = valid ? target[row] : 0.f;
    }
    __syncthreads();
    // forward, layer 1
    float a1[S];
#pragma unroll
    for (int q = 0; q < S; ++q) a1[q] = b1;
    for (int j = 0; j < K; ++j) {
        const float w = W1[u * KP + j];
#pragma unroll
        for (int q = 0; q < S; ++q) a1[q] = fmaf(w, xt[j * S + q], a1[q]);
    }
#pragma unroll
    for (int q = 0; q < S; ++q) h1t[u * S + q] = a1[q] > 0.f ? a1[q] : 0.f;
    __syncthreads();
    // layer 2
    float a2[S];
#pragma unroll
    for (int q = 0; q < S; ++q) a2[q] = b2;
    for (int k = 0; k < H; ++k) {
        const float w = W2[u * kH2 + k];
#pragma unroll
        for (int q = 0; q < S; ++q) a2[q] = fmaf(w, h1t[k * S + q], a2[q]);
    }
    // output of each sample: w3 . relu(a2) over the 64 units (two warps)
#pragma unroll
    for (int q = 0; q < S; ++q) {
        float pq = w3 * (a2[q] > 0.f ? a2[q] : 0.f);
        for (int off = 16; off; off >>= 1) pq += __shfl_xor_sync(full, pq, off);
        if ((u & 31) == 0) red[q * 2 + (u >> 5)] = pq;
    }
    __syncthreads();
    // backward
    float gw3 = 0.f, gb2 = 0.f, gb3 = 0.f;
    double lsum = 0.0;
    float d2[S];
#pragma unroll
    for (int q = 0; q < S; ++q) {
        const bool valid = blockIdx.x * S + q < batch;
        const float out = red[q * 2] + red[q * 2 + 1] + b3;
        const float err = valid ? out - (tt[q] - mu) * inv_sd : 0.f;
        lsum += (double) err * err;
        const float dout = 2.f * err / (float) batch;
        gw3 = fmaf(dout, a2[q] > 0.f ? a2[q] : 0.f, gw3);
        gb3 += dout;
        d2[q] = a2[q] > 0.f ? dout * w3 : 0.f;
        gb2 += d2[q];
        dh2t[u * S + q] = d2[q];
    }
    float *g = gpart + (size_t) blockIdx.x * o.n;
    // dW2 (u, k) = sum_q d2[q] h1[q][k], stored transposed
    for (int k = 0; k < H; ++k) {
        float acc = 0.f;
#pragma unroll
        for (int q = 0; q < S; ++q) acc = fmaf(d2[q], h1t[k * S + q], acc);
        g[o.w2 + k * H + u] = acc;
    }
    __syncthreads();
    // back to layer 1: s[q] = sum_v d2[q][v] W2[v][u]
    float sv[S];
#pragma unroll
    for (int q = 0; q < S; ++q) sv[q] = 0.f;
    for (int v = 0; v < H; ++v) {
        const float w = W2[v * kH2 + u];
#pragma unroll
        for (int q = 0; q < S; ++q) sv[q] = fmaf(w, dh2t[v * S + q], sv[q]);
    }
    float gb1 = 0.f;
#pragma unroll
    for (int q = 0; q < S; ++q) {
        sv[q] = a1[q] > 0.f ? sv[q] : 0.f;
        gb1 += sv[q];
    }
    // dW1 (u, j) = sum_q d1[q] x[q][j], stored transposed
    for (int j = 0; j < K; ++j) {
        float acc = 0.f;
#pragma unroll
        for (int q = 0; q < S; ++q) acc = fmaf(sv[q], xt[j * S + q], acc);
        g[o.w1 + j * H + u] = acc;
    }
    g[o.b1 + u] = gb1;
    g[o.b2 + u] = gb2;
    g[o.w3 + u] = gw3;
    if (u == 0) {
        g[o.b3] = gb3;
        atomicAdd(loss, lsum);
    }
}

// grad[i] = sum over the blocks' partials, in block order
__global__ void k_grad_sum(const float *__restrict__ gpart, int nblocks, int n, int K, float *__restrict__ grad) {
    const Offs o = offs(K);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int t = part_index(i, o, K);
        float g = 0.f;
        for (int b = 0; b < nblocks; ++b) g += gpart[(size_t) b * n + t];
        grad[i] = g;
    }
}

size_t grad_smem(int K) {
    const int KP = odd_stride(K);
    return sizeof(float) * ((size_t) H * KP + (size_t) H * kH2 + (size_t) K * kSPB + kSPB + 2 * (size_t) H * kSPB +
                            2 * kSPB);
}

// ---- Adam: sum of the partial gradients (block order), update; the last block out records
// the loss and advances the step (every block reads the step before any block advances it:
// the counter is only touched after the reads) ---------------------------------------------
__global__ void __launch_bounds__(256) k_adam(float *__restrict__ params, const float *__restrict__ gpart,
                                              int nblocks, float *__restrict__ m, float *__restrict__ v, int n,
                                              unsigned *__restrict__ step, unsigned *__restrict__ done,
                                              double *__restrict__ loss_acc, float *__restrict__ loss_hist,
                                              int batch, float lr, int K) {
    const unsigned t = *step + 1u;
    const float c1 = 1.f - powf(0.9f, (float) t), c2 = 1.f - powf(0.999f, (float) t);
    const Offs o = offs(K);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int pi = part_index(i, o, K);
        float g = 0.f;
#pragma unroll 8
        for (int b = 0; b < nblocks; ++b) g += gpart[(size_t) b * n + pi];
        const float mi = 0.9f * m[i] + 0.1f * g;
        const float vi = 0.999f * v[i] + 0.001f * g * g;
        m[i] = mi;
        v[i] = vi;
        params[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(done, 1u);
        if (prev == gridDim.x - 1) {
            loss_hist[t - 1] = (float) (*loss_acc / batch);
            *loss_acc = 0.0;
            *step = t;
            *done = 0u;
        }
    }
}

// ---- inference with BF16-rounded weights (FP32 accumulation) --------------------------------
__global__ void __launch_bounds__(H) k_mlp_infer(const float *__restrict__ params, int K, const float *__restrict__ x,
                                                  const float *__restrict__ scale, int nrows, float mu, float sd,
                                                  double *__restrict__ beta_hat) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int KP = odd_stride(K);
    __nv_bfloat16 *W1 = reinterpret_cast<__nv_bfloat16 *>(smraw);
    __nv_bfloat16 *W2 = W1 + H * KP;
    float *xs = reinterpret_cast<float *>(smraw + (((size_t) H * KP + (size_t) H * kH2) * 2 + 15) / 16 * 16);
    float *h1 = xs + KP;
    float *red = h1 + H;
    const unsigned full = 0xffffffffu;
    const int u = threadIdx.x;
    const Offs o = offs(K);
    for (int e = u; e < H * K; e += H) W1[(e / K) * KP + e % K] = __float2bfloat16(params[o.w1 + e]);
    for (int e = u; e < H * H; e += H) W2[(e / H) * kH2 + e % H] = __float2bfloat16(params[o.w2 + e]);
    const float b1 = params[o.b1 + u], b2 = params[o.b2 + u], w3 = __bfloat162float(__float2bfloat16(params[o.w3 + u]));
    const float b3 = params[o.b3];
    __syncthreads();
    for (int r = blockIdx.x; r < nrows; r += gridDim.x) {
        for (int j = u; j < K; j += H) xs[j] = x[(size_t) r * K + j];
        __syncthreads();
        float a1 = b1;
        for (int j = 0; j < K; ++j) a1 = fmaf(__bfloat162float(W1[u * KP + j]), xs[j], a1);
        h1[u] = a1 > 0.f ? a1 : 0.f;
        __syncthreads();
        float a2 = b2;
        for (int k = 0; k < H; ++k) a2 = fmaf(__bfloat162float(W2[u * kH2 + k]), h1[k], a2);
        float p = w3 * (a2 > 0.f ? a2 : 0.f);
        for (int off = 16; off; off >>= 1) p += __shfl_xor_sync(full, p, off);
        if ((u & 31) == 0) red[u >> 5] = p;
        __syncthreads();
        if (u == 0) {
            const float out = red[0] + red[1] + b3;
            const float s = scale[r];
            beta_hat[r] = s > 0.f ? exp((double) out * sd + mu) / (double) s : -1.0;
        }
        __syncthreads();
    }
}

size_t infer_smem(int K) {
    const int KP = odd_stride(K);
    return (((size_t) H * KP + (size_t) H * kH2) * 2 + 15) / 16 * 16 + sizeof(float) * (KP + H + 2);
}

// ---- warm-started calibration: safeguarded Newton on H(beta) = log(perplexity) --------------
// H(beta) = beta <d> + log sum exp(-beta d) (the reference's formula, sum seeded with
// DBL_MIN), decreasing in beta, dH/dbeta = -beta Var(d).  The bracket [lo, hi] shrinks with
// every evaluation; a Newton step that leaves it, or a missing prediction, is replaced by
// doubling / bisection as in the reference.
//
// The first steps run in FP32 on the row's distances shifted by their minimum (staged in
// shared memory, one column per thread), where H = beta <t> + log sum exp(-beta t) has no
// cancellation and a bound on its error (screen_value, shared with the bisection): a step
// moves the bracket only when the sign of H - log U is certain, and the FP32 phase ends when
// |H - log U| is within that bound, after one last Newton step from that value.  The FP64 steps that follow take the row to the
// acceptance test |H - log U| < 1e-6; each writes exp(-beta d) to the output row, so the
// accepted evaluation's values only need the normalisation.
__global__ void k_calibrate_warm(const double *__restrict__ dist, int stride, int offset, double *__restrict__ P,
                                 int nrows, int K, double perplexity, const double *__restrict__ beta_hat,
                                 int *__restrict__ iters, int *__restrict__ fallback, int stage) {
    extern __shared__ float s_shift[];
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    const double *d = dist + (size_t) r * stride + offset;
    double *p = P + (size_t) r * K;
    const double logU = log(perplexity);
    const double tol = 1e-6;
    double beta = beta_hat[r];
    int fb = 0;
    if (!(beta > 0.0) || !isfinite(beta)) {
        beta = 1.0;
        fb = 1;
    }
    double lo = 0.0, hi = HUGE_VAL;
    int it = 0;
    if (stage) {
        double d0 = d[0];
        for (int m = 1; m < K; ++m) d0 = fmin(d0, d[m]);
        float *w = s_shift + threadIdx.x;
        const size_t sst = blockDim.x;
        for (int m = 0; m < K; ++m) w[m * sst] = (float) (d[m] - d0);
        while (it < 30 && beta > 1e-30 && beta < 1e30 && beta * d0 <= 600.0) {
            double E;
            float mt, m2;
            const float h = screen_value(w, (int) sst, K, beta, &E, &mt, &m2);
            ++it;
            const double f = (double) h - logU;
            const bool last = !(fabs(f) > E + tol) || !(E < 1e-2);
            if (!last) {  // the sign is certain: the bracket moves
                if (f > 0.0)
                    lo = beta;
                else
                    hi = beta;
            }
            // dH/dbeta = -beta Var(t) (the variance is shift-invariant)
            const double dH = -beta * ((double) m2 - (double) mt * (double) mt);
            const double nb = dH < 0.0 ? beta - f / dH : -1.0;
            if (nb > lo && nb < hi && isfinite(nb)) {
                beta = nb;
            } else if (!last) {
                fb = 1;
                beta = isinf(hi) ? 2.0 * beta : 0.5 * (lo + hi);
            }
            // within the FP32 value's error bound of the target: one last Newton step from it
            // (taken above when it stays in the bracket), then FP64 from here
            if (last) break;
        }
    }
    double last_sum = DBL_MIN;
    int it64 = 0;
    while (it64 < 200) {
        double sum_P = DBL_MIN, s1 = 0.0, s2 = 0.0;
        for (int m = 0; m < K; ++m) {
            const double e = exp(-beta * d[m]);
            p[m] = e;
            sum_P += e;
            s1 += d[m] * e;
            s2 += d[m] * d[m] * e;
        }
        last_sum = sum_P;
        const double Hv = beta * s1 / sum_P + log(sum_P);
        ++it64;
        const double f = Hv - logU;
        if (fabs(f) < tol) break;
        if (f > 0.0)
            lo = beta;
        else
            hi = beta;
        const double ed = s1 / sum_P;
        const double dH = -beta * (s2 / sum_P - ed * ed);
        const double nb = dH < 0.0 ? beta - f / dH : -1.0;
        if (nb > lo && nb < hi && isfinite(nb)) {
            beta = nb;
        } else {
            fb = 1;
            beta = isinf(hi) ? 2.0 * beta : 0.5 * (lo + hi);
        }
    }
    // p holds the last evaluation's row (the accepted one, or the last of 200 steps)
    for (int m = 0; m < K; ++m) p[m] /= last_sum;
    iters[r] = it + it64;
    fallback[r] = fb;
}

uint64_t splitmix(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// He-uniform initial weights (fixed seed: training is reproducible up to FP32 atomics)
std::vector<float> init_params(int K) {
    const Offs o = offs(K);
    std::vector<float> p((size_t) o.n, 0.f);
    uint64_t s = 0x5EEDF17ull;
    auto uni = [&s]() { return (float) ((splitmix(s) >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f; };
    const float a1 = std::sqrt(6.f / (float) K), a2 = std::sqrt(6.f / (float) H);
    for (int e = 0; e < H * K; ++e) p[o.w1 + e] = a1 * uni();
    for (int e = 0; e < H * H; ++e) p[o.w2 + e] = a2 * uni();
    for (int e = 0; e < H; ++e) p[o.w3 + e] = a2 * uni();
    return p;
}

#define MCK(x)                                                         \
    do {                                                               \
        cudaError_t e_ = (x);                                          \
        if (e_ != cudaSuccess) {                                       \
            err = std::string(#x) + ": " + cudaGetErrorString(e_);     \
            return -10;                                                \
        }                                                              \
    } while (0)

// device buffers released on every path
struct Bufs {
    std::vector<void *> p;
    template <typename T>
    cudaError_t get(T **out, size_t n) {
        void *v = nullptr;
        cudaError_t e = cudaMalloc(&v, n * sizeof(T) + 16);
        if (e == cudaSuccess) p.push_back(v);
        *out = reinterpret_cast<T *>(v);
        return e;
    }
    ~Bufs() {
        for (void *v : p) cudaFree(v);
    }
};

}  // namespace

namespace {
int g_calib_mode = -1;
MlpStats g_calib_stats;
std::mutex g_calib_mu;
}  // namespace

int calibration_mode() {
    std::lock_guard<std::mutex> lk(g_calib_mu);
    if (g_calib_mode < 0) {
        const char *e = std::getenv("FITSNE_CALIBRATION");
        g_calib_mode = (e && std::strcmp(e, "learned") == 0) ? 1 : 0;
    }
    return g_calib_mode;
}
void set_calibration_mode(int mode) {
    std::lock_guard<std::mutex> lk(g_calib_mu);
    g_calib_mode = mode == 1 ? 1 : 0;
}
void store_calibration_stats(const MlpStats &s) {
    std::lock_guard<std::mutex> lk(g_calib_mu);
    g_calib_stats = s;
}
MlpStats last_calibration_stats() {
    std::lock_guard<std::mutex> lk(g_calib_mu);
    return g_calib_stats;
}

int calibrate_rows_learned(const double *dist, int stride, int offset, double *P, int nrows, int K, double perplexity,
                           cudaStream_t st, MlpStats *stats, std::string &err) {
    MlpStats sx;
    sx.rows = nrows;
    const int nh = std::min(200000, std::max(10000, nrows / 10));
    if (K > kMlpMaxIn || nrows < 2 * nh || perplexity <= 0) {
        // too few rows to learn from: the plain bisection for all
        std::vector<int> it;
        const double t0 = now_ms();
        int rc = calibrate_rows(dist, stride, offset, P, nrows, K, perplexity, 0.0, 0, nullptr, nullptr, st, err,
                                &it);
        if (rc) return rc;
        sx.rows_harvest = nrows;
        double s = 0;
        for (int v : it) s += v;
        sx.iters_plain = nrows ? s / nrows : 0;
        sx.ms_harvest = now_ms() - t0;
        if (stats) *stats = sx;
        return 0;
    }
    sx.rows_harvest = nh;
    Bufs b;
    const Offs o = offs(K);
    float *x = nullptr, *scale = nullptr, *target = nullptr, *params = nullptr, *grad = nullptr, *m = nullptr,
          *v = nullptr, *hist = nullptr;
    double *beta = nullptr, *loss = nullptr, *beta_hat = nullptr;
    unsigned *step = nullptr, *done = nullptr;
    int *iters = nullptr, *fb = nullptr;
    MCK(b.get(&x, (size_t) nrows * K));
    MCK(b.get(&scale, (size_t) nrows));
    MCK(b.get(&target, (size_t) nh));
    MCK(b.get(&beta, (size_t) nh));
    MCK(b.get(&params, (size_t) o.n));
    MCK(b.get(&m, (size_t) o.n));
    MCK(b.get(&v, (size_t) o.n));
    MCK(b.get(&loss, 1));
    MCK(b.get(&step, 1));
    MCK(b.get(&done, 1));
    MCK(b.get(&beta_hat, (size_t) (nrows - nh)));
    MCK(b.get(&iters, (size_t) (nrows - nh)));
    MCK(b.get(&fb, (size_t) (nrows - nh)));

    // 1. harvest: the plain bisection (reference semantics) on the first nh rows
    double t0 = now_ms();
    std::vector<int> it_plain;
    int rc = calibrate_rows(dist, stride, offset, P, nh, K, perplexity, 0.0, 0, nullptr, beta, st, err, &it_plain);
    if (rc) return rc;
    double s = 0;
    for (int vv : it_plain) s += vv;
    sx.iters_plain = s / nh;
    sx.ms_harvest = now_ms() - t0;

    // 2. features of every row, targets of the harvested ones; standardisation on the host
    t0 = now_ms();
    k_features<<<1024, 256, 0, st>>>(dist, stride, offset, nrows, K, nullptr, x, scale, nullptr);
    k_features<<<1024, 256, 0, st>>>(dist, stride, offset, nh, K, beta, x, scale, target);
    std::vector<float> ht(nh);
    MCK(cudaMemcpyAsync(ht.data(), target, sizeof(float) * nh, cudaMemcpyDeviceToHost, st));
    MCK(cudaStreamSynchronize(st));
    double mu = 0, var = 0;
    for (float t : ht) mu += t;
    mu /= nh;
    for (float t : ht) var += (t - mu) * (t - mu);
    const double sd = std::max(1e-3, std::sqrt(var / nh));

    // 3. training: Adam on random minibatches, kGraphSteps steps per captured graph
    std::vector<float> p0 = init_params(K);
    MCK(cudaMemcpyAsync(params, p0.data(), sizeof(float) * o.n, cudaMemcpyHostToDevice, st));
    MCK(cudaMemsetAsync(m, 0, sizeof(float) * o.n, st));
    MCK(cudaMemsetAsync(v, 0, sizeof(float) * o.n, st));
    MCK(cudaMemsetAsync(loss, 0, sizeof(double), st));
    MCK(cudaMemsetAsync(step, 0, sizeof(unsigned), st));
    MCK(cudaMemsetAsync(done, 0, sizeof(unsigned), st));
    // Minibatches of 512 rows at step size 3e-3; 600 steps up to 20,000 harvested rows, fewer
    // above (12 million / harvested rows, at least 100; FITSNE_MLP_STEPS / FITSNE_MLP_BATCH /
    // FITSNE_MLP_LR override): the search only needs a seed within a few per cent of beta.
    // Measured at N = 1M (100,000 harvested rows): the warm-started search took 16.0 - 16.4 ms
    // and 4.35 - 4.58 evaluations per predicted row for 100 to 600 steps, while the training
    // took 41 us a step; at 60,000 points (10,000 rows) the loss still falls to 0.15 of its
    // first value by step 600 (0.47 at 200).
    int batch = kBatch, want = std::max(100, std::min(600, (int) (12000000LL / std::max(1, nh))));
    if (const char *eb = std::getenv("FITSNE_MLP_BATCH")) batch = std::max(kSPB, std::min(8192, std::atoi(eb)));
    if (const char *es = std::getenv("FITSNE_MLP_STEPS")) want = std::max(kGraphSteps, std::min(20000, std::atoi(es)));
    const int nsteps = want / kGraphSteps * kGraphSteps;
    float lr = kLr;
    if (const char *el = std::getenv("FITSNE_MLP_LR")) lr = std::max(1e-5f, std::min(0.1f, (float) std::atof(el)));
    MCK(b.get(&hist, (size_t) nsteps));
    const size_t gsm = grad_smem(K);
    MCK(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) gsm));
    const int gblocks = (batch + kSPB - 1) / kSPB;
    MCK(b.get(&grad, (size_t) gblocks * o.n));  // the blocks' partial gradients
    const int ablocks = (o.n + 255) / 256;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    MCK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < kGraphSteps; ++k) {
        k_mlp_grad<<<gblocks, H, gsm, st>>>(params, K, x, target, nh, batch, (float) mu, (float) (1.0 / sd), step,
                                            grad, loss);
        k_adam<<<ablocks, 256, 0, st>>>(params, grad, gblocks, m, v, o.n, step, done, loss, hist, batch, lr, K);
    }
    cudaError_t ce = cudaStreamEndCapture(st, &graph);
    if (ce == cudaSuccess) ce = cudaGraphInstantiate(&exec, graph, 0);
    for (int g = 0; ce == cudaSuccess && g < nsteps / kGraphSteps; ++g) ce = cudaGraphLaunch(exec, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
        err = std::string("mlp training: ") + cudaGetErrorString(ce);
        return -10;
    }
    std::vector<float> hh(nsteps);
    MCK(cudaMemcpy(hh.data(), hist, sizeof(float) * nsteps, cudaMemcpyDeviceToHost));
    sx.train_steps = nsteps;
    sx.loss_first = hh.front();
    // the last ten steps' mean (minibatch noise)
    double lt = 0;
    for (int k = nsteps - 10; k < nsteps; ++k) lt += hh[k];
    sx.loss_last = lt / 10;
    sx.ms_train = now_ms() - t0;

    // 4. inference for the remaining rows (BF16 weights)
    t0 = now_ms();
    const int nr = nrows - nh;
    const size_t ism = infer_smem(K);
    MCK(cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) ism));
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    k_mlp_infer<<<nsm * 16, H, ism, st>>>(params, K, x + (size_t) nh * K, scale + nh, nr, (float) mu, (float) sd,
                                          beta_hat);
    MCK(cudaGetLastError());
    MCK(cudaStreamSynchronize(st));
    sx.ms_infer = now_ms() - t0;

    // 5. warm-started calibration of the remaining rows
    t0 = now_ms();
    int bd = 128;
    while (bd > 32 && (size_t) bd * K * sizeof(float) > 160 * 1024) bd /= 2;
    const size_t wsm = (size_t) bd * K * sizeof(float);
    const int stage = wsm <= 160 * 1024 ? 1 : 0;
    if (stage) MCK(cudaFuncSetAttribute(k_calibrate_warm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) wsm));
    k_calibrate_warm<<<(nr + bd - 1) / bd, bd, stage ? wsm : 0, st>>>(dist + (size_t) nh * stride, stride, offset,
                                                                       P + (size_t) nh * K, nr, K, perplexity,
                                                                       beta_hat, iters, fb, stage);
    MCK(cudaGetLastError());
    std::vector<int> hi(nr), hf(nr);
    MCK(cudaMemcpyAsync(hi.data(), iters, sizeof(int) * nr, cudaMemcpyDeviceToHost, st));
    MCK(cudaMemcpyAsync(hf.data(), fb, sizeof(int) * nr, cudaMemcpyDeviceToHost, st));
    MCK(cudaStreamSynchronize(st));
    sx.ms_warm = now_ms() - t0;
    double si = 0;
    int nf = 0;
    for (int k = 0; k < nr; ++k) {
        si += hi[k];
        nf += hf[k];
    }
    sx.iters_warm = si / nr;
    sx.rows_fallback = nf;
    if (stats) *stats = sx;
    return 0;
}

int mlp_loss_grad_host(const float *params, int K, const double *dist, const double *beta, int nrows, double mu,
                       double sd, float *grad, double *loss, std::string &err) {
    if (K < 1 || K > kMlpMaxIn || nrows < 1) {
        err = "invalid MLP shape";
        return -3;
    }
    const Offs o = offs(K);
    Bufs b;
    float *dp = nullptr, *dg = nullptr, *x = nullptr, *scale = nullptr, *target = nullptr;
    double *dd = nullptr, *db = nullptr, *dl = nullptr;
    const int gblocks = (nrows + kSPB - 1) / kSPB;
    float *gp = nullptr;
    MCK(b.get(&dp, (size_t) o.n));
    MCK(b.get(&dg, (size_t) o.n));
    MCK(b.get(&gp, (size_t) gblocks * o.n));
    MCK(b.get(&dd, (size_t) nrows * K));
    MCK(b.get(&db, (size_t) nrows));
    MCK(b.get(&x, (size_t) nrows * K));
    MCK(b.get(&scale, (size_t) nrows));
    MCK(b.get(&target, (size_t) nrows));
    MCK(b.get(&dl, 1));
    MCK(cudaMemcpy(dp, params, sizeof(float) * o.n, cudaMemcpyHostToDevice));
    MCK(cudaMemcpy(dd, dist, sizeof(double) * (size_t) nrows * K, cudaMemcpyHostToDevice));
    MCK(cudaMemcpy(db, beta, sizeof(double) * nrows, cudaMemcpyHostToDevice));
    MCK(cudaMemset(dl, 0, sizeof(double)));
    k_features<<<256, 256>>>(dd, K, 0, nrows, K, db, x, scale, target);
    const size_t gsm = grad_smem(K);
    MCK(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) gsm));
    k_mlp_grad<<<gblocks, H, gsm>>>(dp, K, x, target, nrows, nrows, (float) mu, (float) (1.0 / sd), nullptr, gp, dl);
    k_grad_sum<<<(o.n + 255) / 256, 256>>>(gp, gblocks, o.n, K, dg);
    MCK(cudaGetLastError());
    MCK(cudaDeviceSynchronize());
    MCK(cudaMemcpy(grad, dg, sizeof(float) * o.n, cudaMemcpyDeviceToHost));
    double l = 0;
    MCK(cudaMemcpy(&l, dl, sizeof(double), cudaMemcpyDeviceToHost));
    *loss = l / nrows;
    return 0;
}

}  // namespace fitsne
