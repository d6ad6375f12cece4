// fitsne_fft_gradient_noalloc: the FP32 gradient evaluation for callers that cannot allocate
// device memory.
//
// Some callers own all of the device's memory through their own pool or budget (a host
// framework with a caching allocator, a service with a fixed memory plan) or must not
// trigger an allocation -- and the device synchronisation that comes with it -- in their
// inner loop.  They cannot let this library call cudaMalloc.  This entry point takes the
// caller's device buffers for inputs and outputs and takes every temporary it needs (the
// double-float copy of Y, the interpolation grids, the FFT work buffers and kernel
// spectrum, the repulsion numerators, the reduction partials) from one file-scope device
// array of fixed size, kNoAllocBytes, which every GPU that loads this library holds until
// the process exits.
//
// Layout: the per-point buffers and the reduction scratch are carved first; the grid, FFT
// and kernel-spectrum buffers are carved after the embedding's extent has fixed the grid,
// from its actual node count M and transform length L.  Limits (checked, with an error
// message, before any device work that depends on them): N <= kNoAllocMaxN points; the
// grid buffers must fit in what the per-point buffers leave of the array (in 2-D about
// 160 (nterms * boxes)^2 bytes, in 1-D about 100 bytes per node); the transform length must
// fit the shared-memory FFT passes (as for every other entry point).
//
// The array is shared by every call on a device and keeps the last call's contents: the
// grid and the reduction counters are cleared at the start of each call.  Two calls whose
// work overlaps on the GPU (for example on two streams) race on the array; serialise them.
// The array's device address is looked up with the device current, once per CUDA context
// (again after a device reset, which creates a new context); the first call on a device
// does that lookup, so make it before any stream capture.
#include <cuda.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/fitsne_gb300.h"
#include "capi_internal.h"
#include "embedding.cuh"
#include "fftconv.cuh"
#include "grad.cuh"

namespace fitsne {
namespace {

constexpr size_t kNoAllocBytes = 32ull << 20;  // 32 MiB per device
constexpr int kNoAllocMaxN = 262144;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

std::mutex g_mu;
void *g_addr[kMaxDevices] = {};
unsigned long long g_ctx_id[kMaxDevices] = {};
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
bool g_driver_looked_up = false;

// Unique id of the calling thread's current CUDA context (0 if none or unavailable).  A
// device reset destroys the primary context; the next one gets a new id, and the array is
// then at a new device address.
unsigned long long current_ctx_id() {
    if (!g_driver_looked_up) {
        g_driver_looked_up = true;
        void *f1 = nullptr, *f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q2 == cudaDriverEntryPointSuccess) {
            g_ctx_current = reinterpret_cast<CtxGetCurrentFn>(f1);
            g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
        }
        cudaGetLastError();
    }
    if (!g_ctx_current || !g_ctx_get_id) return 0;
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (g_ctx_current(&c) != CUDA_SUCCESS || !c) return 0;
    if (g_ctx_get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the scratch array on the current device, looked up with that device
// current once per context.  Host code may only pass this address to kernels: the symbol
// itself names a host-side stand-in.
int scratch_base(void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(FITSNE_E_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return set_error(FITSNE_E_ARG, "device index out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    // cudaSetDevice makes the device's primary context current on this thread, so that the
    // context id below names the context the kernels will run in
    e = cudaSetDevice(dev);
    if (e != cudaSuccess) return set_error(FITSNE_E_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    const unsigned long long ctx = current_ctx_id();
    if (!g_addr[dev] || ctx == 0 || ctx != g_ctx_id[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return set_error(FITSNE_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_addr[dev] = p;
        g_ctx_id[dev] = current_ctx_id();
    }
    *out = g_addr[dev];
    return 0;
}

// bump allocator over the scratch array
struct Carve {
    unsigned char *base;
    size_t used = 0;
    template <typename P>
    P *take(size_t count) {
        used = (used + 255) & ~(size_t) 255;
        P *p = reinterpret_cast<P *>(base + used);
        used += sizeof(P) * count;
        return p;
    }
};

__global__ void k_twiddles(float2 *tw, int L) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < L; j += gridDim.x * blockDim.x) {
        double s, c;
        sincospi(2.0 * (double) j / (double) L, &s, &c);
        tw[j] = make_float2((float) c, (float) -s);
    }
}

__global__ void k_f2d(const float *__restrict__ a, double *__restrict__ b, size_t n) {
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n; i += (size_t) gridDim.x * blockDim.x)
        b[i] = (double) a[i];
}

#define NCK(x)                                                                      \
    do {                                                                            \
        cudaError_t e__ = (x);                                                      \
        if (e__ != cudaSuccess)                                                     \
            return set_error(FITSNE_E_CUDA, std::string(#x) + ": " + cudaGetErrorString(e__)); \
    } while (0)

}  // namespace
}  // namespace fitsne

using namespace fitsne;

extern "C" int fitsne_fft_gradient_noalloc(const unsigned int *d_row_P, const unsigned int *d_col_P,
                                           const float *d_val_P, const double *d_Y, int N, int no_dims,
                                           double *d_dC, int nterms, double intervals_per_integer,
                                           int min_num_intervals, double df, double *sum_Q, void *stream) {
    if (!d_row_P || !d_col_P || !d_val_P || !d_Y || !d_dC || N < 1)
        return set_error(FITSNE_E_ARG, "null device buffer or N < 1");
    if (N > kNoAllocMaxN)
        return set_error(FITSNE_E_ARG, "fitsne_fft_gradient_noalloc: N = " + std::to_string(N) + " exceeds the limit " +
                                           std::to_string(kNoAllocMaxN) + " of the fixed scratch array");
    if (no_dims != 1 && no_dims != 2)
        return set_error(FITSNE_E_ARG, "FFT interpolation supports only 1 or 2 output dimensions");
    if (nterms < 1 || nterms > kMaxInterp) return set_error(FITSNE_E_ARG, "n_interpolation_points must be in [1, 8]");
    if (!(intervals_per_integer > 0) || min_num_intervals < 1 || !(df > 0))
        return set_error(FITSNE_E_ARG, "invalid interpolation grid parameters");
    int rc = check_cuda_device();
    if (rc) return rc;
    void *base = nullptr;
    rc = scratch_base(&base);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int D = no_dims;

    // per-point buffers and reduction scratch; the grid's buffers follow once its size is known
    Carve cv{static_cast<unsigned char *>(base)};
    float *Yb = cv.take<float>((size_t) N * 2 * D);
    float *rep = cv.take<float>((size_t) N * D);
    float *dCf = cv.take<float>((size_t) N * D);
    double *red_mem = cv.take<double>(kMaxRedBlocks * 4 + 16);
    unsigned int *red_cnt = cv.take<unsigned int>(8);
    const size_t point_bytes = cv.used;  // <= 8.3 MiB at N = kNoAllocMaxN: fits

    RedScratch red;
    red.part = red_mem;
    red.count = red_cnt;
    red.mnmx = red_mem + kMaxRedBlocks * 4;
    red.z = red.mnmx + 2;
    red.mean = red.z + 1;
    red.kl = red.mean + 2;
    // the array keeps the previous call's contents: reset what must start at zero
    NCK(cudaMemsetAsync(red_cnt, 0, sizeof(unsigned int) * 8, st));
    NCK(cudaMemsetAsync(red.mnmx, 0, sizeof(double) * 16, st));

    NCK(launch_y_from_double<float>(d_Y, Yb, N, D, st));
    NCK(launch_center_minmax<float>(Yb, N, D, 0, 0, red, st));
    double mm[2] = {0.0, 0.0};
    NCK(cudaMemcpyAsync(mm, red.mnmx, sizeof(mm), cudaMemcpyDeviceToHost, st));
    NCK(cudaStreamSynchronize(st));
    if (!std::isfinite(mm[0]) || !std::isfinite(mm[1])) return set_error(FITSNE_E_ARG, "Y is not finite");
    GridParams gp;
    gp.nterms = nterms;
    gp.intervals_per_integer = intervals_per_integer;
    gp.min_num_intervals = min_num_intervals;
    gp.df = df;
    const GridGeom g = make_grid_geom(mm[0], mm[1], D, gp);
    const int L = smooth_even_at_least(2 * g.M);
    FftPlan plan;
    if (!make_fft_plan(L, &plan)) return set_error(FITSNE_E_GRID, "bad FFT length");
    const bool fits_fft = (D == 2) ? (L <= max_fft_len<float>())
                                   : (2 * (size_t) L * sizeof(float2) <= 227 * 1024);
    if (!fits_fft)
        return set_error(FITSNE_E_GRID, "fitsne_fft_gradient_noalloc: the embedding needs " + std::to_string(g.nb) +
                                            " boxes per dimension (transform length " + std::to_string(L) +
                                            "), beyond the shared-memory FFT passes");
    const size_t H = (size_t) L / 2 + 1;
    const size_t cells = (D == 2) ? (size_t) g.M * g.M : (size_t) g.M;
    Cell4<float> *gin = cv.take<Cell4<float>>(cells);
    Cell4<float> *gout = cv.take<Cell4<float>>(cells);
    float2 *wa = cv.take<float2>((D == 2) ? 4 * (size_t) L * H : 6 * (size_t) L);
    float2 *wb = cv.take<float2>((D == 2) ? 4 * (size_t) g.M * H : 1);
    KSpec<float> *ks = cv.take<KSpec<float>>((D == 2) ? (size_t) L * H : 1);
    float2 *tw = cv.take<float2>(L);
    if (cv.used > kNoAllocBytes)
        return set_error(FITSNE_E_GRID,
                         "fitsne_fft_gradient_noalloc: N = " + std::to_string(N) + " and a grid of " +
                             std::to_string(g.nb) + " boxes per dimension x " + std::to_string(nterms) +
                             " nodes need " + std::to_string(point_bytes) + " + " +
                             std::to_string(cv.used - point_bytes) + " bytes of scratch; the fixed array holds " +
                             std::to_string(kNoAllocBytes));

    const int mode = (df == 1.0) ? KERNEL_DF1 : KERNEL_VARDF;
    k_twiddles<<<(L + 255) / 256, 256, 0, st>>>(tw, L);
    NCK(cudaGetLastError());
    NCK(cudaMemsetAsync(gin, 0, sizeof(Cell4<float>) * cells, st));
    NCK(launch_spread<float>(Yb, N, D, g, gin, st));
    if (D == 2)
        NCK(conv2d_launch<float>(gin, gout, g.M, plan, tw, wa, wb, ks, g.hk, df, mode, st));
    else
        NCK(conv1d_launch<float>(gin, gout, g.M, plan, tw, wa, g.hk, df, mode, st));
    NCK(launch_gather<float>(Yb, N, D, g, gout, mode, rep, red, st));
    UpdateParams p{};
    p.mode = 0;
    p.exag = 1.0;
    p.df = df;
    NCK(launch_attr_update<float>(d_row_P, d_col_P, d_val_P, Yb, nullptr, nullptr, nullptr, dCf, rep, N, D, p, red,
                                  st));
    k_f2d<<<256, 256, 0, st>>>(dCf, d_dC, (size_t) N * D);
    NCK(cudaGetLastError());
    double z = 0.0;
    NCK(cudaMemcpyAsync(&z, red.z, sizeof(double), cudaMemcpyDeviceToHost, st));
    NCK(cudaStreamSynchronize(st));
    if (sum_Q) *sum_Q = z;
    return 0;
}
