// Per-iteration gradient kernels of FIt-SNE (everything except the FFT convolution).
//
// Reference functions replaced (src/ paths of KlugerLab/FIt-SNE v1.2.1):
//   computeFftGradient          tsne.cpp:1027-1169   (2-D, df = 1)
//   computeFftGradientVariableDf tsne.cpp:860-1024   (2-D, df != 1)
//   computeFftGradientOneD      tsne.cpp:758-856     (1-D, df = 1)
//   computeFftGradientOneDVariableDf tsne.cpp:647-754 (1-D, df != 1)
//   n_body_fft_2d / nbodyfft steps 1 and 3, interpolate  nbodyfft.cpp:73-248, 310-455
//   TSNE::run update loop + zeroMean                      tsne.cpp:479-531, 1851-1876
//   evaluateErrorFft                                       tsne.cpp:1329-1355
//
// Charges are spread in box-local coordinates.  The reference spreads the charges
// (1, x, y, x^2 + y^2) and forms the repulsion as x_i phi_1 - phi_2, which cancels
// catastrophically in FP32 far from the origin.  Here each node b receives
// (w, w*(x_j - x_b), w*(y_j - y_b), w*|y_j - y_b|^2), and the convolution uses the
// kernels K, Gx = K*dx, Gy = K*dy, H = K*|d|^2 so that
//   rep_x(i) = sum_a L_a(y_i) [ (x_i - x_a) V1(a) + Rx(a) ]
//   Z_i      = sum_a L_a(y_i) [ (1 + |y_i - y_a|^2) V1(a) + 2 (y_i - y_a).R(a) + S(a) ]
// with V1 = K*W1, Rx = Gx*W1 - K*W2', Ry = Gy*W1 - K*W3',
//      S = H*W1 - 2 (Gx*W2' + Gy*W3') + K*W4'.
// This is an exact algebraic rewrite of the reference's interpolated sums (same nodes,
// same Lagrange weights, same kernel samples), so the FP64 form agrees with the
// reference to rounding, and the FP32 form keeps every quantity box-local.
#pragma once

#include "common.cuh"
#include "fftconv.cuh"

namespace fitsne {

// Interpolation grid of one gradient evaluation.
struct GridGeom {
    int nb;         // boxes per dimension
    int nterms;     // interpolation points per box
    int M;          // nterms * nb
    double mn;      // lower corner (both axes in 2-D)
    double bw;      // box width
    double hk;      // node spacing used for the kernel samples (box width / nterms)
    float s32[kMaxInterp], inv_den32[kMaxInterp];
    double s64[kMaxInterp], inv_den64[kMaxInterp];
    // FP32 forms for the FP32 kernels: -mn and bw as double-float (hi, lo) pairs, 1 / bw
    // rounded to float.  Made once here instead of by every thread of the spread and gather
    // (FP64 conversions and a division on the FP64 pipe; the gather at N = 1M went from 0.034
    // to 0.031 ms).
    float neg_mn32[2], bw32[2], inv_bw32;
};

// The reference's grid rule (computeFftGradient*, tsne.cpp:769-780, 1039-1077; box bounds
// and node positions of n_body_fft_2d / nbodyfft): box count truncated from the extent,
// rounded up to the FFT-friendly list below 200 in 2-D; nodes at (k + 1/2) / nterms of a
// box.  Host and device compute it with the same FP64 operations.  A box count above
// nb_max is clamped to nb_max and reported through *clamped (capacity of a captured grid).
FITSNE_HD GridGeom grid_geom(double mn, double mx, int D, int nterms, double ipi, int min_num, int nb_max,
                             int *clamped) {
    GridGeom g;
    int nb = static_cast<int>(fmax((double) min_num, (mx - mn) / ipi));
    if (D == 2) {
        const int allowed[20] = {25, 36, 50, 55, 60, 65, 70, 75, 80, 85, 90, 96, 100, 110, 120, 130, 140, 150, 175, 200};
        if (nb < allowed[19]) {
            int i = 0;
            while (allowed[i] < nb) ++i;
            nb = allowed[i];
        }
    }
    if (nb < 1) nb = 1;
    if (clamped) *clamped = 0;
    if (nb > nb_max) {
        nb = nb_max;
        if (clamped) *clamped = 1;
    }
    g.nb = nb;
    g.nterms = nterms;
    g.M = nb * nterms;
    const double bw = (mx - mn) / (double) nb;
    // n_body_fft_2d / nbodyfft read the lower corner and the width back from the box
    // bounds array: lower[0] = 0*bw + mn, width = (1*bw + mn) - (0*bw + mn)
    g.mn = 0.0 * bw + mn;
    g.bw = (1.0 * bw + mn) - g.mn;
    g.hk = bw / (double) nterms;
    const double h = 1.0 / (double) nterms;
    double s[kMaxInterp];
    s[0] = h / 2.0;
    for (int i = 1; i < nterms && i < kMaxInterp; ++i) s[i] = s[i - 1] + h;
    for (int i = 0; i < kMaxInterp; ++i) {
        g.s64[i] = 0.0;
        g.inv_den64[i] = 0.0;
        g.s32[i] = 0.f;
        g.inv_den32[i] = 0.f;
    }
    for (int i = 0; i < nterms && i < kMaxInterp; ++i) {
        double den = 1.0;
        for (int j = 0; j < nterms; ++j)
            if (i != j) den *= s[i] - s[j];
        g.s64[i] = s[i];
        g.inv_den64[i] = 1.0 / den;
        g.s32[i] = (float) s[i];
        g.inv_den32[i] = (float) (1.0 / den);
    }
    const double nm = -g.mn;
    g.neg_mn32[0] = (float) nm;
    g.neg_mn32[1] = (float) (nm - (double) g.neg_mn32[0]);
    g.bw32[0] = (float) g.bw;
    g.bw32[1] = (float) (g.bw - (double) g.bw32[0]);
    g.inv_bw32 = (float) (1.0 / g.bw);
    return g;
}

// Geometry of one iteration in device memory (see ConvGeom).  status: 0 ok, 1 the grid
// exceeded the capacity it was launched for (results of the iteration are void), 2 the
// coordinates are not finite.
struct DevGeom {
    GridGeom g;
    ConvGeom conv;
    int status;
};

// ---- batched form: many embeddings ("jobs") in concatenated arrays, one launch per stage ----
// The blocks of a batched launch are split among the jobs: job[b] is the job of block b,
// first[j] and count[j] the first block and the number of blocks of job j (device arrays).
struct BatchMap {
    const int *job;
    const int *first;
    const int *count;
};
// One job of the batched iteration (device table).
struct BatchJobDev {
    int p0, n;          // its points: [p0, p0 + n) of the concatenated arrays (CSR rows too)
    int nb_cap, L_cap;  // grid capacity: boxes per dimension and FFT length
    size_t cell0;       // its first cell of the concatenated grids (capacity (nb_cap nterms)^2)
    float lr;           // learning rate
};

// Reduction scratch shared by the kernels of one embedding (device memory).
struct RedScratch {
    double *part;          // per-block partials, up to kMaxRedBlocks * 4 doubles
    unsigned int *count;   // completion counters (4 slots)
    double *mnmx;          // [min, max]
    double *z;             // Z (sum_Q)
    double *mean;          // mean of Y per dimension (2 doubles), consumed by center
    double *kl;            // KL sum
};
constexpr int kMaxRedBlocks = 4096;

struct UpdateParams {
    int mode;               // 0 = write dC only, 1 = optimiser step (reference update rule)
    int use_gains;          // gains/momentum branch (else plain Y -= dY)
    double exag;            // multiplier of P in the attraction
    double momentum;
    double learning_rate;
    double max_step_norm;   // <= 0: no clipping
    double df;
};

// --- launchers (T = float: double-float Y of width 2*D; T = double: plain Y) ---------
// excl: index of the point whose first coordinate is left out of the minimum (the
// caller's point 0 after any internal renumbering).
template <typename T>
cudaError_t launch_center_minmax(T *Y, int N, int D, int apply_mean, int excl, RedScratch r, cudaStream_t st);
// order (may be null): the FP32 nterms-3 spread walks the points as order[0], order[1], ...
// (a 2-D locality order, so that a warp's points share boxes); the other forms ignore it
template <typename T>
cudaError_t launch_spread(const T *Y, int N, int D, const GridGeom &g, Cell4<T> *grid, cudaStream_t st,
                          const uint32_t *order = nullptr);
// yh (may be null): FP32 form only, receives the high words of the positions (D floats per point)
template <typename T>
cudaError_t launch_gather(const T *Y, int N, int D, const GridGeom &g, const Cell4<T> *pot, int mode, T *rep,
                          RedScratch r, cudaStream_t st, float *yh = nullptr);
// As launch_spread / launch_gather with the geometry read from device memory.
template <typename T>
cudaError_t launch_spread_dev(const T *Y, int N, int D, int nterms, const DevGeom *dg, Cell4<T> *grid,
                              cudaStream_t st, const uint32_t *order = nullptr);
template <typename T>
cudaError_t launch_gather_dev(const T *Y, int N, int D, int nterms, const DevGeom *dg, const Cell4<T> *pot, int mode,
                              T *rep, RedScratch r, cudaStream_t st, float *yh = nullptr);
// Grid of the current iteration from r.mnmx into dg (see k_geometry in grad.cu).
cudaError_t launch_geometry(RedScratch r, int D, int nterms, double ipi, int min_num, int nb_cap, int L_cap,
                            DevGeom *dg, int *status_acc, cudaStream_t st);
// Number of attraction launch shapes (rows per work item x edges per lane; see grad.cu) and
// the shape of an index.
constexpr int kNumAttrShapes = 11;
int attr_shape_info(int shape, int *group, int *unroll);
// yh (FP32 form only, may be null): the FP32 positions k_gather wrote for this Y, which the
// attraction then gathers as its neighbours' positions (8 instead of 16 bytes per point in
// 2-D; the neighbour's low word, at most 2^-24 |y| / 2, is dropped from y_i - y_j).
template <typename T>
cudaError_t launch_attr_update(const uint32_t *row, const uint32_t *col, const T *val, const T *Yin, T *Yout,
                               T *uY, T *gains, T *dC, const T *rep, int N, int D, const UpdateParams &p,
                               RedScratch r, cudaStream_t st, int shape = 0, const float *yh = nullptr);
// ---- tiled attraction over the half-stored symmetric P (FP32 form; k_attr_tiles in grad.cu) ----
// Shape index of the tiled form, after the full-CSR shapes (FITSNE_ATTR_SHAPE numbering).
constexpr int kAttrTilesShape = kNumAttrShapes;
// h[0..1] (device): hash sums of the entries and of their transposes; equal iff P is
// symmetric (entries and values), up to a 2^-64 chance.
cudaError_t launch_sym_hash(const uint32_t *row, const uint32_t *col, const float *val, int N,
                            unsigned long long *h, cudaStream_t st);
// ulen[i]: entries of row i with col > i.
cudaError_t launch_upper_count(const uint32_t *row, const uint32_t *col, int N, uint32_t *ulen, cudaStream_t st);
// Blocks of 4,096 points: tile_blocks(N) of them, tile keys A * nblk + B (A <= B).
int tile_blocks(int N);
size_t tile_smem_bytes(int D);
// Per upper entry of the CSR (urow: the exclusive scan of the upper counts): key, index and
// record; tcount (nblk^2, zero on entry) receives the tile sizes.
cudaError_t launch_tile_keys(const uint32_t *row, const uint32_t *col, const float *val, int N, const uint32_t *urow,
                             uint32_t *keys, uint32_t *ids, uint2 *rec, uint32_t *tcount, cudaStream_t st);
cudaError_t launch_tile_gather(const uint2 *rec, const uint32_t *ids, size_t n, uint2 *trec, cudaStream_t st);
// trec: records sorted by tile key (row order within a tile); tstart[nblk^2 + 1]: the tiles'
// first records.  The attraction into acc (N x D floats, zero on entry), then the update of
// launch_attr_update (dC in mode 0), which clears acc again.
cudaError_t launch_attr_tiles_update(const uint2 *trec, const uint32_t *tstart, float *acc, const float *Yin,
                                     float *Yout, float *uY, float *gains, float *dC, const float *rep, int N, int D,
                                     const UpdateParams &p, RedScratch r, cudaStream_t st);
template <typename T>
cudaError_t launch_kl(const uint32_t *row, const uint32_t *col, const T *val, const T *Y, int N, int D, double exag,
                      double df, RedScratch r, cudaStream_t st);
// Batched stages (FP32 form, nterms 3, df = 1).  Each job reduces over its own blocks into its
// own RedScratch rs[j]; Y, rep, yh, uY, gains and the CSR are the concatenated arrays.
cudaError_t launch_batch_center(float *Y, int D, BatchMap m, int nblocks, const BatchJobDev *jobs,
                                const RedScratch *rs, int apply_mean, cudaStream_t st);
cudaError_t launch_batch_geometry(const RedScratch *rs, const BatchJobDev *jobs, int J, int D, int nterms,
                                  double ipi, int min_num, DevGeom *dg, int *status, cudaStream_t st);
cudaError_t launch_batch_spread(const float *Y, int D, BatchMap m, int nblocks, const BatchJobDev *jobs,
                                const DevGeom *dg, Cell4<float> *grid, cudaStream_t st);
cudaError_t launch_batch_gather(const float *Y, int D, BatchMap m, int nblocks, const BatchJobDev *jobs,
                                const DevGeom *dg, const Cell4<float> *pot, float *rep, const RedScratch *rs,
                                float *yh, cudaStream_t st);
cudaError_t launch_batch_attr(const uint32_t *row, const uint32_t *col, const float *val, const float *Yin,
                              float *Yout, float *uY, float *gains, const float *rep, int D, BatchMap m,
                              int nblocks, const BatchJobDev *jobs, const RedScratch *rs, const UpdateParams &p,
                              const float *yh, cudaStream_t st);
cudaError_t launch_batch_kl(const uint32_t *row, const uint32_t *col, const float *val, const float *Y, int D,
                            BatchMap m, int nblocks, const BatchJobDev *jobs, double exag, const RedScratch *rs,
                            cudaStream_t st);
// Blocks the batched attraction may keep resident per SM (for sizing its launch).
int batch_attr_blocks_per_sm();

// host <-> device Y conversion (double array N*D <-> storage layout)
template <typename T>
cudaError_t launch_y_from_double(const double *src, T *Y, int N, int D, cudaStream_t st);
template <typename T>
cudaError_t launch_y_to_double(const T *Y, double *dst, int N, int D, cudaStream_t st);
template <typename T>
cudaError_t launch_cast_from_double(const double *src, T *dst, size_t n, cudaStream_t st);

// width (in T elements) of one point's storage
template <typename T>
constexpr int y_width(int D) { return sizeof(T) == 4 ? 2 * D : D; }

}  // namespace fitsne
