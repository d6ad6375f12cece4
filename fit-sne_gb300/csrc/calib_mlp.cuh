// Learned warm start of the perplexity calibration (no counterpart in the reference; the
// bisection it seeds is distances2similarities, tsne.cpp:1394-1469).
//
// A small MLP (K -> 64 -> 64 -> 1, ReLU, FP32 weights) predicts each point's
// log(beta * mean(d)) from its K sorted kNN distances divided by their mean (beta scales as
// 1 / distance, so the scaled problem is the same for every row).  It is trained on the
// GPU, by this file's forward / backward and Adam kernels, on (distances, beta) pairs
// harvested from the plain bisection of the first rows; its BF16-rounded weights then
// predict beta for the remaining rows, where a safeguarded Newton iteration (bracketed,
// falling back to bisection) solves H(beta) = log(perplexity) to |H - log perplexity| <
// 1e-6.  The network only seeds the search: every row ends in the same entropy test.
#pragma once

#include <cstdint>
#include <string>

#include <cuda_runtime.h>

namespace fitsne {

constexpr int kMlpHidden = 64;
constexpr int kMlpMaxIn = 255;  // distances per row the network accepts

// FP32 parameters, contiguous: W1[64][K], b1[64], W2[64][64], b2[64], w3[64], b3
inline size_t mlp_param_count(int K) {
    return (size_t) kMlpHidden * K + kMlpHidden + kMlpHidden * kMlpHidden + kMlpHidden + kMlpHidden + 1;
}

struct MlpStats {
    int rows = 0;              // rows calibrated
    int rows_harvest = 0;      // rows calibrated by the plain bisection (training pairs)
    int rows_fallback = 0;     // predicted rows whose search needed bisection steps
    int train_steps = 0;
    double iters_plain = 0;    // mean entropy evaluations per harvested row (plain bisection)
    double iters_warm = 0;     // mean entropy evaluations per predicted row (warm start)
    double loss_first = 0;     // mean squared error (standardised target) of the first / last
    double loss_last = 0;      //   training step
    double ms_harvest = 0, ms_train = 0, ms_infer = 0, ms_warm = 0;
};

// Calibrates nrows rows (row r at dist + r*stride + offset, K distances, ascending) for one
// perplexity with the learned warm start; P receives nrows x K similarities.  Falls back to
// the plain bisection when nrows is too small to train on.
int calibrate_rows_learned(const double *dist, int stride, int offset, double *P, int nrows, int K, double perplexity,
                           cudaStream_t st, MlpStats *stats, std::string &err);

// Calibration used by the similarity stage: 0 = the reference's bisection (default; P
// bit-identical to the reference), 1 = learned warm start.  Initial value from
// FITSNE_CALIBRATION (learned / bisection).
int calibration_mode();
void set_calibration_mode(int mode);
// Statistics of the last calibration run by this process.
void store_calibration_stats(const MlpStats &s);
MlpStats last_calibration_stats();

// Test hook: mean squared loss of the standardised target ((log(beta mean d) - mu) / sd)
// over all nrows rows and its gradient with respect to the parameters, on the GPU.
// params / grad: host, mlp_param_count(K) floats; dist (nrows x K) and beta: host.
int mlp_loss_grad_host(const float *params, int K, const double *dist, const double *beta, int nrows, double mu,
                       double sd, float *grad, double *loss, std::string &err);

}  // namespace fitsne
