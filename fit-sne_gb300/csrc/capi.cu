// C ABI: gradient, cost, session and misc entry points (declared in include/fitsne_gb300.h).
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>

#include "calib_mlp.cuh"
#include "../../include/fitsne_gb300.h"
#include "capi_internal.h"
#include "embedding.cuh"
#include "session.cuh"

namespace fitsne {

static thread_local std::string g_last_error;
static int g_precision = -1;

int set_error(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

int precision_bits() {
    if (g_precision < 0) {
        const char *e = std::getenv("FITSNE_PRECISION");
        g_precision = (e && std::atoi(e) == 64) ? 64 : 32;
    }
    return g_precision;
}

int check_cuda_device() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0)
        return set_error(FITSNE_E_CUDA, std::string("no CUDA device available: ") + cudaGetErrorString(e));
    return 0;
}

namespace {

template <typename T>
int gradient_impl(const unsigned int *row_P, const unsigned int *col_P, const double *val_P, const double *Y, int N,
                  int no_dims, double *dC, int nterms, double ipi, int min_num_intervals, double df, double *sum_Q) {
    GridParams gp;
    gp.nterms = nterms;
    gp.intervals_per_integer = ipi;
    gp.min_num_intervals = min_num_intervals;
    gp.df = df;
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
        return set_error(FITSNE_E_CUDA, "cudaStreamCreate failed");
    int rc;
    {
        Embedding<T> emb;
        rc = emb.init_host(N, no_dims, row_P, col_P, val_P, Y, gp, st);
        if (!rc) rc = emb.gradient(dC, sum_Q);
        if (rc) set_error(rc == -13 ? FITSNE_E_GRID : FITSNE_E_CUDA, emb.error());
    }
    cudaStreamDestroy(st);
    return rc ? (rc == -13 ? FITSNE_E_GRID : FITSNE_E_CUDA) : 0;
}

template <typename T>
int kl_impl(const unsigned int *row_P, const unsigned int *col_P, const double *val_P, const double *Y, int N,
            int no_dims, double df, double sum_Q, double *C) {
    GridParams gp;
    gp.df = df;
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
        return set_error(FITSNE_E_CUDA, "cudaStreamCreate failed");
    int rc;
    {
        Embedding<T> emb;
        rc = emb.init_host(N, no_dims, row_P, col_P, val_P, Y, gp, st);
        if (!rc) rc = emb.kl_with_z(1.0, sum_Q, C);
        if (rc) set_error(FITSNE_E_CUDA, emb.error());
    }
    cudaStreamDestroy(st);
    return rc ? FITSNE_E_CUDA : 0;
}

int check_grad_args(const unsigned int *row_P, const unsigned int *col_P, const double *val_P, const double *Y,
                    int N, int no_dims, int nterms, double ipi, int min_num_intervals) {
    if (!row_P || !Y || N < 1) return set_error(FITSNE_E_ARG, "null array or N < 1");
    if (no_dims != 1 && no_dims != 2)
        return set_error(FITSNE_E_ARG, "FFT interpolation supports only 1 or 2 output dimensions");
    if (row_P[N] > 0 && (!col_P || !val_P)) return set_error(FITSNE_E_ARG, "null CSR arrays");
    if (nterms < 1 || nterms > kMaxInterp) return set_error(FITSNE_E_ARG, "n_interpolation_points must be in [1, 8]");
    if (!(ipi > 0)) return set_error(FITSNE_E_ARG, "intervals_per_integer must be positive");
    if (min_num_intervals < 1) return set_error(FITSNE_E_ARG, "min_num_intervals must be >= 1");
    return check_cuda_device();
}

}  // namespace

}  // namespace fitsne

using namespace fitsne;

extern "C" {

int fitsne_fft_gradient(const unsigned int *row_P, const unsigned int *col_P, const double *val_P, const double *Y,
                        int N, int no_dims, double *dC, int nterms, double intervals_per_integer,
                        int min_num_intervals, double df, double *sum_Q) {
    int rc = check_grad_args(row_P, col_P, val_P, Y, N, no_dims, nterms, intervals_per_integer, min_num_intervals);
    if (rc) return rc;
    if (!dC) return set_error(FITSNE_E_ARG, "dC is null");
    if (!(df > 0)) return set_error(FITSNE_E_ARG, "df must be positive");
    if (precision_bits() == 64)
        return gradient_impl<double>(row_P, col_P, val_P, Y, N, no_dims, dC, nterms, intervals_per_integer,
                                     min_num_intervals, df, sum_Q);
    return gradient_impl<float>(row_P, col_P, val_P, Y, N, no_dims, dC, nterms, intervals_per_integer,
                                min_num_intervals, df, sum_Q);
}

int fitsne_evaluate_error_fft(const unsigned int *row_P, const unsigned int *col_P, const double *val_P,
                              const double *Y, int N, int no_dims, double df, double sum_Q, double *C) {
    int rc = check_grad_args(row_P, col_P, val_P, Y, N, no_dims, 3, 1.0, 1);
    if (rc) return rc;
    if (!C) return set_error(FITSNE_E_ARG, "C is null");
    if (precision_bits() == 64) return kl_impl<double>(row_P, col_P, val_P, Y, N, no_dims, df, sum_Q, C);
    return kl_impl<float>(row_P, col_P, val_P, Y, N, no_dims, df, sum_Q, C);
}

int fitsne_session_create(fitsne_session **out, int N, int no_dims, const unsigned int *row_P,
                          const unsigned int *col_P, const double *val_P, const double *Y0, int nterms,
                          double intervals_per_integer, int min_num_intervals, double df, int precision) {
    if (!out) return set_error(FITSNE_E_ARG, "out is null");
    *out = nullptr;
    int rc = check_grad_args(row_P, col_P, val_P, Y0, N, no_dims, nterms, intervals_per_integer, min_num_intervals);
    if (rc) return rc;
    if (!(df > 0)) return set_error(FITSNE_E_ARG, "df must be positive");
    if (precision != 32 && precision != 64) return set_error(FITSNE_E_ARG, "precision must be 32 or 64");
    GridParams gp;
    gp.nterms = nterms;
    gp.intervals_per_integer = intervals_per_integer;
    gp.min_num_intervals = min_num_intervals;
    gp.df = df;
    std::unique_ptr<fitsne_session> s(new fitsne_session);
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
        return set_error(FITSNE_E_CUDA, "cudaStreamCreate failed");
    if (precision == 64) {
        auto *p = new SessionT<double>;
        s->impl.reset(p);
        rc = p->emb.init_host(N, no_dims, row_P, col_P, val_P, Y0, gp, st);
    } else {
        auto *p = new SessionT<float>;
        s->impl.reset(p);
        rc = p->emb.init_host(N, no_dims, row_P, col_P, val_P, Y0, gp, st);
    }
    s->impl->st = st;
    if (rc) {
        std::string m = s->impl->error();
        s->impl.reset();
        cudaStreamDestroy(st);
        return set_error(FITSNE_E_CUDA, m);
    }
    *out = s.release();
    return 0;
}

int fitsne_session_run(fitsne_session *s, int it0, int it1, int max_iter, int stop_lying_iter, int mom_switch_iter,
                       double momentum, double final_momentum, double learning_rate, double early_exag_coeff,
                       int no_momentum_during_exag, int start_late_exag_iter, double late_exag_coeff,
                       double max_step_norm, double *costs) {
    if (!s || !s->impl) return set_error(FITSNE_E_ARG, "null session");
    if (!(early_exag_coeff > 0)) return set_error(FITSNE_E_ARG, "early_exag_coeff must be resolved (> 0)");
    if (it0 < 0 || it1 < it0) return set_error(FITSNE_E_ARG, "bad iteration range");
    Schedule sc;
    sc.max_iter = max_iter;
    sc.stop_lying_iter = stop_lying_iter;
    sc.mom_switch_iter = mom_switch_iter;
    sc.momentum = momentum;
    sc.final_momentum = final_momentum;
    sc.learning_rate = learning_rate;
    sc.early_exag_coeff = early_exag_coeff;
    sc.no_momentum_during_exag = no_momentum_during_exag;
    sc.start_late_exag_iter = start_late_exag_iter;
    sc.late_exag_coeff = late_exag_coeff;
    sc.max_step_norm = max_step_norm;
    int rc = s->impl->run(it0, it1, sc, costs);
    if (rc) return set_error(rc == -13 ? FITSNE_E_GRID : FITSNE_E_CUDA, s->impl->error());
    return 0;
}

int fitsne_session_gradient(fitsne_session *s, double *dC, double *sum_Q) {
    if (!s || !s->impl || !dC) return set_error(FITSNE_E_ARG, "null argument");
    int rc = s->impl->gradient(dC, sum_Q);
    if (rc) return set_error(rc == -13 ? FITSNE_E_GRID : FITSNE_E_CUDA, s->impl->error());
    return 0;
}

int fitsne_session_get_y(fitsne_session *s, double *Y) {
    if (!s || !s->impl || !Y) return set_error(FITSNE_E_ARG, "null argument");
    int rc = s->impl->get_y(Y);
    if (rc) return set_error(FITSNE_E_CUDA, s->impl->error());
    return 0;
}

int fitsne_session_set_timing(fitsne_session *s, int on) {
    if (!s || !s->impl) return set_error(FITSNE_E_ARG, "null session");
    s->impl->set_timing(on != 0);
    return 0;
}

int fitsne_session_set_graphs(fitsne_session *s, int on) {
    if (!s || !s->impl) return set_error(FITSNE_E_ARG, "null session");
    s->impl->set_graphs(on != 0);
    return 0;
}

int fitsne_session_stage_times(fitsne_session *s, double *out10) {
    if (!s || !s->impl || !out10) return set_error(FITSNE_E_ARG, "null argument");
    s->impl->times(out10);
    return 0;
}

int fitsne_session_launch_shapes(fitsne_session *s, int *out5) {
    if (!s || !s->impl || !out5) return set_error(FITSNE_E_ARG, "null argument");
    s->impl->launch_shapes(out5);
    return 0;
}

void fitsne_session_destroy(fitsne_session *s) {
    if (!s) return;
    cudaStream_t st = s->impl ? s->impl->st : nullptr;
    s->impl.reset();
    if (st) cudaStreamDestroy(st);
    delete s;
}

void fitsne_set_calibration(int mode) { set_calibration_mode(mode); }
int fitsne_get_calibration(void) { return calibration_mode(); }

int fitsne_calibration_stats(double *out12) {
    if (!out12) return set_error(FITSNE_E_ARG, "null argument");
    const MlpStats s = last_calibration_stats();
    const double v[12] = {(double) s.rows, (double) s.rows_harvest, (double) s.rows_fallback, (double) s.train_steps,
                          s.iters_plain, s.iters_warm, s.loss_first, s.loss_last, s.ms_harvest, s.ms_train,
                          s.ms_infer, s.ms_warm};
    for (int k = 0; k < 12; ++k) out12[k] = v[k];
    return 0;
}

int fitsne_mlp_param_count(int K) { return (K >= 1 && K <= kMlpMaxIn) ? (int) mlp_param_count(K) : -1; }

int fitsne_mlp_loss_grad(const float *params, int K, const double *dist, const double *beta, int nrows, double mu,
                         double sd, float *grad, double *loss) {
    if (!params || !dist || !beta || !grad || !loss || nrows < 1 || K < 1 || K > kMlpMaxIn || !(sd > 0))
        return set_error(FITSNE_E_ARG, "invalid arguments");
    int rc = check_cuda_device();
    if (rc) return rc;
    std::string err;
    rc = mlp_loss_grad_host(params, K, dist, beta, nrows, mu, sd, grad, loss, err);
    if (rc) return set_error(rc == -3 ? FITSNE_E_ARG : FITSNE_E_CUDA, err);
    return 0;
}

void fitsne_set_precision(int bits) { g_precision = (bits == 64) ? 64 : 32; }
int fitsne_get_precision(void) { return precision_bits(); }
const char *fitsne_last_error(void) { return g_last_error.c_str(); }
const char *fitsne_version(void) { return "1.2.1"; }
void fitsne_free(void *p) { std::free(p); }

}  // extern "C"
