// C ABI: TSNE::run replacement and the input-similarity entry points.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <atomic>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/fitsne_gb300.h"
#include "affinity.cuh"
#include "batch.cuh"
#include "capi_internal.h"
#include "embedding.cuh"
#include "knn.cuh"
#include "knn_tc.cuh"
#include "session.cuh"

namespace fitsne {
namespace {

bool verbose() {
    const char *q = std::getenv("FITSNE_QUIET");
    return !(q && std::atoi(q) != 0);
}

struct Stream {
    cudaStream_t s = nullptr;
    Stream() { cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking); }
    ~Stream() {
        if (s) cudaStreamDestroy(s);
    }
};

// the data's locality order on the device (build_P), freed with its scope
struct DevOrder {
    uint32_t *p = nullptr;
    ~DevOrder() { cudaFree(p); }
};

// Gaussian random number of TSNE::randn (src/tsne.cpp:1880-1890), drawn from libc rand()
// so that a seeded initialisation matches the reference bit for bit.
double randn_polar() {
    double x, y, radius;
    do {
        x = 2 * (std::rand() / ((double) RAND_MAX + 1)) - 1;
        y = 2 * (std::rand() / ((double) RAND_MAX + 1)) - 1;
        radius = (x * x) + (y * y);
    } while ((radius >= 1.0) || (radius == 0.0));
    radius = std::sqrt(-2 * std::log(radius) / radius);
    x *= radius;
    return x;
}

// P_row.dat / P_col.dat / P_val.dat of src/tsne.cpp:236-281 and 333-366
int load_p_files(int N, std::vector<uint32_t> &row, std::vector<uint32_t> &col, std::vector<double> &val) {
    FILE *h = std::fopen("P_row.dat", "rb");
    if (!h) return set_error(FITSNE_E_IO, "could not open P_row.dat");
    row.assign(N + 1, 0);
    size_t got = std::fread(row.data(), sizeof(uint32_t), N + 1, h);
    std::fclose(h);
    if (got != (size_t) N + 1) return set_error(FITSNE_E_IO, "P_row.dat is shorter than N + 1 entries");
    const size_t nnz = row[N];
    col.assign(nnz, 0);
    val.assign(nnz, 0.0);
    if (!(h = std::fopen("P_val.dat", "rb"))) return set_error(FITSNE_E_IO, "could not open P_val.dat");
    got = std::fread(val.data(), sizeof(double), nnz, h);
    std::fclose(h);
    if (got != nnz) return set_error(FITSNE_E_IO, "P_val.dat is too short");
    if (!(h = std::fopen("P_col.dat", "rb"))) return set_error(FITSNE_E_IO, "could not open P_col.dat");
    got = std::fread(col.data(), sizeof(uint32_t), nnz, h);
    std::fclose(h);
    if (got != nnz) return set_error(FITSNE_E_IO, "P_col.dat is too short");
    for (size_t e = 0; e < nnz; ++e)
        if (col[e] >= (uint32_t) N) return set_error(FITSNE_E_IO, "P_col.dat has an index out of range");
    return 0;
}

int save_p_files(int N, const std::vector<uint32_t> &row, const std::vector<uint32_t> &col,
                 const std::vector<double> &val) {
    FILE *h;
    const size_t nnz = row[N];
    if (!(h = std::fopen("P_val.dat", "w+b"))) return set_error(FITSNE_E_IO, "could not open P_val.dat");
    std::fwrite(val.data(), sizeof(double), nnz, h);
    std::fclose(h);
    if (!(h = std::fopen("P_col.dat", "w+b"))) return set_error(FITSNE_E_IO, "could not open P_col.dat");
    std::fwrite(col.data(), sizeof(uint32_t), nnz, h);
    std::fclose(h);
    if (!(h = std::fopen("P_row.dat", "w+b"))) return set_error(FITSNE_E_IO, "could not open P_row.dat");
    std::fwrite(row.data(), sizeof(uint32_t), N + 1, h);
    std::fclose(h);
    return 0;
}

// Whether the embedding of N points of dimension D is numbered in the data's locality order
// (data_locality_order; FITSNE_DATA_ORDER=0 leaves it to the Morton renumbering of the
// embedding): embeddings large enough to be renumbered, data the order describes.
bool data_order_wanted(int N, int D) {
    const char *e = std::getenv("FITSNE_DATA_ORDER");
    if (e && std::atoi(e) == 0) return false;
    return N >= kReorderMinN && D <= kDataOrderMaxD;
}

// Similarity stage of TSNE::run (src/tsne.cpp:153-330): centre and scale X, exact kNN,
// calibration, symmetrisation, normalisation; P stays on the device.  With order non-null and
// data_order_wanted, *order receives the data's locality order (device memory, the caller frees
// it); otherwise it is left null.
int build_P(const double *X, int N, int D, double perplexity, int K, double sigma, int list_len, const double *list,
            DevCSR *P, cudaStream_t st, bool vb, bool annoy_requested, uint32_t **order = nullptr) {
    std::string err;
    const bool normalize = perplexity > 0 || list_len > 0;
    double *Xd = nullptr;
    if (prepare_X(X, N, D, normalize, &Xd, st, err)) return set_error(FITSNE_E_CUDA, err);
    // the order (the kNN writes it when its search used it; otherwise computed here)
    bool order_written = false;
    if (order) {
        *order = nullptr;
        if (data_order_wanted(N, D)) {
            const cudaError_t e = cudaMalloc(order, sizeof(uint32_t) * (size_t) N);
            if (e != cudaSuccess) {
                *order = nullptr;
                cudaFree(Xd);
                return set_error(FITSNE_E_CUDA, cudaGetErrorString(e));
            }
        }
    }
    int K_use;
    double sigma_use;
    if (perplexity < 0) {
        K_use = K;
        sigma_use = sigma;
    } else {
        if (perplexity > 0) {
            K_use = (int) (3 * perplexity);
        } else {
            K_use = (int) (3 * list[0]);
            for (int pp = 1; pp < list_len; ++pp)
                if (3 * list[pp] > K_use) K_use = (int) (3 * list[pp]);
        }
        sigma_use = -1;
    }
    if (K_use < 1 || K_use + 1 > N) {
        cudaFree(Xd);
        return set_error(FITSNE_E_ARG, "number of neighbours must be in [1, N - 1]");
    }
    if (vb) {
        if (annoy_requested) std::printf("Annoy kNN requested: this build computes the exact kNN on the GPU\n");
        std::printf("Computing input similarities (exact kNN, K = %d) on the GPU...\n", K_use);
    }
    DevCSR P0;
    int rc = gaussian_perplexity_device(Xd, N, D, K_use, perplexity, sigma_use, perplexity == 0 ? list_len : 0, list,
                                        &P0, st, err, nullptr, order ? *order : nullptr, &order_written);
    if (!rc && order && *order && !order_written) rc = data_locality_order(Xd, N, D, *order, st, err);
    cudaFree(Xd);
    if (rc) {
        if (order) {
            cudaFree(*order);
            *order = nullptr;
        }
        return set_error(rc == -3 ? FITSNE_E_ARG : FITSNE_E_CUDA, err);
    }
    const auto t0 = std::chrono::steady_clock::now();
    rc = symmetrize_device(P0, P, st, err);
    free_csr(P0);
    if (rc) return set_error(FITSNE_E_CUDA, err);
    if (timing_requested())
        std::fprintf(stderr, "[fitsne] symmetrisation: %.3f s (nnz %zu)\n",
                     std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(), P->nnz);
    double sum = 0.0;
    if (normalize_device(*P, &sum, st, err)) {
        free_csr(*P);
        return set_error(FITSNE_E_CUDA, err);
    }
    return 0;
}

template <typename T>
int optimise(const DevCSR &P, double *Y, int N, int no_dims, const GridParams &gp, const Schedule &s, double *costs,
             cudaStream_t st, bool vb, const uint32_t *order) {
    const auto t0 = std::chrono::steady_clock::now();
    Embedding<T> emb;
    int rc = emb.init_device(N, no_dims, P.row, P.col, P.val, P.nnz, Y, gp, st);
    if (!rc && order) rc = emb.set_order(order);
    const auto t1 = std::chrono::steady_clock::now();
    if (!rc) rc = emb.run_schedule(s, 0, s.max_iter, costs, vb);
    const auto t2 = std::chrono::steady_clock::now();
    if (!rc) rc = emb.get_Y(Y);
    if (rc) return set_error(rc == -13 ? FITSNE_E_GRID : FITSNE_E_CUDA, emb.error());
    if (timing_requested()) {
        auto sec = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
            return std::chrono::duration<double>(b - a).count();
        };
        std::fprintf(stderr,
                     "[fitsne] embedding: set-up %.3f s, %d iterations %.3f s (%zu kernel launches, %d graph "
                     "captures), result %.3f s\n",
                     sec(t0, t1), s.max_iter, sec(t1, t2), (size_t) emb.last_times().launches, (int) emb.graph_captures(),
                     sec(t2, std::chrono::steady_clock::now()));
    }
    return 0;
}

// Batched form: independent embeddings advanced together, chunk by chunk; each job's chunk is
// one CUDA graph (cached per job) launched on the job's own stream, so that the small
// per-iteration kernels of all jobs run side by side with one host synchronisation per job
// and chunk.  Shared schedule and grid parameters; per-job data, perplexity and learning rate.
struct BatchJob {
    cudaStream_t st = nullptr;
    Embedding<float> emb;
};

int batch_iterate(std::vector<std::unique_ptr<BatchJob>> &jobs, const Schedule &s, const std::vector<double> &lr,
                  double *const *costs, double *stats) {
    const int nj = (int) jobs.size();
    double mult = s.early_exag_coeff, momentum = s.momentum;
    auto params = [&](int it, int j) {
        UpdateParams p{};
        p.mode = 1;
        p.exag = mult;
        p.momentum = momentum;
        p.learning_rate = lr[j];
        p.df = 1.0;
        p.use_gains = 1;
        p.max_step_norm = s.max_step_norm;
        (void) it;
        return p;
    };
    auto kl_due = [&](int it) { return (it + 1) % 50 == 0 || it == s.max_iter - 1; };
    auto after = [&](int it) -> int {
        if (it == s.stop_lying_iter) mult /= s.early_exag_coeff;
        if (it == s.mom_switch_iter) momentum = s.final_momentum;
        if (kl_due(it))
            for (int j = 0; j < nj; ++j) {
                double C = 0.0;
                if (jobs[j]->emb.kl(mult, &C)) return set_error(FITSNE_E_CUDA, jobs[j]->emb.error());
                if (it < s.stop_lying_iter && s.stop_lying_iter != -1)
                    C = C / s.early_exag_coeff - std::log(s.early_exag_coeff);
                if (costs && costs[j]) costs[j][it] = C;
            }
        return 0;
    };
    if (s.max_iter <= 0) return 0;
    // first iteration on the host path (grid sizes, launch shapes)
    for (int j = 0; j < nj; ++j) {
        if (jobs[j]->emb.step(params(0, j), true)) return set_error(FITSNE_E_CUDA, jobs[j]->emb.error());
        jobs[j]->emb.set_first_geometry();
    }
    int rc = after(0);
    if (rc) return rc;
    double launches = 0, captures = 0, redo = 0;
    int it = 1;
    while (it < s.max_iter) {
        for (int j = 0; j < nj; ++j)
            if (jobs[j]->emb.reorder_due(it, 0) && jobs[j]->emb.reorder_now())
                return set_error(FITSNE_E_CUDA, jobs[j]->emb.error());
        int end = it + 1;
        auto reorder_any = [&](int i) {
            for (auto &jb : jobs)
                if (jb->emb.reorder_due(i, 0)) return true;
            return false;
        };
        while (end < s.max_iter &&
               !(kl_due(end - 1) || end - 1 == s.stop_lying_iter || end - 1 == s.mom_switch_iter || reorder_any(end)))
            ++end;
        const int len = end - it;
        // every job's chunk graph (cached per job, recaptured only when that job's key
        // changes) launched on its own stream: the jobs' kernels run side by side
        for (int j = 0; j < nj; ++j)
            if (jobs[j]->emb.launch_chunk(params(it, j), len, 0))
                return set_error(FITSNE_E_CUDA, jobs[j]->emb.error());
        launches += nj;
        for (int j = 0; j < nj; ++j)
            if (cudaStreamSynchronize(jobs[j]->st) != cudaSuccess) return set_error(FITSNE_E_CUDA, "batch chunk");
        for (int j = 0; j < nj; ++j) {
            int r = jobs[j]->emb.finish_chunk(len);
            while (r == 1) {  // this job outgrew its grid: its chunk again, with more room
                redo += 1;
                Embedding<float> &e = jobs[j]->emb;
                if (e.launch_chunk(params(it, j), len, 1) || cudaStreamSynchronize(jobs[j]->st) != cudaSuccess)
                    return set_error(FITSNE_E_CUDA, e.error());
                r = e.finish_chunk(len);
            }
            if (r < 0) return set_error(FITSNE_E_CUDA, jobs[j]->emb.error());
        }
        for (int k = it; k < end; ++k) {
            rc = after(k);
            if (rc) return rc;
        }
        it = end;
    }
    double updates = 0;
    for (auto &jb : jobs) {
        captures += (double) jb->emb.graph_captures();
        updates += (double) jb->emb.graph_updates();
    }
    if (stats) {
        stats[2] = launches;
        stats[3] = captures - updates;  // instantiations (the rest were in-place updates)
        stats[4] = redo;
    }
    return 0;
}

}  // namespace
}  // namespace fitsne

using namespace fitsne;

extern "C" {

int fitsne_run(double *X, int N, int D, double *Y, int no_dims, double perplexity, double theta, int rand_seed,
               int skip_random_init, int max_iter, int stop_lying_iter, int mom_switch_iter, double momentum,
               double final_momentum, double learning_rate, int K, double sigma, int nbody_algorithm, int knn_algo,
               double early_exag_coeff, double *costs, int no_momentum_during_exag, int start_late_exag_iter,
               double late_exag_coeff, int n_trees, int search_k, int nterms, double intervals_per_integer,
               int min_num_intervals, unsigned int nthreads, int load_affinities, int perplexity_list_length,
               double *perplexity_list, double df, double max_step_norm) {
    (void) n_trees;
    (void) search_k;
    (void) nthreads;
    const bool vb = verbose();
    if (!X || !Y || N < 2 || D < 1) return set_error(FITSNE_E_ARG, "invalid data arguments");
    if (N - 1 < 3 * perplexity) return set_error(FITSNE_E_ARG, "Perplexity too large for the number of data points!");
    if (theta == .0) return set_error(FITSNE_E_UNSUPPORTED, "exact t-SNE (theta = 0) is not part of this build");
    if (nbody_algorithm != 2)
        return set_error(FITSNE_E_UNSUPPORTED, "only the FFT-accelerated gradient (nbody_algorithm 2) is built");
    if (knn_algo != 1 && knn_algo != 2) return set_error(FITSNE_E_ARG, "Invalid knn_algo param");
    if (no_dims != 1 && no_dims != 2)
        return set_error(FITSNE_E_ARG, "FFT interpolation scheme supports only 1 or 2 output dimensions");
    if (nterms < 1 || nterms > kMaxInterp) return set_error(FITSNE_E_ARG, "n_interpolation_points must be in [1, 8]");
    if (!(intervals_per_integer > 0) || min_num_intervals < 1)
        return set_error(FITSNE_E_ARG, "invalid interpolation grid parameters");
    if (!(df > 0)) return set_error(FITSNE_E_ARG, "df must be positive");
    if (perplexity == 0 && (perplexity_list_length < 1 || !perplexity_list))
        return set_error(FITSNE_E_ARG, "perplexity 0 needs a perplexity list");
    const auto tstart = std::chrono::steady_clock::now();
    int rc = check_cuda_device();
    if (rc) return rc;
    if (max_iter < 0) max_iter = 0;
    if (costs)
        for (int i = 0; i < max_iter; ++i) costs[i] = 0.0;
    Stream st;
    std::string err;
    DevCSR P;
    DevOrder order;
    if (load_affinities == 1) {
        if (vb) std::printf("Loading approximate input similarities from files...\n");
        std::vector<uint32_t> row, col;
        std::vector<double> val;
        rc = load_p_files(N, row, col, val);
        if (rc) return rc;
        if (csr_to_device(row.data(), col.data(), val.data(), N, &P, st.s, err))
            return set_error(FITSNE_E_CUDA, err);
    } else {
        rc = build_P(X, N, D, perplexity, K, sigma, perplexity_list_length, perplexity_list, &P, st.s, vb,
                     knn_algo == 1, &order.p);
        if (rc) return rc;
    }
    if (load_affinities == 2) {
        if (vb) std::printf("Saving approximate input similarities to files...\n");
        std::vector<uint32_t> row(N + 1), col(P.nnz);
        std::vector<double> val(P.nnz);
        if (csr_to_host(P, row.data(), col.data(), val.data(), st.s, err)) {
            free_csr(P);
            return set_error(FITSNE_E_CUDA, err);
        }
        rc = save_p_files(N, row, col, val);
        if (rc) {
            free_csr(P);
            return rc;
        }
    }
    if (!skip_random_init) {
        std::srand(rand_seed >= 0 ? (unsigned int) rand_seed : (unsigned int) std::time(nullptr));
        for (size_t i = 0; i < (size_t) N * no_dims; ++i) Y[i] = randn_polar() * .0001;
    }
    if (early_exag_coeff == 0) {
        double mx = 0.0;
        if (max_row_sum_device(P, &mx, st.s, err)) {
            free_csr(P);
            return set_error(FITSNE_E_CUDA, err);
        }
        early_exag_coeff = 1.0 / (learning_rate * mx);
    }
    if (vb)
        std::printf("Input similarities computed (nnz = %zu); learning embedding (FP%d form)...\n", P.nnz,
                    precision_bits());
    if (timing_requested())
        std::fprintf(stderr, "[fitsne] device check + input similarities: %.3f s\n",
                     std::chrono::duration<double>(std::chrono::steady_clock::now() - tstart).count());
    GridParams gp;
    gp.nterms = nterms;
    gp.intervals_per_integer = intervals_per_integer;
    gp.min_num_intervals = min_num_intervals;
    gp.df = df;
    Schedule s;
    s.max_iter = max_iter;
    s.stop_lying_iter = stop_lying_iter;
    s.mom_switch_iter = mom_switch_iter;
    s.momentum = momentum;
    s.final_momentum = final_momentum;
    s.learning_rate = learning_rate;
    s.early_exag_coeff = early_exag_coeff;
    s.no_momentum_during_exag = no_momentum_during_exag;
    s.start_late_exag_iter = start_late_exag_iter;
    s.late_exag_coeff = late_exag_coeff;
    s.max_step_norm = max_step_norm;
    std::vector<double> costs_local;
    if (!costs) {
        costs_local.assign(max_iter > 0 ? max_iter : 1, 0.0);
        costs = costs_local.data();
    }
    if (precision_bits() == 64)
        rc = optimise<double>(P, Y, N, no_dims, gp, s, costs, st.s, vb, order.p);
    else
        rc = optimise<float>(P, Y, N, no_dims, gp, s, costs, st.s, vb, order.p);
    free_csr(P);
    return rc;
}

int fitsne_session_create_from_data(fitsne_session **out, const double *X, int N, int D, int no_dims,
                                    double perplexity, int K, double sigma, int perplexity_list_length,
                                    const double *perplexity_list, const double *Y0, int nterms,
                                    double intervals_per_integer, int min_num_intervals, double df, int precision,
                                    unsigned long long *nnz) {
    if (!out) return set_error(FITSNE_E_ARG, "out is null");
    *out = nullptr;
    if (!X || !Y0 || N < 2 || D < 1) return set_error(FITSNE_E_ARG, "invalid data arguments");
    if (N - 1 < 3 * perplexity) return set_error(FITSNE_E_ARG, "Perplexity too large for the number of data points!");
    if (no_dims != 1 && no_dims != 2)
        return set_error(FITSNE_E_ARG, "FFT interpolation scheme supports only 1 or 2 output dimensions");
    if (nterms < 1 || nterms > kMaxInterp) return set_error(FITSNE_E_ARG, "n_interpolation_points must be in [1, 8]");
    if (!(intervals_per_integer > 0) || min_num_intervals < 1 || !(df > 0))
        return set_error(FITSNE_E_ARG, "invalid interpolation grid parameters");
    if (precision != 32 && precision != 64) return set_error(FITSNE_E_ARG, "precision must be 32 or 64");
    if (perplexity == 0 && (perplexity_list_length < 1 || !perplexity_list))
        return set_error(FITSNE_E_ARG, "perplexity 0 needs a perplexity list");
    int rc = check_cuda_device();
    if (rc) return rc;
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
        return set_error(FITSNE_E_CUDA, "cudaStreamCreate failed");
    DevCSR P;
    DevOrder order;
    rc = build_P(X, N, D, perplexity, K, sigma, perplexity_list_length, perplexity_list, &P, st, false, false,
                 &order.p);
    if (rc) {
        cudaStreamDestroy(st);
        return rc;
    }
    if (nnz) *nnz = P.nnz;
    GridParams gp;
    gp.nterms = nterms;
    gp.intervals_per_integer = intervals_per_integer;
    gp.min_num_intervals = min_num_intervals;
    gp.df = df;
    std::unique_ptr<fitsne_session> s(new fitsne_session);
    if (precision == 64) {
        auto *p = new SessionT<double>;
        s->impl.reset(p);
        rc = p->emb.init_device(N, no_dims, P.row, P.col, P.val, P.nnz, Y0, gp, st);
        if (!rc && order.p) rc = p->emb.set_order(order.p);
    } else {
        auto *p = new SessionT<float>;
        s->impl.reset(p);
        rc = p->emb.init_device(N, no_dims, P.row, P.col, P.val, P.nnz, Y0, gp, st);
        if (!rc && order.p) rc = p->emb.set_order(order.p);
    }
    free_csr(P);
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

int fitsne_knn(const double *X, int N, int D, int K, unsigned int *indices, double *distances) {
    if (!X || !indices || !distances || N < 1 || D < 1) return set_error(FITSNE_E_ARG, "invalid arguments");
    if (K < 1 || K > N) return set_error(FITSNE_E_ARG, "K must be in [1, N]");
    int rc = check_cuda_device();
    if (rc) return rc;
    Stream st;
    double *Xd = nullptr, *dist = nullptr;
    uint32_t *idx = nullptr;
    const char *kerr = nullptr;
    cudaError_t e = cudaMalloc(&Xd, sizeof(double) * (size_t) N * D);
    if (e == cudaSuccess) e = cudaMalloc(&idx, sizeof(uint32_t) * (size_t) N * K);
    if (e == cudaSuccess) e = cudaMalloc(&dist, sizeof(double) * (size_t) N * K);
    if (e == cudaSuccess) e = cudaMemcpyAsync(Xd, X, sizeof(double) * (size_t) N * D, cudaMemcpyHostToDevice, st.s);
    if (e == cudaSuccess) {
        KnnStats ks;
        rc = knn_exact(Xd, N, D, K, idx, dist, st.s, &ks, &kerr);
        if (!rc && timing_requested()) print_knn_stats(K, ks, -1.0);
        if (!rc) {
            e = cudaMemcpyAsync(indices, idx, sizeof(uint32_t) * (size_t) N * K, cudaMemcpyDeviceToHost, st.s);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(distances, dist, sizeof(double) * (size_t) N * K, cudaMemcpyDeviceToHost, st.s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st.s);
        }
    }
    cudaFree(Xd);
    cudaFree(idx);
    cudaFree(dist);
    if (rc) return set_error(rc == -3 ? FITSNE_E_ARG : FITSNE_E_CUDA, kerr ? kerr : "kNN failed");
    if (e != cudaSuccess) return set_error(FITSNE_E_CUDA, cudaGetErrorString(e));
    return 0;
}

int fitsne_distances2similarities(const double *Dm, double *P, int nrows, int K, double perplexity, double sigma,
                                  int perplexity_list_length, const double *perplexity_list, double *betas) {
    if (!Dm || !P || nrows < 0 || K < 1) return set_error(FITSNE_E_ARG, "invalid arguments");
    if (perplexity == 0 && (perplexity_list_length < 1 || !perplexity_list))
        return set_error(FITSNE_E_ARG, "perplexity 0 needs a perplexity list");
    if (nrows == 0) return 0;
    int rc = check_cuda_device();
    if (rc) return rc;
    Stream st;
    std::string err;
    double *d = nullptr, *p = nullptr, *b = nullptr;
    const size_t n = (size_t) nrows * K;
    cudaError_t e = cudaMalloc(&d, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMalloc(&p, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMalloc(&b, sizeof(double) * nrows);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d, Dm, sizeof(double) * n, cudaMemcpyHostToDevice, st.s);
    if (e == cudaSuccess) {
        rc = calibrate_rows(d, K, 0, p, nrows, K, perplexity, sigma, perplexity == 0 ? perplexity_list_length : 0,
                            perplexity_list, b, st.s, err);
        if (!rc) {
            e = cudaMemcpyAsync(P, p, sizeof(double) * n, cudaMemcpyDeviceToHost, st.s);
            if (e == cudaSuccess && betas)
                e = cudaMemcpyAsync(betas, b, sizeof(double) * nrows, cudaMemcpyDeviceToHost, st.s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st.s);
        }
    }
    cudaFree(d);
    cudaFree(p);
    cudaFree(b);
    if (rc) return set_error(FITSNE_E_CUDA, err);
    if (e != cudaSuccess) return set_error(FITSNE_E_CUDA, cudaGetErrorString(e));
    return 0;
}

static int to_malloced(const DevCSR &P, unsigned int **row_P, unsigned int **col_P, double **val_P, cudaStream_t st,
                       std::string &err) {
    unsigned int *r = (unsigned int *) std::malloc(sizeof(unsigned int) * (P.N + 1));
    unsigned int *c = (unsigned int *) std::malloc(sizeof(unsigned int) * (P.nnz ? P.nnz : 1));
    double *v = (double *) std::malloc(sizeof(double) * (P.nnz ? P.nnz : 1));
    if (!r || !c || !v) {
        std::free(r);
        std::free(c);
        std::free(v);
        return set_error(FITSNE_E_NOMEM, "host allocation failed");
    }
    if (csr_to_host(P, r, c, v, st, err)) {
        std::free(r);
        std::free(c);
        std::free(v);
        return set_error(FITSNE_E_CUDA, err);
    }
    *row_P = r;
    *col_P = c;
    *val_P = v;
    return 0;
}

int fitsne_gaussian_perplexity(const double *X, int N, int D, unsigned int **row_P, unsigned int **col_P,
                               double **val_P, double perplexity, int K, double sigma, unsigned int nthreads,
                               int perplexity_list_length, const double *perplexity_list) {
    (void) nthreads;
    if (!X || !row_P || !col_P || !val_P || N < 2 || D < 1) return set_error(FITSNE_E_ARG, "invalid arguments");
    if (K < 1 || K + 1 > N) return set_error(FITSNE_E_ARG, "K + 1 must not exceed N");
    if (perplexity == 0 && (perplexity_list_length < 1 || !perplexity_list))
        return set_error(FITSNE_E_ARG, "perplexity 0 needs a perplexity list");
    int rc = check_cuda_device();
    if (rc) return rc;
    Stream st;
    std::string err;
    double *Xd = nullptr;
    cudaError_t e = cudaMalloc(&Xd, sizeof(double) * (size_t) N * D);
    if (e == cudaSuccess) e = cudaMemcpyAsync(Xd, X, sizeof(double) * (size_t) N * D, cudaMemcpyHostToDevice, st.s);
    if (e != cudaSuccess) {
        cudaFree(Xd);
        return set_error(FITSNE_E_CUDA, cudaGetErrorString(e));
    }
    DevCSR P;
    rc = gaussian_perplexity_device(Xd, N, D, K, perplexity, sigma, perplexity == 0 ? perplexity_list_length : 0,
                                    perplexity_list, &P, st.s, err);
    cudaFree(Xd);
    if (rc) return set_error(rc == -3 ? FITSNE_E_ARG : FITSNE_E_CUDA, err);
    rc = to_malloced(P, row_P, col_P, val_P, st.s, err);
    free_csr(P);
    return rc;
}

int fitsne_symmetrize(unsigned int **row_P, unsigned int **col_P, double **val_P, int N) {
    if (!row_P || !col_P || !val_P || !*row_P || N < 1) return set_error(FITSNE_E_ARG, "invalid arguments");
    int rc = check_cuda_device();
    if (rc) return rc;
    const unsigned int *row = *row_P;
    for (int n = 0; n < N; ++n)
        if (row[n + 1] < row[n]) return set_error(FITSNE_E_ARG, "row pointers must be non-decreasing");
    for (size_t e = 0; e < row[N]; ++e)
        if ((*col_P)[e] >= (unsigned int) N) return set_error(FITSNE_E_ARG, "column index out of range");
    Stream st;
    std::string err;
    DevCSR in, out;
    if (csr_to_device(*row_P, *col_P, *val_P, N, &in, st.s, err)) return set_error(FITSNE_E_CUDA, err);
    rc = symmetrize_device(in, &out, st.s, err);
    free_csr(in);
    if (rc) return set_error(FITSNE_E_CUDA, err);
    unsigned int *r, *c;
    double *v;
    rc = to_malloced(out, &r, &c, &v, st.s, err);
    free_csr(out);
    if (rc) return rc;
    std::free(*row_P);
    std::free(*col_P);
    std::free(*val_P);
    *row_P = r;
    *col_P = c;
    *val_P = v;
    return 0;
}

int fitsne_batch_run(int njobs, const double *const *X, const int *N, const int *D, double *const *Y, int no_dims,
                     const double *perplexity, const double *learning_rate, const int *rand_seed,
                     int skip_random_init, int max_iter, int stop_lying_iter, int mom_switch_iter, double momentum,
                     double final_momentum, double early_exag_coeff, int nterms, double intervals_per_integer,
                     int min_num_intervals, double max_step_norm, double *const *costs, double *stats5) {
    if (njobs < 1 || !X || !N || !D || !Y || !perplexity || !learning_rate)
        return set_error(FITSNE_E_ARG, "invalid batch arguments");
    if (no_dims != 1 && no_dims != 2)
        return set_error(FITSNE_E_ARG, "FFT interpolation scheme supports only 1 or 2 output dimensions");
    if (nterms < 1 || nterms > kMaxInterp || !(intervals_per_integer > 0) || min_num_intervals < 1)
        return set_error(FITSNE_E_ARG, "invalid interpolation grid parameters");
    for (int j = 0; j < njobs; ++j) {
        if (!X[j] || !Y[j] || N[j] < 2 || D[j] < 1 || !(perplexity[j] > 0))
            return set_error(FITSNE_E_ARG, "invalid data arguments of job " + std::to_string(j));
        if (N[j] - 1 < 3 * perplexity[j])
            return set_error(FITSNE_E_ARG, "Perplexity too large for the number of data points!");
    }
    int rc = check_cuda_device();
    if (rc) return rc;
    const auto t0 = std::chrono::steady_clock::now();
    GridParams gp;
    gp.nterms = nterms;
    gp.intervals_per_integer = intervals_per_integer;
    gp.min_num_intervals = min_num_intervals;
    gp.df = 1.0;
    Schedule s;
    s.max_iter = max_iter;
    s.stop_lying_iter = stop_lying_iter;
    s.mom_switch_iter = mom_switch_iter;
    s.momentum = momentum;
    s.final_momentum = final_momentum;
    s.early_exag_coeff = early_exag_coeff;
    s.max_step_norm = max_step_norm;
    std::vector<double> lr(learning_rate, learning_rate + njobs);
    const char *bmode = std::getenv("FITSNE_BATCH");  // "streams": one graph per job on its own stream
    if (BatchPipeline::supports(no_dims, gp) && !(bmode && std::string(bmode) == "streams")) {
        // every job in the same launches (batch.cuh)
        Stream st;
        std::vector<DevCSR> Ps(njobs);
        struct FreeP {
            std::vector<DevCSR> &v;
            ~FreeP() {
                for (auto &p : v) free_csr(p);
            }
        } free_p{Ps};
        std::vector<const double *> Y0(njobs);
        // similarities of the jobs on a few host threads, each with its own stream, so that
        // the small jobs' kernels share the GPU
        {
            std::vector<int> rcs(njobs, 0);
            std::vector<std::string> msgs(njobs);
            std::atomic<int> next{0};
            int dev = 0;
            cudaGetDevice(&dev);
            auto worker = [&]() {
                cudaSetDevice(dev);
                Stream ws;
                for (int j = next++; j < njobs; j = next++) {
                    rcs[j] = build_P(X[j], N[j], D[j], perplexity[j], -1, -1.0, 0, nullptr, &Ps[j], ws.s, false, false);
                    if (rcs[j]) msgs[j] = fitsne_last_error();
                }
            };
            const int nt = std::min(njobs, 8);
            std::vector<std::thread> pool;
            for (int t = 1; t < nt; ++t) pool.emplace_back(worker);
            worker();
            for (auto &t : pool) t.join();
            for (int j = 0; j < njobs; ++j)
                if (rcs[j]) return set_error(rcs[j], msgs[j]);
            if (cudaDeviceSynchronize() != cudaSuccess) return set_error(FITSNE_E_CUDA, "similarity stage failed");
        }
        for (int j = 0; j < njobs; ++j) {
            if (!skip_random_init) {
                std::srand(rand_seed ? (unsigned int) rand_seed[j] : 0u);
                for (size_t i = 0; i < (size_t) N[j] * no_dims; ++i) Y[j][i] = randn_polar() * .0001;
            }
            Y0[j] = Y[j];
        }
        BatchPipeline bp;
        rc = bp.init(Ps, Y0, lr, gp, st.s);
        for (auto &p : Ps) free_csr(p);
        if (rc) return set_error(FITSNE_E_CUDA, bp.error());
        const auto t1 = std::chrono::steady_clock::now();
        double bs[5] = {0, 0, 0, 0, 0};
        rc = bp.run_schedule(s, costs, bs);
        if (rc) return set_error(rc == -11 ? FITSNE_E_GRID : FITSNE_E_CUDA, bp.error());
        for (int j = 0; j < njobs; ++j)
            if (bp.get_Y(j, Y[j])) return set_error(FITSNE_E_CUDA, bp.error());
        const auto t2 = std::chrono::steady_clock::now();
        if (stats5) {
            stats5[0] = std::chrono::duration<double>(t1 - t0).count();
            stats5[1] = std::chrono::duration<double>(t2 - t1).count();
            stats5[2] = bs[0];
            stats5[3] = bs[1] - bs[2];  // instantiations (the rest were in-place updates)
            stats5[4] = bs[3];
        }
        return 0;
    }
    std::vector<std::unique_ptr<BatchJob>> jobs;
    for (int j = 0; j < njobs; ++j) {
        jobs.emplace_back(new BatchJob());
        if (cudaStreamCreateWithFlags(&jobs[j]->st, cudaStreamNonBlocking) != cudaSuccess)
            return set_error(FITSNE_E_CUDA, "stream creation failed");
    }
    struct Cleanup {
        std::vector<std::unique_ptr<BatchJob>> &v;
        ~Cleanup() {
            for (auto &j : v) {
                cudaStream_t st = j->st;
                j.reset();
                if (st) cudaStreamDestroy(st);
            }
        }
    } cleanup{jobs};
    // similarities and initial embeddings, job by job
    for (int j = 0; j < njobs; ++j) {
        DevCSR P;
        rc = build_P(X[j], N[j], D[j], perplexity[j], -1, -1.0, 0, nullptr, &P, jobs[j]->st, false, false);
        if (rc) return rc;
        if (!skip_random_init) {
            std::srand(rand_seed ? (unsigned int) rand_seed[j] : 0u);
            for (size_t i = 0; i < (size_t) N[j] * no_dims; ++i) Y[j][i] = randn_polar() * .0001;
        }
        rc = jobs[j]->emb.init_device(N[j], no_dims, P.row, P.col, P.val, P.nnz, Y[j], gp, jobs[j]->st);
        free_csr(P);
        if (rc) return set_error(FITSNE_E_CUDA, jobs[j]->emb.error());
    }
    const auto t1 = std::chrono::steady_clock::now();
    double st5[5] = {0, 0, 0, 0, 0};
    rc = batch_iterate(jobs, s, lr, costs, st5);
    if (rc) return rc;
    for (int j = 0; j < njobs; ++j)
        if (jobs[j]->emb.get_Y(Y[j])) return set_error(FITSNE_E_CUDA, jobs[j]->emb.error());
    const auto t2 = std::chrono::steady_clock::now();
    st5[0] = std::chrono::duration<double>(t1 - t0).count();
    st5[1] = std::chrono::duration<double>(t2 - t1).count();
    if (stats5)
        for (int k = 0; k < 5; ++k) stats5[k] = st5[k];
    return 0;
}

}  // extern "C"
