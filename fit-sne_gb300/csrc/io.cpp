// data.dat / result.dat of the fast_tsne binary (TSNE::load_data / TSNE::save_data,
// src/tsne.cpp:1895-2038 of FIt-SNE v1.2.1).  Native-endian, packed, same field order.
#include <cstdio>
#include <cstdlib>

#include "../../include/fitsne_gb300.h"
#include "capi_internal.h"

using fitsne::set_error;

extern "C" {

int fitsne_load_data(const char *data_path, double **data, double **Y, int *n, int *d, int *no_dims, double *theta,
                     double *perplexity, int *rand_seed, int *max_iter, int *stop_lying_iter, int *mom_switch_iter,
                     double *momentum, double *final_momentum, double *learning_rate, int *K, double *sigma,
                     int *nbody_algo, int *knn_algo, double *early_exag_coeff, int *no_momentum_during_exag,
                     int *n_trees, int *search_k, int *start_late_exag_iter, double *late_exag_coeff, int *nterms,
                     double *intervals_per_integer, int *min_num_intervals, int *skip_random_init,
                     int *load_affinities, int *perplexity_list_length, double **perplexity_list, double *df,
                     double *max_step_norm) {
    FILE *h = std::fopen(data_path, "r+b");
    if (!h) return set_error(FITSNE_E_IO, "Error: could not open data file.");
    bool ok = true;
    auto rd = [&](void *p, size_t sz, size_t cnt) {
        if (std::fread(p, sz, cnt, h) != cnt) ok = false;
    };
    rd(n, sizeof(int), 1);
    rd(d, sizeof(int), 1);
    rd(theta, sizeof(double), 1);
    rd(perplexity, sizeof(double), 1);
    *perplexity_list_length = 0;
    *perplexity_list = nullptr;
    if (ok && *perplexity == 0) {
        rd(perplexity_list_length, sizeof(int), 1);
        if (ok && *perplexity_list_length > 0) {
            *perplexity_list = (double *) std::malloc(sizeof(double) * *perplexity_list_length);
            if (!*perplexity_list) {
                std::fclose(h);
                return set_error(FITSNE_E_NOMEM, "Memory allocation failed!");
            }
            rd(*perplexity_list, sizeof(double), *perplexity_list_length);
        }
    }
    rd(no_dims, sizeof(int), 1);
    rd(max_iter, sizeof(int), 1);
    rd(stop_lying_iter, sizeof(int), 1);
    rd(mom_switch_iter, sizeof(int), 1);
    rd(momentum, sizeof(double), 1);
    rd(final_momentum, sizeof(double), 1);
    rd(learning_rate, sizeof(double), 1);
    rd(max_step_norm, sizeof(double), 1);
    rd(K, sizeof(int), 1);
    rd(sigma, sizeof(double), 1);
    rd(nbody_algo, sizeof(int), 1);
    rd(knn_algo, sizeof(int), 1);
    rd(early_exag_coeff, sizeof(double), 1);
    rd(no_momentum_during_exag, sizeof(int), 1);
    rd(n_trees, sizeof(int), 1);
    rd(search_k, sizeof(int), 1);
    rd(start_late_exag_iter, sizeof(int), 1);
    rd(late_exag_coeff, sizeof(double), 1);
    rd(nterms, sizeof(int), 1);
    rd(intervals_per_integer, sizeof(double), 1);
    rd(min_num_intervals, sizeof(int), 1);
    if (!ok || *n < 1 || *d < 1) {
        std::fclose(h);
        return set_error(FITSNE_E_IO, "data file header is truncated or invalid");
    }
    if (*nbody_algo == 2 && *no_dims > 2) {
        std::fclose(h);
        return set_error(FITSNE_E_ARG, "FFT interpolation scheme supports only 1 or 2 output dimensions");
    }
    const size_t nd = (size_t) *n * (size_t) *d;
    *data = (double *) std::malloc(sizeof(double) * nd);
    if (!*data) {
        std::fclose(h);
        return set_error(FITSNE_E_NOMEM, "Memory allocation failed!");
    }
    rd(*data, sizeof(double), nd);
    if (!ok) {
        std::fclose(h);
        return set_error(FITSNE_E_IO, "data file ends inside the data matrix");
    }
    // optional trailer: seed, df, load_affinities, initial Y (each read only if the file
    // has not ended, as the reference does with feof)
    *rand_seed = 0;
    *df = 1.0;
    *load_affinities = 0;
    if (!std::feof(h)) {
        if (std::fread(rand_seed, sizeof(int), 1, h) != 1) *rand_seed = 0;
    }
    if (!std::feof(h)) {
        if (std::fread(df, sizeof(double), 1, h) != 1) *df = 1.0;
    }
    if (!std::feof(h)) {
        if (std::fread(load_affinities, sizeof(int), 1, h) != 1) *load_affinities = 0;
    }
    const size_t ny = (size_t) *n * (size_t) *no_dims;
    *Y = (double *) std::malloc(sizeof(double) * (ny ? ny : 1));
    if (!*Y) {
        std::fclose(h);
        return set_error(FITSNE_E_NOMEM, "Memory allocation failed!");
    }
    *skip_random_init = 0;
    if (!std::feof(h)) {
        const size_t got = std::fread(*Y, sizeof(double), ny, h);
        *skip_random_init = (got < ny) ? 0 : 1;
    }
    std::fclose(h);
    return 0;
}

int fitsne_save_data(const char *result_path, const double *data, const double *costs, int n, int d, int max_iter) {
    FILE *h = std::fopen(result_path, "w+b");
    if (!h) return set_error(FITSNE_E_IO, "Error: could not open data file.");
    std::fwrite(&n, sizeof(int), 1, h);
    std::fwrite(&d, sizeof(int), 1, h);
    std::fwrite(data, sizeof(double), (size_t) n * d, h);
    std::fwrite(&max_iter, sizeof(int), 1, h);
    std::fwrite(costs, sizeof(double), max_iter, h);
    std::fclose(h);
    return 0;
}

}  // extern "C"
