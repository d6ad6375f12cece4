// fast_tsne: drop-in for the reference binary (src/tsne.cpp:2041-2136 of FIt-SNE v1.2.1).
//
//   fast_tsne <version> [data.dat] [result.dat] [nthreads]
//
// Same arguments, same data.dat / result.dat formats, same version check; the work runs on
// the GPU through libfitsne_gb300.so.  nthreads is accepted and ignored.  The arithmetic
// form is chosen with FITSNE_PRECISION=32|64 (default 32).
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "fitsne_gb300.h"

int main(int argc, char *argv[]) {
    const char *version = fitsne_version();
    std::printf("=============== t-SNE v%s (GB300) ===============\n", version);
    if (argc < 2) {
        std::printf("Please pass version number as first argument.\n");
        return -1;
    }
    if (std::strcmp(argv[1], version) != 0) {
        std::printf("Wrapper passed wrong version number: %s\n", argv[1]);
        return -1;
    }
    const char *data_path = argc >= 3 ? argv[2] : "data.dat";
    const char *result_path = argc >= 4 ? argv[3] : "result.dat";
    unsigned int nthreads = argc >= 5 ? (unsigned int) std::strtoul(argv[4], nullptr, 10) : 0u;
    std::printf("fast_tsne data_path: %s\nfast_tsne result_path: %s\nfast_tsne nthreads: %u\n", data_path,
                result_path, nthreads);

    int N, D, no_dims, max_iter, stop_lying_iter, K, nbody_algo, knn_algo, no_momentum_during_exag;
    int mom_switch_iter, n_trees, search_k, start_late_exag_iter, nterms, min_num_intervals;
    int rand_seed = 0, load_affinities = 0, skip_random_init = 0, perplexity_list_length = 0;
    double momentum, final_momentum, learning_rate, max_step_norm, sigma, early_exag_coeff, late_exag_coeff;
    double perplexity, theta, intervals_per_integer, df = 1.0;
    double *data = nullptr, *Y = nullptr, *perplexity_list = nullptr;

    int rc = fitsne_load_data(data_path, &data, &Y, &N, &D, &no_dims, &theta, &perplexity, &rand_seed, &max_iter,
                              &stop_lying_iter, &mom_switch_iter, &momentum, &final_momentum, &learning_rate, &K,
                              &sigma, &nbody_algo, &knn_algo, &early_exag_coeff, &no_momentum_during_exag, &n_trees,
                              &search_k, &start_late_exag_iter, &late_exag_coeff, &nterms, &intervals_per_integer,
                              &min_num_intervals, &skip_random_init, &load_affinities, &perplexity_list_length,
                              &perplexity_list, &df, &max_step_norm);
    if (rc != 0) {
        // the reference prints the error and still exits normally
        std::printf("%s\n", fitsne_last_error());
        std::printf("Done.\n\n");
        return 0;
    }
    std::printf("Read the %i x %i data matrix successfully. X[0,0] = %lf\n", N, D, data[0]);
    double *costs = (double *) std::calloc(max_iter > 0 ? max_iter : 1, sizeof(double));
    if (!costs) {
        std::printf("Memory allocation failed!\n");
        return 1;
    }
    rc = fitsne_run(data, N, D, Y, no_dims, perplexity, theta, rand_seed, skip_random_init, max_iter,
                    stop_lying_iter, mom_switch_iter, momentum, final_momentum, learning_rate, K, sigma, nbody_algo,
                    knn_algo, early_exag_coeff, costs, no_momentum_during_exag, start_late_exag_iter,
                    late_exag_coeff, n_trees, search_k, nterms, intervals_per_integer, min_num_intervals, nthreads,
                    load_affinities, perplexity_list_length, perplexity_list, df, max_step_norm);
    if (rc < 0) {
        std::printf("Error: %s\n", fitsne_last_error());
        std::exit(rc);
    }
    fitsne_save_data(result_path, Y, costs, N, no_dims, max_iter);
    std::printf("Wrote the %i x %i data matrix successfully.\n", N, no_dims);
    std::free(data);
    std::free(Y);
    std::free(costs);
    std::free(perplexity_list);
    std::printf("Done.\n\n");
    return 0;
}
