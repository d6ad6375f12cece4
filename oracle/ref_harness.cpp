/*
 * C entry points into the UNMODIFIED FIt-SNE reference (src/tsne.cpp, src/nbodyfft.cpp,
 * src/sptree.cpp), compiled from where the sources lie by oracle/Makefile into
 * oracle/_ref/libfitsne_ref.so.  TEST INFRASTRUCTURE ONLY: this is the checker that
 * pins the C restatement (oracle/fitsne_oracle.c) and generates the golden fixtures
 * under tests/golden/; it is never linked into the GPU product.
 *
 * The gradient, cost and similarity routines are private members of class TSNE
 * (src/tsne.h:63-110).  They are reached here through the standard explicit
 * instantiation access rule (a pointer to a private member may be named in an explicit
 * template instantiation), so the reference header and sources stay untouched.
 */
#include <cstdlib>

#include "tsne.h"

namespace {

template <typename Tag, typename Tag::type M>
struct Rob {
    friend typename Tag::type get(Tag) { return M; }
};

struct TagSumQ {
    typedef double TSNE::*type;
    friend type get(TagSumQ);
};
template struct Rob<TagSumQ, &TSNE::current_sum_Q>;

typedef void (TSNE::*GradFn)(double *, unsigned int *, unsigned int *, double *, double *, int, int, double *, int,
                             double, int, unsigned int);
typedef void (TSNE::*GradDfFn)(double *, unsigned int *, unsigned int *, double *, double *, int, int, double *, int,
                               double, int, unsigned int, double);

struct TagFft2 { typedef GradFn type; friend type get(TagFft2); };
struct TagFft2Df { typedef GradDfFn type; friend type get(TagFft2Df); };
struct TagFft1 { typedef GradFn type; friend type get(TagFft1); };
struct TagFft1Df { typedef GradDfFn type; friend type get(TagFft1Df); };
template struct Rob<TagFft2, &TSNE::computeFftGradient>;
template struct Rob<TagFft2Df, &TSNE::computeFftGradientVariableDf>;
template struct Rob<TagFft1, &TSNE::computeFftGradientOneD>;
template struct Rob<TagFft1Df, &TSNE::computeFftGradientOneDVariableDf>;

struct TagExact {
    typedef void (TSNE::*type)(double *, double *, int, int, double *, double);
    friend type get(TagExact);
};
template struct Rob<TagExact, &TSNE::computeExactGradient>;

struct TagErrFft {
    typedef double (TSNE::*type)(unsigned int *, unsigned int *, double *, double *, int, int, unsigned int, double);
    friend type get(TagErrFft);
};
template struct Rob<TagErrFft, &TSNE::evaluateErrorFft>;

struct TagD2S {
    typedef double (TSNE::*type)(double *, double *, int, int, double, double, bool, int, double *);
    friend type get(TagD2S);
};
template struct Rob<TagD2S, &TSNE::distances2similarities>;

struct TagGPvp {
    typedef void (TSNE::*type)(double *, int, int, unsigned int **, unsigned int **, double **, double, int, double,
                               unsigned int, int, double *);
    friend type get(TagGPvp);
};
template struct Rob<TagGPvp, &TSNE::computeGaussianPerplexity>;

struct TagZeroMean {
    typedef void (TSNE::*type)(double *, int, int);
    friend type get(TagZeroMean);
};
template struct Rob<TagZeroMean, &TSNE::zeroMean>;

}  // namespace

extern "C" {

/* Dispatch exactly as TSNE::run does (src/tsne.cpp:444-464). Returns current_sum_Q. */
double ref_fft_gradient(const unsigned int *row_P, const unsigned int *col_P, const double *val_P, const double *Y,
                        int N, int no_dims, double *dC, int nterms, double intervals_per_integer,
                        int min_num_intervals, unsigned int nthreads, double df) {
    TSNE t;
    unsigned int *r = const_cast<unsigned int *>(row_P);
    unsigned int *c = const_cast<unsigned int *>(col_P);
    double *v = const_cast<double *>(val_P);
    double *y = const_cast<double *>(Y);
    if (no_dims == 1) {
        if (df == 1.0)
            (t.*get(TagFft1()))(nullptr, r, c, v, y, N, no_dims, dC, nterms, intervals_per_integer,
                                min_num_intervals, nthreads);
        else
            (t.*get(TagFft1Df()))(nullptr, r, c, v, y, N, no_dims, dC, nterms, intervals_per_integer,
                                  min_num_intervals, nthreads, df);
    } else {
        if (df == 1.0)
            (t.*get(TagFft2()))(nullptr, r, c, v, y, N, no_dims, dC, nterms, intervals_per_integer,
                                min_num_intervals, nthreads);
        else
            (t.*get(TagFft2Df()))(nullptr, r, c, v, y, N, no_dims, dC, nterms, intervals_per_integer,
                                  min_num_intervals, nthreads, df);
    }
    return t.*get(TagSumQ());
}

/* src/tsne.cpp:1232-1282 (dense P, O(N^2)) */
void ref_exact_gradient(const double *P, const double *Y, int N, int D, double *dC, double df) {
    TSNE t;
    (t.*get(TagExact()))(const_cast<double *>(P), const_cast<double *>(Y), N, D, dC, df);
}

/* src/tsne.cpp:1329-1355 with a given Z; nthreads 1 (the threaded form races on C). */
double ref_evaluate_error_fft(const unsigned int *row_P, const unsigned int *col_P, const double *val_P,
                              const double *Y, int N, int D, double df, double sum_Q) {
    TSNE t;
    t.*get(TagSumQ()) = sum_Q;
    return (t.*get(TagErrFft()))(const_cast<unsigned int *>(row_P), const_cast<unsigned int *>(col_P),
                                 const_cast<double *>(val_P), const_cast<double *>(Y), N, D, 1u, df);
}

/* src/tsne.cpp:1474-1500 (list overload, which dispatches to 1394-1469). */
double ref_distances2similarities(const double *D, double *P, int N, int n, double perplexity, double sigma,
                                  int if_squared, int perplexity_list_length, const double *perplexity_list) {
    TSNE t;
    return (t.*get(TagD2S()))(const_cast<double *>(D), P, N, n, perplexity, sigma, if_squared != 0,
                              perplexity_list_length, const_cast<double *>(perplexity_list));
}

/* src/tsne.cpp:1643-1726 (VP-tree kNN + bisection); arrays are malloc'd, free with ref_free. */
void ref_gaussian_perplexity_vptree(const double *X, int N, int D, unsigned int **row_P, unsigned int **col_P,
                                    double **val_P, double perplexity, int K, double sigma, unsigned int nthreads,
                                    int perplexity_list_length, const double *perplexity_list) {
    TSNE t;
    (t.*get(TagGPvp()))(const_cast<double *>(X), N, D, row_P, col_P, val_P, perplexity, K, sigma, nthreads,
                        perplexity_list_length, const_cast<double *>(perplexity_list));
}

/* src/tsne.cpp:1730-1828 (public member). */
void ref_symmetrize(unsigned int **row_P, unsigned int **col_P, double **val_P, int N) {
    TSNE t;
    t.symmetrizeMatrix(row_P, col_P, val_P, N);
}

/* src/tsne.cpp:1851-1876 */
void ref_zero_mean(double *X, int N, int D) {
    TSNE t;
    (t.*get(TagZeroMean()))(X, N, D);
}

/* src/tsne.h:42-48 / src/tsne.cpp:118-592 */
int ref_run(double *X, int N, int D, double *Y, int no_dims, double perplexity, double theta, int rand_seed,
            int skip_random_init, int max_iter, int stop_lying_iter, int mom_switch_iter, double momentum,
            double final_momentum, double learning_rate, int K, double sigma, int nbody_algorithm, int knn_algo,
            double early_exag_coeff, double *costs, int no_momentum_during_exag, int start_late_exag_iter,
            double late_exag_coeff, int n_trees, int search_k, int nterms, double intervals_per_integer,
            int min_num_intervals, unsigned int nthreads, int load_affinities, int perplexity_list_length,
            double *perplexity_list, double df, double max_step_norm) {
    TSNE t;
    return t.run(X, N, D, Y, no_dims, perplexity, theta, rand_seed, skip_random_init != 0, max_iter, stop_lying_iter,
                 mom_switch_iter, momentum, final_momentum, learning_rate, K, sigma, nbody_algorithm, knn_algo,
                 early_exag_coeff, costs, no_momentum_during_exag != 0, start_late_exag_iter, late_exag_coeff,
                 n_trees, search_k, nterms, intervals_per_integer, min_num_intervals, nthreads, load_affinities,
                 perplexity_list_length, perplexity_list, df, max_step_norm);
}

void ref_free(void *p) { free(p); }

}  // extern "C"
