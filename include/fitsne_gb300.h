/*
 * fitsne_gb300 -- C ABI of the GB300 (sm_103a) implementation of FIt-SNE's per-iteration
 * gradient and input-similarity stage.
 *
 * Every entry point is a drop-in for one interface of the reference (KlugerLab/FIt-SNE
 * v1.2.1, paths relative to that project); the citation is given beside each.
 *
 * Conventions
 *  - Host buffers are owned by the caller unless stated; arrays are row-major.
 *  - CSR matrices use 32-bit unsigned row pointers and column indices, as the reference.
 *  - Functions return 0 on success and a negative FITSNE_E* code on failure (the
 *    reference calls exit() in several of these places; this library never exits).
 *    fitsne_last_error() gives a message for the calling thread.
 *  - One GPU (the current CUDA device).  Calls are not re-entrant on one session.
 *  - The arithmetic precision of the one-shot entry points is selected with
 *    fitsne_set_precision(): 32 = the FP32 form (double-float coordinates, FP32 spread /
 *    FFT / gather / attraction, FP64 reductions; the default) or 64 = the plain FP64
 *    form of the same kernels.  The environment variable FITSNE_PRECISION sets the
 *    initial value.
 */
#ifndef FITSNE_GB300_H
#define FITSNE_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define FITSNE_OK 0
#define FITSNE_E_ARG (-3)         /* invalid argument (the reference exit(1)s on most) */
#define FITSNE_E_IO (-2)          /* file could not be opened / read (reference returns -2) */
#define FITSNE_E_UNSUPPORTED (-4) /* option outside this build's scope (exact t-SNE, Barnes-Hut) */
#define FITSNE_E_CUDA (-10)       /* CUDA runtime error */
#define FITSNE_E_GRID (-13)       /* interpolation grid larger than the on-chip FFT supports */
#define FITSNE_E_NOMEM (-20)      /* host allocation failed */

/* ---------------------------------------------------------------------------------
 * Whole pipeline.  Replaces TSNE::run (src/tsne.h:42-48, src/tsne.cpp:118-592) with the
 * same arguments and meaning.  X (N x D) is read, not modified (the reference centres and
 * rescales it in place); Y (N x no_dims) is the initial solution when skip_random_init is
 * non-zero and receives the embedding; costs (max_iter) receives the KL divergence at
 * every 50th and the last iteration.  Supported: nbody_algorithm 2 (FFT) with theta != 0;
 * knn_algo 2 (exact kNN); knn_algo 1 (Annoy) is served by the same exact kNN;
 * load_affinities 0/1/2 with the reference's P_row.dat / P_col.dat / P_val.dat files in
 * the working directory.  nthreads is accepted and ignored (the work runs on the GPU).
 */
int fitsne_run(double *X, int N, int D, double *Y, int no_dims, double perplexity, double theta, int rand_seed,
               int skip_random_init, int max_iter, int stop_lying_iter, int mom_switch_iter, double momentum,
               double final_momentum, double learning_rate, int K, double sigma, int nbody_algorithm,
               int knn_algo, double early_exag_coeff, double *costs, int no_momentum_during_exag,
               int start_late_exag_iter, double late_exag_coeff, int n_trees, int search_k, int nterms,
               double intervals_per_integer, int min_num_intervals, unsigned int nthreads, int load_affinities,
               int perplexity_list_length, double *perplexity_list, double df, double max_step_norm);

/* ---------------------------------------------------------------------------------
 * One gradient evaluation.  Replaces the private TSNE methods computeFftGradient,
 * computeFftGradientVariableDf, computeFftGradientOneD and computeFftGradientOneDVariableDf
 * (src/tsne.h:67-80, dispatched as in src/tsne.cpp:444-464: no_dims 1 or 2, df == 1 or
 * not).  P is the CSR (row_P[N+1], col_P[nnz], val_P[nnz]); Y is N x no_dims; dC receives
 * the gradient (no factor 4, as the reference); *sum_Q receives Z (current_sum_Q).
 */
int fitsne_fft_gradient(const unsigned int *row_P, const unsigned int *col_P, const double *val_P,
                        const double *Y, int N, int no_dims, double *dC, int nterms, double intervals_per_integer,
                        int min_num_intervals, double df, double *sum_Q);

/* KL divergence over the CSR edges with a given Z.  Replaces TSNE::evaluateErrorFft
 * (src/tsne.h:92, src/tsne.cpp:1329-1355); the result is the plain sum, without the
 * exaggeration correction that TSNE::run applies afterwards. */
int fitsne_evaluate_error_fft(const unsigned int *row_P, const unsigned int *col_P, const double *val_P,
                              const double *Y, int N, int no_dims, double df, double sum_Q, double *C);

/* ---------------------------------------------------------------------------------
 * Input similarities. */

/* Exact K nearest neighbours of every row of X (N x D), self included.  Replaces
 * VpTree::search over all points (src/vptree.h:110-133 with euclidean_distance,
 * src/vptree.h:97-107): indices[N*K] in increasing distance, distances[N*K] are
 * non-squared Euclidean distances in FP64. */
int fitsne_knn(const double *X, int N, int D, int K, unsigned int *indices, double *distances);

/* Row-wise perplexity calibration.  Batched replacement of
 * TSNE::distances2similarities (src/tsne.h:95-98, src/tsne.cpp:1394-1500) for rows of K
 * neighbour distances with the point itself already removed, used the way the kNN paths
 * use it (n = -1, ifSquared = true on non-squared distances, src/tsne.cpp:1692-1693):
 * P[nrows*K] receives the row-normalised similarities, betas[nrows] (may be NULL) the
 * precision of the last (or only) perplexity.  perplexity > 0: bisection to that
 * perplexity; perplexity < 0: fixed sigma; perplexity == 0: average over the list. */
int fitsne_distances2similarities(const double *D, double *P, int nrows, int K, double perplexity, double sigma,
                                  int perplexity_list_length, const double *perplexity_list, double *betas);

/* kNN + calibration into fixed-length CSR rows.  Replaces the VP-tree overload of
 * TSNE::computeGaussianPerplexity (src/tsne.h:105-107, src/tsne.cpp:1643-1726).  The three
 * arrays are malloc'd here (release with free() or fitsne_free()); row_P[n] = n*K. */
int fitsne_gaussian_perplexity(const double *X, int N, int D, unsigned int **row_P, unsigned int **col_P,
                               double **val_P, double perplexity, int K, double sigma, unsigned int nthreads,
                               int perplexity_list_length, const double *perplexity_list);

/* (P + P^T) / 2 on the union pattern, in the reference's entry order.  Replaces
 * TSNE::symmetrizeMatrix (src/tsne.h:56, src/tsne.cpp:1730-1828): the input arrays are
 * freed with free() and replaced by malloc'd output arrays. */
int fitsne_symmetrize(unsigned int **row_P, unsigned int **col_P, double **val_P, int N);

/* ---------------------------------------------------------------------------------
 * File formats of the fast_tsne binary (src/tsne.cpp:1895-2038). */
int fitsne_load_data(const char *data_path, double **data, double **Y, int *n, int *d, int *no_dims,
                     double *theta, double *perplexity, int *rand_seed, int *max_iter, int *stop_lying_iter,
                     int *mom_switch_iter, double *momentum, double *final_momentum, double *learning_rate,
                     int *K, double *sigma, int *nbody_algo, int *knn_algo, double *early_exag_coeff,
                     int *no_momentum_during_exag, int *n_trees, int *search_k, int *start_late_exag_iter,
                     double *late_exag_coeff, int *nterms, double *intervals_per_integer, int *min_num_intervals,
                     int *skip_random_init, int *load_affinities, int *perplexity_list_length,
                     double **perplexity_list, double *df, double *max_step_norm);
int fitsne_save_data(const char *result_path, const double *data, const double *costs, int n, int d, int max_iter);

/* ---------------------------------------------------------------------------------
 * Device-resident optimisation (the iteration loop of TSNE::run, src/tsne.cpp:437-577,
 * split out so that P and Y stay on the GPU between calls). */
typedef struct fitsne_session fitsne_session;

/* precision: 32 or 64 (see above). */
int fitsne_session_create(fitsne_session **out, int N, int no_dims, const unsigned int *row_P,
                          const unsigned int *col_P, const double *val_P, const double *Y0, int nterms,
                          double intervals_per_integer, int min_num_intervals, double df, int precision);
/* As fitsne_session_create, but P is built on the device from the data X (N x D, read
 * only): centring and max-abs scaling, exact kNN, calibration, symmetrisation and
 * normalisation exactly as fitsne_run does (the first half of TSNE::run,
 * src/tsne.cpp:153-330); P never visits the host.  *nnz (may be NULL) receives the number
 * of non-zeros of P. */
int fitsne_session_create_from_data(fitsne_session **out, const double *X, int N, int D, int no_dims,
                                    double perplexity, int K, double sigma, int perplexity_list_length,
                                    const double *perplexity_list, const double *Y0, int nterms,
                                    double intervals_per_integer, int min_num_intervals, double df, int precision,
                                    unsigned long long *nnz);
/* One gradient evaluation at the session's current Y (no update): dC (N x no_dims) and Z,
 * as fitsne_fft_gradient. */
int fitsne_session_gradient(fitsne_session *s, double *dC, double *sum_Q);
/* Runs iterations [it0, it1) of the schedule; early_exag_coeff must be resolved (> 0).
 * costs (length >= max_iter, may be NULL) receives the KL at the reference's iterations. */
int fitsne_session_run(fitsne_session *s, int it0, int it1, int max_iter, int stop_lying_iter,
                       int mom_switch_iter, double momentum, double final_momentum, double learning_rate,
                       double early_exag_coeff, int no_momentum_during_exag, int start_late_exag_iter,
                       double late_exag_coeff, double max_step_norm, double *costs);
int fitsne_session_get_y(fitsne_session *s, double *Y);
/* Per-stage device milliseconds of the last iteration when timing is on:
 * out[0..5] = centre/min-max, spread, FFT convolution, gather, attraction+update, total;
 * out[6] = boxes per dimension, out[7] = FFT length; always: out[8] = device milliseconds
 * of the whole last fitsne_session_run call (CUDA events on the session's stream),
 * out[9] = number of kernels that call launched. */
int fitsne_session_set_timing(fitsne_session *s, int on);
/* 1 (default unless FITSNE_GRAPH=0): iterations run in chunks of replayed two-iteration CUDA
 * graphs with the grid sized on the device; 0: one host round trip per iteration (the
 * per-stage timing path). */
int fitsne_session_set_graphs(fitsne_session *s, int on);
int fitsne_session_stage_times(fitsne_session *s, double *out10);
/* Launch shapes the session's autotuner chose (no reference counterpart), out[5]: the
 * attraction's shape index (FITSNE_ATTR_SHAPE numbering; -1 before the first choice), its rows
 * per work item (points per block in the tiled form) and edges per lane, its form (0 over the
 * full CSR, 2 tiled over the half-stored symmetric P), and the threads per block of the 2-D FFT
 * passes. */
int fitsne_session_launch_shapes(fitsne_session *s, int *out5);
void fitsne_session_destroy(fitsne_session *s);

/* ---------------------------------------------------------------------------------
 * Gradient evaluation that allocates no device memory.  This entry point has no
 * counterpart in the reference; it exists for callers that cannot let a library call
 * cudaMalloc: a host framework that owns the device memory through its own pool or a
 * fixed budget, or an inner loop where an allocation (and the device synchronisation it
 * brings) is not allowed.
 *
 * Same computation and result as fitsne_fft_gradient in the FP32 form, on the caller's
 * DEVICE buffers: d_row_P[N+1], d_col_P[nnz], d_val_P[nnz] (float), d_Y[N*no_dims] (double)
 * in; d_dC[N*no_dims] (double) out; *sum_Q (host, may be NULL) receives Z.  stream is a
 * cudaStream_t (NULL = the legacy default stream).  The call synchronises the host with
 * that stream twice: once to read the embedding's extent, which sizes the grid, and once
 * before it returns, when its work is complete.  All temporaries come from one fixed device
 * array of 32 MiB that every GPU loading this library holds until the process exits.
 * Limits: N <= 262144; the per-point buffers (32 N bytes in 2-D) and the grid's buffers
 * (about 160 (n_interpolation_points x boxes per dimension)^2 bytes in 2-D, about 100 bytes
 * per node in 1-D) must fit in the array together.  At N = 262144 that allows, per
 * dimension, 128 boxes at n_interpolation_points 3, 76 at 5 and 48 at 8 (a little more for
 * fewer points); the box count is the embedding's extent / intervals_per_integer, at least
 * min_num_intervals.  Larger inputs are rejected with FITSNE_E_ARG (N) or FITSNE_E_GRID
 * (grid) and a message naming the sizes.  The array is shared by all calls on a device and
 * keeps the last call's contents (each call clears what must start at zero): calls whose
 * work overlaps on the GPU race on it.  The array's device address is looked up with the
 * device current, once per CUDA context; the first call on a device does that lookup, so
 * make it before any stream capture. */
int fitsne_fft_gradient_noalloc(const unsigned int *d_row_P, const unsigned int *d_col_P, const float *d_val_P,
                                const double *d_Y, int N, int no_dims, double *d_dC, int nterms,
                                double intervals_per_integer, int min_num_intervals, double df, double *sum_Q,
                                void *stream);

/* ---------------------------------------------------------------------------------
 * Batched form (no reference counterpart; each job is what TSNE::run, src/tsne.cpp:118-
 * 577, does for one data set, FP32 form, FFT gradient, df = 1, exact kNN).  njobs
 * independent embeddings of any sizes: job j has HOST X[j] (N[j] x D[j]), Y[j] (N[j] x
 * no_dims, in/out; initialised by libc srand(rand_seed[j]) + the polar method x 1e-4 unless
 * skip_random_init), perplexity[j] (K = 3 perplexity) and learning_rate[j]; the schedule
 * and grid arguments are shared.  The similarity stage runs job after job; the iterations
 * advance all jobs together in chunks between the schedule's events; each job's chunk is
 * one CUDA graph (cached per job, the grid sized on the device) launched on the job's own
 * stream, so the jobs' kernels overlap.  costs[j] (may be NULL, or
 * costs itself) receives job j's KL every 50 iterations as in TSNE::run.  stats5 (may be
 * NULL): seconds of the similarity stage, seconds of the iterations, chunk graph launches,
 * graph instantiations (other recaptures update an instantiated graph in place), chunks
 * repeated because a job's grid outgrew its capacity. */
int fitsne_batch_run(int njobs, const double *const *X, const int *N, const int *D, double *const *Y, int no_dims,
                     const double *perplexity, const double *learning_rate, const int *rand_seed,
                     int skip_random_init, int max_iter, int stop_lying_iter, int mom_switch_iter, double momentum,
                     double final_momentum, double early_exag_coeff, int nterms, double intervals_per_integer,
                     int min_num_intervals, double max_step_norm, double *const *costs, double *stats5);

/* ---------------------------------------------------------------------------------
 * Learned warm start of the perplexity calibration (no reference counterpart: the
 * bisection it seeds is distances2similarities, src/tsne.cpp:1394-1469).
 *
 * fitsne_set_calibration(1) makes the similarity stage (fitsne_run, fitsne_gaussian_
 * perplexity, fitsne_session_create_from_data) calibrate single-perplexity runs of at
 * least 20,000 points as follows:
 *   - the plain bisection (the reference's) on the first max(10000, min(N/10, 200000)) rows;
 *   - training, on the GPU, of an MLP (K -> 64 -> 64 -> 1) that maps the row's scaled
 *     kNN distances to log(beta * mean distance);
 *   - for the other rows, a safeguarded Newton search from the predicted beta, to
 *     |H - log(perplexity)| < 1e-6.
 * 0 (default, or FITSNE_CALIBRATION unset / "bisection") keeps the reference's bisection
 * everywhere: P is then identical to the reference's.  Perplexity lists and fixed sigma
 * always use the bisection. */
void fitsne_set_calibration(int mode);
int fitsne_get_calibration(void);
/* Statistics of this process's last calibration, out[12]: rows, harvested rows (plain
 * bisection), predicted rows that needed bisection steps, training steps, mean entropy
 * evaluations per harvested row, mean per predicted row, first and last training loss
 * (standardised MSE), ms for harvest (with the plain bisection: of all rows), training,
 * inference, warm-started search.  Entropy evaluations count FP32 and FP64 steps alike
 * (both searches evaluate a step in FP32 first and in FP64 where FP32 cannot decide it).
 * Returns 0. */
int fitsne_calibration_stats(double *out12);
/* Number of FP32 parameters of the network for K distances per row: W1[64][K], b1[64],
 * W2[64][64], b2[64], w3[64], b3. */
int fitsne_mlp_param_count(int K);
/* The network's loss and gradient on the GPU, for checking the training kernels: mean over
 * the nrows rows (HOST dist[nrows*K] ascending, beta[nrows]) of (out - t)^2 with the target
 * t = (log(beta * mean(dist)) - mu) / sd and input dist / mean(dist); params and grad are
 * HOST arrays of fitsne_mlp_param_count(K) floats. */
int fitsne_mlp_loss_grad(const float *params, int K, const double *dist, const double *beta, int nrows, double mu,
                         double sd, float *grad, double *loss);

/* ---------------------------------------------------------------------------------
 * PCA initialisation on the GPU (replaces the scikit-learn PCA of fast_tsne.py:186-197,
 * the step before TSNE::run): the first n_components principal components of HOST X
 * (N x D, not modified) into HOST Y (N x n_components, row-major): (X - mean) V with V the
 * leading eigenvectors of the covariance, each component's largest-magnitude entry positive
 * (scikit-learn's svd_flip with u_based_decision=False).  D <= 2048. */
int fitsne_pca(const double *X, int N, int D, int n_components, double *Y);

/* ---------------------------------------------------------------------------------
 * Misc. */
void fitsne_set_precision(int bits);
int fitsne_get_precision(void);
const char *fitsne_last_error(void);
const char *fitsne_version(void); /* "1.2.1" data-file protocol version */
void fitsne_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
