// Device-resident state of one embedding and the host loop that drives the kernels.
//
// Embedding<T> mirrors the gradient part of TSNE::run (src/tsne.cpp:437-577 of the
// reference): per iteration it centres Y (zeroMean of the previous step), reads the
// bounding square, builds the interpolation grid with the reference's box-count rule,
// spreads, convolves, gathers, and applies the attraction + optimiser step in one pass.
#pragma once

#include <map>
#include <string>
#include <vector>

#include "fftconv.cuh"
#include "grad.cuh"

namespace fitsne {

// Optimiser schedule (arguments of TSNE::run that drive the iteration loop).
struct Schedule {
    int max_iter = 1000;
    int stop_lying_iter = 250;
    int mom_switch_iter = 250;
    double momentum = 0.5;
    double final_momentum = 0.8;
    double learning_rate = 200.0;
    double early_exag_coeff = 12.0;
    int no_momentum_during_exag = 0;
    int start_late_exag_iter = -1;
    double late_exag_coeff = -1.0;
    double max_step_norm = 5.0;
};

// Embeddings smaller than this are not renumbered (they fit in cache either way).
constexpr int kReorderMinN = 16384;
// Longest chunk of graph-replayed iterations between two host reads of the grid status.
constexpr int kMaxChunk = 50;

struct GridParams {
    int nterms = 3;
    double intervals_per_integer = 1.0;
    int min_num_intervals = 50;
    double df = 1.0;
};

// Per-stage device time of the last timed iteration (CUDA events), milliseconds.
struct StageTimes {
    float center = 0, spread = 0, conv = 0, gather = 0, attract = 0, total = 0;
    float run_ms = 0;               // device time of the last run_schedule call (events)
    unsigned long long launches = 0;  // kernels launched by the last run_schedule call
};

template <typename T>
class Embedding {
   public:
    typedef typename Cx<T>::t C;

    Embedding();
    ~Embedding();
    Embedding(const Embedding &) = delete;
    Embedding &operator=(const Embedding &) = delete;

    // Uploads P (host CSR; val in FP64) and the initial Y (host, N x D row-major).
    int init_host(int N, int D, const uint32_t *row, const uint32_t *col, const double *val, const double *Y0,
                  const GridParams &gp, cudaStream_t st);
    // Takes P already on the device (row/col u32, val FP64); the arrays are copied.
    int init_device(int N, int D, const uint32_t *d_row, const uint32_t *d_col, const double *d_val,
                    size_t nnz, const double *Y0_host, const GridParams &gp, cudaStream_t st);

    // One gradient evaluation without update: dC (host, N x D) and Z.
    int gradient(double *dC_host, double *sum_Q);
    // One optimiser iteration with the given step parameters.
    int step(const UpdateParams &p, bool first);
    // KL divergence with the current Y, the Z of the last gradient, P scaled by exag.
    int kl(double exag, double *out);
    // KL with a caller-supplied Z (evaluateErrorFft with current_sum_Q set by the caller).
    int kl_with_z(double exag, double z, double *out);
    // Subtracts the pending mean and copies Y to the host.
    int get_Y(double *Y_host);

    // Runs iterations [it0, it1) of the reference schedule; costs may be null.
    int run_schedule(const Schedule &s, int it0, int it1, double *costs, bool verbose);

    void set_timing(bool on) { timing_ = on; }
    // CUDA-graph iteration chunks (on by default; FITSNE_GRAPH=0 or timing turn them off)
    void set_graphs(bool on) { graphs_ = on; }
    bool graphs() const { return graphs_; }

    // ---- graph-captured chunks (used by run_schedule and by the multi-job driver) ----
    // A chunk is `len` iterations with constant parameters on this object's stream: a
    // snapshot of the state, the iterations, then the status and box count copied to pinned
    // memory.  The iterations are replays of small captured graphs of one or two iterations
    // each, cached per (iterations, current buffer, mean flag of the first) and captured
    // again only when what they depend on changes.  A capture and its update cost host time
    // in proportion to the nodes, with the GPU idle meanwhile: graphs of whole 50-iteration
    // chunks took 23 ms of a 600-iteration run at N = 1M (9 captures).
    // record_iters records n iterations starting from buffer c (the stream must be
    // capturing): per iteration centre/min-max (the first applies the pending mean when
    // apply_mean_first), device-side grid sizing, spread, convolution, gather, attraction +
    // update.
    int record_iters(const UpdateParams &p, int n, int c, bool apply_mean_first);
    // records (or reuses the cached graph of) n iterations from buffer c and launches it
    int launch_iters(const UpdateParams &p, int n, int c, bool apply_mean_first);
    // After the chunk ran: 0 ok, 1 the grid outgrew its capacity (state restored: redo the
    // chunk with a larger one), <0 error.  Updates cur_ / mean_pending_ on success.
    int finish_chunk(int len);
    // Capacity for the next chunk from the last known box count (grows buffers; call
    // outside any capture).  grow > 0 forces a larger capacity after an overflow.
    int plan_capacity(int grow);
    // plan_capacity, then the chunk on this object's stream (snapshot, iterations graphs,
    // status copies) without synchronising; finish_chunk after the stream is idle.
    int launch_chunk(const UpdateParams &p, int len, int grow);
    unsigned long long graph_captures() const { return captures_; }
    unsigned long long graph_updates() const { return updates_; }
    // Runs iterations [it0, it1) with graph chunks; costs may be null.
    int run_schedule_graphs(const Schedule &s, int it0, int it1, double *costs, bool verbose);
    // What recorded iterations depend on (parameters, capacity, buffers): equal keys replay.
    std::vector<unsigned long long> iters_key(const UpdateParams &p, int n, int c, bool apply_mean_first) const;
    bool mean_pending() const { return mean_pending_; }
    void set_first_geometry() { nb_last_ = geom_.nb; }
    // Renumbering rule of run_schedule (iterations 50, 150, 300, 600 above kReorderMinN).
    bool reorder_due(int it, int it0) const {
        return reorder_enabled_ && N_ >= kReorderMinN &&
               (it == 50 || it == 150 || it == 300 || it == 600 || (!reordered_ && it == it0 && it0 > 50));
    }
    int reorder_now() { return reorder(); }
    // Numbers the points in a given order instead (order[k] = caller index of internal point
    // k, on the device); the points keep it, and the renumbering schedule then only orders the
    // spread's walk.
    int set_order(const uint32_t *order);
    // Phase of the run for the attraction's launch shape: 0 while the embedding is compact
    // (early exaggeration and the first 50 iterations after it), 1 once it has expanded.  The
    // shapes rank differently in the two (N = 1M: 8 x 4 rows/edges 0.95 ms against 1.18 ms for
    // the register-capped 16 x 2 up to iteration 260; 0.68 against 0.75 ms from 320 on), so each
    // phase is timed on its own.  In the default schedule phase 1 starts with the renumbering
    // at iteration 300.
    int tune_phase(const Schedule &s, int it) const {
        return (s.stop_lying_iter < 0 || it >= s.stop_lying_iter + 50) ? 1 : 0;
    }
    const StageTimes &last_times() const { return times_; }
    const GridGeom &last_geom() const { return geom_; }
    int last_L() const { return L_; }
    size_t nnz() const { return nnz_; }
    int N() const { return N_; }
    cudaStream_t stream() const { return st_; }
    const std::string &error() const { return err_; }
    // launch shapes in use: attraction shape index, its rows per work item (points per tile
    // block in the tiled form) and edges per lane, the attraction's form (0 full CSR, 2 tiled),
    // FFT threads per block
    void launch_shapes(int *out5) const;
    // device pointers (for zero-copy consumers such as the no-allocation path)
    const uint32_t *d_row() const { return row_; }
    const uint32_t *d_col() const { return col_; }
    const T *d_val() const { return val_; }
    const T *d_Y() const { return Y_[cur_]; }

   private:
    int alloc_common(int N, int D, size_t nnz);
    int prepare_grid();  // reads min/max (synchronises) and sizes the grid
    int repulsion();     // spread + conv + gather
    int fail(const char *what, cudaError_t e);

    int N_ = 0, D_ = 0;
    size_t nnz_ = 0;
    GridParams gp_;
    cudaStream_t st_ = nullptr;
    uint32_t *row_ = nullptr, *col_ = nullptr;
    T *val_ = nullptr;
    T *Y_[2] = {nullptr, nullptr};
    float *yh_ = nullptr;  // FP32 form: high words of Y_[cur_] (written by the gather pass)
    int cur_ = 0;
    bool mean_pending_ = false;
    T *uY_ = nullptr, *gains_ = nullptr, *rep_ = nullptr, *dC_ = nullptr;
    Cell4<T> *grid_in_ = nullptr, *grid_out_ = nullptr;
    size_t grid_cap_ = 0;
    C *work_a_ = nullptr, *work_b_ = nullptr;
    size_t wa_cap_ = 0, wb_cap_ = 0;
    KSpec<T> *kspec_ = nullptr;
    size_t ks_cap_ = 0;
    std::map<int, C *> tw_;
    RedScratch red_{};
    double *red_mem_ = nullptr;
    unsigned int *red_cnt_ = nullptr;
    double *h_pin_ = nullptr;  // pinned: [min, max, z, kl]
    GridGeom geom_{};
    FftPlan plan_{};
    int L_ = 0;
    bool timing_ = false;
    StageTimes times_;
    // per-iteration stage events, double-buffered so that the previous iteration's events
    // are read after the next iteration's existing synchronisation (no extra host waits)
    cudaEvent_t evs_[2][6] = {};
    cudaEvent_t evr_[2] = {};  // start / end of a run_schedule call
    int tb_ = 0;
    bool tpend_ = false;
    double tacc_[6] = {};
    int tacc_n_ = 0;
    void read_stage_events(int buf);
    unsigned long long launches_ = 0;  // running count of this object's kernel launches

    // autotuned launch shape of the attraction pass (-1: not chosen yet); re-chosen after a
    // locality renumbering and when the run enters a new phase, since the gathers' locality
    // and the embedding's extent decide between the shapes
    int attr_shape_ = -1;
    int attr_phase_ = -1;  // tune_phase_ that attr_shape_ was chosen for
    // The tiled attraction (FP32 form, symmetric P; shape kAttrTilesShape): records of the
    // upper entries sorted by tile, the tiles' first records, the force accumulator.
    bool sym_ok_ = false, tiles_ok_ = false;
    uint32_t *urow_ = nullptr;
    size_t unnz_ = 0;
    uint2 *trec_ = nullptr;
    uint32_t *tstart_ = nullptr;
    float *acc_ = nullptr;
    int check_symmetric();  // sets sym_ok_ (FP32 form, FITSNE_ATTR_SYM unset or 1), builds the tiles
    int build_tiles();      // from the current CSR (after every renumbering)
    static constexpr int kTilesMaxN = 262144;
    bool tiles_wanted() const;
    // the attraction + update of the given shape (either form)
    cudaError_t attr_call(const T *Yin, T *Yout, T *uY, T *gains, T *dC, const UpdateParams &p, int shape);
    int tune_phase_ = 1;   // phase of the current iteration (tune_phase)
    int tune_attr(bool measure);
    // autotuned threads per block of the 2-D FFT passes, per transform length (fft_thr_L_)
    int fft_thr_ = 256, fft_thr_L_ = 0;
    int tune_fft(int M, int L);
    C *twiddles(int L);  // host-built twiddles of length L (cached in tw_)
    // graph chunks
    bool graphs_ = true;
    DevGeom *dgeom_ = nullptr;         // device: geometry of the current iteration
    int *gstatus_ = nullptr;           // device: OR of the chunk's geometry statuses
    int *h_gstat_ = nullptr;           // pinned: [status, boxes per dimension]
    C *tw_dev_ = nullptr;              // twiddles written on the device for the current L
    int tw_dev_cap_ = 0;
    int nb_cap_ = 0, M_cap_ = 0, L_cap_ = 0, nb_last_ = 0;
    T *snap_ = nullptr;                // state at the start of a chunk: Y, uY, gains
    double *snap_mean_ = nullptr;      // and the pending mean
    struct GraphSlot {  // a cached iterations graph and its key
        cudaGraphExec_t exec = nullptr;
        std::vector<unsigned long long> key;
    };
    GraphSlot gslots_[2][2][2];     // [iterations - 1][current buffer][mean flag of the first]
    int grid_buffers(int M, int L);  // grows grid / FFT buffers to M x M, L
    int gchunk_len_ = 0;
    unsigned long long captures_ = 0, updates_ = 0;
    int gchunk_cur0_ = 0;

    // locality renumbering (reorder.cuh): perm_[k] = caller index of internal point k
    int renumber_alloc();
    int renumber(const uint32_t *order);
    int reorder();
    int perm_to_host(std::vector<uint32_t> &out);
    bool reorder_enabled_ = true;
    bool reordered_ = false;
    // numbered in the data's locality order (set_order): the renumbering schedule then only
    // refreshes sorder_, the Morton order in which the spread walks the points
    bool data_order_ = false;
    uint32_t *sorder_ = nullptr;
    int excl_ = 0;  // internal index of the caller's point 0 (min/max rule of the reference)
    uint32_t *perm_ = nullptr, *iperm_ = nullptr, *rkeys_ = nullptr, *rids_ = nullptr, *rkeys2_ = nullptr,
             *rids2_ = nullptr, *rlen_ = nullptr, *row2_ = nullptr, *col2_ = nullptr;
    T *val2_ = nullptr;
    void *rscratch_ = nullptr;
    std::string err_;
};

// Box-count rule of the reference (tsne.cpp:1065-1077 for 2-D, 663/774 for 1-D) and
// the node layout of precompute_2d / precompute (nbodyfft.cpp:9-70, 251-307).
GridGeom make_grid_geom(double mn, double mx, int D, const GridParams &gp);

}  // namespace fitsne
