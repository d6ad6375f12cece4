// Batched form of the iteration: many independent embeddings ("jobs") advanced together,
// one kernel launch per stage for all of them (no counterpart in the reference, which runs one
// data set per process).
//
// The jobs' points, CSR matrices, positions and optimiser state are concatenated; every job
// keeps its own interpolation grid (sized on the device each iteration from its own extent,
// inside a per-job capacity), its own FFT buffers, Z, mean and KL.  Each batched launch
// splits its blocks among the jobs (grad.cuh, fftconv.cuh); the per-job reductions finish in
// each job's last block.  An iteration is 12 launches whatever the number of jobs, and a run
// of up to 50 iterations is captured as one CUDA graph.  FP32 form, 2-D, nterms 3, df = 1.
#pragma once

#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "affinity.cuh"
#include "embedding.cuh"
#include "fftconv.cuh"
#include "grad.cuh"

namespace fitsne {

class BatchPipeline {
   public:
    BatchPipeline() = default;
    ~BatchPipeline();
    BatchPipeline(const BatchPipeline &) = delete;
    BatchPipeline &operator=(const BatchPipeline &) = delete;

    // Whether a batch with these settings runs on this pipeline (else one graph per job).
    static bool supports(int no_dims, const GridParams &gp);
    // P[j]: job j's normalised symmetric P (device, consumed: the pipeline copies it);
    // Y0[j]: its N_j x 2 start (host); lr[j]: its learning rate.
    int init(const std::vector<DevCSR> &P, const std::vector<const double *> &Y0, const std::vector<double> &lr,
             const GridParams &gp, cudaStream_t st);
    // The reference's schedule (TSNE::run's loop) for every job; costs[j] (may be null)
    // receives job j's KL every 50 iterations.  stats (5 values, may be null): graph launches,
    // graph captures, graph updates (in place of an instantiation), chunk repeats, seconds.
    int run_schedule(const Schedule &s, double *const *costs, double *stats);
    int get_Y(int j, double *Y);
    const std::string &error() const { return err_; }

   private:
    int plan(bool grow);
    int upload_maps();
    int record_chunk(const UpdateParams &p, int len, bool apply_first);
    int launch_chunk(const UpdateParams &p, int len, bool apply_first, bool grow);
    int kl_all(double exag, std::vector<double> &out);

    std::string err_;
    cudaStream_t st_ = nullptr;
    GridParams gp_;
    int J_ = 0, D_ = 2, Ntot_ = 0;
    size_t nnz_tot_ = 0;
    std::vector<int> n_, p0_;
    std::vector<double> lr_;
    // concatenated per-point state (FP32 form: double-float Y, 4 floats per 2-D point)
    float *Y_[2] = {nullptr, nullptr};
    float *uY_ = nullptr, *gains_ = nullptr, *rep_ = nullptr, *yh_ = nullptr;
    uint32_t *row_ = nullptr, *col_ = nullptr;
    float *val_ = nullptr;
    int cur_ = 0;
    bool mean_pending_ = false;
    // per-job reduction scratch and geometry
    double *red_mem_ = nullptr;     // partials + per-job scalars
    unsigned int *counts_ = nullptr;
    RedScratch *rs_ = nullptr;      // device array, J entries
    std::vector<RedScratch> hrs_;   // its host copy
    DevGeom *dg_ = nullptr;         // device array, J entries
    int *status_ = nullptr;         // device, J entries (OR over the iterations of a chunk)
    int *h_status_ = nullptr;       // pinned: status, then box counts
    DevGeom *h_dg_ = nullptr;       // pinned copy of dg_
    // capacities and the tables / maps built from them
    std::vector<int> nb_cap_, nb_last_;
    std::vector<BatchJobDev> hjobs_;
    BatchJobDev *jobs_ = nullptr;
    FftBatchJob *fjobs_ = nullptr;
    int *maps_ = nullptr;           // device: every map's job / first / count arrays
    size_t maps_len_ = 0;
    BatchMap pp_{}, at_{};
    FftBatchMap krow_{}, cols_{}, rows_{};
    int n_pp_ = 0, n_at_ = 0, n_krow_ = 0, n_cols_ = 0, n_rows_ = 0, L_max_ = 0;
    size_t cells_ = 0, work_ = 0, kspec_n_ = 0, tw_n_ = 0, cells_used_ = 0;
    Cell4<float> *grid_in_ = nullptr, *grid_out_ = nullptr;
    float2 *work_a_ = nullptr, *work_b_ = nullptr, *tw_ = nullptr;
    KSpec<float> *kspec_ = nullptr;
    // snapshot of the state a chunk starts from (repeated after a grid overflow)
    float *snap_ = nullptr;
    double *snap_mean_ = nullptr;
    // the cached chunk graph
    cudaGraphExec_t gexec_ = nullptr;
    std::vector<unsigned long long> gkey_;
    int gexec_len_ = -1;
    unsigned long long captures_ = 0, updates_ = 0, redos_ = 0, launches_ = 0, graph_launches_ = 0;
};

}  // namespace fitsne
