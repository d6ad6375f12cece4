// Batched iteration pipeline (see batch.cuh).
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>

#include "batch.cuh"

namespace fitsne {
namespace {

constexpr int kThreads = 256;

#define BCK(call)                                                                     \
    do {                                                                              \
        cudaError_t e__ = (call);                                                     \
        if (e__ != cudaSuccess) {                                                     \
            err_ = std::string(#call) + ": " + cudaGetErrorString(e__);               \
            return -10;                                                               \
        }                                                                             \
    } while (0)

__global__ void k_offset_u32(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst, size_t n, uint32_t add) {
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n; i += (size_t) gridDim.x * blockDim.x)
        dst[i] = src[i] + add;
}

// The box count of the grid rule's allowed list at or above target (below 200).
int allowed_at_least(int target) {
    static const int allowed[20] = {25, 36, 50, 55, 60, 65, 70, 75, 80, 85, 90, 96, 100, 110, 120, 130, 140, 150, 175, 200};
    if (target >= 200) return target;
    int i = 0;
    while (allowed[i] < target) ++i;
    return allowed[i];
}

// blocks of the per-point stages and of the attraction for n points
int pp_blocks(int n) { return std::max(1, std::min(256, (n + 2 * kThreads - 1) / (2 * kThreads))); }
int at_blocks(int n) { return std::max(1, std::min(1024, (n + 2 * kThreads - 1) / (2 * kThreads))); }

}  // namespace

bool BatchPipeline::supports(int no_dims, const GridParams &gp) {
    return no_dims == 2 && gp.nterms == 3 && gp.df == 1.0;
}

BatchPipeline::~BatchPipeline() {
    if (gexec_) cudaGraphExecDestroy(gexec_);
    for (void *p : {(void *) Y_[0], (void *) Y_[1], (void *) uY_, (void *) gains_, (void *) rep_, (void *) yh_,
                    (void *) row_, (void *) col_, (void *) val_, (void *) red_mem_, (void *) counts_, (void *) rs_,
                    (void *) dg_, (void *) status_, (void *) jobs_, (void *) fjobs_, (void *) maps_,
                    (void *) grid_in_, (void *) grid_out_, (void *) work_a_, (void *) work_b_, (void *) tw_,
                    (void *) kspec_, (void *) snap_, (void *) snap_mean_})
        cudaFree(p);
    if (h_status_) cudaFreeHost(h_status_);
    if (h_dg_) cudaFreeHost(h_dg_);
}

int BatchPipeline::init(const std::vector<DevCSR> &P, const std::vector<const double *> &Y0,
                        const std::vector<double> &lr, const GridParams &gp, cudaStream_t st) {
    st_ = st;
    gp_ = gp;
    J_ = (int) P.size();
    D_ = 2;
    lr_ = lr;
    n_.resize(J_);
    p0_.resize(J_);
    std::vector<size_t> e0(J_);
    Ntot_ = 0;
    nnz_tot_ = 0;
    for (int j = 0; j < J_; ++j) {
        n_[j] = P[j].N;
        p0_[j] = Ntot_;
        e0[j] = nnz_tot_;
        Ntot_ += P[j].N;
        nnz_tot_ += P[j].nnz;
    }
    if (nnz_tot_ >= (size_t) UINT_MAX) {
        err_ = "batched form: more than 2^32 non-zeros in all";
        return -3;
    }
    const size_t np = (size_t) Ntot_;
    BCK(cudaMalloc(&Y_[0], sizeof(float) * np * 4));
    BCK(cudaMalloc(&Y_[1], sizeof(float) * np * 4));
    BCK(cudaMalloc(&uY_, sizeof(float) * np * 2));
    BCK(cudaMalloc(&gains_, sizeof(float) * np * 2));
    BCK(cudaMalloc(&rep_, sizeof(float) * np * 2));
    BCK(cudaMalloc(&yh_, sizeof(float) * np * 2));
    BCK(cudaMalloc(&row_, sizeof(uint32_t) * (np + 1)));
    BCK(cudaMalloc(&col_, sizeof(uint32_t) * std::max<size_t>(nnz_tot_, 1)));
    BCK(cudaMalloc(&val_, sizeof(float) * std::max<size_t>(nnz_tot_, 1)));
    BCK(cudaMalloc(&snap_, sizeof(float) * np * 8));
    BCK(cudaMalloc(&snap_mean_, sizeof(double) * 2 * J_));
    BCK(cudaMemsetAsync(uY_, 0, sizeof(float) * np * 2, st_));
    BCK(cudaMemsetAsync(yh_, 0, sizeof(float) * np * 2, st_));
    {
        std::vector<float> ones(np * 2, 1.0f);
        BCK(cudaMemcpyAsync(gains_, ones.data(), sizeof(float) * ones.size(), cudaMemcpyHostToDevice, st_));
        BCK(cudaStreamSynchronize(st_));
    }
    // concatenated CSR: rows shifted by the job's first non-zero, columns by its first point
    double *tmp = nullptr;
    size_t nmax = 0;
    for (int j = 0; j < J_; ++j) nmax = std::max(nmax, (size_t) n_[j] * 2);
    BCK(cudaMalloc(&tmp, sizeof(double) * std::max<size_t>(nmax, 1)));
    for (int j = 0; j < J_; ++j) {
        k_offset_u32<<<64, kThreads, 0, st_>>>(P[j].row, row_ + p0_[j], (size_t) n_[j], (uint32_t) e0[j]);
        if (P[j].nnz) {
            k_offset_u32<<<256, kThreads, 0, st_>>>(P[j].col, col_ + e0[j], P[j].nnz, (uint32_t) p0_[j]);
            BCK(launch_cast_from_double<float>(P[j].val, val_ + e0[j], P[j].nnz, st_));
        }
        BCK(cudaMemcpyAsync(tmp, Y0[j], sizeof(double) * (size_t) n_[j] * 2, cudaMemcpyHostToDevice, st_));
        BCK(launch_y_from_double<float>(tmp, Y_[0] + (size_t) p0_[j] * 4, n_[j], 2, st_));
        BCK(cudaStreamSynchronize(st_));  // tmp is reused
    }
    cudaFree(tmp);
    const uint32_t last = (uint32_t) nnz_tot_;
    BCK(cudaMemcpyAsync(row_ + np, &last, sizeof(uint32_t), cudaMemcpyHostToDevice, st_));
    // per-job reduction scratch: partials for the most blocks any stage gives the job, then
    // mnmx[2], z, mean[2], kl
    std::vector<size_t> part0(J_);
    size_t nparts = 0;
    for (int j = 0; j < J_; ++j) {
        part0[j] = nparts;
        nparts += 4 * (size_t) std::max(pp_blocks(n_[j]), at_blocks(n_[j]));
    }
    const size_t scal0 = nparts;
    BCK(cudaMalloc(&red_mem_, sizeof(double) * (nparts + 6 * (size_t) J_)));
    BCK(cudaMemsetAsync(red_mem_, 0, sizeof(double) * (nparts + 6 * (size_t) J_), st_));
    BCK(cudaMalloc(&counts_, sizeof(unsigned int) * 8 * J_));
    BCK(cudaMemsetAsync(counts_, 0, sizeof(unsigned int) * 8 * J_, st_));
    hrs_.resize(J_);
    for (int j = 0; j < J_; ++j) {
        double *sc = red_mem_ + scal0 + 6 * (size_t) j;
        hrs_[j].part = red_mem_ + part0[j];
        hrs_[j].count = counts_ + 8 * j;
        hrs_[j].mnmx = sc;
        hrs_[j].z = sc + 2;
        hrs_[j].mean = sc + 3;
        hrs_[j].kl = sc + 5;
    }
    BCK(cudaMalloc(&rs_, sizeof(RedScratch) * J_));
    BCK(cudaMemcpyAsync(rs_, hrs_.data(), sizeof(RedScratch) * J_, cudaMemcpyHostToDevice, st_));
    BCK(cudaMalloc(&dg_, sizeof(DevGeom) * J_));
    BCK(cudaMemsetAsync(dg_, 0, sizeof(DevGeom) * J_, st_));
    BCK(cudaMalloc(&status_, sizeof(int) * J_));
    BCK(cudaHostAlloc(&h_status_, sizeof(int) * J_, cudaHostAllocDefault));
    BCK(cudaHostAlloc(&h_dg_, sizeof(DevGeom) * J_, cudaHostAllocDefault));
    BCK(cudaMalloc(&jobs_, sizeof(BatchJobDev) * J_));
    BCK(cudaMalloc(&fjobs_, sizeof(FftBatchJob) * J_));
    nb_cap_.assign(J_, 0);
    nb_last_.assign(J_, gp_.min_num_intervals);
    hjobs_.resize(J_);
    cur_ = 0;
    mean_pending_ = false;
    BCK(cudaStreamSynchronize(st_));
    return plan(false);
}

// Per-job grid capacity from the last box counts (as Embedding::plan_capacity), buffers,
// tables and block maps.  grow: a job of the last chunk outgrew its capacity.
int BatchPipeline::plan(bool grow) {
    bool changed = false;
    for (int j = 0; j < J_; ++j) {
        const int nb = std::max(1, nb_last_[j]);
        const bool over = grow && h_dg_ && (h_status_[j] & 1);
        int target = over ? std::max(nb_cap_[j] + 1, nb + nb / 2 + 1) : nb + nb / 4 + 1;
        target = allowed_at_least(target);
        if (!over && target <= nb_cap_[j]) continue;  // keep a larger capacity (and the graph)
        while (target > 1 && smooth_even_at_least(2 * target * gp_.nterms) > max_fft_len<float>()) --target;
        if (target != nb_cap_[j]) {
            nb_cap_[j] = target;
            changed = true;
        }
    }
    if (!changed && grid_in_) return 0;
    // offsets of every job's buffers, sized for its capacity
    size_t cells = 0, work = 0, ks = 0, tw = 0;
    L_max_ = 0;
    std::vector<FftBatchJob> hf(J_);
    for (int j = 0; j < J_; ++j) {
        const int M = nb_cap_[j] * gp_.nterms;
        const int L = smooth_even_at_least(2 * M);
        const int H = L / 2 + 1;
        L_max_ = std::max(L_max_, L);
        hjobs_[j].p0 = p0_[j];
        hjobs_[j].n = n_[j];
        hjobs_[j].nb_cap = nb_cap_[j];
        hjobs_[j].L_cap = L;
        hjobs_[j].cell0 = cells;
        hjobs_[j].lr = (float) lr_[j];
        hf[j].cg = &dg_[j].conv;
        hf[j].cell0 = cells;
        hf[j].work0 = work;
        hf[j].kspec0 = ks;
        hf[j].tw0 = tw;
        cells += (size_t) M * M;
        work += 4 * (size_t) L * H;
        ks += (size_t) H * L;
        tw += (size_t) L;
    }
    cells_used_ = cells;
    if (cells > cells_ || work > work_ || ks > kspec_n_ || tw > tw_n_) {
        // grow with headroom: capacities rise a few times per run
        cells_ = cells + cells / 2;
        work_ = work + work / 2;
        kspec_n_ = ks + ks / 2;
        tw_n_ = tw + tw / 2;
        for (void *p : {(void *) grid_in_, (void *) grid_out_, (void *) work_a_, (void *) work_b_, (void *) kspec_,
                        (void *) tw_})
            cudaFree(p);
        BCK(cudaMalloc(&grid_in_, sizeof(Cell4<float>) * cells_));
        BCK(cudaMalloc(&grid_out_, sizeof(Cell4<float>) * cells_));
        BCK(cudaMalloc(&work_a_, sizeof(float2) * work_));
        BCK(cudaMalloc(&work_b_, sizeof(float2) * work_));
        BCK(cudaMalloc(&kspec_, sizeof(KSpec<float>) * kspec_n_));
        BCK(cudaMalloc(&tw_, sizeof(float2) * tw_n_));
    }
    BCK(cudaMemcpyAsync(jobs_, hjobs_.data(), sizeof(BatchJobDev) * J_, cudaMemcpyHostToDevice, st_));
    BCK(cudaMemcpyAsync(fjobs_, hf.data(), sizeof(FftBatchJob) * J_, cudaMemcpyHostToDevice, st_));
    return upload_maps();
}

// Block maps of the five launch kinds: job of each block, first block and count per job.
int BatchPipeline::upload_maps() {
    std::vector<int> host;
    auto build = [&](auto blocks_of, size_t &job_at, size_t &first_at, size_t &count_at) {
        std::vector<int> first(J_), count(J_);
        int total = 0;
        for (int j = 0; j < J_; ++j) {
            first[j] = total;
            count[j] = blocks_of(j);
            total += count[j];
        }
        job_at = host.size();
        for (int j = 0; j < J_; ++j)
            for (int b = 0; b < count[j]; ++b) host.push_back(j);
        first_at = host.size();
        host.insert(host.end(), first.begin(), first.end());
        count_at = host.size();
        host.insert(host.end(), count.begin(), count.end());
        return total;
    };
    size_t pj, pf, pc, aj, af, ac, kj, kf, kc, cj, cf, cc, rj, rf, rc;
    n_pp_ = build([&](int j) { return pp_blocks(n_[j]); }, pj, pf, pc);
    n_at_ = build([&](int j) { return at_blocks(n_[j]); }, aj, af, ac);
    n_krow_ = build([&](int j) { return nb_cap_[j] * gp_.nterms; }, kj, kf, kc);
    n_cols_ = build([&](int j) { return hjobs_[j].L_cap / 2 + 1; }, cj, cf, cc);
    n_rows_ = build([&](int j) { return nb_cap_[j] * gp_.nterms; }, rj, rf, rc);
    if (host.size() > maps_len_) {
        cudaFree(maps_);
        maps_len_ = host.size() + host.size() / 2;
        BCK(cudaMalloc(&maps_, sizeof(int) * maps_len_));
    }
    BCK(cudaMemcpyAsync(maps_, host.data(), sizeof(int) * host.size(), cudaMemcpyHostToDevice, st_));
    BCK(cudaStreamSynchronize(st_));  // host is a local
    pp_ = BatchMap{maps_ + pj, maps_ + pf, maps_ + pc};
    at_ = BatchMap{maps_ + aj, maps_ + af, maps_ + ac};
    krow_ = FftBatchMap{maps_ + kj, maps_ + kf};
    cols_ = FftBatchMap{maps_ + cj, maps_ + cf};
    rows_ = FftBatchMap{maps_ + rj, maps_ + rf};
    return 0;
}

// The launches of len iterations: a snapshot of the state first (for a repeat after a grid
// overflow), then per iteration centre + min/max, geometry, twiddles, spread, the five FFT
// passes, gather and attraction + update; the jobs' statuses and geometries go to pinned
// memory at the end.
int BatchPipeline::record_chunk(const UpdateParams &p, int len, bool apply_first) {
    const size_t np = (size_t) Ntot_;
    BCK(cudaMemcpyAsync(snap_, Y_[cur_], sizeof(float) * np * 4, cudaMemcpyDeviceToDevice, st_));
    BCK(cudaMemcpyAsync(snap_ + np * 4, uY_, sizeof(float) * np * 2, cudaMemcpyDeviceToDevice, st_));
    BCK(cudaMemcpyAsync(snap_ + np * 6, gains_, sizeof(float) * np * 2, cudaMemcpyDeviceToDevice, st_));
    BCK(cudaMemsetAsync(status_, 0, sizeof(int) * J_, st_));
    int c = cur_;
    for (int k = 0; k < len; ++k) {
        BCK(launch_batch_center(Y_[c], 2, pp_, n_pp_, jobs_, rs_, (k > 0 || apply_first) ? 1 : 0, st_));
        BCK(launch_batch_geometry(rs_, jobs_, J_, 2, gp_.nterms, gp_.intervals_per_integer, gp_.min_num_intervals,
                                  dg_, status_, st_));
        BCK(twiddles_batch<float>(fjobs_, J_, tw_, st_));
        BCK(cudaMemsetAsync(grid_in_, 0, sizeof(Cell4<float>) * cells_used_, st_));
        BCK(launch_batch_spread(Y_[c], 2, pp_, n_pp_, jobs_, dg_, grid_in_, st_));
        BCK(conv2d_launch_batch<float>(grid_in_, grid_out_, fjobs_, krow_, n_krow_, cols_, n_cols_, rows_, n_rows_,
                                       L_max_, tw_, work_a_, work_b_, kspec_, 1.0, KERNEL_DF1, st_));
        BCK(launch_batch_gather(Y_[c], 2, pp_, n_pp_, jobs_, dg_, grid_out_, rep_, rs_, yh_, st_));
        BCK(launch_batch_attr(row_, col_, val_, Y_[c], Y_[1 - c], uY_, gains_, rep_, 2, at_, n_at_, jobs_, rs_, p,
                              yh_, st_));
        c = 1 - c;
    }
    BCK(cudaMemcpyAsync(h_status_, status_, sizeof(int) * J_, cudaMemcpyDeviceToHost, st_));
    BCK(cudaMemcpyAsync(h_dg_, dg_, sizeof(DevGeom) * J_, cudaMemcpyDeviceToHost, st_));
    return 0;
}

int BatchPipeline::launch_chunk(const UpdateParams &p, int len, bool apply_first, bool grow) {
    int rc = plan(grow);
    if (rc) return rc;
    // the graph depends on the parameters, the capacities (buffers, maps) and the buffers
    std::vector<unsigned long long> key = {(unsigned long long) len, (unsigned long long) apply_first,
                                           (unsigned long long) cur_};
    auto add_d = [&](double v) {
        unsigned long long u;
        std::memcpy(&u, &v, sizeof u);
        key.push_back(u);
    };
    add_d(p.exag);
    add_d(p.momentum);
    add_d(p.max_step_norm);
    key.push_back((unsigned long long) p.use_gains);
    key.push_back((unsigned long long) (uintptr_t) grid_in_);
    key.push_back((unsigned long long) (uintptr_t) maps_);
    for (int j = 0; j < J_; ++j) key.push_back((unsigned long long) nb_cap_[j]);
    if (!gexec_ || key != gkey_) {
        cudaGraph_t g = nullptr;
        BCK(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
        rc = record_chunk(p, len, apply_first);
        cudaError_t e = cudaStreamEndCapture(st_, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        BCK(e);
        ++captures_;
        bool updated = false;
        if (gexec_ && gexec_len_ == len) {
            cudaGraphExecUpdateResultInfo info;
            if (cudaGraphExecUpdate(gexec_, g, &info) == cudaSuccess) {
                updated = true;
                ++updates_;
            } else {
                cudaGetLastError();
            }
        }
        if (!updated) {
            if (gexec_) cudaGraphExecDestroy(gexec_);
            gexec_ = nullptr;
            cudaError_t ie = cudaGraphInstantiate(&gexec_, g, 0);
            if (ie != cudaSuccess) {
                cudaGraphDestroy(g);
                BCK(ie);
            }
            gexec_len_ = len;
        }
        cudaGraphDestroy(g);
        gkey_ = key;
    }
    BCK(cudaGraphLaunch(gexec_, st_));
    ++graph_launches_;
    launches_ += (unsigned long long) len * 12;
    return 0;
}

int BatchPipeline::kl_all(double exag, std::vector<double> &out) {
    BCK(launch_batch_kl(row_, col_, val_, Y_[cur_], 2, pp_, n_pp_, jobs_, exag, rs_, st_));
    out.assign(J_, 0.0);
    // the per-job scalars are consecutive (mnmx[2], z, mean[2], kl: stride 6 doubles)
    std::vector<double> sc(6 * (size_t) J_);
    BCK(cudaMemcpyAsync(sc.data(), hrs_[0].mnmx, sizeof(double) * sc.size(), cudaMemcpyDeviceToHost, st_));
    BCK(cudaStreamSynchronize(st_));
    for (int j = 0; j < J_; ++j) out[j] = sc[6 * (size_t) j + 5];
    launches_ += 1;
    return 0;
}

int BatchPipeline::run_schedule(const Schedule &s, double *const *costs, double *stats) {
    const auto t0 = std::chrono::steady_clock::now();
    double mult = s.early_exag_coeff, momentum = s.momentum;
    auto params = [&](int it) {
        UpdateParams p{};
        p.mode = 1;
        p.exag = mult;
        p.momentum = momentum;
        p.learning_rate = 0.0;  // per job (BatchJobDev::lr)
        p.df = 1.0;
        if (s.no_momentum_during_exag) {
            p.use_gains = (it > s.stop_lying_iter) ? 1 : 0;
            p.max_step_norm = -1.0;
        } else {
            p.use_gains = 1;
            p.max_step_norm = s.max_step_norm;
        }
        return p;
    };
    auto kl_due = [&](int it) { return (it + 1) % 50 == 0 || it == s.max_iter - 1; };
    int it = 0;
    std::vector<double> kl;
    while (it < s.max_iter) {
        int end = it + 1;
        while (end < s.max_iter && end - it < kMaxChunk &&
               !(kl_due(end - 1) || end - 1 == s.stop_lying_iter || end - 1 == s.start_late_exag_iter ||
                 end - 1 == s.mom_switch_iter))
            ++end;
        const int len = end - it;
        const UpdateParams p = params(it);
        bool grow = false;
        while (true) {
            int rc = launch_chunk(p, len, mean_pending_, grow);
            if (rc) return rc;
            BCK(cudaStreamSynchronize(st_));
            int worst = 0;
            for (int j = 0; j < J_; ++j) worst |= h_status_[j];
            if (worst & 2) {
                err_ = "embedding coordinates are not finite";
                return -11;
            }
            for (int j = 0; j < J_; ++j) nb_last_[j] = h_dg_[j].g.nb;
            if (!(worst & 1)) break;
            // a job outgrew its grid inside the chunk: back to the snapshot, larger grids
            const size_t np = (size_t) Ntot_;
            BCK(cudaMemcpyAsync(Y_[cur_], snap_, sizeof(float) * np * 4, cudaMemcpyDeviceToDevice, st_));
            BCK(cudaMemcpyAsync(uY_, snap_ + np * 4, sizeof(float) * np * 2, cudaMemcpyDeviceToDevice, st_));
            BCK(cudaMemcpyAsync(gains_, snap_ + np * 6, sizeof(float) * np * 2, cudaMemcpyDeviceToDevice, st_));
            // the means pending at the chunk's start
            for (int j = 0; j < J_; ++j)
                BCK(cudaMemcpyAsync(hrs_[j].mean, snap_mean_ + 2 * j, sizeof(double) * 2, cudaMemcpyDeviceToDevice,
                                    st_));
            ++redos_;
            grow = true;
        }
        if (len % 2) cur_ = 1 - cur_;
        mean_pending_ = true;
        // the means of this chunk's end: the start of the next chunk's snapshot
        for (int j = 0; j < J_; ++j)
            BCK(cudaMemcpyAsync(snap_mean_ + 2 * j, hrs_[j].mean, sizeof(double) * 2, cudaMemcpyDeviceToDevice, st_));
        for (int k = it; k < end; ++k) {
            if (k == s.stop_lying_iter) mult /= s.early_exag_coeff;
            if (k == s.start_late_exag_iter) mult *= s.late_exag_coeff;
            if (k == s.mom_switch_iter) momentum = s.final_momentum;
            if (kl_due(k) && costs) {
                int rc = kl_all(mult, kl);
                if (rc) return rc;
                for (int j = 0; j < J_; ++j) {
                    double C = kl[j];
                    if (k < s.stop_lying_iter && s.stop_lying_iter != -1)
                        C = C / s.early_exag_coeff - std::log(s.early_exag_coeff);
                    if (k >= s.start_late_exag_iter && s.start_late_exag_iter != -1)
                        C = C / s.late_exag_coeff - std::log(s.late_exag_coeff);
                    if (costs[j]) costs[j][k] = C;
                }
            }
        }
        it = end;
    }
    BCK(cudaStreamSynchronize(st_));
    if (stats) {
        stats[0] = (double) graph_launches_;
        stats[1] = (double) captures_;
        stats[2] = (double) updates_;
        stats[3] = (double) redos_;
        stats[4] = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return 0;
}

int BatchPipeline::get_Y(int j, double *Y) {
    if (mean_pending_) {
        BCK(launch_batch_center(Y_[cur_], 2, pp_, n_pp_, jobs_, rs_, 1, st_));
        mean_pending_ = false;
    }
    double *tmp = nullptr;
    BCK(cudaMalloc(&tmp, sizeof(double) * (size_t) n_[j] * 2));
    cudaError_t e = launch_y_to_double<float>(Y_[cur_] + (size_t) p0_[j] * 4, tmp, n_[j], 2, st_);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(Y, tmp, sizeof(double) * (size_t) n_[j] * 2, cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    cudaFree(tmp);
    BCK(e);
    return 0;
}

}  // namespace fitsne
