// Host driver of the per-iteration kernels (see embedding.cuh).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "embedding.cuh"
#include "reorder.cuh"
#include "sort.cuh"

namespace fitsne {

GridGeom make_grid_geom(double mn, double mx, int D, const GridParams &gp) {
    GridGeom g;
    std::memset(&g, 0, sizeof(g));
    int nb = static_cast<int>(std::fmax((double) gp.min_num_intervals, (mx - mn) / gp.intervals_per_integer));
    if (D == 2) {
        // FFT-friendly box counts of computeFftGradient (tsne.cpp:1068-1077)
        static const int allowed[20] = {25, 36, 50, 55, 60, 65, 70, 75, 80, 85,
                                        90, 96, 100, 110, 120, 130, 140, 150, 175, 200};
        if (nb < allowed[19]) {
            int i = 0;
            while (allowed[i] < nb) ++i;
            nb = allowed[i];
        }
    }
    if (nb < 1) nb = 1;
    g.nb = nb;
    g.nterms = gp.nterms;
    g.M = nb * gp.nterms;
    const double bw = (mx - mn) / (double) nb;
    // n_body_fft_2d / nbodyfft read the lower corner and the width back from the box
    // bounds array: lower[0] = 0*bw + mn, width = (1*bw + mn) - (0*bw + mn)
    g.mn = 0.0 * bw + mn;
    g.bw = (1.0 * bw + mn) - g.mn;
    g.hk = bw / (double) gp.nterms;
    const double h = 1.0 / (double) gp.nterms;
    double s[kMaxInterp];
    s[0] = h / 2.0;
    for (int i = 1; i < gp.nterms && i < kMaxInterp; ++i) s[i] = s[i - 1] + h;
    for (int i = 0; i < gp.nterms && i < kMaxInterp; ++i) {
        double den = 1.0;
        for (int j = 0; j < gp.nterms; ++j)
            if (i != j) den *= s[i] - s[j];
        g.s64[i] = s[i];
        g.inv_den64[i] = 1.0 / den;
        g.s32[i] = (float) s[i];
        g.inv_den32[i] = (float) (1.0 / den);
    }
    return g;
}

template <typename T>
Embedding<T>::Embedding() {
    const char *e = std::getenv("FITSNE_REORDER");
    if (e && std::atoi(e) == 0) reorder_enabled_ = false;
}

template <typename T>
Embedding<T>::~Embedding() {
    cudaFree(row_);
    cudaFree(col_);
    cudaFree(val_);
    cudaFree(Y_[0]);
    cudaFree(Y_[1]);
    cudaFree(uY_);
    cudaFree(gains_);
    cudaFree(rep_);
    cudaFree(dC_);
    cudaFree(grid_in_);
    cudaFree(grid_out_);
    cudaFree(work_a_);
    cudaFree(work_b_);
    cudaFree(kspec_);
    for (auto &kv : tw_) cudaFree(kv.second);
    for (void *p : {(void *) perm_, (void *) iperm_, (void *) rkeys_, (void *) rids_, (void *) rkeys2_,
                    (void *) rids2_, (void *) rlen_, (void *) row2_, (void *) col2_, (void *) val2_, rscratch_})
        cudaFree(p);
    cudaFree(red_mem_);
    cudaFree(red_cnt_);
    if (h_pin_) cudaFreeHost(h_pin_);
    for (auto &b : evs_)
        for (auto &e : b)
            if (e) cudaEventDestroy(e);
    for (auto &e : evr_)
        if (e) cudaEventDestroy(e);
}

template <typename T>
int Embedding<T>::fail(const char *what, cudaError_t e) {
    err_ = std::string(what) + ": " + cudaGetErrorString(e);
    return -10;
}

#define FITSNE_CK(call)                                  \
    do {                                                 \
        cudaError_t e__ = (call);                        \
        if (e__ != cudaSuccess) return fail(#call, e__); \
    } while (0)

template <typename T>
int Embedding<T>::alloc_common(int N, int D, size_t nnz) {
    N_ = N;
    D_ = D;
    nnz_ = nnz;
    const int W = y_width<T>(D);
    FITSNE_CK(cudaMalloc(&row_, sizeof(uint32_t) * (N + 1)));
    FITSNE_CK(cudaMalloc(&col_, sizeof(uint32_t) * (nnz ? nnz : 1)));
    FITSNE_CK(cudaMalloc(&val_, sizeof(T) * (nnz ? nnz : 1)));
    FITSNE_CK(cudaMalloc(&Y_[0], sizeof(T) * (size_t) N * W));
    FITSNE_CK(cudaMalloc(&Y_[1], sizeof(T) * (size_t) N * W));
    FITSNE_CK(cudaMalloc(&uY_, sizeof(T) * (size_t) N * D));
    FITSNE_CK(cudaMalloc(&gains_, sizeof(T) * (size_t) N * D));
    FITSNE_CK(cudaMalloc(&rep_, sizeof(T) * (size_t) N * D));
    FITSNE_CK(cudaMalloc(&dC_, sizeof(T) * (size_t) N * D));
    FITSNE_CK(cudaMemsetAsync(uY_, 0, sizeof(T) * (size_t) N * D, st_));
    // gains start at 1 (tsne.cpp:149-150)
    {
        std::vector<T> ones((size_t) N * D, T(1));
        FITSNE_CK(cudaMemcpyAsync(gains_, ones.data(), sizeof(T) * ones.size(), cudaMemcpyHostToDevice, st_));
        FITSNE_CK(cudaStreamSynchronize(st_));
    }
    FITSNE_CK(cudaMalloc(&red_mem_, sizeof(double) * (kMaxRedBlocks * 4 + 16)));
    FITSNE_CK(cudaMalloc(&red_cnt_, sizeof(unsigned int) * 8));
    FITSNE_CK(cudaMemsetAsync(red_cnt_, 0, sizeof(unsigned int) * 8, st_));
    FITSNE_CK(cudaMemsetAsync(red_mem_, 0, sizeof(double) * (kMaxRedBlocks * 4 + 16), st_));
    red_.part = red_mem_;
    red_.count = red_cnt_;
    red_.mnmx = red_mem_ + kMaxRedBlocks * 4;
    red_.z = red_.mnmx + 2;
    red_.mean = red_.z + 1;
    red_.kl = red_.mean + 2;
    FITSNE_CK(cudaMallocHost(&h_pin_, sizeof(double) * 8));
    for (auto &b : evs_)
        for (auto &e : b) FITSNE_CK(cudaEventCreate(&e));
    for (auto &e : evr_) FITSNE_CK(cudaEventCreate(&e));
    return 0;
}

template <typename T>
int Embedding<T>::init_host(int N, int D, const uint32_t *row, const uint32_t *col, const double *val,
                            const double *Y0, const GridParams &gp, cudaStream_t st) {
    st_ = st;
    gp_ = gp;
    const size_t nnz = row[N];
    int rc = alloc_common(N, D, nnz);
    if (rc) return rc;
    FITSNE_CK(cudaMemcpyAsync(row_, row, sizeof(uint32_t) * (N + 1), cudaMemcpyHostToDevice, st_));
    if (nnz) FITSNE_CK(cudaMemcpyAsync(col_, col, sizeof(uint32_t) * nnz, cudaMemcpyHostToDevice, st_));
    double *tmp = nullptr;
    const size_t tmpn = std::max(nnz, (size_t) N * D);
    FITSNE_CK(cudaMalloc(&tmp, sizeof(double) * (tmpn ? tmpn : 1)));
    if (nnz) {
        FITSNE_CK(cudaMemcpyAsync(tmp, val, sizeof(double) * nnz, cudaMemcpyHostToDevice, st_));
        FITSNE_CK(launch_cast_from_double<T>(tmp, val_, nnz, st_));
    }
    FITSNE_CK(cudaMemcpyAsync(tmp + 0, Y0, sizeof(double) * (size_t) N * D, cudaMemcpyHostToDevice, st_));
    FITSNE_CK(launch_y_from_double<T>(tmp, Y_[0], N, D, st_));
    FITSNE_CK(cudaStreamSynchronize(st_));
    cudaFree(tmp);
    cur_ = 0;
    mean_pending_ = false;
    return 0;
}

template <typename T>
int Embedding<T>::init_device(int N, int D, const uint32_t *d_row, const uint32_t *d_col, const double *d_val,
                              size_t nnz, const double *Y0, const GridParams &gp, cudaStream_t st) {
    st_ = st;
    gp_ = gp;
    int rc = alloc_common(N, D, nnz);
    if (rc) return rc;
    FITSNE_CK(cudaMemcpyAsync(row_, d_row, sizeof(uint32_t) * (N + 1), cudaMemcpyDeviceToDevice, st_));
    if (nnz) {
        FITSNE_CK(cudaMemcpyAsync(col_, d_col, sizeof(uint32_t) * nnz, cudaMemcpyDeviceToDevice, st_));
        FITSNE_CK(launch_cast_from_double<T>(d_val, val_, nnz, st_));
    }
    double *tmp = nullptr;
    FITSNE_CK(cudaMalloc(&tmp, sizeof(double) * (size_t) N * D));
    FITSNE_CK(cudaMemcpyAsync(tmp, Y0, sizeof(double) * (size_t) N * D, cudaMemcpyHostToDevice, st_));
    FITSNE_CK(launch_y_from_double<T>(tmp, Y_[0], N, D, st_));
    FITSNE_CK(cudaStreamSynchronize(st_));
    cudaFree(tmp);
    cur_ = 0;
    mean_pending_ = false;
    return 0;
}

template <typename T>
int Embedding<T>::prepare_grid() {
    FITSNE_CK(cudaMemcpyAsync(h_pin_, red_.mnmx, sizeof(double) * 2, cudaMemcpyDeviceToHost, st_));
    FITSNE_CK(cudaStreamSynchronize(st_));
    const double mn = h_pin_[0], mx = h_pin_[1];
    if (!std::isfinite(mn) || !std::isfinite(mx)) {
        err_ = "embedding coordinates are not finite";
        return -11;
    }
    geom_ = make_grid_geom(mn, mx, D_, gp_);
    if (gp_.nterms < 1 || gp_.nterms > kMaxInterp) {
        err_ = "n_interpolation_points must be in [1, 8]";
        return -12;
    }
    const int M = geom_.M;
    const int L = smooth_even_at_least(2 * M);
    if (L > max_fft_len<T>()) {
        err_ = "interpolation grid too large: " + std::to_string(L) + " > " + std::to_string(max_fft_len<T>());
        return -13;
    }
    if (L != L_) {
        if (!make_fft_plan(L, &plan_)) {
            err_ = "bad FFT length";
            return -14;
        }
        L_ = L;
    }
    auto it = tw_.find(L);
    if (it == tw_.end()) {
        std::vector<C> h(L);
        const double pi = 3.14159265358979323846264338327950288;
        for (int j = 0; j < L; ++j) {
            const double a = 2.0 * pi * (double) j / (double) L;
            h[j] = mkc((T) std::cos(a), (T) -std::sin(a));
        }
        C *d = nullptr;
        FITSNE_CK(cudaMalloc(&d, sizeof(C) * L));
        FITSNE_CK(cudaMemcpyAsync(d, h.data(), sizeof(C) * L, cudaMemcpyHostToDevice, st_));
        FITSNE_CK(cudaStreamSynchronize(st_));
        tw_[L] = d;
    }
    const size_t H = L / 2 + 1;
    const size_t gridn = (D_ == 2) ? (size_t) M * M : (size_t) M;
    if (gridn > grid_cap_) {
        cudaFree(grid_in_);
        cudaFree(grid_out_);
        const size_t cap = gridn + gridn / 4;
        FITSNE_CK(cudaMalloc(&grid_in_, sizeof(Cell4<T>) * cap));
        FITSNE_CK(cudaMalloc(&grid_out_, sizeof(Cell4<T>) * cap));
        grid_cap_ = cap;
    }
    const size_t wa = (D_ == 2) ? 4 * (size_t) L * H : 6 * (size_t) L;
    const size_t wb = (D_ == 2) ? 4 * (size_t) M * H : 1;
    const size_t ks = (D_ == 2) ? (size_t) L * H : 1;
    if (wa > wa_cap_) {
        cudaFree(work_a_);
        FITSNE_CK(cudaMalloc(&work_a_, sizeof(C) * (wa + wa / 4)));
        wa_cap_ = wa + wa / 4;
    }
    if (wb > wb_cap_) {
        cudaFree(work_b_);
        FITSNE_CK(cudaMalloc(&work_b_, sizeof(C) * (wb + wb / 4)));
        wb_cap_ = wb + wb / 4;
    }
    if (ks > ks_cap_) {
        cudaFree(kspec_);
        FITSNE_CK(cudaMalloc(&kspec_, sizeof(KSpec<T>) * (ks + ks / 4)));
        ks_cap_ = ks + ks / 4;
    }
    return 0;
}

template <typename T>
int Embedding<T>::repulsion() {
    const int M = geom_.M;
    const size_t gridn = (D_ == 2) ? (size_t) M * M : (size_t) M;
    const int mode = (gp_.df == 1.0) ? KERNEL_DF1 : KERNEL_VARDF;
    FITSNE_CK(cudaMemsetAsync(grid_in_, 0, sizeof(Cell4<T>) * gridn, st_));
    FITSNE_CK(launch_spread<T>(Y_[cur_], N_, D_, geom_, grid_in_, st_));
    if (timing_) FITSNE_CK(cudaEventRecord(evs_[tb_][2], st_));
    if (D_ == 2)
        FITSNE_CK(conv2d_launch<T>(grid_in_, grid_out_, M, plan_, tw_[L_], work_a_, work_b_, kspec_, geom_.hk,
                                   gp_.df, mode, st_));
    else
        FITSNE_CK(conv1d_launch<T>(grid_in_, grid_out_, M, plan_, tw_[L_], work_a_, geom_.hk, gp_.df, mode, st_));
    if (timing_) FITSNE_CK(cudaEventRecord(evs_[tb_][3], st_));
    FITSNE_CK(launch_gather<T>(Y_[cur_], N_, D_, geom_, grid_out_, mode, rep_, red_, st_));
    if (timing_) FITSNE_CK(cudaEventRecord(evs_[tb_][4], st_));
    launches_ += 1 + (D_ == 2 ? 5 : 2) + 1;  // spread, convolution passes, gather
    return 0;
}

template <typename T>
int Embedding<T>::gradient(double *dC_host, double *sum_Q) {
    FITSNE_CK(launch_center_minmax<T>(Y_[cur_], N_, D_, mean_pending_ ? 1 : 0, excl_, red_, st_));
    mean_pending_ = false;
    int rc = prepare_grid();
    if (rc) return rc;
    tpend_ = false;
    rc = repulsion();
    if (rc) return rc;
    UpdateParams p{};
    p.mode = 0;
    p.exag = 1.0;
    p.df = gp_.df;
    FITSNE_CK(launch_attr_update<T>(row_, col_, val_, Y_[cur_], nullptr, nullptr, nullptr, dC_, rep_, N_, D_, p,
                                    red_, st_));
    launches_ += 2;
    std::vector<T> tmp((size_t) N_ * D_);
    FITSNE_CK(cudaMemcpyAsync(tmp.data(), dC_, sizeof(T) * tmp.size(), cudaMemcpyDeviceToHost, st_));
    FITSNE_CK(cudaMemcpyAsync(h_pin_ + 2, red_.z, sizeof(double), cudaMemcpyDeviceToHost, st_));
    FITSNE_CK(cudaStreamSynchronize(st_));
    if (reordered_) {
        std::vector<uint32_t> perm;
        rc = perm_to_host(perm);
        if (rc) return rc;
        for (size_t k = 0; k < (size_t) N_; ++k)
            for (int d = 0; d < D_; ++d) dC_host[(size_t) perm[k] * D_ + d] = (double) tmp[k * D_ + d];
    } else {
        for (size_t k = 0; k < tmp.size(); ++k) dC_host[k] = (double) tmp[k];
    }
    if (sum_Q) *sum_Q = h_pin_[2];
    return 0;
}

template <typename T>
int Embedding<T>::perm_to_host(std::vector<uint32_t> &out) {
    out.resize(N_);
    FITSNE_CK(cudaMemcpyAsync(out.data(), perm_, sizeof(uint32_t) * N_, cudaMemcpyDeviceToHost, st_));
    FITSNE_CK(cudaStreamSynchronize(st_));
    return 0;
}

// Renumbers the points along a Morton curve of the current embedding (reorder.cuh).
template <typename T>
int Embedding<T>::reorder() {
    const int W = y_width<T>(D_);
    if (!perm_) {
        FITSNE_CK(cudaMalloc(&perm_, sizeof(uint32_t) * N_));
        FITSNE_CK(cudaMalloc(&iperm_, sizeof(uint32_t) * N_));
        FITSNE_CK(cudaMalloc(&rkeys_, sizeof(uint32_t) * N_));
        FITSNE_CK(cudaMalloc(&rids_, sizeof(uint32_t) * N_));
        FITSNE_CK(cudaMalloc(&rkeys2_, sizeof(uint32_t) * N_));
        FITSNE_CK(cudaMalloc(&rids2_, sizeof(uint32_t) * N_));
        FITSNE_CK(cudaMalloc(&rlen_, sizeof(uint32_t) * (N_ + 1)));
        FITSNE_CK(cudaMalloc(&row2_, sizeof(uint32_t) * (N_ + 1)));
        FITSNE_CK(cudaMalloc(&col2_, sizeof(uint32_t) * (nnz_ ? nnz_ : 1)));
        FITSNE_CK(cudaMalloc(&val2_, sizeof(T) * (nnz_ ? nnz_ : 1)));
        const size_t scr = std::max(radix_sort_scratch_bytes(N_), scan_scratch_bytes((size_t) N_ + 1));
        FITSNE_CK(cudaMalloc(&rscratch_, scr));
        FITSNE_CK(launch_iota(perm_, N_, st_));
    }
    // current bounds (also applies any pending mean shift)
    FITSNE_CK(launch_center_minmax<T>(Y_[cur_], N_, D_, mean_pending_ ? 1 : 0, excl_, red_, st_));
    mean_pending_ = false;
    FITSNE_CK(cudaMemcpyAsync(h_pin_, red_.mnmx, sizeof(double) * 2, cudaMemcpyDeviceToHost, st_));
    FITSNE_CK(cudaStreamSynchronize(st_));
    const double lo = h_pin_[0], hi = h_pin_[1];
    if (!std::isfinite(lo) || !std::isfinite(hi)) {
        err_ = "embedding coordinates are not finite";
        return -11;
    }
    FITSNE_CK(launch_morton_keys<T>(Y_[cur_], N_, D_, W, lo, hi, rkeys_, rids_, st_));
    FITSNE_CK(radix_sort_pairs(rkeys_, rids_, rkeys2_, rids2_, (size_t) N_, 32, rscratch_, st_));
    const uint32_t *order = rids_;
    FITSNE_CK(launch_invert(order, rkeys2_, N_, st_));  // rkeys2_ = inverse of order
    // point arrays
    FITSNE_CK(launch_gather_rows<T>(Y_[cur_], Y_[1 - cur_], order, N_, W, st_));
    cur_ = 1 - cur_;
    FITSNE_CK(launch_gather_rows<T>(uY_, rep_, order, N_, D_, st_));
    std::swap(uY_, rep_);
    FITSNE_CK(launch_gather_rows<T>(gains_, dC_, order, N_, D_, st_));
    std::swap(gains_, dC_);
    // P: rows in the new order, columns renamed
    FITSNE_CK(launch_perm_lengths(row_, order, N_, rlen_, st_));
    FITSNE_CK(exclusive_scan_u32(rlen_, row2_, (size_t) N_, rscratch_, st_));
    FITSNE_CK(launch_perm_csr<T>(row_, col_, val_, order, rkeys2_, row2_, N_, col2_, val2_, st_));
    std::swap(row_, row2_);
    std::swap(col_, col2_);
    std::swap(val_, val2_);
    // caller index of each internal point, and its inverse
    FITSNE_CK(launch_compose(perm_, order, rids2_, N_, st_));
    std::swap(perm_, rids2_);
    FITSNE_CK(launch_invert(perm_, iperm_, N_, st_));
    unsigned int e0 = 0;
    FITSNE_CK(cudaMemcpyAsync(&e0, iperm_, sizeof(uint32_t), cudaMemcpyDeviceToHost, st_));
    FITSNE_CK(cudaStreamSynchronize(st_));
    excl_ = (int) e0;
    reordered_ = true;
    return 0;
}

template <typename T>
int Embedding<T>::step(const UpdateParams &p, bool) {
    if (timing_) FITSNE_CK(cudaEventRecord(evs_[tb_][0], st_));
    FITSNE_CK(launch_center_minmax<T>(Y_[cur_], N_, D_, mean_pending_ ? 1 : 0, excl_, red_, st_));
    mean_pending_ = false;
    if (timing_) FITSNE_CK(cudaEventRecord(evs_[tb_][1], st_));
    int rc = prepare_grid();
    if (rc) return rc;
    // the stream is idle here: the previous iteration's events are complete
    if (timing_ && tpend_) {
        read_stage_events(tb_ ^ 1);
        tpend_ = false;
    }
    rc = repulsion();
    if (rc) return rc;
    FITSNE_CK(launch_attr_update<T>(row_, col_, val_, Y_[cur_], Y_[1 - cur_], uY_, gains_, nullptr, rep_, N_, D_, p,
                                    red_, st_));
    launches_ += 2;  // centre + attraction
    if (timing_) {
        FITSNE_CK(cudaEventRecord(evs_[tb_][5], st_));
        tpend_ = true;
        tb_ ^= 1;
    }
    cur_ = 1 - cur_;
    mean_pending_ = true;
    return 0;
}

template <typename T>
void Embedding<T>::read_stage_events(int b) {
    float t[6];
    cudaEventElapsedTime(&t[0], evs_[b][0], evs_[b][1]);
    cudaEventElapsedTime(&t[1], evs_[b][1], evs_[b][2]);
    cudaEventElapsedTime(&t[2], evs_[b][2], evs_[b][3]);
    cudaEventElapsedTime(&t[3], evs_[b][3], evs_[b][4]);
    cudaEventElapsedTime(&t[4], evs_[b][4], evs_[b][5]);
    cudaEventElapsedTime(&t[5], evs_[b][0], evs_[b][5]);
    for (int k = 0; k < 6; ++k) tacc_[k] += t[k];
    ++tacc_n_;
}

template <typename T>
int Embedding<T>::kl(double exag, double *out) {
    FITSNE_CK(launch_kl<T>(row_, col_, val_, Y_[cur_], N_, D_, exag, gp_.df, red_, st_));
    launches_ += 1;
    FITSNE_CK(cudaMemcpyAsync(h_pin_ + 3, red_.kl, sizeof(double), cudaMemcpyDeviceToHost, st_));
    FITSNE_CK(cudaStreamSynchronize(st_));
    *out = h_pin_[3];
    return 0;
}

template <typename T>
int Embedding<T>::kl_with_z(double exag, double z, double *out) {
    h_pin_[2] = z;
    FITSNE_CK(cudaMemcpyAsync(red_.z, h_pin_ + 2, sizeof(double), cudaMemcpyHostToDevice, st_));
    return kl(exag, out);
}

template <typename T>
int Embedding<T>::get_Y(double *Y_host) {
    if (mean_pending_) {
        FITSNE_CK(launch_center_minmax<T>(Y_[cur_], N_, D_, 1, excl_, red_, st_));
        mean_pending_ = false;
    }
    double *tmp = nullptr;
    FITSNE_CK(cudaMalloc(&tmp, sizeof(double) * (size_t) N_ * D_ * (reordered_ ? 2 : 1)));
    FITSNE_CK(launch_y_to_double<T>(Y_[cur_], tmp, N_, D_, st_));
    double *out = tmp;
    if (reordered_) {
        out = tmp + (size_t) N_ * D_;
        FITSNE_CK(launch_scatter_rows<double>(tmp, out, perm_, N_, D_, st_));
    }
    FITSNE_CK(cudaMemcpyAsync(Y_host, out, sizeof(double) * (size_t) N_ * D_, cudaMemcpyDeviceToHost, st_));
    FITSNE_CK(cudaStreamSynchronize(st_));
    cudaFree(tmp);
    return 0;
}

template <typename T>
int Embedding<T>::run_schedule(const Schedule &s, int it0, int it1, double *costs, bool verbose) {
    // replay the switches of tsne.cpp:533-544 for the iterations before it0
    double mult = s.early_exag_coeff;
    double momentum = s.momentum;
    for (int it = 0; it < it0; ++it) {
        if (it == s.stop_lying_iter) mult /= s.early_exag_coeff;
        if (it == s.start_late_exag_iter) mult *= s.late_exag_coeff;
        if (it == s.mom_switch_iter) momentum = s.final_momentum;
    }
    const unsigned long long l0 = launches_;
    tpend_ = false;
    tacc_n_ = 0;
    for (double &a : tacc_) a = 0.0;
    FITSNE_CK(cudaEventRecord(evr_[0], st_));
    for (int it = it0; it < it1; ++it) {
        UpdateParams p{};
        p.mode = 1;
        p.exag = mult;
        p.momentum = momentum;
        p.learning_rate = s.learning_rate;
        p.df = gp_.df;
        if (s.no_momentum_during_exag) {
            // tsne.cpp:479-490: gains/momentum only after the exaggeration, never clipped
            p.use_gains = (it > s.stop_lying_iter) ? 1 : 0;
            p.max_step_norm = -1.0;
        } else {
            p.use_gains = 1;
            p.max_step_norm = s.max_step_norm;
        }
        // renumber for locality a few times while the embedding takes shape
        if (reorder_enabled_ && N_ >= kReorderMinN &&
            (it == 50 || it == 150 || it == 300 || it == 600 || (!reordered_ && it == it0 && it0 > 50))) {
            int rr = reorder();
            if (rr) return rr;
        }
        int rc = step(p, it == 0);
        if (rc) return rc;
        if (it == s.stop_lying_iter) mult /= s.early_exag_coeff;
        if (it == s.start_late_exag_iter) mult *= s.late_exag_coeff;
        if (it == s.mom_switch_iter) momentum = s.final_momentum;
        if (costs && ((it + 1) % 50 == 0 || it == s.max_iter - 1)) {
            double C = 0.0;
            rc = kl(mult, &C);
            if (rc) return rc;
            if (it < s.stop_lying_iter && s.stop_lying_iter != -1)
                C = C / s.early_exag_coeff - std::log(s.early_exag_coeff);
            if (it >= s.start_late_exag_iter && s.start_late_exag_iter != -1)
                C = C / s.late_exag_coeff - std::log(s.late_exag_coeff);
            costs[it] = C;
            if (verbose) std::printf("Iteration %d, cost %f\n", it + 1, C);
        }
    }
    FITSNE_CK(cudaEventRecord(evr_[1], st_));
    FITSNE_CK(cudaEventSynchronize(evr_[1]));
    cudaEventElapsedTime(&times_.run_ms, evr_[0], evr_[1]);
    times_.launches = launches_ - l0;
    if (timing_ && tpend_) {
        read_stage_events(tb_ ^ 1);
        tpend_ = false;
    }
    if (tacc_n_ > 0) {
        // average per iteration over this call
        times_.center = (float) (tacc_[0] / tacc_n_);
        times_.spread = (float) (tacc_[1] / tacc_n_);
        times_.conv = (float) (tacc_[2] / tacc_n_);
        times_.gather = (float) (tacc_[3] / tacc_n_);
        times_.attract = (float) (tacc_[4] / tacc_n_);
        times_.total = (float) (tacc_[5] / tacc_n_);
    }
    return 0;
}

template class Embedding<float>;
template class Embedding<double>;

}  // namespace fitsne
