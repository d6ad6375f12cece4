// Host driver of the per-iteration kernels (see embedding.cuh).
#include <algorithm>
#include <chrono>
#include <climits>
#include <mutex>
#include <map>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "affinity.cuh"
#include "embedding.cuh"
#include "reorder.cuh"
#include "sort.cuh"

namespace fitsne {

GridGeom make_grid_geom(double mn, double mx, int D, const GridParams &gp) {
    return grid_geom(mn, mx, D, gp.nterms, gp.intervals_per_integer, gp.min_num_intervals, INT_MAX, nullptr);
}

template <typename T>
Embedding<T>::Embedding() {
    const char *e = std::getenv("FITSNE_REORDER");
    if (e && std::atoi(e) == 0) reorder_enabled_ = false;
    const char *g = std::getenv("FITSNE_GRAPH");
    if (g && std::atoi(g) == 0) graphs_ = false;
}

template <typename T>
Embedding<T>::~Embedding() {
    cudaFree(row_);
    cudaFree(col_);
    cudaFree(val_);
    cudaFree(Y_[0]);
    cudaFree(Y_[1]);
    cudaFree(yh_);
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
    cudaFree(urow_);
    cudaFree(trec_);
    cudaFree(tstart_);
    cudaFree(acc_);
    cudaFree(sorder_);
    if (h_pin_) cudaFreeHost(h_pin_);
    cudaFree(dgeom_);
    cudaFree(gstatus_);
    if (h_gstat_) cudaFreeHost(h_gstat_);
    cudaFree(tw_dev_);
    cudaFree(snap_);
    cudaFree(snap_mean_);
    for (auto &a : gslots_)
        for (auto &b : a)
            for (auto &s : b)
                if (s.exec) cudaGraphExecDestroy(s.exec);
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
    if (sizeof(T) == 4) {  // FP32 form: the neighbour positions the attraction gathers (k_gather writes them)
        FITSNE_CK(cudaMalloc(&yh_, sizeof(float) * (size_t) N * D));
        FITSNE_CK(cudaMemsetAsync(yh_, 0, sizeof(float) * (size_t) N * D, st_));
    }
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
    return check_symmetric();
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
    return check_symmetric();
}

// The tiled attraction needs P symmetric in pattern and values (symmetrizeMatrix's output
// is; a caller's P need not be): checked once by hashing the entries and their transposes on
// the device.  A renumbering keeps the symmetry.
template <typename T>
int Embedding<T>::check_symmetric() {
    sym_ok_ = false;
    tiles_ok_ = false;
    if (sizeof(T) != 4 || nnz_ == 0) return 0;
    const char *e = std::getenv("FITSNE_ATTR_SYM");
    if (e && std::atoi(e) == 0) return 0;
    unsigned long long *h = nullptr;
    FITSNE_CK(cudaMalloc(&h, 2 * sizeof(unsigned long long)));
    FITSNE_CK(launch_sym_hash(row_, col_, reinterpret_cast<const float *>(val_), N_, h, st_));
    unsigned long long hh[2] = {0, 1};
    FITSNE_CK(cudaMemcpyAsync(hh, h, sizeof hh, cudaMemcpyDeviceToHost, st_));
    FITSNE_CK(cudaStreamSynchronize(st_));
    cudaFree(h);
    if (hh[0] != hh[1]) return 0;
    sym_ok_ = true;
    return build_tiles();
}

// The tiled form pays a build (a radix sort of the upper entries) at set-up and after every
// renumbering; it is built only where it can win: up to kTilesMaxN points (measured: it wins
// at 50,000 points, ties at 200,000 and loses at 1,000,000), or when FITSNE_ATTR_SHAPE asks for
// it.
template <typename T>
bool Embedding<T>::tiles_wanted() const {
    if (!sym_ok_) return false;
    if (N_ <= kTilesMaxN) return true;
    const char *fixed = std::getenv("FITSNE_ATTR_SHAPE");
    return fixed && *fixed && std::atoi(fixed) == kAttrTilesShape;
}

// Records of the upper entries sorted by tile (A, B) of 4,096-point blocks, row order kept
// within a tile (stable radix sort on the tile key), and the tiles' first records.  Rebuilt
// after every renumbering: the tiles follow the point order.
template <typename T>
int Embedding<T>::build_tiles() {
    tiles_ok_ = false;
    if (!tiles_wanted()) return 0;
    const int nblk = tile_blocks(N_);
    const size_t nkeys = (size_t) nblk * nblk;
    if (nkeys >= (1ull << 30)) return 0;
    int key_bits = 1;
    while (((size_t) 1 << key_bits) < nkeys) ++key_bits;
    uint32_t *ulen = nullptr, *keys = nullptr, *ids = nullptr, *keys2 = nullptr, *ids2 = nullptr, *tcount = nullptr;
    uint2 *rec = nullptr;
    void *scr = nullptr;
    auto release = [&]() {
        cudaFree(ulen);
        cudaFree(keys);
        cudaFree(ids);
        cudaFree(keys2);
        cudaFree(ids2);
        cudaFree(tcount);
        cudaFree(rec);
        cudaFree(scr);
    };
    cudaError_t e = cudaSuccess;
    if (!urow_) e = cudaMalloc(&urow_, sizeof(uint32_t) * (N_ + 1));
    if (e == cudaSuccess && !acc_) {
        e = cudaMalloc(&acc_, sizeof(float) * (size_t) N_ * D_);
        if (e == cudaSuccess) e = cudaMemsetAsync(acc_, 0, sizeof(float) * (size_t) N_ * D_, st_);
    }
    // upper entries per row and their row offsets
    if (e == cudaSuccess) e = cudaMalloc(&ulen, sizeof(uint32_t) * (N_ + 1));
    if (e == cudaSuccess) e = cudaMalloc(&scr, std::max(scan_scratch_bytes((size_t) N_ + 1), scan_scratch_bytes(nkeys + 1)));
    if (e == cudaSuccess) e = launch_upper_count(row_, col_, N_, ulen, st_);
    if (e == cudaSuccess) e = exclusive_scan_u32(ulen, urow_, (size_t) N_, scr, st_);
    unsigned int total = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&total, urow_ + N_, sizeof(uint32_t), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    const size_t n = total;
    if (e == cudaSuccess && n > 0) {
        cudaFree(scr);
        scr = nullptr;
        const size_t scr_bytes = std::max(radix_sort_scratch_bytes(n), scan_scratch_bytes(nkeys + 1));
        for (auto pr : {std::make_pair((void **) &keys, n * 4), std::make_pair((void **) &ids, n * 4),
                        std::make_pair((void **) &keys2, n * 4), std::make_pair((void **) &ids2, n * 4),
                        std::make_pair((void **) &tcount, nkeys * 4), std::make_pair((void **) &rec, n * 8),
                        std::make_pair((void **) &scr, scr_bytes)})
            if (e == cudaSuccess) e = cudaMalloc(pr.first, pr.second);
        if (e == cudaSuccess && (!trec_ || n > unnz_)) {
            cudaFree(trec_);
            trec_ = nullptr;
            e = cudaMalloc(&trec_, sizeof(uint2) * n);
            unnz_ = n;
        }
        if (e == cudaSuccess) {
            cudaFree(tstart_);
            tstart_ = nullptr;
            e = cudaMalloc(&tstart_, sizeof(uint32_t) * (nkeys + 1));
        }
        if (e == cudaSuccess) e = cudaMemsetAsync(tcount, 0, nkeys * 4, st_);
        if (e == cudaSuccess)
            e = launch_tile_keys(row_, col_, reinterpret_cast<const float *>(val_), N_, urow_, keys, ids, rec, tcount,
                                 st_);
        if (e == cudaSuccess) e = exclusive_scan_u32(tcount, tstart_, nkeys, scr, st_);
        if (e == cudaSuccess) e = radix_sort_pairs(keys, ids, keys2, ids2, n, key_bits, scr, st_);
        if (e == cudaSuccess) e = launch_tile_gather(rec, ids, n, trec_, st_);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
        if (e == cudaSuccess && timing_requested()) {
            // how the edges spread over the tiles: the tiled form pays per tile (a block load
            // and an accumulator flush), so it gains where the tiles are dense
            std::vector<uint32_t> tc(nkeys);
            e = cudaMemcpy(tc.data(), tcount, nkeys * 4, cudaMemcpyDeviceToHost);
            size_t ne = 0, e4 = 0, e16 = 0, e64 = 0;
            for (uint32_t c : tc) {
                ne += c > 0;
                e4 += c >= 4096 ? c : 0;
                e16 += c >= 16384 ? c : 0;
                e64 += c >= 65536 ? c : 0;
            }
            std::fprintf(stderr,
                         "[fitsne] tiles: N=%d, %d blocks, %zu of %zu tiles hold edges, %zu upper edges; share of edges "
                         "in tiles of >= 4096 / 16384 / 65536 edges: %.3f / %.3f / %.3f\n",
                         N_, nblk, ne, nkeys, n, (double) e4 / n, (double) e16 / n, (double) e64 / n);
        }
    }
    release();
    if (e != cudaSuccess) return fail("build_tiles", e);
    tiles_ok_ = n > 0;
    return 0;
}

template <typename T>
cudaError_t Embedding<T>::attr_call(const T *Yin, T *Yout, T *uY, T *gains, T *dC, const UpdateParams &p,
                                    int shape) {
    if constexpr (sizeof(T) == 4) {
        if (shape == kAttrTilesShape && tiles_ok_)
            return launch_attr_tiles_update(trec_, tstart_, acc_, Yin, Yout, uY, gains, dC, rep_, N_, D_, p, red_,
                                            st_);
    }
    return launch_attr_update<T>(row_, col_, val_, Yin, Yout, uY, gains, dC, rep_, N_, D_, p, red_, st_,
                                 shape >= kNumAttrShapes ? 10 : shape, yh_);
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
    if (!twiddles(L)) return -10;
    int rc = grid_buffers(M, L);
    if (!rc && fft_thr_L_ != L) rc = tune_fft(M, L);
    return rc;
}

template <typename T>
typename Embedding<T>::C *Embedding<T>::twiddles(int L) {
    auto it = tw_.find(L);
    if (it != tw_.end()) return it->second;
    std::vector<C> h(L);
    const double pi = 3.14159265358979323846264338327950288;
    for (int j = 0; j < L; ++j) {
        const double a = 2.0 * pi * (double) j / (double) L;
        h[j] = mkc((T) std::cos(a), (T) -std::sin(a));
    }
    C *d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(C) * L);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d, h.data(), sizeof(C) * L, cudaMemcpyHostToDevice, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) {
        fail("twiddles", e);
        cudaFree(d);
        return nullptr;
    }
    tw_[L] = d;
    return d;
}

// Threads per block of the five 2-D FFT passes (kFftThreadChoices), timed on this
// embedding's grid buffers at transform length L the first time L occurs in the process
// (FITSNE_FFT_THREADS fixes it; FITSNE_AUTOTUNE=0 keeps 256).  Smaller blocks put more
// blocks on an SM for the short transforms of small grids; larger ones share each
// transform's stages among more threads.
template <typename T>
int Embedding<T>::tune_fft(int M, int L) {
    fft_thr_L_ = L;
    fft_thr_ = 256;
    if (D_ != 2) return 0;
    const char *fx = std::getenv("FITSNE_FFT_THREADS");
    if (fx && *fx) {
        fft_thr_ = std::atoi(fx);
        return 0;
    }
    const char *e = std::getenv("FITSNE_AUTOTUNE");
    if (e && std::atoi(e) == 0) return 0;
    // one choice per octave of transform lengths: the grid grows through a dozen lengths in
    // a run, the ranking of the three block sizes stays the same within an octave (N = 1M:
    // 256 threads ahead at every length from 300 to 864), and each timing costs ~1.5 ms
    // with the GPU otherwise idle
    int octave = 0;
    while ((2 << octave) <= L) ++octave;
    static std::mutex mu;
    static std::map<std::pair<int, int>, int> chosen;
    const std::pair<int, int> key((int) sizeof(T), octave);
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = chosen.find(key);
        if (it != chosen.end()) {
            fft_thr_ = it->second;
            return 0;
        }
    }
    FftPlan pl;
    if (!make_fft_plan(L, &pl)) return 0;
    C *tw = twiddles(L);
    if (!tw) return -10;
    const int mode = (gp_.df == 1.0) ? KERNEL_DF1 : KERNEL_VARDF;
    cudaEvent_t a = nullptr, b = nullptr;
    FITSNE_CK(cudaEventCreate(&a));
    FITSNE_CK(cudaEventCreate(&b));
    int best = 256;
    float best_ms = 0.f;
    for (int ci = 0; ci < 3; ++ci) {
        const int thr = kFftThreadChoices[(ci + 1) % 3];  // 256 first
        FITSNE_CK(conv2d_launch<T>(grid_in_, grid_out_, M, pl, tw, work_a_, work_b_, kspec_, 0.05, gp_.df, mode,
                                   st_, thr));
        FITSNE_CK(cudaEventRecord(a, st_));
        for (int r = 0; r < 3; ++r)
            FITSNE_CK(conv2d_launch<T>(grid_in_, grid_out_, M, pl, tw, work_a_, work_b_, kspec_, 0.05, gp_.df, mode,
                                       st_, thr));
        FITSNE_CK(cudaEventRecord(b, st_));
        FITSNE_CK(cudaEventSynchronize(b));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (timing_requested()) std::fprintf(stderr, "[fitsne] FFT passes, L = %d, %d threads: %.4f ms\n", L, thr, ms / 3.f);
        if (ci == 0 || ms < 0.97f * best_ms) {
            best = thr;
            best_ms = ms;
        }
    }
    launches_ += 4 * 3 * 5;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    {
        std::lock_guard<std::mutex> lk(mu);
        chosen[key] = best;
    }
    fft_thr_ = best;
    return 0;
}

template <typename T>
void Embedding<T>::launch_shapes(int *out5) const {
    int g = 4096, u = 4;
    if (attr_shape_ != kAttrTilesShape) attr_shape_info(attr_shape_, &g, &u);
    out5[0] = attr_shape_;
    out5[1] = g;
    out5[2] = u;
    out5[3] = (attr_shape_ == kAttrTilesShape && tiles_ok_) ? 2 : 0;
    out5[4] = fft_thr_;
}

template <typename T>
int Embedding<T>::grid_buffers(int M, int L) {
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
    FITSNE_CK(launch_spread<T>(Y_[cur_], N_, D_, geom_, grid_in_, st_, data_order_ ? sorder_ : nullptr));
    if (timing_) FITSNE_CK(cudaEventRecord(evs_[tb_][2], st_));
    if (D_ == 2)
        FITSNE_CK(conv2d_launch<T>(grid_in_, grid_out_, M, plan_, tw_[L_], work_a_, work_b_, kspec_, geom_.hk,
                                   gp_.df, mode, st_, fft_thr_));
    else
        FITSNE_CK(conv1d_launch<T>(grid_in_, grid_out_, M, plan_, tw_[L_], work_a_, geom_.hk, gp_.df, mode, st_));
    if (timing_) FITSNE_CK(cudaEventRecord(evs_[tb_][3], st_));
    FITSNE_CK(launch_gather<T>(Y_[cur_], N_, D_, geom_, grid_out_, mode, rep_, red_, st_, yh_));
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
    if (attr_shape_ < 0) {
        int tr = tune_attr(false);
        if (tr) return tr;
    }
    FITSNE_CK(attr_call(Y_[cur_], nullptr, nullptr, nullptr, dC_, p, attr_shape_));
    launches_ += (attr_shape_ == kAttrTilesShape && tiles_ok_) ? 3 : 2;
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

// Buffers of the renumbering, allocated with the first one.
template <typename T>
int Embedding<T>::renumber_alloc() {
    if (perm_) return 0;
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
    return 0;
}

// Renumbers the points along a Morton curve of the current embedding (reorder.cuh).  Points
// numbered in the data's locality order keep it (the attraction's neighbour lists want it);
// only the spread walks them in the Morton order then, so that a warp's points share boxes.
template <typename T>
int Embedding<T>::reorder() {
    const int W = y_width<T>(D_);
    if (int ra = renumber_alloc()) return ra;
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
    if (data_order_) {
        FITSNE_CK(cudaMemcpyAsync(sorder_, rids_, sizeof(uint32_t) * N_, cudaMemcpyDeviceToDevice, st_));
        return 0;
    }
    return renumber(rids_);
}

// Numbers the points in the given order of the data space (data_locality_order): the
// neighbour lists of consecutive rows overlap from the first iteration on, which the Morton
// order of an embedding still taking shape does not give (N = 1M: the attraction 0.67 ms in
// both phases, against 0.98 ms while the embedding is compact and 0.70 – 0.86 ms after, in the
// Morton order).  The points keep this numbering; the spread walks them in the Morton order of
// the embedding, refreshed at the iterations of the renumbering schedule.
template <typename T>
int Embedding<T>::set_order(const uint32_t *order) {
    if (int ra = renumber_alloc()) return ra;
    if (!sorder_) FITSNE_CK(cudaMalloc(&sorder_, sizeof(uint32_t) * N_));
    FITSNE_CK(launch_iota(sorder_, N_, st_));
    FITSNE_CK(cudaMemcpyAsync(rids_, order, sizeof(uint32_t) * N_, cudaMemcpyDeviceToDevice, st_));
    if (int rn = renumber(rids_)) return rn;
    data_order_ = true;
    return 0;
}

// Internal point k becomes the current internal point order[k] (a permutation on the device):
// point arrays, the CSR rows (in the new order) and columns (renamed), the tiles, and the map
// to the caller's indices.
template <typename T>
int Embedding<T>::renumber(const uint32_t *order) {
    const int W = y_width<T>(D_);
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
    if (int rb = build_tiles()) return rb;
    // caller index of each internal point, and its inverse
    FITSNE_CK(launch_compose(perm_, order, rids2_, N_, st_));
    std::swap(perm_, rids2_);
    FITSNE_CK(launch_invert(perm_, iperm_, N_, st_));
    unsigned int e0 = 0;
    FITSNE_CK(cudaMemcpyAsync(&e0, iperm_, sizeof(uint32_t), cudaMemcpyDeviceToHost, st_));
    FITSNE_CK(cudaStreamSynchronize(st_));
    excl_ = (int) e0;
    reordered_ = true;
    attr_shape_ = -1;
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
    if (attr_shape_ < 0 || attr_phase_ != tune_phase_) {
        rc = tune_attr(true);
        if (rc) return rc;
    }
    FITSNE_CK(attr_call(Y_[cur_], Y_[1 - cur_], uY_, gains_, nullptr, p, attr_shape_));
    // centre + attraction (+ the separate update of the tiled form)
    launches_ += (attr_shape_ == kAttrTilesShape && tiles_ok_) ? 3 : 2;
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
    if (graphs_ && !timing_ && it1 - it0 > 1) return run_schedule_graphs(s, it0, it1, costs, verbose);
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
        tune_phase_ = tune_phase(s, it);
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

// ---------------------------------------------------------------------------------
// Graph-captured iteration chunks.  The grid of every iteration is sized on the device
// (k_geometry) inside a capacity chosen here; the host reads the status once per chunk.
//
// Chooses the attraction pass's launch shape: FITSNE_ATTR_SHAPE fixes it; otherwise, when
// `measure` is set, the candidate shapes are timed on the attraction pass with the optimiser
// step of this embedding's data (on scratch copies of the state) and the fastest is kept.
// Choices are made per phase of the run (tune_phase: compact or expanded embedding) and shared
// by embeddings of the same size class (type, dimension, log2 N, log2 nnz / N, renumbered or
// not, phase, tiled form available or not, numbered in the data's order or not) within the
// process.  An embedding that will be renumbered runs the default shape
// until its first renumbering.  One-off gradients (measure false) take the cached choice or the
// default.
template <typename T>
int Embedding<T>::tune_attr(bool measure) {
    // candidates, the default first: the shapes that came out ahead on some size class and
    // phase (grad.cu describes them).  FP32 at N = 1M: 16 rows x 2 edges per lane with 48
    // warps per SM on the expanded embedding, 8 x 4 on the compact one; FP64 (twice the
    // registers per value): 16 x 2 and 8 x 4 with 32 warps.
    static const int kCandidates32[] = {10, 2, 3, 0};
    // FP32 with a symmetric P: the full-CSR default, the tiled form, the compact-phase shape
    static const int kCandidatesTiles[] = {10, kAttrTilesShape, 2};
    static const int kCandidates64[] = {3, 2};
    const int *kCandidates = sizeof(T) == 4 ? (tiles_ok_ ? kCandidatesTiles : kCandidates32) : kCandidates64;
    const int kNumCandidates = sizeof(T) == 4 ? (tiles_ok_ ? 3 : 4) : 2;
    static std::mutex mu;
    static std::map<std::vector<int>, int> chosen;
    int lgN = 0, lgK = 0;
    while ((1 << (lgN + 1)) <= N_) ++lgN;
    const size_t per = N_ ? nnz_ / (size_t) N_ : 0;
    while (((size_t) 1 << (lgK + 1)) <= per) ++lgK;
    const std::vector<int> key = {(int) sizeof(T), D_, lgN, lgK, reordered_ ? 1 : 0, tune_phase_,
                                  tiles_ok_ ? 1 : 0, data_order_ ? 1 : 0};
    attr_phase_ = tune_phase_;
    const char *fixed = std::getenv("FITSNE_ATTR_SHAPE");  // a fixed shape index: no tuning, no cache
    if (fixed && *fixed) {
        const int sh = std::atoi(fixed);
        attr_shape_ = (sh >= 0 && sh <= kAttrTilesShape) ? sh : 0;
        return 0;
    }
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = chosen.find(key);
        if (it != chosen.end()) {
            attr_shape_ = it->second;
            return 0;
        }
    }
    const bool renumber_ahead = !reordered_ && reorder_enabled_ && N_ >= kReorderMinN;
    if (!measure || renumber_ahead) {
        attr_shape_ = kCandidates[0];  // not cached: a later call may measure
        return 0;
    }
    const char *e = std::getenv("FITSNE_AUTOTUNE");
    int best = kCandidates[0];
    if (!(e && std::atoi(e) == 0) && N_ >= 4096) {
        // the launches time the optimiser step itself (mode 1, the kernel the iterations run):
        // the new Y goes to the free buffer, the gains and momentum to copies, and the pending
        // mean of Y (written by the step's reduction) is kept aside and put back afterwards
        UpdateParams p{};
        p.mode = 1;
        p.use_gains = 1;
        p.exag = 1.0;
        p.momentum = 0.8;
        p.learning_rate = 200.0;
        p.max_step_norm = 5.0;
        p.df = gp_.df;
        const size_t nd = (size_t) N_ * D_;
        T *scr = nullptr;
        FITSNE_CK(cudaMalloc(&scr, sizeof(T) * 2 * nd));
        FITSNE_CK(cudaMemcpyAsync(scr, uY_, sizeof(T) * nd, cudaMemcpyDeviceToDevice, st_));
        FITSNE_CK(cudaMemcpyAsync(scr + nd, gains_, sizeof(T) * nd, cudaMemcpyDeviceToDevice, st_));
        double *mean_keep = red_.mnmx + 8;
        FITSNE_CK(cudaMemcpyAsync(mean_keep, red_.mean, sizeof(double) * 2, cudaMemcpyDeviceToDevice, st_));
        cudaEvent_t a = nullptr, b = nullptr;
        FITSNE_CK(cudaEventCreate(&a));
        FITSNE_CK(cudaEventCreate(&b));
        float best_ms = 0.f;
        for (int ci = 0; ci < kNumCandidates; ++ci) {
            const int sh = kCandidates[ci];
            FITSNE_CK(attr_call(Y_[cur_], Y_[1 - cur_], scr, scr + nd, nullptr, p, sh));
            FITSNE_CK(cudaEventRecord(a, st_));
            for (int r = 0; r < 2; ++r) FITSNE_CK(attr_call(Y_[cur_], Y_[1 - cur_], scr, scr + nd, nullptr, p, sh));
            FITSNE_CK(cudaEventRecord(b, st_));
            FITSNE_CK(cudaEventSynchronize(b));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, a, b);
            if (timing_requested()) std::fprintf(stderr, "[fitsne] attraction shape %d: %.4f ms\n", sh, ms / 2.f);
            // another shape must beat the best so far by 3 % (timing noise)
            if (ci == 0 || ms < 0.97f * best_ms) {
                best = sh;
                best_ms = ms;
            }
        }
        launches_ += 3 * kNumCandidates;
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        FITSNE_CK(cudaMemcpyAsync(red_.mean, mean_keep, sizeof(double) * 2, cudaMemcpyDeviceToDevice, st_));
        FITSNE_CK(cudaStreamSynchronize(st_));
        FITSNE_CK(cudaFree(scr));
        if (timing_requested()) {
            int g = 4096, u = 4;  // the tiled form: 4,096-point blocks, 4 records per lane
            if (best != kAttrTilesShape) attr_shape_info(best, &g, &u);
            std::fprintf(stderr, "[fitsne] attraction launch shape %d (N=%d, nnz=%zu%s, phase %d): %d rows per work "
                                 "item, %d edges per lane\n", best, N_, nnz_, reordered_ ? ", renumbered" : "",
                         tune_phase_, g, u);
        }
    }
    {
        std::lock_guard<std::mutex> lk(mu);
        chosen[key] = best;
    }
    attr_shape_ = best;
    return 0;
}

template <typename T>
int Embedding<T>::plan_capacity(int grow) {
    if (attr_shape_ < 0 || attr_phase_ != tune_phase_) {
        int tr = tune_attr(true);
        if (tr) return tr;
    }
    int nb = nb_last_ > 0 ? nb_last_ : geom_.nb;
    if (nb < 1) nb = 1;
    int target = grow ? std::max(nb_cap_ + 1, nb + nb / 2 + 1) : nb + nb / 4 + 1;
    if (D_ == 2 && target < 200) {
        static const int allowed[20] = {25, 36, 50, 55, 60, 65, 70, 75, 80, 85,
                                        90, 96, 100, 110, 120, 130, 140, 150, 175, 200};
        int i = 0;
        while (allowed[i] < target) ++i;
        target = allowed[i];
    }
    if (!grow && target <= nb_cap_) target = nb_cap_;  // keep a larger capacity (and the cached graph)
    int M = target * gp_.nterms;
    int L = smooth_even_at_least(2 * M);
    while (L > max_fft_len<T>() && target > nb) {
        --target;
        M = target * gp_.nterms;
        L = smooth_even_at_least(2 * M);
    }
    if (L > max_fft_len<T>()) {
        err_ = "interpolation grid too large: " + std::to_string(L) + " > " + std::to_string(max_fft_len<T>());
        return -13;
    }
    int rc = grid_buffers(M, L);
    if (rc) return rc;
    if (fft_thr_L_ != L) {
        rc = tune_fft(M, L);
        if (rc) return rc;
    }
    if (L > tw_dev_cap_) {
        cudaFree(tw_dev_);
        FITSNE_CK(cudaMalloc(&tw_dev_, sizeof(C) * L));
        tw_dev_cap_ = L;
    }
    if (!dgeom_) {
        const int W = y_width<T>(D_);
        FITSNE_CK(cudaMalloc(&dgeom_, sizeof(DevGeom)));
        FITSNE_CK(cudaMalloc(&gstatus_, sizeof(int)));
        FITSNE_CK(cudaMallocHost(&h_gstat_, sizeof(int) * 2));
        FITSNE_CK(cudaMalloc(&snap_, sizeof(T) * (size_t) N_ * (W + 2 * D_)));
        FITSNE_CK(cudaMalloc(&snap_mean_, sizeof(double) * 2));
    }
    nb_cap_ = target;
    M_cap_ = M;
    L_cap_ = L;
    return 0;
}

template <typename T>
int Embedding<T>::record_iters(const UpdateParams &p, int n, int c, bool apply_mean_first) {
    const int mode = (gp_.df == 1.0) ? KERNEL_DF1 : KERNEL_VARDF;
    const ConvGeom *cg =
        reinterpret_cast<const ConvGeom *>(reinterpret_cast<const char *>(dgeom_) + offsetof(DevGeom, conv));
    const size_t gridn = (D_ == 2) ? (size_t) M_cap_ * M_cap_ : (size_t) M_cap_;
    for (int k = 0; k < n; ++k) {
        FITSNE_CK(launch_center_minmax<T>(Y_[c], N_, D_, (k > 0 || apply_mean_first) ? 1 : 0, excl_, red_, st_));
        FITSNE_CK(launch_geometry(red_, D_, gp_.nterms, gp_.intervals_per_integer, gp_.min_num_intervals, nb_cap_,
                                  L_cap_, dgeom_, gstatus_, st_));
        FITSNE_CK(twiddles_dev<T>(cg, tw_dev_, st_));
        FITSNE_CK(cudaMemsetAsync(grid_in_, 0, sizeof(Cell4<T>) * gridn, st_));
        FITSNE_CK(launch_spread_dev<T>(Y_[c], N_, D_, gp_.nterms, dgeom_, grid_in_, st_,
                                       data_order_ ? sorder_ : nullptr));
        if (D_ == 2)
            FITSNE_CK(conv2d_launch_dev<T>(grid_in_, grid_out_, M_cap_, L_cap_, cg, tw_dev_, work_a_, work_b_, kspec_,
                                           gp_.df, mode, st_, fft_thr_));
        else
            FITSNE_CK(conv1d_launch_dev<T>(grid_in_, grid_out_, L_cap_, cg, tw_dev_, work_a_, gp_.df, mode, st_));
        FITSNE_CK(launch_gather_dev<T>(Y_[c], N_, D_, gp_.nterms, dgeom_, grid_out_, mode, rep_, red_, st_, yh_));
        FITSNE_CK(attr_call(Y_[c], Y_[1 - c], uY_, gains_, nullptr, p,
                            attr_shape_ < 0 ? (sizeof(T) == 4 ? 10 : 3) : attr_shape_));
        c = 1 - c;
    }
    return 0;
}

template <typename T>
int Embedding<T>::launch_iters(const UpdateParams &p, int n, int c, bool apply_mean_first) {
    GraphSlot &s = gslots_[n - 1][c][apply_mean_first ? 1 : 0];
    const std::vector<unsigned long long> key = iters_key(p, n, c, apply_mean_first);
    if (!s.exec || key != s.key) {
        cudaGraph_t graph = nullptr;
        FITSNE_CK(cudaStreamBeginCapture(st_, cudaStreamCaptureModeRelaxed));
        int rc = record_iters(p, n, c, apply_mean_first);
        cudaError_t ce = cudaStreamEndCapture(st_, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        // same topology (a new capacity, new buffers after a renumbering, new schedule
        // parameters): update the instantiated graph in place, else instantiate anew
        bool updated = false;
        if (ce == cudaSuccess && s.exec) {
            cudaGraphExecUpdateResultInfo info;
            updated = cudaGraphExecUpdate(s.exec, graph, &info) == cudaSuccess;
            if (!updated) cudaGetLastError();  // clear the failed update
        }
        if (ce == cudaSuccess && !updated) {
            if (s.exec) {
                cudaGraphExecDestroy(s.exec);
                s.exec = nullptr;
            }
            ce = cudaGraphInstantiate(&s.exec, graph, 0);
        }
        if (graph) cudaGraphDestroy(graph);
        if (ce != cudaSuccess) {
            if (s.exec) cudaGraphExecDestroy(s.exec);
            s.exec = nullptr;
            s.key.clear();
            return fail("iterations graph", ce);
        }
        s.key = key;
        ++captures_;
        if (updated) ++updates_;
    }
    FITSNE_CK(cudaGraphLaunch(s.exec, st_));
    return 0;
}

template <typename T>
int Embedding<T>::finish_chunk(int len) {
    const int status = h_gstat_[0];
    if (status & 2) {
        err_ = "embedding coordinates are not finite";
        return -11;
    }
    if (status & 1) {
        // the grid outgrew the capacity: back to the state at the start of the chunk
        const int W = y_width<T>(D_);
        const size_t ny = (size_t) N_ * W, nd = (size_t) N_ * D_;
        FITSNE_CK(cudaMemcpyAsync(Y_[gchunk_cur0_], snap_, sizeof(T) * ny, cudaMemcpyDeviceToDevice, st_));
        FITSNE_CK(cudaMemcpyAsync(uY_, snap_ + ny, sizeof(T) * nd, cudaMemcpyDeviceToDevice, st_));
        FITSNE_CK(cudaMemcpyAsync(gains_, snap_ + ny + nd, sizeof(T) * nd, cudaMemcpyDeviceToDevice, st_));
        FITSNE_CK(cudaMemcpyAsync(red_.mean, snap_mean_, sizeof(double) * 2, cudaMemcpyDeviceToDevice, st_));
        FITSNE_CK(cudaStreamSynchronize(st_));
        cur_ = gchunk_cur0_;
        return 1;
    }
    nb_last_ = h_gstat_[1];
    if (len & 1) cur_ = 1 - cur_;
    mean_pending_ = true;
    launches_ += (unsigned long long) len * ((D_ == 2 ? 11 : 8) + ((attr_shape_ == kAttrTilesShape && tiles_ok_) ? 1 : 0));
    return 0;
}

template <typename T>
int Embedding<T>::launch_chunk(const UpdateParams &p, int len, int grow) {
    int rc = plan_capacity(grow);
    if (rc) return rc;
    // the state at the start of the chunk (put back when the grid outgrows its capacity)
    const int W = y_width<T>(D_);
    const size_t ny = (size_t) N_ * W, nd = (size_t) N_ * D_;
    FITSNE_CK(cudaMemcpyAsync(snap_, Y_[cur_], sizeof(T) * ny, cudaMemcpyDeviceToDevice, st_));
    FITSNE_CK(cudaMemcpyAsync(snap_ + ny, uY_, sizeof(T) * nd, cudaMemcpyDeviceToDevice, st_));
    FITSNE_CK(cudaMemcpyAsync(snap_ + ny + nd, gains_, sizeof(T) * nd, cudaMemcpyDeviceToDevice, st_));
    FITSNE_CK(cudaMemcpyAsync(snap_mean_, red_.mean, sizeof(double) * 2, cudaMemcpyDeviceToDevice, st_));
    FITSNE_CK(cudaMemsetAsync(gstatus_, 0, sizeof(int), st_));
    // pairs of iterations (the buffers swap twice: one graph per starting buffer serves the
    // whole chunk), one single iteration for an odd length
    int c = cur_;
    for (int k = 0; k < len;) {
        const int n = (len - k >= 2) ? 2 : 1;
        rc = launch_iters(p, n, c, k > 0 || mean_pending_);
        if (rc) return rc;
        if (n == 1) c = 1 - c;
        k += n;
    }
    FITSNE_CK(cudaMemcpyAsync(h_gstat_, gstatus_, sizeof(int), cudaMemcpyDeviceToHost, st_));
    FITSNE_CK(cudaMemcpyAsync(h_gstat_ + 1,
                              reinterpret_cast<const char *>(dgeom_) + offsetof(DevGeom, g) + offsetof(GridGeom, nb),
                              sizeof(int), cudaMemcpyDeviceToHost, st_));
    gchunk_cur0_ = cur_;
    gchunk_len_ = len;
    return 0;
}

template <typename T>
std::vector<unsigned long long> Embedding<T>::iters_key(const UpdateParams &p, int n, int c,
                                                        bool apply_mean_first) const {
    std::vector<unsigned long long> key;
    auto put = [&key](const void *v, size_t n) {
        unsigned long long w = 0;
        std::memcpy(&w, v, n < 8 ? n : 8);
        key.push_back(w);
    };
    put(&n, sizeof n);
    put(&c, sizeof c);
    put(&apply_mean_first, sizeof apply_mean_first);
    put(&p.exag, 8);
    put(&p.momentum, 8);
    put(&p.learning_rate, 8);
    put(&p.df, 8);
    put(&p.max_step_norm, 8);
    put(&p.use_gains, sizeof p.use_gains);
    put(&nb_cap_, sizeof nb_cap_);
    put(&excl_, sizeof excl_);
    put(&attr_shape_, sizeof attr_shape_);
    put(&fft_thr_, sizeof fft_thr_);
    put(&tiles_ok_, sizeof tiles_ok_);
    const void *ord = data_order_ ? (const void *) sorder_ : nullptr;
    for (const void *q : {(const void *) row_, (const void *) col_, (const void *) val_, (const void *) Y_[0],
                          (const void *) Y_[1], (const void *) uY_, (const void *) gains_, (const void *) rep_,
                          (const void *) grid_in_, (const void *) grid_out_, (const void *) work_a_,
                          (const void *) work_b_, (const void *) kspec_, (const void *) tw_dev_, (const void *) trec_,
                          (const void *) tstart_, (const void *) acc_, (const void *) yh_, ord})
        put(&q, sizeof q);
    return key;
}

template <typename T>
int Embedding<T>::run_schedule_graphs(const Schedule &s, int it0, int it1, double *costs, bool verbose) {
    double mult = s.early_exag_coeff;
    double momentum = s.momentum;
    for (int it = 0; it < it0; ++it) {
        if (it == s.stop_lying_iter) mult /= s.early_exag_coeff;
        if (it == s.start_late_exag_iter) mult *= s.late_exag_coeff;
        if (it == s.mom_switch_iter) momentum = s.final_momentum;
    }
    auto params = [&](int it) {
        UpdateParams p{};
        p.mode = 1;
        p.exag = mult;
        p.momentum = momentum;
        p.learning_rate = s.learning_rate;
        p.df = gp_.df;
        if (s.no_momentum_during_exag) {
            p.use_gains = (it > s.stop_lying_iter) ? 1 : 0;
            p.max_step_norm = -1.0;
        } else {
            p.use_gains = 1;
            p.max_step_norm = s.max_step_norm;
        }
        return p;
    };
    auto reorder_due = [&](int it) { return this->reorder_due(it, it0); };
    auto kl_due = [&](int it) { return costs && ((it + 1) % 50 == 0 || it == s.max_iter - 1); };
    auto after = [&](int it) -> int {  // the reference's switches and KL after iteration it
        if (it == s.stop_lying_iter) mult /= s.early_exag_coeff;
        if (it == s.start_late_exag_iter) mult *= s.late_exag_coeff;
        if (it == s.mom_switch_iter) momentum = s.final_momentum;
        if (kl_due(it)) {
            double C = 0.0;
            int rc = kl(mult, &C);
            if (rc) return rc;
            if (it < s.stop_lying_iter && s.stop_lying_iter != -1)
                C = C / s.early_exag_coeff - std::log(s.early_exag_coeff);
            if (it >= s.start_late_exag_iter && s.start_late_exag_iter != -1)
                C = C / s.late_exag_coeff - std::log(s.late_exag_coeff);
            costs[it] = C;
            if (verbose) std::printf("Iteration %d, cost %f\n", it + 1, C);
        }
        return 0;
    };
    const unsigned long long l0 = launches_;
    // host time by phase (reported under FITSNE_TIMING)
    using clk = std::chrono::steady_clock;
    double t_first = 0, t_reorder = 0, t_launch = 0, t_wait = 0, t_after = 0;
    auto since = [](clk::time_point a) { return std::chrono::duration<double>(clk::now() - a).count(); };
    const unsigned long long cap0 = captures_, upd0 = updates_;
    FITSNE_CK(cudaEventRecord(evr_[0], st_));
    int it = it0;
    if (it < it1) {
        // first iteration on the host path: it sizes the grid and fixes the launch shapes
        const auto t = clk::now();
        if (reorder_due(it)) {
            int rr = reorder();
            if (rr) return rr;
        }
        int rc = step(params(it), it == 0);
        if (rc) return rc;
        nb_last_ = geom_.nb;
        rc = after(it);
        if (rc) return rc;
        ++it;
        FITSNE_CK(cudaStreamSynchronize(st_));
        t_first += since(t);
    }
    while (it < it1) {
        if (reorder_due(it)) {
            const auto t = clk::now();
            int rr = reorder();
            if (rr) return rr;
            FITSNE_CK(cudaStreamSynchronize(st_));
            t_reorder += since(t);
        }
        // chunks of at most kMaxChunk iterations, so that the grid capacity follows the
        // embedding's growth and a repeated chunk costs little
        int end = it + 1;
        while (end < it1 && end - it < kMaxChunk &&
               !(kl_due(end - 1) || end - 1 == s.stop_lying_iter || end - 1 == s.start_late_exag_iter ||
                 end - 1 == s.mom_switch_iter || reorder_due(end)))
            ++end;
        const int len = end - it;
        const UpdateParams p = params(it);
        // the phase whose launch shape the chunk's attraction uses
        tune_phase_ = tune_phase(s, it);
        int grow = 0;
        while (true) {
            auto t = clk::now();
            int rc = launch_chunk(p, len, grow);
            if (rc) return rc;
            t_launch += since(t);
            t = clk::now();
            FITSNE_CK(cudaStreamSynchronize(st_));
            t_wait += since(t);
            rc = finish_chunk(len);
            if (rc < 0) return rc;
            if (rc == 0) break;
            grow = 1;  // the embedding outgrew the capacity inside the chunk: larger grid, same chunk
        }
        const auto t = clk::now();
        for (int k = it; k < end; ++k) {
            int rc = after(k);
            if (rc) return rc;
        }
        t_after += since(t);
        it = end;
    }
    FITSNE_CK(cudaEventRecord(evr_[1], st_));
    FITSNE_CK(cudaEventSynchronize(evr_[1]));
    cudaEventElapsedTime(&times_.run_ms, evr_[0], evr_[1]);
    times_.launches = launches_ - l0;
    if (timing_requested())
        std::fprintf(stderr,
                     "[fitsne] iterations %d-%d: first (host path, tuning) %.3f s, renumbering %.3f s, chunk "
                     "capture/update/launch %.3f s (%llu captures, %llu updates), chunk execution wait %.3f s, "
                     "KL and switches %.3f s\n",
                     it0, it1, t_first, t_reorder, t_launch, captures_ - cap0, updates_ - upd0, t_wait, t_after);
    return 0;
}

template class Embedding<float>;
template class Embedding<double>;

}  // namespace fitsne
