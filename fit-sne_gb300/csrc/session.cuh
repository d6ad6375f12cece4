// Opaque session object behind the fitsne_session_* entry points.
#pragma once

#include <memory>
#include <string>

#include "embedding.cuh"

namespace fitsne {

struct SessionBase {
    virtual ~SessionBase() {}
    virtual int run(int it0, int it1, const Schedule &s, double *costs) = 0;
    virtual int gradient(double *dC, double *sum_Q) = 0;
    virtual int get_y(double *Y) = 0;
    virtual void set_timing(bool on) = 0;
    virtual void set_graphs(bool on) = 0;
    virtual void times(double *out10) = 0;
    virtual void launch_shapes(int *out5) = 0;
    virtual std::string error() = 0;
    cudaStream_t st = nullptr;
};

template <typename T>
struct SessionT : SessionBase {
    Embedding<T> emb;
    int run(int it0, int it1, const Schedule &s, double *costs) override {
        return emb.run_schedule(s, it0, it1, costs, false);
    }
    int gradient(double *dC, double *sum_Q) override { return emb.gradient(dC, sum_Q); }
    int get_y(double *Y) override { return emb.get_Y(Y); }
    void set_timing(bool on) override { emb.set_timing(on); }
    void set_graphs(bool on) override { emb.set_graphs(on); }
    void times(double *o) override {
        const StageTimes &t = emb.last_times();
        o[0] = t.center;
        o[1] = t.spread;
        o[2] = t.conv;
        o[3] = t.gather;
        o[4] = t.attract;
        o[5] = t.total;
        o[6] = emb.last_geom().nb;
        o[7] = emb.last_L();
        o[8] = t.run_ms;
        o[9] = (double) t.launches;
    }
    void launch_shapes(int *o) override { emb.launch_shapes(o); }
    std::string error() override { return emb.error(); }
};

}  // namespace fitsne

struct fitsne_session {
    std::unique_ptr<fitsne::SessionBase> impl;
};
