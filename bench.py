#!/usr/bin/env python3
"""FIt-SNE on one GB300: t-SNE iterations/s at N = 1,000,000, 2-D, and end-to-end seconds.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload (both arms): N = 1,000,000 x D = 50 Gaussian mixture (10 clusters, Dirichlet(2)
weights, per-cluster std U(0.5, 2), centres N(0, 25 I), seed 42); perplexity 30, K = 90,
2-D, df = 1, learning rate N/12, nterms 3, min_num_intervals 50, intervals_per_integer 1.
A *step* is one optimiser iteration after the early exaggeration (exaggeration 1,
momentum 0.8): spread + FFT convolution + gather on the interpolation grid, attraction over
the ~1.56e8 non-zeros of P, gains/momentum/clipping update, zero-mean.

gb300 arm: P is built on the GPU from the data (exact kNN, calibration, symmetrisation) and
stays resident; the reference schedule runs untimed from a random start to iteration 300
(early exaggeration until 250), then W untimed steps, then K steps timed with CUDA events
on the library's stream (the grid grows from ~50 to ~100 boxes per side over those steps).
`e2e` runs the whole pipeline (fitsne_run: data on the host -> embedding on the host, 1000
iterations of the reference schedule) with the learned calibration warm start and reports
iterations/s over that wall time; `e2e.bisection` is the same call with the reference's
bisection, `e2e.plain_fp64` the FP64 form.  The FP64 form of the same kernels is timed on
the same steps (`plain_fp64`); the FP32 gradient is compared with the FP64 one at the
starting state (`grad_rel_l2_vs_fp64`) and with the restated reference gradient (oracle/,
FP64) on the reference's P at that state (`grad_rel_l2_vs_oracle`).  `on_cpu_inputs` times
the GPU on exactly the CPU leg's P, start state and steps.  `batch` runs the batched form
(64 jobs, below) and the same jobs one by one; `similarities` times the input-similarity stage
alone, with the tcgen05 kNN candidate search against the tensor roofline.

reference arm (and the cpu_baseline leg of the gb300 arm, same inputs): the reference's CPU
path (the C restatement in oracle/, the reference tree is not on the GPU machine) on all host
cores, on the same step definition; P for that arm is built on the CPU from random
within-cluster neighbour lists of the same size (K = 90 per row, symmetrised by the restated
symmetrizeMatrix): the exact kNN of 1M points on the CPU takes hours.  Y is a synthetic
post-exaggeration embedding of the same clusters whose grid (60 boxes per side) is the middle
of the GPU's timed steps; W untimed steps precede the timed ones.  The number of timed CPU
steps is capped so that the arm ends within a few minutes.

    python bench.py --stage similarities [--n N]

times the input-similarity stage alone on the GPU (exact kNN with the tcgen05 candidate
search, perplexity calibration, symmetrisation) on the same mixture, K = 91 with self, and
reports the kNN candidate search against the tensor-core roofline (2 N^2 D flops, D = 50
unpadded, against the measured bf16 peak).

    python bench.py --stage batch [--jobs 64]

runs the batched form (fitsne_batch_run: 64 embeddings, N log-uniform in [2,000, 50,000],
D = 50 mixtures of 5-30 clusters, perplexity 10 / 30 / 50 cycled, 1000 iterations) and the
same jobs one by one through fitsne_run, and reports the aggregate iterations/s.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "fit-sne_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "t-SNE iters/s at N=1M 2D vs plain GPU form at grad rel-L2≤1e-4; end-to-end s"
PERPLEXITY = 30.0
K_NEIGH = 90
D_IN = 50
SCHEDULE = dict(max_iter=1000, stop_lying_iter=250, mom_switch_iter=250, momentum=0.5, final_momentum=0.8,
                early_exag_coeff=12.0, max_step_norm=5.0)
STEP_IT0 = 300  # steps are iterations of the post-exaggeration phase
HBM_FALLBACK_GBS = 6800.0
BF16_FALLBACK_TFLOPS = 1900.0


def mixture(N, D=D_IN, seed=42):
    """10-cluster Gaussian mixture: Dirichlet(2) weights, std U(0.5, 2), centres N(0, 25 I)."""
    rng = np.random.default_rng(seed)
    w = rng.dirichlet(np.full(10, 2.0))
    sizes = rng.multinomial(N, w)
    labels = np.repeat(np.arange(10), sizes)
    centres = rng.standard_normal((10, D)) * 5.0
    std = rng.uniform(0.5, 2.0, 10)
    X = centres[labels] + rng.standard_normal((N, D)) * std[labels, None]
    return X, labels, sizes


def expanded_state(labels, seed=7):
    """Synthetic post-exaggeration embedding of the same clusters: centres N(0, 12^2 I),
    spread 2.5, range ~59 at N = 1M, i.e. a 60-box grid, the middle of the 50 -> 70 boxes that
    the GPU's timed steps (iterations 305-605 of the real schedule) pass through."""
    rng = np.random.default_rng(seed)
    centres = rng.standard_normal((10, 2)) * 12.0
    Y = centres[labels] + rng.standard_normal((len(labels), 2)) * 2.5
    return Y - Y.mean(0)


def cpu_sample_P(orc, labels, sizes, K=K_NEIGH, seed=3):
    """Random within-cluster neighbour lists of K per row, calibrated-like weights,
    symmetrised by the restated symmetrizeMatrix and normalised."""
    rng = np.random.default_rng(seed)
    N = len(labels)
    starts = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    col = (starts[labels][:, None] + (rng.random((N, K)) * sizes[labels][:, None]).astype(np.int64))
    col = np.where(col == np.arange(N)[:, None], (col + 1) % N, col).astype(np.uint32).ravel()
    row = (np.arange(N + 1, dtype=np.int64) * K).astype(np.uint32)
    val = rng.random(N * K)
    val /= val.reshape(N, K).sum(1).repeat(K)
    r, c, v = orc.symmetrize(row, col, val, N)
    return r, c, v / v.sum()


def time_cpu_steps(orc, P, Y, warm, steps, nthreads, budget_s=None):
    """Runs `warm` untimed reference iterations (post-exaggeration parameters) from Y, then
    times up to `steps` more, carrying Y, uY and gains through; returns (timed, seconds)."""
    row, col, val = P
    N = Y.shape[0]
    Y = Y.copy()
    uY = np.zeros_like(Y)
    gains = np.ones_like(Y)
    lr = N / 12.0
    for _ in range(warm):
        orc.gradient_step(row, col, val, Y, uY, gains, 3, 1.0, 50, nthreads, 1.0, 1.0, 0.8, lr, 1, 5.0)
    done, t0 = 0, time.perf_counter()
    for _ in range(steps):
        orc.gradient_step(row, col, val, Y, uY, gains, 3, 1.0, 50, nthreads, 1.0, 1.0, 0.8, lr, 1, 5.0)
        done += 1
        if budget_s is not None and time.perf_counter() - t0 > budget_s:
            break
    return done, time.perf_counter() - t0


def reference_P(fitsne, X, perplexity, K):
    """P as TSNE::run builds it (src/tsne.cpp:153-330): X centred by zeroMean's sequential
    column sums and scaled by its largest magnitude; exact kNN and calibration (identical to
    the reference's); symmetrisation; normalisation by the sequential sum."""
    Xp = X - np.cumsum(X, axis=0)[-1] / len(X)
    Xp /= np.abs(Xp).max()
    row, col, val = fitsne.gaussian_perplexity(Xp, perplexity, K)
    del Xp
    row, col, val = fitsne.symmetrize(row, col, val, len(X))
    return row, col, val / np.cumsum(val)[-1]


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        self.index = index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        except OSError:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    try:
        p = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


def bf16_peak():
    """Dense bf16 TFLOP/s of this machine's GB300 (burst figure: the kNN kernel runs alone)."""
    try:
        p = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(p["bf16_tflops"]), "measured"
    except Exception:
        return BF16_FALLBACK_TFLOPS, "fallback"


# DRAM bytes (read + write) of one attraction launch / its algorithmic bytes, from an ncu
# capture of k_attr on this workload (N = 1,000,000, nnz = 155,720,438; the 301st launch):
# 1,355,542,000 + 28,894,976 bytes against 1,321,763,508 algorithmic.  (At N = 200,000 the
# ratio was 0.995: 256,773,632 / 257,955,380.)
ATTR_TRAFFIC_RATIO = (1355542000 + 28894976) / 1321763508


def attraction_bytes(N, nnz):
    """Algorithmic bytes of one attraction + update launch (FP32 form, 2-D): row pointers,
    col (u32) + val (f32) per non-zero, own Y read and new Y write (double-float, 16 B),
    uY and gains read + write (8 B each), repulsion numerators read (8 B).  Neighbour Y
    gathers count 0 (Y, 16 MB, stays in L2)."""
    return 4 * (N + 1) + 8 * nnz + N * (16 + 16 + 16 + 16 + 8)


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    import oracle
    oracle.build_restated()
    orc = oracle.Restated()
    X, labels, sizes = mixture(args.n)
    del X
    P = cpu_sample_P(orc, labels, sizes)
    Y = expanded_state(labels)
    cores = os.cpu_count() or 1
    _, per = time_cpu_steps(orc, P, Y, 0, 1, cores)
    cap = max(1, int(150.0 / max(per, 1e-3)))
    # W warm-up steps from the synthetic state, then the timed steps (the definition the
    # GPU arm's on_cpu_inputs leg uses on the same P and state)
    timed, secs = time_cpu_steps(orc, P, Y, args.warmup, min(args.steps, cap), cores, budget_s=170.0)
    value = timed / secs
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "iters/s", "n_gpus": args.gpus,
            "steps": args.steps, "steps_timed": timed, "warmup": args.warmup, "ms_per_step": 1e3 * secs / timed,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Gaussian mixture; random within-cluster P of the same size)",
            "config": config(args, "CPU restatement of the reference path"),
            "cpu_baseline": {"value": value, "unit": "iters/s", "cores": cores, "kind": "port",
                             "sample": "%d post-exaggeration iterations at N=%d, 2-D, after %d untimed ones from "
                                       "the synthetic state" % (timed, args.n, args.warmup)},
            "e2e": {"value": value, "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def config(args, impl_note):
    return {"workload": "N=%d x D=50 Gaussian mixture (10 clusters, seed 42); perplexity 30, K=90, 2-D, df=1, "
                        "lr=N/12; step = one post-exaggeration FFT-gradient iteration" % args.n,
            "N": args.n, "D": D_IN, "no_dims": 2, "perplexity": PERPLEXITY, "K": K_NEIGH, "df": 1.0,
            "nterms": 3, "min_num_intervals": 50, "intervals_per_integer": 1.0,
            "l2": "inputs larger than L2 (P: ~1 GB per step vs 129 MB L2)", "parallelism": "replicas",
            "impl": impl_note}


def run_gb300(args, world, rank, local):
    import fitsne
    hbm, peak_kind = peaks()
    X, labels, sizes = mixture(args.n)
    Yst = expanded_state(labels)
    N = args.n
    sched = dict(SCHEDULE, learning_rate=N / 12.0)
    # the real schedule from a random initialisation up to the first timed step (untimed)
    Y0 = np.random.default_rng(1).standard_normal((N, 2)) * 1e-4
    t0 = time.perf_counter()
    s32 = fitsne.Session.from_data(X, Y0, perplexity=PERPLEXITY, precision=32)
    setup_s = time.perf_counter() - t0
    nnz = s32.nnz
    s32.run(0, STEP_IT0, **sched)
    Yburn = s32.get_y()
    g32, z32 = s32.gradient()
    # FP64 form of the same kernels on the same steps, from the same state
    s64 = fitsne.Session.from_data(X, Yburn, perplexity=PERPLEXITY, precision=64)
    g64, z64 = s64.gradient()
    grad_rel = float(np.linalg.norm(g32 - g64) / np.linalg.norm(g64))
    s64.run(STEP_IT0, STEP_IT0 + args.warmup, **sched)
    k64 = max(10, min(args.steps, 100))
    s64.run(STEP_IT0 + args.warmup, STEP_IT0 + args.warmup + k64, **sched)
    fp64_ms = s64.stage_times()[8]
    s64.close()
    fp64_value = k64 / (fp64_ms / 1e3)

    # timed steps on the production path (graph-captured chunks, no per-iteration host
    # round trip), then a short run with per-stage events (host path) for the stage split
    s32.set_timing(False)
    s32.run(STEP_IT0, STEP_IT0 + args.warmup, **sched)
    barrier(world)
    it_a = STEP_IT0 + args.warmup
    it_b = it_a + args.steps
    with ClockSampler(local) as clk:
        t1 = time.perf_counter()
        s32.run(it_a, it_b, **sched)
        wall = time.perf_counter() - t1
    run_ms = reduce_max(s32.stage_times()[8], world)
    launches = int(s32.stage_times()[9])
    shapes = s32.launch_shapes()
    s32.set_timing(True)
    k_st = max(10, min(args.steps, 60))
    s32.run(it_b, it_b + k_st, **sched)
    st = s32.stage_times()
    s32.close()
    value = world * args.steps / (run_ms / 1e3)
    attr_ms = st[4]
    abytes = attraction_bytes(N, nnz)
    achieved = abytes / (attr_ms / 1e3) / 1e9

    # end to end: data on the host -> embedding on the host, full schedule.  The headline
    # is the FP32 form with the learned calibration warm start; the same call with the
    # reference's bisection, and the plain FP64 form (bisection) beside it.
    e2e = None
    if not args.skip_e2e:
        rng = np.random.default_rng(1)
        Y0 = rng.standard_normal((N, 2)) * 1e-4
        os.environ.setdefault("FITSNE_QUIET", "1")
        iters = SCHEDULE["max_iter"]

        def timed_run(calibration, bits):
            fitsne.set_calibration(calibration)
            fitsne.set_precision(bits)
            try:
                t = time.perf_counter()
                Yo, c = fitsne.run(X, Y0=Y0, perplexity=PERPLEXITY, learning_rate=N / 12.0, knn_algo=2, **SCHEDULE)
                secs = reduce_max(time.perf_counter() - t, world)
                cs = fitsne.calibration_stats()
            finally:
                fitsne.set_calibration("bisection")
                fitsne.set_precision(32)
            cal_ms = cs["ms_harvest"] + cs["ms_train"] + cs["ms_infer"] + cs["ms_warm"]
            return Yo, c, secs, cal_ms, cs

        Yout, costs, e2e_s, cal_ms, cs = timed_run("learned", 32)
        _, costs_b, e2eb_s, calb_ms, csb = timed_run("bisection", 32)
        _, costs64, e2e64_s, cal64_ms, _ = timed_run("bisection", 64)
        e2e = {"value": world * iters / e2e_s, "unit": "iters/s", "seconds": e2e_s,
               "h2d_bytes_per_step": int((X.nbytes + Y0.nbytes) / iters),
               "d2h_bytes_per_step": int((Yout.nbytes + 16 * iters + 8 * (iters // 50)) / iters),
               "note": "whole fitsne_run (similarities with the learned calibration warm start + %d iterations), "
                       "bytes averaged per iteration" % iters,
               "final_kl": float(costs[-1]), "calibration_ms": cal_ms,
               "calibration": {"rows_bisection": cs["rows_harvest"], "evals_per_bisection_row": cs["evals_plain"],
                               "evals_per_predicted_row": cs["evals_warm"], "train_steps": cs["train_steps"],
                               "ms_harvest": cs["ms_harvest"], "ms_train": cs["ms_train"],
                               "ms_infer": cs["ms_infer"], "ms_warm": cs["ms_warm"]},
               "bisection": {"seconds": e2eb_s, "value": world * iters / e2eb_s, "final_kl": float(costs_b[-1]),
                             "calibration_ms": calb_ms, "evals_per_row": csb["evals_plain"]},
               "plain_fp64": {"seconds": e2e64_s, "final_kl": float(costs64[-1]), "calibration_ms": cal64_ms,
                              "speedup": e2e64_s / e2e_s}}

    cpu = None
    on_cpu_inputs = None
    grad_vs_oracle = None
    if rank == 0 and not args.skip_cpu:
        import oracle
        oracle.build_restated()
        orc = oracle.Restated()
        cores = os.cpu_count() or 1
        # the FP32 gradient at the bench's starting state against the restated reference
        # gradient (FP64) on the identical Y and P: the reference's P built as TSNE::run does
        Pr = reference_P(fitsne, X, PERPLEXITY, K_NEIGH)
        dg, zg = fitsne.fft_gradient(*Pr, Yburn)
        dr, zr = orc.fft_gradient(*Pr, Yburn, 3, 1.0, 50, cores, 1.0)
        grad_vs_oracle = {"rel_l2": float(np.linalg.norm(dg - dr) / np.linalg.norm(dr)),
                          "z_rel": abs(zg - zr) / zr, "state": "iteration %d of the reference schedule" % STEP_IT0}
        del Pr, dg, dr
        # the CPU leg: the restated reference on all host cores
        P = cpu_sample_P(orc, labels, sizes)
        n, secs = time_cpu_steps(orc, P, Yst, args.warmup, args.cpu_steps, cores)
        cpu = {"value": n / secs, "unit": "iters/s", "cores": cores, "kind": "port",
               "sample": "%d post-exaggeration iterations of the restated reference at N=%d, 2-D, after %d untimed "
                         "ones from the synthetic state" % (n, N, args.warmup)}
        # the GPU on exactly those inputs and steps: P and start state of the CPU leg, the same
        # untimed steps, then the same number of timed steps (device time of the call)
        sc = fitsne.Session(*P, Yst, precision=32)
        try:
            sc.run(STEP_IT0, STEP_IT0 + args.warmup, **sched)
            sc.run(STEP_IT0 + args.warmup, STEP_IT0 + args.warmup + n, **sched)
            ms_a = sc.stage_times()[8]
            k_long = max(n, 100)
            sc.run(STEP_IT0 + args.warmup + n, STEP_IT0 + args.warmup + n + k_long, **sched)
            ms_b = sc.stage_times()[8]
        finally:
            sc.close()
        on_cpu_inputs = {"value": n / (ms_a / 1e3), "unit": "iters/s", "steps": n, "same_inputs": True,
                         "vs_cpu": (n / (ms_a / 1e3)) / cpu["value"], "nnz": int(P[0][-1]),
                         "value_next_%d_steps" % k_long: k_long / (ms_b / 1e3),
                         "note": "P (random within-cluster lists) and start state of the CPU leg, the same %d untimed "
                                 "steps, then the same %d timed steps (device time)" % (args.warmup, n)}
        del P

    batch = None
    if rank == 0 and not args.skip_batch:
        batch = batch_measure(fitsne, args.jobs)
    sims = None
    if rank == 0 and not args.skip_batch:
        sims = similarity_measure(fitsne, N)
        sims.pop("stage_log", None)

    if rank != 0:
        return 0
    line = {"metric": METRIC, "value": value, "unit": "iters/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": run_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (double-float coordinates, FP64 reductions)",
            "data": "synthetic (seeded Gaussian mixture)", "config": config(args, "GB300 sm_103a kernels"),
            "roofline": {"bound": "hbm", "kernel": "attraction + update (k_attr)", "achieved": achieved,
                         "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": ATTR_TRAFFIC_RATIO * abytes, "bytes_per_launch": abytes,
                         "ms_per_launch": attr_ms},
            "stage_ms": {"centre_minmax": st[0], "spread": st[1], "fft_conv": st[2], "gather": st[3],
                         "attraction_update": st[4], "iteration": st[5], "boxes_per_dim": st[6], "fft_len": st[7],
                         "note": "per-stage CUDA events over %d further steps on the host path (one min/max round "
                                 "trip per iteration, inside the spread stage); value and ms_per_step are the "
                                 "graph-captured production path" % k_st},
            "launch_shapes": shapes, "nnz": nnz, "wall_ms_per_step": 1e3 * wall / args.steps, "setup_s": setup_s,
            "state_extent": float(np.abs(Yburn).max()),
            "plain_fp64": {"value": fp64_value, "unit": "iters/s", "steps": k64, "speedup": value / fp64_value},
            "grad_rel_l2_vs_fp64": grad_rel, "Z": z32,
            "grad_rel_l2_vs_oracle": grad_vs_oracle["rel_l2"] if grad_vs_oracle else None,
            "grad_vs_oracle": grad_vs_oracle, "on_cpu_inputs": on_cpu_inputs, "batch": batch, "similarities": sims,
            "gpu_launches": launches, "clocks": clk.summary(), "cpu_baseline": cpu, "e2e": e2e}
    print(json.dumps(line))
    return 0


def similarity_measure(fitsne, n, shuffle=False, reps=2):
    """The input-similarity stage alone on the GPU, as fitsne_run runs it (P built on the
    device from the host X and kept there: X upload, centring and scaling, exact kNN,
    calibration, symmetrisation, normalisation), with the tcgen05 candidate search against the
    tensor roofline.  Stage seconds come from the library's own timing lines."""
    X, _, _ = mixture(n)
    if shuffle:  # rows in random order instead of grouped by cluster
        X = X[np.random.default_rng(11).permutation(n)]
    Y0 = np.zeros((n, 2))
    had = os.environ.get("FITSNE_TIMING")
    os.environ["FITSNE_TIMING"] = "1"
    times = []
    try:
        for rep in range(reps):
            with tempfile.TemporaryFile(mode="w+") as log:
                fd = sys.stderr.fileno()
                saved = os.dup(fd)
                os.dup2(log.fileno(), fd)
                try:
                    t0 = time.perf_counter()
                    sess = fitsne.Session.from_data(X, Y0, perplexity=PERPLEXITY, precision=32)
                    t1 = time.perf_counter()
                    sess.close()
                finally:
                    os.dup2(saved, fd)
                    os.close(saved)
                log.seek(0)
                text = log.read()
            times.append((t1 - t0, text))
    finally:
        if had is None:
            del os.environ["FITSNE_TIMING"]
        else:
            os.environ["FITSNE_TIMING"] = had
    total_s, text = times[-1]

    def after(key, stop=" s"):
        return float(text.split(key)[1].split(stop)[0]) if key in text else None
    cand_s = after(", candidates ")
    knn_s = after("tcgen05 candidates): ") or after("FP32 candidates): ")
    cal_s = after("calibration: ")
    sym_s = after("symmetrisation: ")
    kept = float(text.split("tile pairs computed ")[1].split("%")[0]) / 100 if "tile pairs computed " in text else 1.0
    peak, kind = bf16_peak()
    # tensor work issued: per computed (128-query, 64-point) tile pair three BF16 products of
    # K = 64 (D = 50 padded with the folded norm columns)
    npad = -(-n // 128) * 128
    flops = kept * (npad / 128) * (npad / 64) * 2.0 * 128 * 64 * 64 * 3
    dense = 2.0 * n * n * D_IN
    return {"metric": "similarity stage seconds (host X to P resident on the device)", "value": total_s,
            "unit": "s", "workload": "N=%d x D=50 Gaussian mixture, perplexity 30, K=90" % n,
            "row_order": "shuffled" if shuffle else "grouped by cluster",
            "knn_s": knn_s, "candidate_search_s": cand_s, "calibration_s": cal_s, "symmetrisation_s": sym_s,
            "stage_log": text.strip().splitlines(),
            "roofline": {"bound": "tensor", "kernel": "tcgen05 kNN candidate search (k_knn_tc)",
                         "achieved": flops / cand_s / 1e12 if cand_s else None, "peak": peak, "peak_kind": kind,
                         "unit": "TFLOP/s", "frac": flops / cand_s / 1e12 / peak if cand_s else None,
                         "flops": flops, "tile_pairs_computed": kept,
                         "dense_equivalent_tflops": dense / cand_s / 1e12 if cand_s else None,
                         "note": "tensor flops issued (computed tile pairs x 128 x 64 x 64 x 2 x 3 split products) "
                                 "over the host-clock time of the candidate phase (ordering, bounds, BF16 planes, "
                                 "kernel); dense_equivalent = 2 N^2 D over the same time"}}


def run_similarities(args, world, rank):
    """The input-similarity stage alone (kNN + calibration + symmetrisation) on the GPU."""
    if rank != 0:
        return 0
    import fitsne
    m = similarity_measure(fitsne, args.n, args.shuffle, 1 + args.warmup // 3)
    line = {"metric": m.pop("metric"), "value": m.pop("value"), "unit": m.pop("unit"), "n_gpus": 1,
            "higher_is_better": False, "data": "synthetic (seeded Gaussian mixture)",
            "config": {"workload": m.pop("workload"), "row_order": m.pop("row_order")}}
    line.update(m)
    print(json.dumps(line))
    return 0


def batch_jobs(njobs=64, seed=5):
    """Batched workload: N log-uniform in [2,000, 50,000], D = 50 Gaussian mixtures with
    5-30 clusters (Dirichlet(2) weights, std U(0.5, 2), centres N(0, 25 I)), perplexity
    10 / 30 / 50 cycled (K = 3 perplexity), learning rate max(200, N / 12)."""
    rng = np.random.default_rng(seed)
    jobs = []
    for j in range(njobs):
        N = int(round(np.exp(rng.uniform(np.log(2000), np.log(50000)))))
        k = int(rng.integers(5, 31))
        w = rng.dirichlet(np.full(k, 2.0))
        lab = np.repeat(np.arange(k), rng.multinomial(N, w))
        c = rng.standard_normal((k, D_IN)) * 5.0
        X = c[lab] + rng.standard_normal((N, D_IN)) * rng.uniform(0.5, 2.0, k)[lab, None]
        jobs.append((X, (10.0, 30.0, 50.0)[j % 3], max(200.0, N / 12.0)))
    return jobs


def batch_measure(fitsne, njobs, one_by_one=True):
    """The batched form (fitsne_batch_run) on the batch_jobs workload, and the same jobs one
    by one through fitsne_run."""
    jobs = batch_jobs(njobs)
    Xs = [j[0] for j in jobs]
    perps = [j[1] for j in jobs]
    lrs = [j[2] for j in jobs]
    rng = np.random.default_rng(9)
    Y0s = [rng.standard_normal((len(X), 2)) * 1e-4 for X in Xs]
    iters = 1000
    t0 = time.perf_counter()
    Ys, costs, st = fitsne.batch_run(Xs, perps, learning_rates=lrs, Y0s=Y0s, max_iter=iters)
    batch_s = time.perf_counter() - t0
    n = [len(X) for X in Xs]
    out = {"metric": "batched t-SNE: aggregate iterations/s over %d independent embeddings" % len(jobs),
           "value": len(jobs) * iters / batch_s, "unit": "iters/s",
           "workload": "%d jobs, N log-uniform in [2000, 50000] (total %d points), D=50, 5-30 clusters, "
                       "perplexity 10/30/50 cycled, 2-D, df=1, %d iterations" % (len(jobs), sum(n), iters),
           "batch_seconds": batch_s, "similarity_seconds": st["similarity_s"], "iterate_seconds": st["iterate_s"],
           "iterate_iters_per_s": len(jobs) * iters / st["iterate_s"], "graph_launches": st["graph_launches"],
           "graph_instantiations": st["graph_instantiations"], "chunks_redone": st["chunks_redone"]}
    if one_by_one:
        t1 = time.perf_counter()
        single_kl = []
        for X, p, lr, Y0 in zip(Xs, perps, lrs, Y0s):
            _, c = fitsne.run(X, Y0=Y0, perplexity=p, learning_rate=lr, max_iter=iters, knn_algo=2)
            single_kl.append(c[-1])
        single_s = time.perf_counter() - t1
        out.update({"one_by_one_seconds": single_s, "speedup_vs_one_by_one": single_s / batch_s,
                    "max_final_kl_rel_dev_vs_one_by_one": max(abs(c[-1] - k) / k for c, k in zip(costs, single_kl))})
    return out


def run_batch(args, world, rank):
    """The batched form (fitsne_batch_run) against the same jobs run one by one."""
    if rank != 0:
        return 0
    import fitsne
    b = batch_measure(fitsne, args.jobs)
    line = {"metric": b.pop("metric"), "value": b.pop("value"), "unit": b.pop("unit"), "n_gpus": 1,
            "higher_is_better": True, "data": "synthetic (seeded Gaussian mixtures)",
            "config": {"workload": b.pop("workload")}}
    line.update(b)
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=1_000_000)
    ap.add_argument("--cpu-steps", type=int, default=4)
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-batch", action="store_true")
    ap.add_argument("--stage", default="iteration", choices=["iteration", "similarities", "batch"])
    ap.add_argument("--jobs", type=int, default=64)
    ap.add_argument("--shuffle", action="store_true", help="similarity stage: rows in random order")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    world, rank, local = dist_setup()
    if world > 1:
        if args.impl == "reference":
            return run_reference(args, world, rank)
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.impl == "reference":
        rc = run_reference(args, world, rank)
    elif args.stage == "similarities":
        rc = run_similarities(args, world, rank)
    elif args.stage == "batch":
        rc = run_batch(args, world, rank)
    else:
        rc = run_gb300(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
