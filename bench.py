#!/usr/bin/env python3
"""Lasso time-to-gap benchmark of the GB300 PCDM library.

Workload (default): the large single Lasso of the reference's headline metric:
A is 1,000,000 x 10,000,000 with Zipf(1.5) column lengths clipped to [1, 2000]
and rescaled to mean 20 (about 2.0e8 nonzeros), uniform distinct rows, N(0,1)
values scaled to unit columns; x* has 10,000 entries +-1; b = A x* + N(0, 0.01^2);
lambda = 0.05 ||A^T b||_inf.  Seeded synthetic data (no dataset is shipped).
PCDM with tau = 4096, FP32 bulk with FP64 refresh and duality gap every 5 epochs,
q-shrinking (q = 0.9) after 5 epochs with 1024 updates in flight on the active
set, 50 active-set passes between refreshes, screened evaluations and the
hot-set tier (threshold 0.1); target relative duality gap 1e-6.

A step is one solve from x = 0 to the target gap with the matrix resident in
HBM; value is the mean time-to-gap in seconds (lower is better), timed with
CUDA events on the library's stream.  e2e repeats the same metric through the
C-ABI from pinned host buffers (upload, device layout build, solve, x read back).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs N independent replicas (one per GPU, no collective on the data
path); value is the slowest replica's time-to-gap.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "ac-dc_gb300")
ORACLE = os.path.join(ROOT, "oracle")
sys.path.insert(0, PKG)

WORKLOADS = {
    "lasso_m1e6_n1e7_zipf": dict(m=1_000_000, n=10_000_000, nnz_mode=1, zipf_s=1.5, nnz_min=1,
                                 nnz_max=2000, nnz_mean=20.0, n_star=10_000, noise_sigma=0.01,
                                 lambda_frac=0.05, seed=0xACDC0001, tau=4096, refresh_every=5,
                                 gap=1e-6, max_epochs=12000, tau_active=1024, active_passes=50),
    # the same generator at 3e5 x 3e6 (about 6e7 nonzeros): small enough for full
    # profiler captures
    "lasso_m3e5_n3e6_zipf": dict(m=300_000, n=3_000_000, nnz_mode=1, zipf_s=1.5, nnz_min=1,
                                 nnz_max=2000, nnz_mean=20.0, n_star=3_000, noise_sigma=0.01,
                                 lambda_frac=0.05, seed=0xACDC0001, tau=4096, refresh_every=5,
                                 gap=1e-6, max_epochs=3000, tau_active=1024, active_passes=100),
    # the reference's CPU-sized case (2,000 x 10,000, 20 per column), for quick checks
    "lasso_m2e3_n1e4": dict(m=2000, n=10000, nnz_mode=0, nnz_per_col=20, n_star=100,
                            noise_sigma=0.01, lambda_frac=0.1, seed=0xACDC0000, tau=64,
                            refresh_every=2, gap=1e-6, max_epochs=3000, tau_active=64, active_passes=20),
    # hinge-loss SVM dual: 20,000 samples x 1,355,191 features, log-normal sample
    # lengths (median 450, sigma 0.8), Exp(1) values scaled to unit rows, labels of
    # a sparse w* (5,000 entries) with 5% flips, lambda = 1e-4, synchronous
    # mini-batch SDCA with batches of 1024 distinct samples, gap checked every
    # epoch (n / 1024 steps), absolute duality gap 1e-5
    "svm_n2e4_d1355191": dict(loss="svm", m=1_355_191, n=20_000, nnz_median=450.0,
                              nnz_sigma=0.8, w_star_nnz=5000, flip_prob=0.05, lam=1e-4,
                              seed=0xACDC0002, tau=1024, refresh_every=1, gap=1e-5,
                              max_epochs=3000, minibatch=1),
}
METRICS = {"lasso": "lasso_time_to_gap_1e-6", "svm": "svm_time_to_gap_1e-5"}
# Kernels launched per evaluation (refresh: init, scatter, finish; Lasso gap:
# short, long, finalize; SVM gap: one pass, finalize) and per reset (set_x +
# refresh).
KERNELS_PER_EVAL = 6
KERNELS_PER_EVAL_SVM = 5
# Lasso with shrinking: a full evaluation adds the active-set violations, the
# active-set omega (row count, max) and the hot set (mark, collect); a screened
# one is refresh (3), the active-column pass, finalize and the hot set (2).
KERNELS_PER_EVAL_SHRINK = 11
KERNELS_PER_EVAL_SCREENED = 7
KERNELS_PER_RESET = 4
# Columns of the update kernel's algorithmic bytes (FP32 values and state, int32
# indices): every update reads 12 bytes per entry (value, row index, residual
# gather) and 16 bytes of column record (start, length, Li, x); a nonzero step
# adds 4 bytes per entry (residual scatter) and 4 bytes (x write).
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC_FILE = os.path.join(ROOT, "profiles", "k_pcdm_update_traffic.json")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="lasso_m1e6_n1e7_zipf", choices=sorted(WORKLOADS))
    ap.add_argument("--e2e-steps", type=int, default=3,
                    help="end-to-end solves through the C-ABI from host buffers (mean reported)")
    ap.add_argument("--lanes", type=int, default=0, choices=[-1, 0, 1, 8, 16, 32],
                    help="update kernel (settings.lanes_per_update): 0 the lean kernel for "
                         "the q-shrinking launches, 1 the lean kernel for all, -1 the ring "
                         "kernel for all, 8/16/32 the grouped kernel")
    ap.add_argument("--cpu-budget", type=float, default=20.0,
                    help="seconds of computation for the CPU baseline run of the workload")
    ap.add_argument("--ref-step-seconds", type=float, default=0,
                    help="--impl reference: computation seconds per step (0 = 120 / steps, at least 2)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--max-epochs", type=int, default=0,
                    help="cap each solve (profiling runs; the line then reports converged=false)")
    ap.add_argument("--batch-instances", type=int, default=64,
                    help="instances of the batched lambda-path sample (0 = skip)")
    ap.add_argument("--batch-max-epochs", type=int, default=200)
    ap.add_argument("--svm-steps", type=int, default=10,
                    help="solves of the SVM-dual workload reported under the line's svm key "
                         "(0 = skip)")
    ap.add_argument("--serve-requests", type=int, default=256,
                    help="requests of the serving sample at each rate (0 = skip)")
    ap.add_argument("--serve-rate", type=float, default=0.0,
                    help="one arrival rate per second (0 = the sweep 50..2000)")
    ap.add_argument("--serve-quantum", type=int, default=4,
                    help="rounds per server step (acdc_server_options.quantum_epochs)")
    ap.add_argument("--active-passes", type=int, default=0,
                    help="passes over the active set per bulk while q-shrinking (Lasso; "
                         "0 = the workload's own, 50 for the 1e6 x 1e7 Lasso)")
    ap.add_argument("--probe-repeat", type=int, default=1,
                    help="--probe-launches: active-set launches to time (the first is counted)")
    ap.add_argument("--probe-launches", action="store_true",
                    help="profiling aid: run one uniform-draw update launch (refresh_every "
                         "epochs) and one active-set launch (active_passes |A|/q updates) on "
                         "the workload and print their work counters")
    return ap.parse_args()


def update_kernel_label(s, w):
    """The update kernels a solve with settings s launches."""
    if is_svm(w) and s.minibatch:
        return "k_sdca_phase1 + k_sdca_phase2 (synchronous mini-batch steps)"
    lanes = s.lanes_per_update
    if lanes in (8, 16, 32):
        return "k_pcdm_update_grouped<%d>" % lanes
    if lanes == 1:
        return "k_pcdm_update_lean"
    if lanes == 0 and s.use_shrinking:
        return "k_pcdm_update (uniform bulks) + k_pcdm_update_lean (q-shrinking bulks)"
    return "k_pcdm_update"


def bulk_phases(traces, s):
    """Update bulks of the timed solves by kind (from the solve traces): uniform
    draws, q-shrinking draws, and either in FP64.  Per kind: bulks, updates,
    event-timed milliseconds, updates/s, the updates in flight (tau or
    tau_active) and the microseconds one update takes at that many in flight
    (in flight x time / updates)."""
    out = {}
    for rows in traces:
        prev = 0
        for row in rows[1:]:
            n = row["updates"] - prev
            prev = row["updates"]
            kind = ("active" if row["shrink"] else "uniform") + ("_fp64" if row["fp64"] else "")
            k = out.setdefault(kind, {"bulks": 0, "updates": 0, "ms": 0.0})
            k["bulks"] += 1
            k["updates"] += n
            k["ms"] += row["update_ms"]
    for kind, k in out.items():
        fly = s.tau_active if kind.startswith("active") and s.tau_active > 0 else s.tau
        k["in_flight"] = fly
        k["updates_per_s"] = k["updates"] / (k["ms"] * 1e-3) if k["ms"] > 0 else None
        k["us_per_update_in_flight"] = (fly * k["ms"] * 1e3 / k["updates"]) if k["updates"] else None
    return out


def probe_launches(w):
    """Two update launches of known size for a profiler capture: a uniform bulk
    from x = 0, then (after a full evaluation built the active set) one bulk of
    active-set draws, without the hot tier."""
    import acdc
    inst = generate(w, pinned=False)
    ctx = acdc.Context(0)
    s = settings_for(w)
    s.hot_threshold = 0.0
    p = acdc.Problem(ctx, inst, s)

    def timed(count):
        # host clock around one launch with the stream drained on both sides
        # (includes the launch overhead, a few microseconds)
        p.synchronize()
        t = time.perf_counter()
        p.run_updates(count)
        p.synchronize()
        return (time.perf_counter() - t) * 1e3

    t1 = timed(w["refresh_every"] * inst.n)
    first = p.stats()
    ev = p.evaluate()
    count = int(w["active_passes"] * ev["active"] / 0.9)
    p.reset_stats()
    t2 = timed(count)
    second = p.stats()
    # further active-set launches of the same size (same active set) for timing
    more = [timed(count) for _ in range(max(0, w.get("probe_repeat", 1) - 1))]
    print(json.dumps({"workload": w.get("name"), "lanes_per_update": s.lanes_per_update,
                      "uniform_launch": dict(first, host_ms=t1),
                      "active_launch": dict(second, active_set=ev["active"], host_ms=t2,
                                            repeat_host_ms=more)}),
          flush=True)
    p.close()
    ctx.close()
    return 0


def batch_sample(count, seed=0xACDC0003, only=None):
    """Instances of the batched lambda-path workload: m log-uniform in [500, 50,000],
    n log-uniform in [1,000, 200,000], 5..50 entries per column, each with the
    16-point path lambda_max 0.5^k, k = 1..16.  `only` restricts the sample to
    those indices (a rank's shard); instance i is the same either way."""
    import acdc
    import numpy as np
    insts = []
    for i in (range(count) if only is None else only):
        m, n = acdc.mix_sizes(seed, i)
        insts.append(acdc.gen_lasso(m, n, nnz_mode=acdc.NNZ_UNIFORM, nnz_min=5, nnz_max=50,
                                    n_star=max(1, n // 100), lambda_frac=1.0, seed=seed + i))
    lams = np.array([[x.lam * 0.5 ** k for k in range(1, 17)] for x in insts]).reshape(-1, 16)
    return insts, lams


def shard_by_footprint(footprints, world):
    """Independent instances dealt to `world` ranks by device footprint: largest
    first, each to the rank with the least bytes so far (ties to the lower rank).
    Returns one sorted index list per rank.  No data moves between ranks."""
    loads = [0] * world
    shards = [[] for _ in range(world)]
    for i in sorted(range(len(footprints)), key=lambda k: (-footprints[k], k)):
        r = min(range(world), key=lambda k: (loads[k], k))
        shards[r].append(i)
        loads[r] += footprints[i]
    return [sorted(x) for x in shards]


def batch_footprints(count, seed=0xACDC0003):
    """Expected device bytes of the batched sample's instances from their sizes
    alone (27.5 entries per column on average), so every rank can shard the
    sample without generating it."""
    import acdc
    out = []
    for i in range(count):
        m, n = acdc.mix_sizes(seed, i)
        out.append(20 * 27.5 * n + 136 * n + 32 * m)
    return out


def run_batched(ctx, count, max_epochs, rank=0, world=1, dist=None, dev=None):
    """Batched solves/s of the lambda-path sample against the plain one-instance
    path on the same instances (both with q-shrinking, gap 1e-6 per lambda).
    With several ranks each solves its shard of the instances (dealt by
    footprint, no collective on the data path); solves/s is all ranks' solves
    over the slowest rank's time."""
    import acdc
    shards = shard_by_footprint(batch_footprints(count), world) if world > 1 else [list(range(count))]
    mine = shards[rank]
    insts, lams = batch_sample(count, only=mine)
    out = {"workload": "lasso_paths_mix", "instances": count, "lambdas_per_instance": 16,
           "solves": count * 16, "gap_target_relative": 1e-6, "max_epochs_per_lambda": max_epochs,
           "sizes": "m logU[500,5e4], n logU[1e3,2e5], 5..50 per column (the 512-instance "
                    "workload's distribution, first %d instances)" % count,
           "nnz": int(round(sum_over_ranks(dist, sum(x.nnz for x in insts), dev))),
           "shards": [len(x) for x in shards],
           "scaling": "strong: the sample's instances dealt to the ranks by footprint"}
    warm_tuner(ctx, (insts, []))
    conv_mask = {}
    for plain in (0, 1):
        probs = [acdc.Problem(ctx, x) for x in insts]
        for q in probs:
            q.synchronize()
        if dist is not None:
            dist.barrier()
        t = time.perf_counter()
        res, _ = (acdc.batch_solve_path(ctx, probs, lams, gap_target=1e-6, max_epochs=max_epochs,
                                        refresh_every=2, autotune=1, plain=plain, use_shrinking=1)
                  if probs else ([], None))
        dt = max_over_ranks(dist, time.perf_counter() - t, dev)
        for q in probs:
            q.close()
        key = "plain" if plain else "batched"
        conv_mask[key] = [[bool(r.converged) for r in row] for row in res]
        # tau per instance: the measured autotuner's choice (cached per size class)
        taus = {}
        for row in res:
            if len(row):
                taus[int(row[0].tau)] = taus.get(int(row[0].tau), 0) + 1
        conv = sum(r.converged for row in res for r in row)
        conv = int(round(sum_over_ranks(dist, conv, dev)))
        out[key] = {"seconds": dt, "all_solves_per_s": count * 16 / dt, "converged": conv,
                    "converged_per_s": conv / dt,
                    "converged_per_lambda": [sum(row[k] for row in conv_mask[key])
                                             for k in range(16)],
                    "tau_chosen": {str(t): c for t, c in sorted(taus.items())}}
    # the metric: solves that reached the gap in both paths, per second of each
    both = sum(a and b for ra, rb in zip(conv_mask["batched"], conv_mask["plain"])
               for a, b in zip(ra, rb))
    both = int(round(sum_over_ranks(dist, both, dev)))
    out["converged_in_both"] = both
    neither = sum((not a) and (not b) for ra, rb in zip(conv_mask["batched"], conv_mask["plain"])
                  for a, b in zip(ra, rb))
    out["neither_converged"] = int(round(sum_over_ranks(dist, neither, dev)))
    for key in ("batched", "plain"):
        out[key]["solves_per_s"] = both / out[key]["seconds"]
    out["speedup"] = out["batched"]["solves_per_s"] / out["plain"]["solves_per_s"]
    out["metric_rule"] = ("solves_per_s counts the lambda points both paths solved to the gap "
                          "target, over each path's own time (which includes the points that "
                          "hit the epoch cap)")
    return out


SERVE_RATES = (50, 100, 200, 500, 1000, 2000)
SERVE_MAX_EPOCHS = 1000  # per request, both paths


def serve_pool(seed=0xACDC0004, lasso=24, svm=8, pinned=True):
    """Instances the serving requests draw from: Lasso problems of the lambda-path
    mix's size distribution, unscaled (m log-uniform in [500, 50,000], n in
    [1,000, 200,000], 5..50 entries per column), and SVM duals from the SVM
    generator with samples log-uniform in [1,000, 50,000] and the features
    scaled with them (1,355,191 per 20,000 samples), median 450 entries per
    sample, lambda = 1e-4.  A pool keeps the host memory of a long request
    stream bounded: requests share matrices, not device state."""
    import acdc
    las, svs = [], []
    for i in range(lasso):
        m, n = acdc.mix_sizes(seed, i)
        las.append(acdc.gen_lasso(m, n, nnz_mode=acdc.NNZ_UNIFORM, nnz_min=5, nnz_max=50,
                                  n_star=max(1, n // 100), lambda_frac=1.0, seed=seed + i,
                                  pinned=pinned))
    for i in range(svm):
        _, ns = acdc.mix_sizes(seed + 0x10, i, n_lo=1000, n_hi=50000)
        d = max(1000, int(round(ns * 1355191 / 20000)))
        svs.append(acdc.gen_svm(ns, d, nnz_median=450, nnz_sigma=0.8,
                                w_star_nnz=max(10, ns // 4), lam=1e-4, seed=seed + 0x10 + i,
                                pinned=pinned))
    return las, svs


def serve_sample(pool, count, rate, seed=0xACDC0004):
    """A request stream: 70% Lasso (a pool instance at lambda = lambda_max 0.5^k,
    k uniform in 1..5: further along the 16-point path some underdetermined
    instances need thousands of epochs),
    30% SVM duals (a pool instance); Poisson arrivals at `rate` per second.
    Returns (instance, lambda, seed) per request and the arrival times."""
    import numpy as np
    las, svs = pool
    rng = np.random.default_rng(seed + int(rate))
    reqs = []
    for i in range(count):
        if rng.random() < 0.7:
            inst = las[int(rng.integers(len(las)))]
            reqs.append((inst, inst.lam * 0.5 ** int(rng.integers(1, 6)), i + 1))
        else:
            inst = svs[int(rng.integers(len(svs)))]
            reqs.append((inst, inst.lam, i + 1))
    arrivals = np.cumsum(rng.exponential(1.0 / rate, count))
    return reqs, arrivals


def latency_summary(lat_s, span_s, conv, count):
    import numpy as np
    lat = np.array(lat_s) * 1e3
    return {"solves_per_s": count / span_s, "converged": int(conv),
            "converged_per_s": conv / span_s, "p50_ms": float(np.percentile(lat, 50)),
            "p90_ms": float(np.percentile(lat, 90)), "p99_ms": float(np.percentile(lat, 99)),
            "span_s": span_s}


def serve_one_rate(ctx, pool, count, rate, quantum):
    """Continuous batching (acdc_server_*) against the plain path (one request at
    a time through acdc_batch_solve_path with plain = 1) on the same arrivals;
    latency = finish - arrival on the host's monotonic clock."""
    import acdc
    import numpy as np
    reqs, arr = serve_sample(pool, count, rate)
    out = {"rate_per_s": rate, "requests": count}
    srv = acdc.Server(ctx, memory_budget_bytes=120 << 30, max_slots=256, quantum_rounds=quantum,
                      max_epochs=SERVE_MAX_EPOCHS, use_shrinking=1)
    start = time.monotonic()
    tickets, nxt = {}, 0
    while True:
        now = time.monotonic() - start
        while nxt < count and arr[nxt] <= now:
            inst, lam, seed = reqs[nxt]
            tickets[nxt] = srv.submit(inst, lam=lam, gap_target=1e-6, seed=seed)
            nxt += 1
        pend = srv.step()
        if nxt >= count and pend == 0:
            break
        if pend == 0 and nxt < count:
            time.sleep(max(0.0, min(0.002, arr[nxt] - (time.monotonic() - start))))
    lat, fin, conv = [], [], 0
    for i in range(count):
        res, _ = srv.poll(tickets[i])
        lat.append(res.finish_time - (start + arr[i]))
        fin.append(res.finish_time - start)
        conv += res.converged
    out["server_stats"] = srv.stats()
    srv.close()
    out["server"] = latency_summary(lat, max(fin) - arr[0], conv, count)
    start = time.monotonic()
    lat, fin, conv = [], [], 0
    for i in range(count):
        now = time.monotonic() - start
        if now < arr[i]:
            time.sleep(arr[i] - now)
        inst, lam, seed = reqs[i]
        q = acdc.Problem(ctx, inst, seed=seed)
        res, _ = acdc.batch_solve_path(ctx, [q], np.array([[lam]]), gap_target=1e-6,
                                       max_epochs=SERVE_MAX_EPOCHS, refresh_every=1, autotune=1,
                                       plain=1, want_x=True, use_shrinking=1)
        q.close()
        t = time.monotonic() - start
        lat.append(t - arr[i])
        fin.append(t)
        conv += res[0][0].converged
    out["plain"] = latency_summary(lat, max(fin) - arr[0], conv, count)
    out["speedup"] = out["server"]["solves_per_s"] / out["plain"]["solves_per_s"]
    return out


def warm_tuner(ctx, pool):
    """Untimed: one capped solve of every pool instance, so that the autotuner's
    per-size-class choice of tau is cached on the context before either path
    is timed (both paths then use the same cached choices)."""
    import acdc
    import numpy as np
    for inst in pool[0] + pool[1]:
        q = acdc.Problem(ctx, inst, seed=1)
        acdc.batch_solve_path(ctx, [q], np.array([[inst.lam]]), gap_target=1e-6, max_epochs=1,
                              refresh_every=1, autotune=1, plain=1, use_shrinking=1)
        q.close()


def run_serving(ctx, count, rates, quantum=4):
    """The serving workload at each arrival rate of the sweep."""
    pool = serve_pool()
    warm_tuner(ctx, pool)
    out = {"workload": "serve_mix_70_30", "requests_per_rate": count, "quantum_rounds": quantum,
           "gap_target": 1e-6, "request_buffers": "pinned host memory (both paths)",
           "pool": {"lasso": len(pool[0]), "svm": len(pool[1]),
                    "lasso_nnz": int(sum(x.nnz for x in pool[0])),
                    "svm_nnz": int(sum(x.nnz for x in pool[1])),
                    "svm_samples": [x.n for x in pool[1]]},
           "sizes": "Lasso: the 512-instance mix's distribution unscaled; SVM: samples "
                    "logU[1e3, 5e4], features scaled with them, median 450 entries per sample"}
    out["sweep"] = [serve_one_rate(ctx, pool, count, r, quantum) for r in rates]
    top = out["sweep"][-1]
    out["rate_per_s"] = top["rate_per_s"]
    out["speedup"] = top["speedup"]
    return out


def run_svm_section(ctx, steps=10, warmup=2, cpu=True):
    """The SVM-dual workload (20,000 x 1,355,191) beside the Lasso line: time to
    absolute gap 1e-5 of the synchronous mini-batch SDCA (batch 1024) and of the
    asynchronous form (1024 in flight), each the mean of `steps` solves from
    alpha = 0 with the data resident, CUDA-event timed; the mini-batch form also
    to the gap that bounds the objective error by 1e-6 relative; the last
    solve's error against the committed FP64 optimum; and the reference's
    algorithm on the host cores (measured, capped at 60 s)."""
    import acdc
    name = "svm_n2e4_d1355191"
    w = dict(WORKLOADS[name], name=name)
    inst = generate(w, pinned=False)
    out = {"workload": name, "metric": METRICS["svm"], "unit": "s", "n": inst.n, "d": inst.m,
           "nnz": inst.nnz, "tau": w["tau"], "gap_target_absolute": w["gap"]}
    runs = [("minibatch", 1, w["gap"]), ("asynchronous", 0, w["gap"])]
    f = OPTIMA.get(name)
    if f and os.path.exists(f):
        import numpy as np
        runs.append(("minibatch_rel_1e-6", 1, 1e-6 * abs(float(np.load(f)["primal"]))))
    for key, mb, gap in runs:
        # the mini-batch form checks the gap every epoch (n / 1024 steps), as the
        # reference's loop does; the asynchronous form every 5 epochs
        ws = dict(w, minibatch=mb, gap=gap, refresh_every=1 if mb else 5)
        p = acdc.Problem(ctx, inst, settings_for(ws))
        res = []
        for i in range(warmup + steps):
            p.reset()
            p.reset_stats()
            r = p.solve()
            if i >= warmup:
                res.append(r)
        ms = [r.device_ms for r in res]
        x = p.get_x()
        out[key] = {"value": statistics.mean(ms) / 1e3, "gap_target_absolute": gap,
                    "ms": [round(v, 3) for v in ms], "epochs": [r.epochs for r in res],
                    "converged": all(r.converged for r in res), "gap": [r.eval.gap for r in res],
                    "beta": p.info().sigma,
                    "oracle": oracle_error(name, inst, x, res[-1].eval.primal)}
        st = res[-1].stats
        out[key]["updates_per_s"] = st.updates / (st.update_ms * 1e-3) if st.update_ms > 0 else None
        p.close()
    out["value"] = out["minibatch"]["value"]
    if cpu:
        threads = os.cpu_count() or 1
        run = cpu_time_to_gap(inst, threads, w["gap"], False, 60.0)
        run.pop("trace", None)
        out["cpu_reference"] = dict(run, kind="port",
                                    sample="the reference's asynchronous multicore engine (oracle "
                                           "port) on %d threads from alpha = 0 to the gap" % threads)
    return out


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def dist_init(world, backend):
    if world <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend=backend)
    return dist


def max_over_ranks(dist, value, device=None):
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, value, device=None):
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(self.NAMES, parts[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


GOLDEN = os.path.join(ROOT, "tests", "golden")
OPTIMA = {"lasso_m1e6_n1e7_zipf": os.path.join(GOLDEN, "lasso_m1e6_n1e7_optimum.npz"),
          "svm_n2e4_d1355191": os.path.join(GOLDEN, "svm_n2e4_d1355191_optimum.npz")}


def instance_digest(inst):
    """SHA-256 of the generated arrays and lambda (the fixtures record it)."""
    import hashlib
    import numpy as np
    h = hashlib.sha256()
    for a in (inst.col_ptr, inst.row_idx, inst.vals, inst.rhs):
        h.update(np.ascontiguousarray(a).tobytes())
    h.update(np.float64(inst.lam).tobytes())
    return h.hexdigest()


def duplicate_classes(inst):
    """Class id per coordinate: one-entry columns at the same row are the same
    column up to sign (the generator scales them to +-1), so any split of
    their mass is optimal; they share one class, keyed by the row.  Every other
    column is its own class.  Returns (class ids, sign of the one entry or 1)."""
    import numpy as np
    lens = np.diff(inst.col_ptr)
    one = lens == 1
    cls = np.arange(inst.n, dtype=np.int64) + inst.m
    first = inst.col_ptr[:-1][one]
    cls[one] = inst.row_idx[first]
    sign = np.ones(inst.n)
    sign[one] = np.sign(inst.vals[first])
    return cls, sign


def class_mass(cls, sign, x, idx):
    """Signed mass of each class over the coordinates idx of x."""
    mass = {}
    for c, v in zip(cls[idx].tolist(), (sign[idx] * x[idx]).tolist()):
        mass[c] = mass.get(c, 0.0) + v
    return mass


def class_support(cls, sign, x, idx=None):
    """Classes whose signed mass is nonzero."""
    import numpy as np
    idx = np.nonzero(x)[0] if idx is None else idx
    return {c for c, v in class_mass(cls, sign, x, idx).items() if v != 0.0}


def host_objective(inst, x):
    """FP64 primal objective of x on the generated (FP64) data, on the host:
    0.5||Ax - b||^2 + lambda||x||_1 for the Lasso; for the SVM dual (x = alpha)
    lambda/2 ||w||^2 + mean hinge with w = sum_i alpha_i y_i x_i / (lambda n)."""
    import numpy as np
    lens = np.diff(inst.col_ptr)
    if is_svm_inst(inst):
        coef = x * inst.rhs / (inst.lam * inst.n)
        w = np.bincount(inst.row_idx, weights=inst.vals * np.repeat(coef, lens), minlength=inst.m)
        prod = inst.vals * w[inst.row_idx]
        cs = np.concatenate([[0.0], np.cumsum(prod)])
        margin = cs[inst.col_ptr[1:]] - cs[inst.col_ptr[:-1]]
        hinge = np.maximum(0.0, 1.0 - inst.rhs * margin)
        return float(0.5 * inst.lam * w.dot(w) + hinge.mean())
    sup = np.nonzero(x)[0]
    sl = lens[sup]
    first = np.repeat(inst.col_ptr[sup] - np.concatenate([[0], np.cumsum(sl)[:-1]]), sl)
    ent = first + np.arange(int(sl.sum()))
    r = np.bincount(inst.row_idx[ent], weights=inst.vals[ent] * np.repeat(x[sup], sl),
                    minlength=inst.m) - inst.rhs
    return float(0.5 * r.dot(r) + inst.lam * np.abs(x).sum())


def is_svm_inst(inst):
    return inst.loss == 2


def oracle_error(workload, inst, x, primal):
    """The solve's error against the committed FP64 optimum of the workload
    (tests/golden/make_config_optima.py: oracle run to a gap <= 1e-9): relative
    objective error, support match raw and up to duplicate columns."""
    import numpy as np
    path = OPTIMA.get(workload)
    if not path or not os.path.exists(path):
        return None
    f = np.load(path)
    digest = instance_digest(inst)
    out = {"fixture": os.path.relpath(path, ROOT), "same_input": digest == str(f["sha256"]),
           "oracle_objective": float(f["primal"]), "oracle_gap": float(f["gap"]),
           "oracle_rel_gap": float(f["rel_gap"])}
    p_o = float(f["primal"])
    p_h = host_objective(inst, x)
    out["objective_fp64_host"] = p_h
    out["objective_device"] = primal
    out["oracle_rel_err"] = abs(p_h - p_o) / abs(p_o)
    out["oracle_rel_err_device"] = abs(primal - p_o) / abs(p_o)
    sup_o = np.asarray(f["support"], np.int64)
    sup = np.nonzero(x)[0]
    sym = np.setxor1d(sup, sup_o)
    out["support"] = int(len(sup))
    out["oracle_support"] = int(len(sup_o))
    out["support_symmetric_difference"] = int(len(sym))
    if "x_support" in f.files:
        xo = np.zeros(inst.n)
        xo[sup_o] = f["x_support"]
        out["max_abs_x_in_difference"] = float(np.abs(np.concatenate([x[sym], xo[sym]])).max()) \
            if len(sym) else 0.0
        cls, sign = duplicate_classes(inst)
        mg = class_mass(cls, sign, x, sup)
        mo = class_mass(cls, sign, xo, sup_o)
        cs = {c for c, v in mg.items() if v != 0.0}
        co = {c for c, v in mo.items() if v != 0.0}
        out["class_support"] = len(cs)
        out["oracle_class_support"] = len(co)
        out["class_symmetric_difference"] = len(cs ^ co)
        out["support_match"] = cs == co
        # the classes that differ: the solution's and the oracle's mass on each
        # (for a column class, c - m is the column; for a one-entry class, c is the row)
        out["class_differences"] = [
            {"class": int(c), "column": int(c - inst.m) if c >= inst.m else None,
             "row": int(c) if c < inst.m else None, "mass": mg.get(c, 0.0),
             "oracle_mass": mo.get(c, 0.0)} for c in sorted(cs ^ co)[:10]]
        out["support_rule"] = ("same nonzero classes; one-entry columns at one row form one class "
                               "(the same column up to sign, so the split of their mass is not unique)")
    else:
        out["support_match"] = bool(len(sym) == 0)
        out["support_rule"] = "same nonzero coordinates"
    if "alpha" in f.files:
        out["max_abs_alpha_err"] = float(np.abs(x - f["alpha"]).max())
    return out


def load_json(path, default=None):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return default


def is_svm(w):
    return w.get("loss") == "svm"


def generate(w, pinned):
    import acdc
    if is_svm(w):
        return acdc.gen_svm(w["n"], w["m"], nnz_median=w["nnz_median"], nnz_sigma=w["nnz_sigma"],
                            w_star_nnz=w["w_star_nnz"], flip_prob=w["flip_prob"], lam=w["lam"],
                            seed=w["seed"], pinned=pinned)
    if w["nnz_mode"] == 1:
        return acdc.gen_lasso(w["m"], w["n"], nnz_mode=acdc.NNZ_ZIPF, zipf_s=w["zipf_s"],
                              nnz_min=w["nnz_min"], nnz_max=w["nnz_max"], nnz_mean=w["nnz_mean"],
                              n_star=w["n_star"], noise_sigma=w["noise_sigma"],
                              lambda_frac=w["lambda_frac"], seed=w["seed"], pinned=pinned)
    return acdc.gen_lasso(w["m"], w["n"], nnz_per_col=w["nnz_per_col"], n_star=w["n_star"],
                          noise_sigma=w["noise_sigma"], lambda_frac=w["lambda_frac"],
                          seed=w["seed"], pinned=pinned)


def settings_for(w):
    import acdc
    if is_svm(w):
        return acdc.default_settings(acdc.LOSS_SVM_DUAL, tau=w["tau"], warps_per_block=8,
                                     refresh_every=w["refresh_every"], gap_target=w["gap"],
                                     gap_relative=0, max_epochs=w["max_epochs"], seed=1,
                                     precision=acdc.PREC_FP32, lanes_per_update=w.get("lanes", 0),
                                     minibatch=w.get("minibatch", 0))
    return acdc.default_settings(acdc.LOSS_L1_SQUARE, tau=w["tau"], warps_per_block=8,
                                 refresh_every=w["refresh_every"], gap_target=w["gap"],
                                 gap_relative=1, max_epochs=w["max_epochs"], use_shrinking=1,
                                 shrinking_probability=0.9, shrinking_starting_iter=5, seed=1,
                                 precision=acdc.PREC_FP32, tau_active=w["tau_active"],
                                 active_passes=w["active_passes"], lanes_per_update=w.get("lanes", 0))


def cpu_engine(inst):
    """The reference's multicore engine restated (oracle port) on an instance:
    the Lasso (MulticoreL1RegSquareLoss) or the SVM dual (MulticoreSVMDualLoss)
    with the reference's own Lipschitz constants, from x = 0."""
    sys.path.insert(0, ORACLE)
    import oracle
    import acdc
    if inst.loss == acdc.LOSS_SVM_DUAL:
        return oracle.SVM(inst.m, inst.n, inst.col_ptr, inst.row_idx, inst.vals, inst.rhs, inst.lam)
    return oracle.Lasso(inst.m, inst.n, inst.col_ptr, inst.row_idx, inst.vals, inst.rhs, inst.lam)


def cpu_time_to_gap(inst, threads, target, rel, budget_s, bulk_epochs=1, engine=None, eval_every=1):
    """Measured time-to-gap of the reference's algorithm on the host cores: the
    asynchronous multicore engine (OpenMP over updates, CAS-loop atomics,
    uniform sampling; the serial engine when threads = 1) runs bulks of
    bulk_epochs epochs; after a bulk the residual is recomputed and the FP64
    duality gap evaluated, outside the timed computation, as the reference's
    Solver loop times only its bulks (cpp/src/solver/Solver.h:43-65).
    Evaluations follow every eval_every bulks while they cost at most a
    quarter of the computation (every bulk on small instances), and always at
    the end of the budget.  Stops at the gap target or once the computation
    time reaches budget_s.  Returns the computation seconds, epochs, the last
    gap and whether the target was reached (if not, the seconds are a lower
    bound on the time-to-gap)."""
    L = engine if engine is not None else cpu_engine(inst)
    secs, epochs, bulks, eval_s = 0.0, 0, 0, 0.0
    gap = None
    trace = []
    while True:
        count = int(bulk_epochs * inst.n)
        if threads == 1:
            t = time.perf_counter()
            L.updates(count, 1)
            secs += time.perf_counter() - t
        else:
            secs += L.hogwild(count, 1, threads)
        epochs += bulk_epochs
        bulks += 1
        if (bulks % eval_every == 0 and eval_s <= 0.25 * secs) or secs >= budget_s:
            t = time.perf_counter()
            L.refresh()
            ev = L.evaluate(threads)
            eval_s += time.perf_counter() - t
            gap = ev["rel_gap"] if rel else ev["gap"]
            trace.append((round(secs, 3), epochs, gap))
            if gap <= target or secs >= budget_s:
                break
    return {"seconds": secs, "epochs": epochs, "gap": gap, "reached": bool(gap <= target),
            "updates_per_s": epochs * inst.n / secs if secs > 0 else None, "threads": threads,
            "trace": trace[-8:]}


def cpu_config0(threads):
    """The reference's CPU case (2,000 x 10,000, 20 per column, FP64, absolute
    gap 1e-6), run to the gap by the serial engine and by the OpenMP engine."""
    w0 = dict(WORKLOADS["lasso_m2e3_n1e4"])
    inst0 = generate(w0, pinned=False)
    out = {"workload": "lasso_m2e3_n1e4", "gap_target_absolute": 1e-6}
    out["serial"] = cpu_time_to_gap(inst0, 1, 1e-6, False, 60.0)
    out["openmp"] = cpu_time_to_gap(inst0, threads, 1e-6, False, 60.0)
    for k in ("serial", "openmp"):
        out[k].pop("trace", None)
    return out


def run_reference(args, w):
    """--impl reference: the reference's algorithm (its asynchronous multicore
    engine restated in the oracle; the x86 build of the reference itself does
    not run on an Arm host) on all host cores, on the same workload.  The solve
    starts from x = 0 and each timed step continues it for a bounded time;
    value is the computation time to the gap target, or, when the target is not
    reached within the steps, the total computation time with reached = false
    (a measured lower bound, never an extrapolation)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    inst = generate(w, pinned=False)
    rel = not is_svm(w)
    step_s = args.ref_step_seconds if args.ref_step_seconds > 0 else max(2.0, 120.0 / args.steps)
    # warm-up: short solves from x = 0 (page-in, thread pool), discarded
    for _ in range(args.warmup):
        cpu_time_to_gap(inst, threads, w["gap"], rel, 0.2)
    engine = cpu_engine(inst)
    total, epochs, gap, steps_run, trace = 0.0, 0, None, 0, []
    reached = False
    for _ in range(args.steps):
        r = cpu_time_to_gap(inst, threads, w["gap"], rel, step_s, engine=engine)
        total += r["seconds"]
        epochs += r["epochs"]
        gap = r["gap"]
        steps_run += 1
        trace.append((round(total, 2), epochs, gap))
        if r["reached"]:
            reached = True
            break
    c0 = cpu_config0(threads)
    value = total
    sample = ("the reference's asynchronous multicore engine (oracle port, uniform sampling, "
              "CAS atomics) on %d threads from x = 0, continued over %d steps of up to %.1f s of "
              "computation each, FP64 gap evaluated outside the timing; %s"
              % (threads, steps_run, step_s,
                 "target reached" if reached else
                 "target not reached: value is a measured lower bound (gap %.3g after %.0f s)"
                 % (gap, total)))
    line = {"metric": METRICS[w.get("loss", "lasso")], "value": value, "unit": "s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": value * 1e3 / max(1, steps_run),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded %s generator)" % ("SVM" if is_svm(w) else "Zipf Lasso"),
            "impl": "reference",
            "config": {"workload": args.workload, "m": w["m"], "n": w["n"], "nnz": inst.nnz,
                       "threads": threads, "gap_target": w["gap"], "gap_relative": rel,
                       "reached": reached, "gap_reached": gap, "epochs": epochs,
                       "updates_per_s": epochs * inst.n / total if total > 0 else None,
                       "trace": trace, "config0_time_to_gap": c0},
            "cpu_baseline": {"value": value, "unit": "s", "cores": threads, "kind": "port",
                             "lower_bound": not reached, "sample": sample},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, w):
    import numpy as np
    import torch
    import acdc

    rank, world, local = dist_env()
    if world > 1:
        torch.cuda.set_device(local)
    dist = dist_init(world, "nccl" if torch.cuda.is_available() else "gloo")
    dev = torch.device("cuda", local) if torch.cuda.is_available() else None

    t_gen = time.time()
    inst = generate(w, pinned=True)
    t_gen = time.time() - t_gen
    s = settings_for(w)
    ctx = acdc.Context(local)
    p = acdc.Problem(ctx, inst, s)
    info = p.info()

    traces = []

    def one_solve():
        p.reset()
        p.reset_stats()
        r, rows = p.solve_traced(cap=100000)
        traces.append(rows)
        return r

    for _ in range(args.warmup):
        one_solve()
    p.synchronize()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    del traces[:]
    clocks = ClockSampler(local)
    clocks.start()
    t0 = time.perf_counter()
    results = []
    for _ in range(args.steps):
        results.append(one_solve())
    p.synchronize()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if dist is not None:
        dist.barrier()
    clk = clocks.stop()

    # the last timed solve's error against the committed FP64 optimum
    # (outside the timed region)
    oracle_cmp = oracle_error(args.workload, inst, p.get_x(), results[-1].eval.primal)

    dev_ms = [r.device_ms for r in results]
    ms_per_step = max_over_ranks(dist, statistics.mean(dev_ms), dev)
    value = ms_per_step / 1e3
    converged = all(r.converged for r in results)
    epochs = [r.epochs for r in results]

    # Roofline of the update kernel (algorithmic bytes over its event-timed duration).
    upd_ms = sum(r.stats.update_ms for r in results)
    launches = sum(r.stats.update_launches for r in results)
    updates = sum(r.stats.updates for r in results)
    nnz_read = sum(r.stats.nnz_read for r in results)
    nnz_sc = sum(r.stats.nnz_scattered for r in results)
    nonzero = sum(r.stats.nonzero_updates for r in results)
    alg_bytes = 12 * nnz_read + 16 * updates + 4 * nnz_sc + 4 * nonzero
    achieved = alg_bytes / (upd_ms * 1e-3) / 1e9 if upd_ms > 0 else 0.0
    peaks = load_json(PEAKS_FILE, {})
    peak = peaks.get("hbm_gbs")
    peak_src = "measured"
    if not peak:
        peak, peak_src = 6800.0, "fallback"
    # DRAM traffic per launch from the committed per-update figures of the two
    # launch kinds: each solve's first launch draws uniformly (refresh_every
    # epochs), the others draw mostly from the active set.
    traffic_rec = load_json(TRAFFIC_FILE, {})
    traffic = None
    if traffic_rec.get("uniform_dram_bytes_per_update") and launches and not is_svm(w):
        uniform = min(updates, len(results) * w["refresh_every"] * inst.n)
        traffic = (traffic_rec["uniform_dram_bytes_per_update"] * uniform +
                   traffic_rec["active_dram_bytes_per_update"] * (updates - uniform)) / launches
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak if peak else None, "traffic": traffic,
                "peak_source": peak_src, "kernel": update_kernel_label(s, w),
                "alg_bytes_per_launch": alg_bytes / launches if launches else 0,
                "avg_launch_ms": upd_ms / launches if launches else 0,
                "phases": bulk_phases(traces, s)}

    if is_svm(w):
        k_full, k_scr = KERNELS_PER_EVAL_SVM, 0
    elif s.use_shrinking:
        k_full, k_scr = KERNELS_PER_EVAL_SHRINK, KERNELS_PER_EVAL_SCREENED
    else:
        k_full, k_scr = KERNELS_PER_EVAL, 0
    gpu_launches = sum(r.stats.update_launches + k_scr * r.stats.screened_evals +
                       k_full * (r.stats.eval_launches - r.stats.screened_evals) +
                       KERNELS_PER_RESET + (1 if r.fp64_epochs else 0) for r in results)

    # e2e: the same metric through the C-ABI from pinned host buffers.
    h2d = inst.col_ptr.nbytes + inst.row_idx.nbytes + inst.vals.nbytes + inst.rhs.nbytes
    d2h = inst.n * 8
    # One untimed pass first (pool growth, module load), then e2e_steps timed
    # passes, each split into create (upload + device layout), solve and
    # readback (x to host) on the host clock.
    e2e_times, e2e_parts = [], []
    x_last = None
    for i in range(args.e2e_steps + 1 if args.e2e_steps > 0 else 0):
        torch.cuda.synchronize()
        t = time.perf_counter()
        q = acdc.Problem(ctx, inst, s)
        q.synchronize()
        t_create = time.perf_counter()
        rq = q.solve()
        t_solve = time.perf_counter()
        x_last = q.get_x()
        q.close()
        torch.cuda.synchronize()
        t_end = time.perf_counter()
        if i > 0:
            e2e_times.append(t_end - t)
            e2e_parts.append((t_create - t, t_solve - t_create, t_end - t_solve, rq.epochs))
    e2e_value = max_over_ranks(dist, statistics.mean(e2e_times), dev) if e2e_times else None

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        # measured, bounded: the reference's algorithm on the same workload
        # from x = 0 for at most cpu_budget seconds of computation
        threads = os.cpu_count() or 1
        rel = not is_svm(w)
        run = cpu_time_to_gap(inst, threads, w["gap"], rel, args.cpu_budget)
        cpu = {"value": run["seconds"], "unit": "s", "cores": threads, "kind": "port",
               "lower_bound": not run["reached"], "gap_reached": run["gap"],
               "epochs": run["epochs"], "updates_per_s": run["updates_per_s"],
               "sample": ("the reference's asynchronous multicore engine (oracle port, uniform "
                          "sampling) on %d threads from x = 0 for up to %.0f s of computation: "
                          "%s" % (threads, args.cpu_budget,
                                  "reached the target" if run["reached"] else
                                  "gap %.3g after %d epochs, so its time-to-gap exceeds %.1f s "
                                  "(measured lower bound)" % (run["gap"], run["epochs"],
                                                              run["seconds"])))}
        # the serial engine (the reference's -t 1) on the same workload, capped
        serial = cpu_time_to_gap(inst, 1, w["gap"], rel, args.cpu_budget / 2)
        cpu["serial"] = {"value": serial["seconds"], "cores": 1, "lower_bound": not serial["reached"],
                         "gap_reached": serial["gap"], "epochs": serial["epochs"],
                         "updates_per_s": serial["updates_per_s"]}
        cpu["config0_time_to_gap"] = cpu_config0(threads)

    p.close()
    batched = serving = svm = None
    if rank == 0 and not is_svm(w) and args.svm_steps > 0:
        svm = run_svm_section(ctx, args.svm_steps, cpu=not args.no_cpu_baseline)
    if not is_svm(w) and args.batch_instances > 0:
        # every rank takes its shard of the instances
        batched = run_batched(ctx, args.batch_instances, args.batch_max_epochs, rank, world, dist,
                              dev)
    if rank == 0 and not is_svm(w) and args.serve_requests > 0:
        rates = [args.serve_rate] if args.serve_rate > 0 else list(SERVE_RATES)
        serving = run_serving(ctx, args.serve_requests, rates, args.serve_quantum)
    if is_svm(w):
        solver_keys = {"gap_target_absolute": w["gap"], "q_shrinking": 0, "lambda": w["lam"]}
    else:
        solver_keys = {"gap_target_relative": w["gap"], "q_shrinking": 0.9,
                       "tau_active": w["tau_active"], "active_passes": w["active_passes"],
                       "screened_eval": 1, "hot_threshold": 0.1,
                       "hot_polish_sweeps": 16, "polish_active_passes": 2,
                       "polish_rel_gap": 1e-5}
    if rank == 0:
        line = {
            "metric": METRICS[w.get("loss", "lasso")], "value": value, "unit": "s", "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded %s generator; inputs larger than L2)"
                    % ("SVM" if is_svm(w) else "Zipf Lasso"),
            "config": dict(solver_keys, **{
                       "workload": args.workload, "m": w["m"], "n": w["n"], "nnz": inst.nnz,
                       "tau": w["tau"], "refresh_every": w["refresh_every"],
                       "lanes_per_update": s.lanes_per_update,
                       "precision": "fp32 bulk; fp64 refresh, gap and hot-column polish",
                       "updates": int(updates), "update_launches": int(launches),
                       "updates_per_s": updates / (upd_ms * 1e-3) if upd_ms > 0 else None,
                       # where a solve's device time goes: update bulks, evaluations
                       # (both event-timed), and the rest (polish launches, host
                       # turnarounds between a bulk and the next)
                       "time_split_ms": {
                           "solve": statistics.mean(dev_ms),
                           "update_bulks": statistics.mean(r.stats.update_ms for r in results),
                           "evaluations": statistics.mean(r.stats.eval_ms for r in results),
                           "evaluation_count": statistics.mean(r.stats.eval_launches
                                                               for r in results)},
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs larger than L2 (no flush)", "omega": info.omega,
                       "beta": info.sigma, "epochs": epochs,
                       "fp64_epochs": [r.fp64_epochs for r in results],
                       "converged": converged, "final_rel_gap": [r.eval.rel_gap for r in results],
                       "objective": results[-1].eval.primal, "support": results[-1].eval.support,
                       "oracle_rel_err": oracle_cmp["oracle_rel_err"] if oracle_cmp else None,
                       "support_match": oracle_cmp["support_match"] if oracle_cmp else None,
                       "oracle": oracle_cmp,
                       "host_wall_s": wall / args.steps, "generate_s": t_gen}),
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "solves": len(e2e_times),
                    "create_s": [round(x[0], 4) for x in e2e_parts],
                    "solve_s": [round(x[1], 4) for x in e2e_parts],
                    "readback_s": [round(x[2], 4) for x in e2e_parts],
                    "epochs": [x[3] for x in e2e_parts]},
            "gpu_launches": int(gpu_launches),
            "clocks": clk,
            "svm": svm,
            "batched": batched,
            "serving": serving,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    ctx.close()
    return 0


def main():
    args = parse_args()
    if args.warmup < 3:
        args.warmup = 3
    w = dict(WORKLOADS[args.workload], name=args.workload)
    if args.active_passes > 0 and "active_passes" in w:
        w["active_passes"] = args.active_passes
    w["lanes"] = args.lanes
    w["probe_repeat"] = args.probe_repeat
    if args.probe_launches:
        return probe_launches(w)
    if args.max_epochs > 0:
        w["max_epochs"] = args.max_epochs
    if args.impl == "reference":
        return run_reference(args, w)
    return run_ours(args, w)


if __name__ == "__main__":
    sys.exit(main())
