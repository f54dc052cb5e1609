"""Benchmark of the WEAVESS hot path on one GB300.

Workload (default): N=1,000,000 base vectors, d=128, integer-valued Gaussian
mixture (256 centres uniform in [0,255], sigma 20, rounded, clipped), 10,000
queries from the same mixture (seeded synthetic stand-in for the 1M x 128
configuration).  Build: INIT_RANDOM (S=20) -> NN-Descent (K=64, L=80, ITER=8,
R=100) -> NSG link (RNG prune, R=32, L_refine=64, C_refine=500) + DFS
connectivity.  (The reference's Vamana link re-prunes rows farthest-first and
its graphs stay below recall@10 0.2 on this data, so the RNG prune is the
alpha=1 member of the RNG/alpha family used here.)  Search:
SEARCH_ENTRY_RAND + ROUTER_GREEDY, top-10, at the smallest beam width L that
reaches recall@10 >= 0.95 against FP64 brute-force ground truth.

One step = one search of all 10,000 queries.  `value` is QPS with queries and
seeds resident in HBM (device-timed with CUDA events, L2 flushed between
steps); `e2e` is QPS through the public C-ABI call with host buffers (seed
draws, H2D of queries + seeds, D2H of the result ids inside the timed
region).  `--impl reference` times the CPU implementation of the same path
(the oracle restatement of the reference, OpenMP over queries) on the host.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from weavess_gb300 import datasets as ds  # noqa: E402

CFG = dict(n=1_000_000, d=128, centers=256, nq=10_000, seed=7, S=20, K=64, L=80, ITER=8, R=100, expansions=(0, 1, 2, 3, 4),
           R_refine=32, L_refine=64, C_refine=500, k=10, target_recall=0.95,
           n_train=200_000, n_val=2000, clusters=64, L_trace=1024, L_max_learned=256, epochs=6,
           L_grid=[16, 24, 32, 48, 64, 96, 128, 160, 192, 256, 320, 384, 448, 512, 640, 768, 896, 1024, 1280,
                   1536])
METRIC = "QPS at recall@10>=0.95 (learned+BF16 vs plain FP32, 1 GB300); build sec"
# DRAM bytes (read + write) of one learned-plan search launch on the 1M x 128
# workload, by expansion width (0: the exact traversal), from ncu captures of
# this command (profiles/)
TRAFFIC_LEARNED_1M = {0: 2781244672 + 781312, 1: 2289462016 + 993536, 2: 2276730112 + 1079296,
                      3: 2273065216 + 1006080, 4: 2284729600 + 1025280}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---- ranks: under torchrun every rank holds a replica of the index on its
# own GPU and searches its own batch (search shards by query, weak scaling);
# the only collectives are the timing barrier and the max / sum of the
# per-rank figures
def world():
    return int(os.environ.get("WORLD_SIZE", "1"))


def rank():
    return int(os.environ.get("RANK", "0"))


def local_device():
    return int(os.environ.get("LOCAL_RANK", "0"))


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def rank_barrier():
    d = _dist()
    if d is not None:
        d.barrier()


def rank_reduce(x, op):
    """x reduced over ranks ("max" or "sum"); x itself without a process group."""
    d = _dist()
    if d is None:
        return float(x)
    import torch
    dev = torch.device("cuda", torch.cuda.current_device()) if d.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    d.all_reduce(t, op=d.ReduceOp.MAX if op == "max" else d.ReduceOp.SUM)
    return float(t.item())


def job_rate(units, ms_per_step):
    """Whole-job throughput: all ranks' units of one step over the slowest
    rank's step time.  Returns (units per second, max ms per step)."""
    ms_max = rank_reduce(ms_per_step, "max")
    return rank_reduce(units, "sum") / (ms_max / 1e3), ms_max


class Clocks:
    """nvidia-smi samples while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.rows, self.proc = [], None
        self.win = None

    def mark(self, t0, t1):
        """The timed region, in time.perf_counter() seconds."""
        self.win = (t0, t1)

    def in_window(self):
        if self.win is None:
            return len(self.rows)
        return sum(1 for r in self.rows if self.win[0] <= r[0] <= self.win[1] + 0.25)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([time.perf_counter()] + [x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        """Samples from the timed region on; when the region was shorter than
        the sampling period, the samples of the same steps repeated right after
        it (the caller keeps the load on until enough samples arrived)."""
        rows = [r[1:] for r in self.rows if self.win is None or r[0] >= self.win[0]]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 5 + i and r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "samples_in_timed_region": self.in_window()}


PROFILE_REGION = "search"  # which region a cudaProfilerStart/Stop pair brackets (for ncu --profile-from-start off)


def timed_steps(step, steps, stream, flush, clk, after=None):
    """`steps` CUDA-event-timed calls of `step` (L2 flushed before each), with
    the clock sampler running; the same steps continue untimed until the
    sampler has three readings from the timed region on.  `after(i)` runs
    after step i is enqueued (e.g. to read its kernel time).  Returns per-step
    ms."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    rank_barrier()
    t0 = time.perf_counter()
    if PROFILE_REGION == "search":
        torch.cuda.profiler.start()
    for i in range(steps):
        flush.zero_()
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
        if after is not None:
            after(i)
    torch.cuda.synchronize()
    rank_barrier()
    if PROFILE_REGION == "search":
        torch.cuda.profiler.stop()
    clk.mark(t0, time.perf_counter())
    deadline = time.perf_counter() + 3.0
    while sum(1 for r in clk.rows if r[0] >= t0) < 3 and time.perf_counter() < deadline:
        flush.zero_()
        step()
        torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev]


def make_data(cfg):
    t = time.time()
    base, query = ds.int_mixture(cfg["n"], cfg["d"], cfg["centers"], seed=cfg["seed"], n_query=cfg["nq"])
    log(f"data {base.shape} {query.shape} in {time.time() - t:.1f}s")
    return base, query


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def recall(res, gt, k=10):
    g = gt[:, :k]
    hit = (res[:, :k, None] == g[:, None, :]).any(2).sum()
    return float(hit) / (res.shape[0] * k)


def build_index(ctx, base, cfg):
    """GPU build; returns build seconds and per-stage stats."""
    import torch
    torch.cuda.synchronize()
    if PROFILE_REGION == "build":
        torch.cuda.profiler.start()
    t0 = time.time()
    ctx.upload_base(base)
    ctx.srand(1)
    st0 = ctx.init_random(cfg["S"])
    st1 = ctx.nnd_refine(cfg["S"], cfg["K"], cfg["L"], cfg["ITER"], cfg["R"])
    stages = {"init_random": st0, "nndescent": st1}
    if cfg.get("link") == "vamana":
        # the RNG/alpha prune as the 1M configuration states it: alpha 1.2,
        # R 32, in the clean build mode (the reference's Vamana link defects
        # fixed; compat mode reproduces them bit for bit)
        ctx.set_build_mode("clean")
        stages["vamana"] = ctx.vamana_refine(cfg["L_refine"], cfg["R_refine"], cfg["alpha"], 0)
        ctx.set_build_mode("compat")
    else:
        stages["nsg"] = ctx.nsg_refine(cfg["L_refine"], cfg["R_refine"], cfg["C_refine"])
    ctx.load_built_graph()
    torch.cuda.synchronize()
    dt = time.time() - t0
    if PROFILE_REGION == "build":
        torch.cuda.profiler.stop()
    return dt, stages


def cpu_search_qps(base, query, g_ids, g_deg, L, threads, sample):
    """The oracle restatement (OpenMP over queries) on the host cores."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    g = O.Graph(g_ids, np.zeros(g_ids.shape, np.float32), g_deg, 0)
    q = query[:sample]
    O.search(base, q[:8], g, L, O.Rand(1), threads=threads)  # warm
    t = time.perf_counter()
    res, dc, hc = O.search(base, q, g, L, O.Rand(1), threads=threads)
    dt = time.perf_counter() - t
    return sample / dt, dt, res


def bisect_beam(rec, grid, target, step=8):
    """The smallest beam reaching `target` recall: the first grid point that
    does, then bisected against the grid point below it to `step`.
    rec(L) -> recall; returns (L, {L: recall} of every beam tried)."""
    sweep = {}

    def r(L):
        if L not in sweep:
            sweep[L] = round(rec(L), 4)
            log(f"L={L} recall={sweep[L]}")
        return sweep[L]

    below, hi = None, grid[-1]
    for L in grid:
        if r(L) >= target:
            hi = L
            break
        below = L
    if below is not None and r(hi) >= target:
        lo = below
        while hi - lo > step:
            mid = (lo + hi) // 2 // step * step
            if mid <= lo:
                break
            if r(mid) >= target:
                hi = mid
            else:
                lo = mid
    return hi, dict(sorted(sweep.items()))


def time_plan(plan, nq, args, stream, flush, tune=True):
    """Tuned launch shape, warm-up, then the timed replays: (mean step ms,
    mean search-kernel ms, counters, tune report, clocks)."""
    tr = plan.tune(nq) if tune else None
    plan.run(nq)
    counters = plan.wait()
    for _ in range(args.warmup):
        plan.run(nq)
        plan.wait()
    kms = []
    with Clocks() as clk:
        step_ms = timed_steps(lambda: plan.run(nq), args.steps, stream, flush, clk,
                              after=lambda i: kms.append(plan.search_ms()))
    plan.wait()
    return float(np.mean(step_ms)), float(np.mean(kms)), counters, tr, clk.summary()


def calibrate_margin(ctx, val, gtv, k, goal):
    """The smallest beam margin whose validation recall clears `goal`: a
    coarse grid, then bisected against the grid point below."""
    def val_recall(m):
        ctx.learn_set_margin(m)
        ctx.srand(4321)
        rv, _, _ = ctx.search_learned(val, k)
        r = recall(rv, gtv, k)
        log(f"margin {m:.3f} val recall {r:.4f}")
        return r

    chosen, below = None, None
    for m in (0.5, 0.75, 1.0, 1.25, 1.5, 2.0, 2.5, 3.0, 4.0, 6.0, 8.0):
        chosen = m
        if val_recall(m) >= goal:
            break
        below = m
    if below is not None and chosen != below:
        lo, hi = below, chosen
        for _ in range(3):
            mid = (lo + hi) / 2
            if val_recall(mid) >= goal:
                hi = mid
            else:
                lo = mid
        chosen = hi
    ctx.learn_set_margin(chosen)
    return chosen


def run_learned(ctx, cfg, base, query, gt, args, dev, stream, flush):
    """Learned entry point and beam width (trained on plain-search traces of
    queries disjoint from the evaluation set), bf16 candidate distances with an
    exact FP32 rerank.  The fallback threshold and, per expansion width, the
    beam margin are calibrated on held-out validation queries (exact ground
    truth); each width is then timed on the evaluation queries like the plain
    search, and the fastest is the headline."""
    import torch
    from weavess_gb300.groundtruth import knn_fp64
    nt, nval, K = cfg["n_train"], cfg["n_val"], cfg["k"]
    _, tq = ds.int_mixture(0, cfg["d"], cfg["centers"], seed=cfg["seed"], n_query=nt + nval, query_stream=3)
    train, val = tq[:nt], tq[nt:]
    t = time.time()
    rep = ctx.learn_fit(train, clusters=cfg["clusters"], L_trace=cfg["L_trace"], L_max=cfg["L_max_learned"],
                        list_len=cfg["L_max_learned"], epochs=cfg["epochs"], batch=1024)
    fit_s = time.time() - t
    log(f"learn_fit {fit_s:.1f}s {rep}")
    gtv = knn_fp64(base, val, 10)
    ctx.set_precision("bf16", rerank=0)
    goal = cfg["target_recall"] + 0.005
    # ---- the fallback: the least confident validation queries take the plain
    # search at the learned kernel's largest beam; a threshold is kept only if
    # its validation recall at the exact traversal's margin beats the
    # model's own by at least 0.002 (a plain query runs several times as many
    # hops and its visited set sizes the launch's shared memory, so a
    # threshold that buys nothing measurable is left off)
    ctx.set_expansion(0)
    m0 = calibrate_margin(ctx, val, gtv, K, goal)
    _, vprob, _ = ctx.learn_predict(val)
    fb_rows = []
    best_fb = (0.0, None)
    for frac in (0.0, 0.005, 0.01, 0.02):
        p = float(np.quantile(vprob, frac)) if frac > 0 else 0.0
        ctx.learn_set_fallback(p, cfg["L_max_learned"])
        ctx.srand(4321)
        rv, _, _ = ctx.search_learned(val, K)
        r = recall(rv, gtv, K)
        fb_rows.append({"val_fraction": frac, "threshold": round(p, 5), "val_recall": round(r, 4)})
        if best_fb[1] is None or r >= best_fb[1] + 0.002:
            best_fb = (p, r)
    ctx.learn_set_fallback(best_fb[0], cfg["L_max_learned"])
    log(f"fallback {fb_rows} -> threshold {best_fb[0]}")
    _, eprob, _ = ctx.learn_predict(query)
    fallback = {"threshold": round(best_fb[0], 5), "beam": cfg["L_max_learned"], "calibration": fb_rows,
                "eval_fraction": round(float(np.mean(eprob < best_fb[0])), 4)}
    nq = query.shape[0]
    dq = torch.from_numpy(query).to(dev)
    dout = torch.empty((nq, K), dtype=torch.int32, device=dev)
    variants = {}
    for E in cfg["expansions"]:
        ctx.set_expansion(E)
        m = m0 if E == 0 else calibrate_margin(ctx, val, gtv, K, goal)
        ctx.learn_set_margin(m)
        # the batched form: a plan bound to device buffers, launch shape tuned on
        # these queries, the whole step (forward pass, seeds, search) one graph
        plan = ctx.plan(nq, K, dq.data_ptr(), dout.data_ptr(), mode="learned")
        ms, kms, counters, tune, clocks = time_plan(plan, nq, args, stream, flush)
        plan.close()
        res = dout.cpu().numpy().astype(np.uint32)
        variants[E] = {"qps": nq / (ms / 1e3), "ms": ms, "search_kernel_ms": kms, "recall@10": recall(res, gt, K),
                       "margin": m, "dist_count": counters[0], "hop_count": counters[1],
                       "tuned_shape": tune["chosen"], "clocks": clocks}
        log(f"learned E={E}: {variants[E]}")
    bestE = max(variants, key=lambda e: variants[e]["qps"])
    best = variants[bestE]
    ctx.set_expansion(bestE)
    ctx.learn_set_margin(best["margin"])
    # e2e through the public plan API: pinned host queries in, ids out
    plan = ctx.plan(nq, K, dq.data_ptr(), dout.data_ptr(), mode="learned")
    plan.set_shape(best["tuned_shape"]["warps_per_block"], best["tuned_shape"]["hash_words"],
                   bool(best["tuned_shape"]["wide_hash"]), best["tuned_shape"].get("query_warps", 1) or 1)
    qpin = torch.from_numpy(query).pin_memory()
    opin = torch.empty((nq, K), dtype=torch.int32).pin_memory()
    e2e_t = []
    for _ in range(args.steps + 1):
        t0 = time.perf_counter()
        dq.copy_(qpin, non_blocking=True)
        plan.run(nq)
        opin.copy_(dout, non_blocking=True)
        plan.wait()
        e2e_t.append(time.perf_counter() - t0)
    e2e_t = e2e_t[1:]
    plan.close()
    # and through the one-call host API (wv_search_learned)
    qnp = qpin.numpy()
    _, _, _, Ls = ctx.search_learned(qnp, K, return_L=True)
    plain_beam = ctx.learn_plain_beam()  # host-drawn plain seeds per query the call copies (0: none)
    call_t = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        ctx.search_learned(qnp, K)
        call_t.append(time.perf_counter() - t0)
    ctx.set_expansion(0)
    ctx.set_precision("fp32")
    out = dict(best)
    out.update({"expansion": bestE, "e2e_qps": nq / float(np.mean(e2e_t)), "e2e_call_qps": nq / float(np.mean(call_t)),
                "mean_L": float(Ls.mean()), "fit_s": fit_s, "report": rep, "n_train": nt,
                "plain_seeds_per_query": plain_beam, "fallback": fallback,
                "by_expansion": {str(e): {kk: (round(vv, 4) if isinstance(vv, float) else vv)
                                          for kk, vv in v.items() if kk not in ("clocks",)}
                                 for e, v in variants.items()}})
    return out


def plain_leg(ctx, query, gt, cfg, args, dev, stream, flush, entry, expansion, dq, dout):
    """One plain FP32 search form: the beam calibrated (bisected) to the
    recall target on the timed seeds, then a tuned plan timed."""
    import torch
    nq, K = query.shape[0], cfg["k"]
    ctx.set_expansion(expansion)

    def rec(L):
        ctx.srand(777)
        res, _, _ = ctx.search(query, L, K, entry=entry)
        return recall(res, gt, K)

    L, sweep = bisect_beam(rec, cfg["L_grid"], cfg["target_recall"])
    ctx.srand(777)
    seeds = ctx.draw_seeds(nq, L, entry)
    ds_ = torch.from_numpy(seeds.astype(np.int32)).to(dev)
    plan = ctx.plan(nq, K, dq.data_ptr(), dout.data_ptr(), L_max=L, mode="seeds", d_seeds=ds_.data_ptr())
    ms, kms, counters, tune, clocks = time_plan(plan, nq, args, stream, flush)
    plan.close()
    res = dout.cpu().numpy().astype(np.uint32)
    ctx.set_expansion(0)
    return {"entry": entry, "expansion": expansion, "qps": round(nq / (ms / 1e3), 1), "ms_per_step": round(ms, 4),
            "L_search": L, "recall@10": round(recall(res, gt, K), 4), "recall_sweep": sweep,
            "dist_count": counters[0], "hop_count": counters[1], "tuned_shape": tune["chosen"],
            "search_kernel_ms": round(kms, 4), "clocks": clocks}


def run_ours(args):
    import torch
    from weavess_gb300 import Context
    from weavess_gb300.groundtruth import knn_fp64
    cfg = dict(CFG)
    if args.small:
        cfg.update(n=100_000, centers=64, nq=1000, S=10, K=32, L=40, ITER=8, R=100, R_refine=32, L_refine=32,
                   n_train=40_000, clusters=32, L_trace=512, L_max_learned=256)
    if args.nq:
        cfg["nq"] = args.nq
    if args.n:
        cfg["n"] = args.n
    if args.link == "vamana":
        cfg.update(link="vamana", alpha=1.2, L_refine=args.vamana_L)
    dev = torch.device("cuda", local_device())
    torch.cuda.set_device(dev)
    base, query = make_data(cfg)
    if world() > 1:
        # weak scaling: every rank holds a replica and searches its own slice
        # of a batch of nq x N queries (weavess_gb300.replicas)
        from weavess_gb300.replicas import query_slice
        _, allq = ds.int_mixture(0, cfg["d"], cfg["centers"], seed=cfg["seed"], n_query=cfg["nq"] * world())
        s0, s1 = query_slice(allq.shape[0], rank(), world())
        query = allq[s0:s1]
    ctx = Context(local_device())
    # one stream for everything timed: the L2 flush, the events and the
    # context's kernels (the legacy default stream would not order the
    # context's non-blocking stream)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    build_s, stages = build_index(ctx, base, cfg)
    log(f"build {build_s:.2f}s {stages}")
    t = time.time()
    gt = knn_fp64(base, query, 100)
    log(f"ground truth {time.time() - t:.1f}s")
    nq, d, K = query.shape[0], cfg["d"], cfg["k"]
    dq = torch.from_numpy(query).to(dev)
    dout = torch.empty((nq, K), dtype=torch.int32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # 256 MB > 129 MB L2
    # ---- the plain FP32 search in the reference's traversal, with the Rand
    # and the Centroid entries, each at its own bisected beam; the faster is
    # the comparator.  The throughput form of the plain search is reported
    # beside it.
    legs = {e: plain_leg(ctx, query, gt, cfg, args, dev, stream, flush, e, 0, dq, dout) for e in ("rand", "centroid")}
    plain = legs["rand"] if legs["rand"]["qps"] >= legs["centroid"]["qps"] else legs["centroid"]
    plain_tp = plain_leg(ctx, query, gt, cfg, args, dev, stream, flush, "rand", 2, dq, dout)
    value, ms = plain["qps"], plain["ms_per_step"]
    Lsel, entry = plain["L_search"], plain["entry"]
    dc, hc = plain["dist_count"], plain["hop_count"]
    # ---- roofline of the search kernel (algorithmic bytes per launch)
    g_ids, _, g_deg, _ = ctx.get_graph()
    avg_deg = float(g_deg.mean())
    alg_bytes = dc * d * 4 + hc * (avg_deg * 4 + 4) + nq * d * 4
    hbm, peak_kind = peaks()
    achieved = alg_bytes / (plain["search_kernel_ms"] / 1e3) / 1e9
    # ---- e2e through the public call (host buffers, pinned)
    qpin = torch.from_numpy(query).pin_memory().numpy()
    ctx.srand(777)
    for _ in range(max(1, args.warmup // 2)):
        ctx.search(qpin, Lsel, K, entry=entry)
    torch.cuda.synchronize()
    e2e_t = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        ctx.search(qpin, Lsel, K, entry=entry)
        e2e_t.append(time.perf_counter() - t0)
    e2e_qps = nq / float(np.mean(e2e_t))
    plain["e2e_qps"] = round(e2e_qps, 1)
    # ---- learned entry / beam + bf16 candidate distances
    learned = None
    if not args.no_learned:
        learned = run_learned(ctx, cfg, base, query, gt, args, dev, stream, flush)
    # ---- CPU baseline: the oracle on the host cores, bounded sample (rank 0),
    # the reference's default entry (Rand) at its calibrated beam
    threads = os.cpu_count() or 1
    sample = 2000 if not args.small else 1000
    L_cpu = legs["rand"]["L_search"]
    cpu_qps, cpu_dt = 0.0, 0.0
    if rank() == 0:
        cpu_qps, cpu_dt, _ = cpu_search_qps(base, query, g_ids, g_deg, L_cpu, threads, sample)
    if learned is not None:
        head_qps, head_ms, head_e2e = learned["qps"], learned["ms"], learned["e2e_qps"]
        ldc, lhc = learned["dist_count"], learned["hop_count"]
        # bf16 candidate rows (2d bytes), graph rows, query rows
        alg = ldc * d * 2 + lhc * (avg_deg * 4 + 4) + nq * d * 4
        l_achieved = alg / (learned["search_kernel_ms"] / 1e3) / 1e9
        kname = ("k_beam (throughput form, E=%d parents per step, tensor-core bf16 rows)" % learned["expansion"]
                 if learned["expansion"] > 0 else "k_search (exact traversal, bf16 candidate rows)")
        roof = {"bound": "hbm", "achieved": round(l_achieved, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(l_achieved / hbm, 4),
                "traffic": TRAFFIC_LEARNED_1M.get(learned["expansion"]) if cfg["n"] == 1_000_000 else None,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of this search launch, "
                                  "profiles/launches_search_1M.md",
                "peak_kind": peak_kind, "alg_bytes_per_launch": int(alg), "dist_count": ldc, "hop_count": lhc,
                "mean_graph_degree": round(avg_deg, 2), "kernel": kname + ", learned seeds, per-query L",
                "kernel_ms": round(learned["search_kernel_ms"], 4),
                "timing": "CUDA events captured around the search (dispatch-order and search kernels) in each timed replay"}
        # queries, the replay's query count, the rand() values of the plain seeds (if any)
        h2d = nq * d * 4 + 4 + (nq * 4 if learned["plain_seeds_per_query"] else 0)
        # query normalisation, 3 GEMMs, the seed kernel, the widest-first dispatch order, the search per step
        # (plus the plain seed draw when the fallback or short lists read plain seeds)
        launches = args.steps * (8 if learned["plain_seeds_per_query"] else 7)
    else:
        head_qps, head_ms, head_e2e = value, ms, e2e_qps
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 4), "traffic": None, "peak_kind": peak_kind,
                "alg_bytes_per_launch": int(alg_bytes), "dist_count": dc, "hop_count": hc, "kernel": "k_search",
                "mean_graph_degree": round(avg_deg, 2), "kernel_ms": plain["search_kernel_ms"],
                "timing": "CUDA events captured around the search kernel in each timed replay"}
        h2d = nq * d * 4 + nq * 4  # queries and one rand() value per query (seeds drawn on the device)
        launches = args.steps
    # whole job: every rank searched its own nq queries per step
    head_qps, head_ms = job_rate(nq, head_ms)
    head_e2e = rank_reduce(head_e2e, "sum")
    if rank() != 0:
        return
    line = {
        "metric": METRIC, "value": round(head_qps, 1), "unit": "queries/s", "n_gpus": world(), "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(head_ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": ("bf16 candidates (f32 accumulate; exact on this integer data, so no f32 rerank)" if learned
                  else "f32"),
        "data": "synthetic (seeded integer Gaussian mixture)",
        "config": {"workload": f"{cfg['n']}x{cfg['d']} int-mixture({cfg['centers']}), {nq} queries, top-{K}, "
                               f"KGraph NN-Descent S={cfg['S']} K={cfg['K']} L={cfg['L']} ITER={cfg['ITER']} "
                               f"R={cfg['R']} -> " + (
                                   f"Vamana (clean build mode) alpha={cfg['alpha']} R={cfg['R_refine']} "
                                   f"L_refine={cfg['L_refine']}" if cfg.get("link") == "vamana" else
                                   f"NSG R={cfg['R_refine']} L_refine={cfg['L_refine']} C_refine={cfg['C_refine']}"),
                   "headline": "learned entry + beam, bf16 candidates" if learned else "plain FP32",
                   "learned": ({k: (round(v, 4) if isinstance(v, float) else v) for k, v in learned.items()}
                               if learned else None),
                   "plain_fp32": plain,
                   "plain_fp32_by_entry": {e: {k: v for k, v in leg.items() if k != "clocks"} for e, leg in legs.items()},
                   "plain_fp32_throughput": {k: v for k, v in plain_tp.items() if k != "clocks"},
                   "speedup_vs_plain": round(head_qps / value, 3) if learned else 1.0,
                   "speedup_vs_plain_note": "against the faster of the Rand and Centroid entries of the plain FP32 "
                                            "search in the reference's traversal, each at its smallest beam reaching "
                                            "recall@10 0.95 on the timed queries (bisected to 8)",
                   "l2": f"flushed (256 MB write) between steps; base {cfg['n'] * d * 4 / 1e6:.0f} MB",
                   "build_s": round(build_s, 3),
                   "build_stages": {k: {kk: (round(vv, 2) if isinstance(vv, float) else vv) for kk, vv in v.items()}
                                    for k, v in stages.items()}},
        "e2e": {"value": round(head_e2e, 1), "unit": "queries/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": nq * K * 4},
        "gpu_launches": launches,
        "roofline": roof,
        "cpu_baseline": {"value": round(cpu_qps, 1), "unit": "queries/s", "cores": threads, "kind": "port",
                         "sample": f"first {sample} queries, same graph, plain search (Rand entry) at L={L_cpu}, "
                                   f"oracle OpenMP ({cpu_dt:.2f}s)"},
        "clocks": learned["clocks"] if learned else plain["clocks"],
    }
    print(json.dumps(line), flush=True)


def run_reference(args):
    """The CPU implementation of the path (the oracle restatement of the
    reference, every host thread -- the reference tree itself is not on the
    GPU machine) on the same workload: the 1M x 128 build (INIT_RANDOM ->
    NN-Descent -> NSG, untimed setup, a few minutes on the host cores), then
    each step searches a bounded sample of the queries at the smallest beam
    reaching recall@10 >= 0.95 on that sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    cfg = dict(CFG)
    if args.small:
        cfg.update(n=100_000, centers=64, S=10, K=32, L=40, ITER=8, R=100, R_refine=32, L_refine=32)
    if args.n:
        cfg["n"] = args.n
    threads = os.cpu_count() or 1
    sample = 2000
    base, query = ds.int_mixture(cfg["n"], cfg["d"], cfg["centers"], seed=cfg["seed"], n_query=cfg["nq"])
    query = query[:sample]
    t = time.time()
    r = O.Rand(1)
    g = O.init_random(base, cfg["S"], r)
    g = O.nndescent(base, g, cfg["S"], cfg["K"], cfg["L"], cfg["ITER"], cfg["R"], r, threads=threads)
    t_nnd = time.time() - t
    g = O.nsg(base, g, cfg["L_refine"], cfg["R_refine"], cfg["C_refine"], r, threads=threads)
    build_s = time.time() - t
    log(f"reference build {build_s:.1f}s (NN-Descent {t_nnd:.1f}s) on {threads} threads")
    gt = ds.groundtruth_fp64(base, query, 10)

    def rec(L):
        res, _, _ = O.search(base, query, g, L, O.Rand(5), threads=threads)
        return recall(res, gt)

    # the smallest beam reaching the target, bisected as for the GPU search
    Lsel, sweep = bisect_beam(rec, cfg["L_grid"], cfg["target_recall"])
    for _ in range(args.warmup):
        O.search(base, query, g, Lsel, O.Rand(5), threads=threads)
    ts = []
    for _ in range(args.steps):
        t = time.perf_counter()
        O.search(base, query, g, Lsel, O.Rand(5), threads=threads)
        ts.append(time.perf_counter() - t)
    qps = query.shape[0] / float(np.mean(ts))
    line = {"impl": "reference", "metric": METRIC, "value": round(qps, 1), "unit": "queries/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(float(np.mean(ts)) * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded integer Gaussian mixture)",
            "config": {"workload": f"{cfg['n']}x{cfg['d']} int-mixture({cfg['centers']}), {sample}-query sample per "
                                   f"step, top-10, NN-Descent S={cfg['S']} K={cfg['K']} L={cfg['L']} "
                                   f"ITER={cfg['ITER']} R={cfg['R']} -> NSG R={cfg['R_refine']} "
                                   f"L_refine={cfg['L_refine']} C_refine={cfg['C_refine']}",
                       "L_search": Lsel, "recall_sweep": sweep, "build_s": round(build_s, 2),
                       "build_nndescent_s": round(t_nnd, 2), "headline": "plain FP32 (the reference has no "
                       "learned or low-precision path)"},
            "cpu_baseline": {"value": round(qps, 1), "unit": "queries/s", "cores": threads, "kind": "port",
                             "sample": f"{sample} queries of the {cfg['n']}-vector workload, plain search at "
                                       f"L={Lsel}, OpenMP over queries"},
            "e2e": {"value": round(qps, 1), "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ the other configurations
# Informational lines (one JSON line each, its own metric); the default run
# measures the 1M x 128 configuration above.

def _setup(cfg, ds_fn, nq):
    import torch
    from weavess_gb300 import Context
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    t = time.time()
    base, query = ds_fn(cfg["n"], cfg["d"], n_query=nq)
    log(f"data {base.shape} {query.shape} in {time.time() - t:.1f}s")
    ctx = Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    build_s, stages = build_index(ctx, base, cfg)
    log(f"build {build_s:.2f}s")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    return torch, dev, base, query, ctx, stream, flush, build_s, stages


def _timed_plan(torch, plan, nq, args, stream, flush):
    plan.run(nq)
    counters = plan.wait()
    for _ in range(args.warmup):
        plan.run(nq)
        plan.wait()
    kms = []
    with Clocks() as clk:
        step_ms = timed_steps(lambda: plan.run(nq), args.steps, stream, flush, clk,
                              after=lambda i: kms.append(plan.search_ms()))
    plan.wait()
    return float(np.mean(step_ms)), float(np.mean(kms)), counters, clk.summary()


def run_precision96(args):
    """1M x 96 unit-norm vectors (isotropic part + 1,000 directions, cosine
    ~0.7), NN-Descent -> NSG R=32; the plain search with FP32, bf16 and fp8
    e4m3 (per-row scale) candidate distances, each with the exact FP32 rerank
    of the final pool: QPS at recall@10 >= 0.95 per precision, and the
    candidate-distance error against FP64."""
    from weavess_gb300.groundtruth import knn_fp64
    cfg = dict(CFG)
    cfg.update(n=args.n or 1_000_000, d=96, nq=args.nq or 10_000)
    torch, dev, base, query, ctx, stream, flush, build_s, _ = _setup(
        cfg, lambda n, d, n_query: ds.unit_mixture(n, d, 1000, seed=11, n_query=n_query), cfg["nq"])
    gt = knn_fp64(base, query, 100)
    nq, K = query.shape[0], cfg["k"]
    # candidate-distance error vs FP64: each of 1,000 queries against its
    # true 100 nearest and 100 random rows
    rng = np.random.default_rng(3)
    qs = query[:1000]
    ids = np.concatenate([gt[:1000, :100], rng.integers(0, base.shape[0], size=(1000, 100))], 1).astype(np.uint32)
    exact = ((qs[:, None, :].astype(np.float64) - base[ids].astype(np.float64)) ** 2).sum(2)
    out = {}
    dq = torch.from_numpy(query).to(dev)
    dout = torch.empty((nq, K), dtype=torch.int32, device=dev)
    for storage in ("fp32", "bf16", "fp8"):
        ctx.set_precision(storage, rerank=0)
        got = ctx.candidate_distances(qs, ids).astype(np.float64)
        err = np.abs(got - exact)
        for E in (0, 2):
            # the exact traversal, and the throughput form (bf16 rows of d = 96
            # on the tensor cores with a hi + lo bf16 query)
            ctx.set_expansion(E)

            def rec(L):
                ctx.srand(777)  # the timed steps' seeds
                res, _, _ = ctx.search(query, L, K)
                return recall(res, gt, K)

            Lsel, sweep = bisect_beam(rec, cfg["L_grid"], cfg["target_recall"])
            ctx.srand(777)
            seeds = torch.from_numpy(ctx.draw_seeds(nq, Lsel, "rand").astype(np.int32)).to(dev)
            plan = ctx.plan(nq, K, dq.data_ptr(), dout.data_ptr(), L_max=Lsel, mode="seeds", d_seeds=seeds.data_ptr())
            tune = plan.tune(nq)
            ms, kms, (dc, hc), clk = _timed_plan(torch, plan, nq, args, stream, flush)
            plan.close()
            ctx.set_expansion(0)
            r = recall(dout.cpu().numpy().astype(np.uint32), gt, K)
            key = storage if E == 0 else f"{storage}_E{E}"
            out[key] = {"qps": round(nq / (ms / 1e3), 1), "L_search": Lsel, "recall@10": round(r, 4),
                        "recall_sweep": sweep, "search_kernel_ms": round(kms, 4), "dist_count": dc,
                        "tuned_shape": tune["chosen"], "clocks": clk,
                        "err_vs_fp64": {"max_abs": float(err.max()), "mean_abs": float(err.mean()),
                                        "max_rel_to_mean_dist": float(err.max() / exact.mean()),
                                        "mean_rel": float((err / np.maximum(exact, 1e-12)).mean())}}
            log(f"{key}: {out[key]}")
    ctx.set_precision("fp32")
    best = max(out, key=lambda k: out[k]["qps"])
    line = {"metric": "QPS at recall@10>=0.95 per candidate precision (1M x 96 unit vectors)",
            "value": out[best]["qps"], "unit": "queries/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": best, "data": "synthetic (seeded unit-norm mixture)",
            "config": {"workload": f"{cfg['n']}x96 unit-mixture, {nq} queries, top-10, NN-Descent S=20 K=64 L=80 "
                                   f"ITER=8 R=100 -> NSG R=32 L_refine=64 C_refine=500, exact FP32 rerank of "
                                   f"the whole pool", "build_s": round(build_s, 2), "by_precision": out}}
    print(json.dumps(line), flush=True)


def run_batch960(args):
    """1M x 960 non-negative vectors summing to 1 (512-component mixture),
    NN-Descent -> NSG R=48; one launch serves 20,000 queries with k drawn
    from {1, 10, 50, 100} and L uniform on [10, 500] (L >= k): a tuned,
    captured plan; QPS and recall@k per k."""
    from weavess_gb300.groundtruth import knn_fp64
    cfg = dict(CFG)
    cfg.update(n=args.n or 1_000_000, d=960, nq=args.nq or 20_000, R_refine=48)
    torch, dev, base, query, ctx, stream, flush, build_s, stages = _setup(
        cfg, lambda n, d, n_query: ds.simplex_mixture(n, d, 512, seed=13, n_query=n_query), cfg["nq"])
    gt = knn_fp64(base, query, 100)
    nq = query.shape[0]
    rng = np.random.default_rng(4)
    K = rng.choice([1, 10, 50, 100], size=nq).astype(np.int32)
    L = np.maximum(K, rng.integers(10, 501, size=nq)).astype(np.int32)
    dq = torch.from_numpy(query).to(dev)
    dL, dK = torch.from_numpy(L).to(dev), torch.from_numpy(K).to(dev)
    dout = torch.full((nq, 100), -1, dtype=torch.int32, device=dev)

    def one_form(E):
        """the exact traversal (E = 0) or the throughput form with E parents
        per step; launch shape (warps per block, warps per query, hash)
        tuned on the batch"""
        ctx.set_expansion(E)
        plan = ctx.plan(nq, 100, dq.data_ptr(), dout.data_ptr(), L_max=500, mode="rand", d_L=dL.data_ptr(),
                        d_K=dK.data_ptr(), out_stride=100)
        tune = plan.tune(nq)
        log(f"E={E} tuning {tune}")
        ms, kms, (dc, hc), clk = _timed_plan(torch, plan, nq, args, stream, flush)
        plan.close()
        ctx.set_expansion(0)
        out = dout.cpu().numpy()
        rec = {}
        for k in (1, 10, 50, 100):
            sel = np.nonzero(K == k)[0]
            hit = sum(len(set(out[i, :k].tolist()) & set(gt[i, :k].tolist())) for i in sel)
            rec[k] = round(hit / max(1, len(sel) * k), 4)
        return {"qps": round(nq / (ms / 1e3), 1), "ms": ms, "kms": kms, "dc": dc, "hc": hc, "clk": clk,
                "recall_at_k": rec, "tuned_shape": tune["chosen"], "tune": tune["tried"]}

    forms = {E: one_form(E) for E in (0, 1, 2)}
    bestE = max(forms, key=lambda e: forms[e]["qps"])
    f = forms[bestE]
    ms, kms, dc, hc, clk, rec, tune = f["ms"], f["kms"], f["dc"], f["hc"], f["clk"], f["recall_at_k"], f
    line = {"metric": "QPS, one launch of 20,000 queries with mixed k and L (1M x 960)",
            "value": round(nq / (ms / 1e3), 1), "unit": "queries/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded simplex mixture)",
            "config": {"workload": f"{cfg['n']}x960 simplex-mixture(512), {nq} queries, k in {{1,10,50,100}}, "
                                   f"L~U[10,500], NN-Descent S=20 K=64 L=80 ITER=8 R=100 -> NSG R=48 "
                                   f"L_refine=64 C_refine=500", "build_s": round(build_s, 2),
                       "build_stages": {k: {kk: (round(vv, 2) if isinstance(vv, float) else vv)
                                            for kk, vv in v.items()} for k, v in stages.items()},
                       "recall_at_k": rec, "search_kernel_ms": round(kms, 4), "dist_count": dc, "hop_count": hc,
                       "expansion": bestE, "tuned_shape": tune["tuned_shape"], "tune": tune["tune"],
                       "by_expansion": {str(e): {"qps": v["qps"], "recall_at_k": v["recall_at_k"],
                                                 "search_kernel_ms": round(v["kms"], 4),
                                                 "tuned_shape": v["tuned_shape"]} for e, v in forms.items()}},
            "clocks": clk}
    print(json.dumps(line), flush=True)


def run_learned10m(args):
    """10M x 128 integer mixture (1,024 centres), NN-Descent -> NSG R=32; the
    learned entry / beam (64 clusters, trained on 200,000 plain-search traces)
    with bf16 candidates against the plain FP32 search, 10,000 held-out
    queries; QPS at recall@10 >= 0.95 (or the best recall the beam cap
    reaches)."""
    from weavess_gb300.groundtruth import knn_fp64
    cfg = dict(CFG)
    # (the beams of this larger index reach past 256: the model's cap stays 512)
    cfg.update(n=args.n or 10_000_000, centers=1024, nq=args.nq or 10_000, L_max_learned=512)
    torch, dev, base, query, ctx, stream, flush, build_s, stages = _setup(
        cfg, lambda n, d, n_query: ds.int_mixture(n, d, cfg["centers"], seed=cfg["seed"], n_query=n_query),
        cfg["nq"])
    gt = knn_fp64(base, query, 100)
    nq, K = query.shape[0], cfg["k"]
    sweep, Lsel = {}, cfg["L_grid"][-1]
    for L in cfg["L_grid"]:
        ctx.srand(777)  # the timed steps' seeds
        res, _, _ = ctx.search(query, L, K)
        sweep[L] = round(recall(res, gt, K), 4)
        log(f"plain L={L} recall={sweep[L]}")
        if sweep[L] >= cfg["target_recall"]:
            Lsel = L
            break
    dq = torch.from_numpy(query).to(dev)
    dout = torch.empty((nq, K), dtype=torch.int32, device=dev)
    ctx.srand(777)
    seeds = torch.from_numpy(ctx.draw_seeds(nq, Lsel, "rand").astype(np.int32)).to(dev)
    plan = ctx.plan(nq, K, dq.data_ptr(), dout.data_ptr(), L_max=Lsel, mode="seeds", d_seeds=seeds.data_ptr())
    plan.tune(nq)
    ms_p, kms_p, _, _ = _timed_plan(torch, plan, nq, args, stream, flush)
    plan.close()
    r_p = recall(dout.cpu().numpy().astype(np.uint32), gt, K)
    learned = run_learned(ctx, cfg, base, query, gt, args, dev, stream, flush)
    line = {"metric": "QPS at recall@10>=0.95 (learned+BF16 vs plain FP32, 10M x 128)",
            "value": round(learned["qps"], 1), "unit": "queries/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(learned["ms"], 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 candidates (f32 accumulate; exact on this integer data, so no f32 rerank)",
            "data": "synthetic (seeded integer Gaussian mixture)",
            "config": {"workload": f"{cfg['n']}x128 int-mixture(1024), {nq} held-out queries, top-10, NN-Descent "
                                   f"S=20 K=64 L=80 ITER=8 R=100 -> NSG R=32 L_refine=64 C_refine=500",
                       "build_s": round(build_s, 2),
                       "build_stages": {k: {kk: (round(vv, 2) if isinstance(vv, float) else vv)
                                            for kk, vv in v.items()} for k, v in stages.items()},
                       "learned": {k: (round(v, 4) if isinstance(v, float) else v) for k, v in learned.items()},
                       "plain_fp32": {"qps": round(nq / (ms_p / 1e3), 1), "L_search": Lsel,
                                      "recall@10": round(r_p, 4), "recall_sweep": sweep,
                                      "search_kernel_ms": round(kms_p, 4)},
                       "speedup_vs_plain": round(learned["qps"] / (nq / (ms_p / 1e3)), 3)},
            "e2e": {"value": round(learned["e2e_qps"], 1), "unit": "queries/s"}}
    print(json.dumps(line), flush=True)


def layered_graph_words(base, l0_ids, l0_deg, m, m0, seed, upper_rows):
    """A graph in the INDEX_HNSW file layout for the routing measurement (the
    HNSW build itself is not part of this library): layer 0 = the first m0
    entries of the given rows; levels drawn geometrically with HNSW's rule
    (P(level >= l) = m^-l); layer l >= 1 = upper_rows(ids) over the nodes of
    level >= l (rows of global ids, at most m each); the enterpoint is the
    first top-level node."""
    n = base.shape[0]
    rng = np.random.default_rng(seed)
    level = np.minimum(rng.geometric(1 - 1 / m, size=n) - 1, 8)
    top = int(level.max())
    ep = int(np.flatnonzero(level == top)[0])
    upper = {}
    for lv in range(1, top + 1):
        ids = np.flatnonzero(level >= lv)
        rows, deg = upper_rows(ids)
        upper[lv] = (ids, rows, deg)
    pos = {lv: {int(v): r for r, v in enumerate(upper[lv][0])} for lv in upper}
    deg0 = np.minimum(l0_deg, m0).astype(np.uint32)
    chunks = [np.array([ep, top], np.uint32)]
    for v in range(n):
        chunks.append(np.array([v, level[v] + 1, deg0[v]], np.uint32))
        chunks.append(l0_ids[v, :deg0[v]].astype(np.uint32))
        for lv in range(1, level[v] + 1):
            r = pos[lv][v]
            fr = upper[lv][1][r, :upper[lv][2][r]][:m]
            chunks.append(np.array([len(fr)], np.uint32))
            chunks.append(fr.astype(np.uint32))
    return np.concatenate(chunks), level


def run_graphs1m(args):
    """The rows built beyond the KGraph/NSG path, on the 1M x 128 data: the
    SSG refine (REFINE_SSG) and its SubCentroid search, the EFANNA refine
    (REFINE_EFANNA) from INIT_RANDOM, and HNSW routing (ROUTER_HNSW) over a
    layered graph whose layer 0 is the NN-Descent graph.  Search QPS are
    measured through the host entry points (queries copied in, ids out), at
    the smallest L of the grid with recall@10 >= 0.95."""
    import torch
    from weavess_gb300 import Context
    from weavess_gb300.groundtruth import knn_fp64
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    cfg = dict(CFG)
    if args.n:
        cfg["n"] = args.n
    if args.nq:
        cfg["nq"] = args.nq
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    base, query = make_data(cfg)
    gt = knn_fp64(base, query, 100)
    ctx = Context(0)
    K = cfg["k"]
    nq = query.shape[0]

    def timed_search(fn):
        fn()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(max(1, args.steps // 2)):
            out = fn()
        return nq * max(1, args.steps // 2) / (time.perf_counter() - t), out

    def sweep(fn, target=cfg["target_recall"]):
        for L in cfg["L_grid"]:
            res = fn(L)[0]
            r = recall(res, gt, K)
            log(f"  L={L} recall={r:.4f}")
            if r >= target:
                return L, r
        return cfg["L_grid"][-1], r

    out = {}
    # ---- KNN graph (shared by SSG and the HNSW layer 0)
    ctx.upload_base(base)
    ctx.srand(1)
    t = time.time()
    ctx.init_random(cfg["S"])
    ctx.nnd_refine(cfg["S"], cfg["K"], cfg["L"], cfg["ITER"], cfg["R"])
    torch.cuda.synchronize()
    knn_s = time.time() - t
    kids, kdist, kdeg, _ = ctx.get_graph()
    # ---- SSG
    t = time.time()
    st = ctx.ssg_refine(100, 50, 60.0, 10)
    torch.cuda.synchronize()
    ssg_s = time.time() - t
    ctx.load_built_graph()
    sids, sdist, sdeg, _ = ctx.get_graph()
    # the SSG graph searched from random seeds (SEARCH_ENTRY_RAND) ...
    Ls, rs = sweep(lambda L: ctx.search(query, L, K, entry="rand"))
    qps, _ = timed_search(lambda: ctx.search(query, Ls, K, entry="rand"))
    # ... and with the entry the reference's SSG test uses (SubCentroid: its
    # seed distances are taken to rows shifted by one float, so seeds with
    # wrong, small distances hold the head of the pool and recall stays low
    # -- the reference's own behaviour, reproduced exactly)
    Lsub = 256
    ctx.srand(5)
    res_sub, dc_sub, hc_sub = ctx.search(query, Lsub, K, entry="sub_centroid")
    qps_sub, _ = timed_search(lambda: ctx.search(query, Lsub, K, entry="sub_centroid"))
    g = O.Graph(sids, sdist, sdeg, 0)
    g.eps = st["eps"]
    smp = 1000
    tc = time.perf_counter()
    O.search(base, query[:smp], g, Ls, O.Rand(1), entry="rand", threads=os.cpu_count() or 1)
    cpu_ssg = smp / (time.perf_counter() - tc)
    out["ssg"] = {"refine_s": round(ssg_s, 2), "params": "L_refine=100 R_refine=50 A=60 n_try=10",
                  "avg_degree": float(sdeg.mean()), "conn_added": st["conn_added"],
                  "rand_entry": {"L_search": Ls, "recall@10": round(rs, 4), "qps_e2e": round(qps, 1),
                                 "cpu_oracle_qps": round(cpu_ssg, 1), "cpu_threads": os.cpu_count()},
                  "sub_centroid_entry": {"L_search": Lsub, "recall@10": round(recall(res_sub, gt, K), 4),
                                         "qps_e2e": round(qps_sub, 1), "dist_count": dc_sub}}
    log(f"ssg {out['ssg']}")
    # ---- HNSW routing over a layered graph (layer 0: the NSG rows built
    # from the same KNN graph, so that layer 0 is navigable)
    ctx.set_graph(kids, kdeg, dist=kdist)
    ctx.nsg_refine(cfg["L_refine"], cfg["R_refine"], cfg["C_refine"])
    nids, _, ndeg, _ = ctx.get_graph()
    sub = Context(local_device())

    def nsg_rows(ids):
        # upper layers: an NSG (R=16) over the layer's nodes; tiny layers are
        # fully connected
        if len(ids) <= 17:
            rows = np.array([[u for u in ids if u != v] + [0] * (17 - len(ids)) for v in ids], np.int64)
            return rows, np.full(len(ids), len(ids) - 1)
        sub.upload_base(np.ascontiguousarray(base[ids]))
        sub.srand(1)
        S = min(20, len(ids) - 2)
        sub.init_random(S)
        sub.nnd_refine(S, min(32, len(ids) - 1), min(40, len(ids) - 1), 8, 100)
        sub.nsg_refine(min(40, len(ids) - 1), 16, 200)
        r, _, d, _ = sub.get_graph()
        return ids[r.astype(np.int64)], d

    t = time.time()
    words, level = layered_graph_words(base, nids, ndeg, 16, 32, 5, nsg_rows)
    lay_s = time.time() - t
    ctx.load_hnsw(words)
    # (this synthetic layered graph tops out near recall 0.93: the target here is 0.90)
    Lh, rh = sweep(lambda L: ctx.search_hnsw(query, L, K), target=0.90)
    qps_h, (res_h, dc_h, hc_h) = timed_search(lambda: ctx.search_hnsw(query, Lh, K))
    tc = time.perf_counter()
    O.search_hnsw(base, query[:smp], words, Lh)
    cpu_h = smp / (time.perf_counter() - tc)
    out["hnsw"] = {"graph": f"layer 0 = the NSG rows (R={cfg['R_refine']}); {int((level > 0).sum())} upper-layer "
                            f"nodes (an NSG with R=16 per upper layer), top level {int(level.max())} (made in {lay_s:.1f}s)",
                   "L_search": Lh, "recall@10": round(rh, 4), "qps_e2e": round(qps_h, 1),
                   "dist_count": dc_h, "hop_count": hc_h, "cpu_oracle_qps_1thread": round(cpu_h, 1)}
    log(f"hnsw {out['hnsw']}")
    # ---- EFANNA refine from INIT_RANDOM
    ctx.srand(1)
    ctx.init_random(cfg["S"])
    t = time.time()
    est = ctx.efanna_refine(cfg["S"], cfg["K"], cfg["L"], cfg["ITER"], cfg["R"])
    torch.cuda.synchronize()
    ef_s = time.time() - t
    eids, _, edeg, _ = ctx.get_graph()
    sample = np.random.default_rng(1).choice(base.shape[0], 1000, replace=False)
    ex = knn_fp64(base, base[sample], 11)[:, 1:11]
    grec = float(np.mean([len(set(eids[v, :10].tolist()) & set(ex[i].tolist())) / 10 for i, v in enumerate(sample)]))
    out["efanna"] = {"refine_s": round(ef_s, 2), "params": f"S={cfg['S']} K={cfg['K']} L={cfg['L']} "
                     f"ITER={cfg['ITER']} R={cfg['R']} from INIT_RANDOM", "graph_recall@10_1000_nodes": round(grec, 4),
                     "pairs": est["pairs"], "rand_draws": est["rand_draws"], "nndescent_s_same_params": round(knn_s, 2)}
    log(f"efanna {out['efanna']}")
    # ---- the reference's EFANNA pipeline: INIT_KDT -> REFINE_EFANNA ->
    # SEARCH_ENTRY_KDT (parameters of its sift1M row, exp_data.h:320)
    kp = dict(nTrees=8, mLevel=8, K=60, L=70, ITER=10, S=15, R=150)
    ctx.srand(1)
    t = time.time()
    kst = ctx.init_kdt(kp["nTrees"], kp["K"], kp["mLevel"])
    torch.cuda.synchronize()
    kdt_s = time.time() - t
    kids2, _, _, _ = ctx.get_graph()
    krec = float(np.mean([len(set(kids2[v, :10].tolist()) & set(ex[i].tolist())) / 10 for i, v in enumerate(sample)]))
    t = time.time()
    ctx.efanna_refine(kp["S"], kp["K"], kp["L"], kp["ITER"], kp["R"])
    torch.cuda.synchronize()
    ef2_s = time.time() - t
    eids2, _, _, _ = ctx.get_graph()
    erec = float(np.mean([len(set(eids2[v, :10].tolist()) & set(ex[i].tolist())) / 10 for i, v in enumerate(sample)]))
    ctx.load_built_graph()
    Lk, rk = sweep(lambda L: ctx.search(query, L, K, entry="kdt"))
    qps_k, _ = timed_search(lambda: ctx.search(query, Lk, K, entry="kdt"))
    out["efanna_kdt"] = {"init_kdt_s": round(kdt_s, 2), "efanna_refine_s": round(ef2_s, 2),
                         "params": " ".join(f"{k}={v}" for k, v in kp.items()),
                         "kdt_graph_recall@10_1000_nodes": round(krec, 4),
                         "efanna_graph_recall@10_1000_nodes": round(erec, 4), "L_search": Lk,
                         "recall@10": round(rk, 4), "qps_e2e": round(qps_k, 1), "rand_draws": kst["rand_draws"]}
    log(f"efanna_kdt {out['efanna_kdt']}")
    line = {"metric": "HNSW routing QPS at recall@10>=0.90, with the SSG and EFANNA rows (1M x 128)",
            "value": out["hnsw"]["qps_e2e"], "unit": "queries/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded integer Gaussian mixture)",
            "config": {"workload": f"{cfg['n']}x128 int-mixture(256), {nq} queries, top-10", "rows": out}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--small", action="store_true", help="N=1e5 configuration (quick check)")
    ap.add_argument("--nq", type=int, default=0, help="override the number of queries")
    ap.add_argument("--n", type=int, default=0, help="override the number of base vectors")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned + bf16 leg")
    ap.add_argument("--link", choices=["nsg", "vamana"], default="nsg",
                    help="the graph: NSG (RNG prune, the default) or Vamana alpha=1.2 in the clean build mode")
    ap.add_argument("--vamana-L", type=int, default=64, help="L_refine of the Vamana link")
    ap.add_argument("--workload", default="int128",
                    choices=["int128", "precision96", "batch960", "learned10m", "graphs1m"],
                    help="int128: the 1M x 128 measurement (default); the others print informational lines")
    ap.add_argument("--profile-region", choices=["search", "build"], default="search",
                    help="region bracketed by cudaProfilerStart/Stop (ncu --profile-from-start off)")
    args = ap.parse_args()
    global PROFILE_REGION
    PROFILE_REGION = args.profile_region
    if args.impl == "reference":
        if rank() == 0:
            run_reference(args)
        return
    if args.workload != "int128" and rank() != 0:
        return  # the informational workloads run on rank 0 alone
    if args.workload == "int128" and world() > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_device())
        dist.init_process_group(backend="nccl")
    {"int128": run_ours, "precision96": run_precision96, "batch960": run_batch960,
     "learned10m": run_learned10m, "graphs1m": run_graphs1m}[args.workload](args)
    if _dist() is not None:
        _dist().destroy_process_group()


if __name__ == "__main__":
    main()
