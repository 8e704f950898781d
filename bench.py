"""Benchmark: points/sec of fit_sDbscan on the 1M x 784 Cosine workload.

One step = one full fit_sDbscan (transform, index, distances, core points,
clusters) of the whole workload through the engine's C ABI.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` times fits on data already resident in HBM with CUDA events on the
engine's stream; `e2e` times the public call with host (pinned) input, i.e.
the upload, the fit and the label download.  The reference arm
(`--impl reference`) times the CPU restatement of the reference (oracle/) on
all host cores, on a bounded sample of the same matrix.  Multi-GPU runs are
independent replicas of the workload (the path has no data exchange at this
tier), one process per GPU.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "points/sec fit_sDbscan: plain FP32 vs BF16+recheck & batched, at ARI≥0.99"
WORKLOADS = {
    2: dict(workload="cfg2_cosine_1Mx784", n=1_000_000, d=784, distance="Cosine", n_proj=1024, topK=10, topM=50,
            eps=0.25, minPts=50, seed=2007, fit="sdbscan"),
    1: dict(workload="cfg1_cosine_50Kx128", n=50_000, d=128, distance="Cosine", n_proj=1024, topK=5, topM=50,
            eps=0.15, minPts=20, seed=1007, fit="sdbscan"),
    # L2 through the random-Fourier embedding (ker 1024, sigma = median pairwise
    # distance of the first 10K points).  The literal data puts every point
    # farther than eps = 0.3 from all others, so the data is scaled by 0.0148:
    # the median 30-NN distance of the unscaled 1M set is 20.23 and
    # 0.3 / 20.23 = 0.0148 (scaling X and sigma together leaves the embedding's
    # law unchanged).
    3: dict(workload="cfg3_l2_rff_1Mx256_scaled", n=1_000_000, d=256, distance="L2", n_proj=1024, topK=10,
            topM=100, eps=0.3, minPts=30, seed=3007, fit="sdbscan", ker_n_features=1024, scale=0.3 / 20.234),
    # k, m, eps and minPts are not given for this config: k = 10, m = 50 (the
    # Python defaults), minPts = 50, and eps = 0.17, the median 50-NN Chi2
    # distance of 100 sampled points (about 60% of the points get reached).
    4: dict(workload="cfg4_chi2_soptics_500Kx512", n=500_000, d=512, distance="Chi2", n_proj=1024, topK=10,
            topM=50, eps=0.17, minPts=50, seed=4007, fit="soptics", ker_n_features=1024),
}
# flops per dimension of one candidate distance (multiply-add = 2; L2 sub + fma;
# Chi2 mul, add, div, add)
DIST_FLOPS = {"Cosine": 2, "L2": 3, "L1": 3, "Chi2": 4, "JS": 8}
FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.070e9 / 1e12  # nominal FP32 CUDA-core peak at max SM clock
# DRAM bytes (read + write) of one k_dist<Cosine> launch on the 1M x 784
# workload, from a one-pass ncu capture of
# `python bench.py --single-fit 1000000 --precision 0` (profiles/k_dist_fp32_cfg2.md):
# 23.29 GB read + 0.370 GB written (tiles run in point-chunk order).
K_DIST_TRAFFIC_1M = 23.29e9 + 0.370e9
# One CPU fit of the whole 1M x 784 config-2 workload (the reference arm's code,
# all 16 host cores of the GPU machine): `python bench.py --impl reference
# --cpu-full-fit`, recorded in profiles/cpu_full_fit_cfg2_1Mx784.md (23 minutes,
# too long to repeat inside a benchmark run).
CPU_FULL_FIT_CFG2 = {"seconds": 1389.7, "value": 719.6, "unit": "points/s", "cores": 16, "kind": "port",
                     "source": "profiles/cpu_full_fit_cfg2_1Mx784.md"}
# sngDBSCAN, the reference's sampling baseline that its benchmark loop runs
# next to fit_sDbscan (src/main.cpp:57-73): samplingProb 0.01 (the default,
# 10,000 draws per point at 1M points), seed 42, the workload's eps / minPts.
SNG_PROB, SNG_SEED = 0.01, 42


def _peaks():
    """Measured HBM copy GB/s and cuBLAS BF16 TFLOP/s of this GPU pool."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            m = json.load(f)
        return m["hbm_gbs"], m["bf16_tflops_sustained"], "measured"
    except Exception:
        return 6800.0, 1700.0, "fallback"


def _dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _sgemm_tflops(device, n=8192, reps=6):
    """cuBLAS FP32 GEMM rate on this GPU (TF32 off): the practical FP32 ceiling
    the exact distance kernels are compared with (a reference figure only)."""
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        a = torch.randn(n, n, device=device)
        b = torch.randn(n, n, device=device)
        for _ in range(2):
            c = a @ b
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            c = a @ b
        e1.record()
        torch.cuda.synchronize()
        del a, b, c
        return 2.0 * n ** 3 * reps / (e0.elapsed_time(e1) / 1e3) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def _h2d_copy_ms(src_pinned, dst, reps=3):
    """Best of `reps` plain host -> device copies of a pinned tensor (CUDA events)."""
    import torch
    best = None
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        dst.copy_(src_pinned, non_blocking=True)
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1)
        best = t if best is None else min(best, t)
    return best


def _max_over_ranks(x: float, ws: int, device) -> float:
    """The largest of every rank's x: a replicated job takes its slowest
    replica's time."""
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _replica_rate(units_per_rank: float, steps: int, ws: int, seconds: float) -> float:
    """Whole-job throughput of ws replicas that each process units_per_rank per step."""
    return ws * units_per_rank * steps / seconds


def _host_data(cfg, n):
    """The workload's law, n points, as a numpy (n, d) float32 array."""
    from sdbscan_gb300 import datasets
    w = cfg["workload"]
    if w.startswith("cfg2"):
        return datasets.cfg2_mnist_like(n, cfg["d"], seed=cfg["seed"])[0]
    if w.startswith("cfg3"):
        return datasets.cfg3_aniso_l2(n, cfg["d"], seed=cfg["seed"], scale=cfg["scale"])[0]
    if w.startswith("cfg4"):
        return datasets.cfg4_dirichlet(n, cfg["d"], seed=cfg["seed"])[0]
    return datasets.cfg1_cosine(n, cfg["d"], seed=cfg["seed"])[0]


def _make_data(cfg, device):
    import torch
    from sdbscan_gb300 import datasets
    if cfg["workload"].startswith("cfg2"):
        X, _ = datasets.cfg2_mnist_like_torch(cfg["n"], cfg["d"], seed=cfg["seed"], device=device)
    else:
        X = torch.from_numpy(_host_data(cfg, cfg["n"])).to(device)
    return X.contiguous()


def _kernel_params(cfg, X=None):
    """ker_n_features / ker_sigma for the embedded distances; sigma is the
    median pairwise distance of the first 10K points (L1/L2)."""
    out = {}
    if "ker_n_features" in cfg:
        out["ker_n_features"] = cfg["ker_n_features"]
    if cfg["distance"] in ("L1", "L2") and X is not None:
        import torch
        a = torch.as_tensor(X[:10000]).float().cuda() if not torch.is_tensor(X) else X[:10000].float()
        d2 = (a.pow(2).sum(1)[:, None] + a.pow(2).sum(1)[None, :] - 2 * a @ a.T).clamp_min(0).sqrt()
        iu = torch.triu_indices(a.shape[0], a.shape[0], 1, device=a.device)
        out["ker_sigma"] = float(d2[iu[0], iu[1]].median())
    return out


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        # the raw samples (the JSON line carries their summary); SDB_CLOCKS_DIR keeps them
        self.path = os.path.join(os.environ.get("SDB_CLOCKS_DIR", tempfile.gettempdir()),
                                 f"sdbscan_clocks_gpu{gpu_index}_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        text = open(self.path).read()
        if "SDB_CLOCKS_DIR" not in os.environ:
            os.remove(self.path)  # kept only where asked for
        return self.parse(text)

    @staticmethod
    def parse(text):
        """Median SM clock, the maximum clock and the throttle reasons seen in
        nvidia-smi's CSV rows (FIELDS order, no header, no units)."""
        rows = [r.split(", ") for r in text.strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = float(rows[0][2]) if rows[0][2].replace(".", "").isdigit() else None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


def _cpu_sample_rate(Xh, cfg, n_sample, kp=None):
    """The oracle (CPU restatement of the reference) on the first n_sample
    points, all host threads.  Returns (points/s, threads, seconds)."""
    from oracle.oracle import Port, build_port
    build_port()
    port = Port()
    threads = os.cpu_count() or 1
    kp = kp or {}
    kw = dict(dist=cfg["distance"], n_proj=cfg["n_proj"], topK=cfg["topK"], topM=cfg["topM"], seed=42,
              threads=threads)
    if "ker_n_features" in kp:
        kw["ker"] = kp["ker_n_features"]
    if "ker_sigma" in kp:
        kw["sigma"] = kp["ker_sigma"]
    fit = port.fit_soptics if cfg["fit"] == "soptics" else port.fit_sdbscan
    port.set_timing_mode(True)  # distances at the reference's vectorised-Eigen speed
    try:
        t0 = time.perf_counter()
        fit(Xh[:n_sample], cfg["eps"], cfg["minPts"], **kw)
        dt = time.perf_counter() - t0
    finally:
        port.set_timing_mode(False)
    return n_sample / dt, threads, dt


def _np_median_pair(a):
    """Median pairwise L2 distance of the rows of a (numpy, CPU)."""
    import numpy as np
    a = a.astype(np.float64)
    sq = (a * a).sum(1)
    d2 = np.maximum(sq[:, None] + sq[None, :] - 2.0 * a @ a.T, 0.0)
    iu = np.triu_indices(a.shape[0], 1)
    return float(np.median(np.sqrt(d2[iu])))


def run_reference(args, cfg):
    """CPU reference arm: the oracle restatement of the reference's fit path,
    each step a bounded sample of the workload."""
    ws, rank, _ = _dist_env()
    if rank != 0:
        return 0
    import numpy as np
    from sdbscan_gb300 import datasets
    n_sample = min(args.cpu_sample, cfg["n"])
    Xh = _host_data(cfg, n_sample)
    kp = _kernel_params(cfg, Xh) if cfg["distance"] not in ("L1", "L2") else {
        "ker_n_features": cfg["ker_n_features"], "ker_sigma": _np_median_pair(Xh[:2000])}
    rates = []
    for i in range(args.warmup + args.steps):
        r, threads, dt = _cpu_sample_rate(Xh, cfg, n_sample, kp)
        if i >= args.warmup:
            rates.append((r, dt))
    total_pts = n_sample * args.steps
    total_s = sum(dt for _, dt in rates)
    value = total_pts / total_s
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": f"synthetic ({cfg['workload']} law, numpy, seed {cfg['seed']})",
        "config": {"workload": cfg["workload"], "n": cfg["n"], "d": cfg["d"], "n_proj": cfg["n_proj"],
                   "topK": cfg["topK"], "topM": cfg["topM"], "eps": cfg["eps"], "minPts": cfg["minPts"]},
        "cpu_baseline": {"value": value, "unit": "points/s", "cores": threads, "kind": "port",
                         "sample": f"full fit_{'sOptics' if cfg['fit'] == 'soptics' else 'sDbscan'} on {n_sample} "
                                   f"points of the workload's law per step "
                                   f"(oracle/ restatement with vectorised distances, the reference's Eigen "
                                   f"speed; OpenMP, {threads} threads)"},
        "e2e": {"value": value, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_cpu_full_fit(args, cfg):
    """One fit of the whole workload (all n points) by the CPU restatement of
    the reference (the reference arm's code, timing mode, all host threads):
    the same-config CPU figure beside the sampled per-step rate.  The data is
    the GPU arm's (the config's law drawn with torch, on the GPU when there is
    one, then copied to the host).  Prints one JSON line."""
    import torch
    from sdbscan_gb300 import datasets
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    if cfg["workload"].startswith("cfg2"):
        X, _ = datasets.cfg2_mnist_like_torch(cfg["n"], cfg["d"], seed=cfg["seed"], device=dev)
        Xh = X.cpu().numpy()
        del X
    else:
        Xh = _host_data(cfg, cfg["n"])
    if dev == "cuda":
        torch.cuda.empty_cache()
    kp = _kernel_params(cfg, Xh) if cfg["distance"] not in ("L1", "L2") else {
        "ker_n_features": cfg["ker_n_features"], "ker_sigma": _np_median_pair(Xh[:2000])}
    rate, threads, dt = _cpu_sample_rate(Xh, cfg, cfg["n"], kp)
    print(json.dumps({"impl": "reference", "cpu_full_fit": {
        "workload": cfg["workload"], "n": cfg["n"], "seconds": dt, "value": rate, "unit": "points/s",
        "cores": threads, "kind": "port",
        "form": f"one full fit_{'sOptics' if cfg['fit'] == 'soptics' else 'sDbscan'} of the whole workload "
                f"(oracle/ restatement of the reference's loop, vectorised distances, OpenMP)"}}))
    return 0


def run_batched(args, local, cpu=True):
    """Config 5: 64 vMF mixtures (n log-uniform 2K..200K, d in {64,128,256}),
    an 8-value eps sweep each (0.05 .. 0.40), minPts 20, D 1024, k 5, m 50.

    Three GPU forms of the same 512 clusterings:
      - batched BF16+recheck: one CUDA graph of all sets' sweeps, BF16-screened distances;
      - batched plain: the same graph with plain FP32 distances;
      - plain fits: 512 separate fit_sDbscan calls (one per set and eps).
    Rate = sum(n) * 8 / time.  The labels of all three forms are compared."""
    import numpy as np
    import torch
    from sdbscan_gb300 import capi, datasets
    sets = datasets.cfg5_batch_torch(64, seed=5007, device=f"cuda:{local}")
    torch.cuda.synchronize()
    eps_list = [0.05 * (i + 1) for i in range(8)]
    ptrs = [(X.data_ptr(), X.shape[0], X.shape[1]) for X, _ in sets]
    total_n = sum(X.shape[0] for X, _ in sets)
    params = dict(n_proj=1024, topK=5, topM=50, distance="Cosine", random_seed=42)

    def graph(precision):
        t0 = time.perf_counter()
        b = capi.Batch(ptrs, eps_list, 20, device=local, precision=precision, **params)
        setup_s = time.perf_counter() - t0
        for _ in range(max(3, args.warmup)):
            b.run()
        times = [b.run() for _ in range(args.steps)]
        labels = [[b.labels(i, j) for j in range(len(eps_list))] for i in range(len(sets))]
        lanes = (b.lanes(), b.tile_variants())
        b.close()
        return sum(times) / len(times), setup_s, lanes, labels

    bms, bsetup, blanes, blabels = graph(capi.PREC_BF16)
    pms, psetup, planes, plabels = graph(capi.PREC_FP32)
    bf16_identical = all(np.array_equal(blabels[i][j][0], plabels[i][j][0]) and blabels[i][j][1] == plabels[i][j][1]
                         for i in range(len(sets)) for j in range(len(eps_list)))

    # plain GPU form: one fit_sDbscan per (set, eps), device-resident input
    engines = []
    for X, _ in sets:
        e = capi.Engine(X.shape[0], X.shape[1], device=local)
        e.set_params(**params)
        engines.append(e)
    fits_identical = True
    for i, ((X, _), e) in enumerate(zip(sets, engines)):  # warm-up pass, checks the labels
        for j, eps in enumerate(eps_list):
            e.fit_sdbscan_device(X.data_ptr(), eps, 20)
            lab, ncl = e.labels()
            fits_identical &= bool(np.array_equal(lab, plabels[i][j][0])) and ncl == plabels[i][j][1]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for (X, _), e in zip(sets, engines):
        for eps in eps_list:
            e.fit_sdbscan_device(X.data_ptr(), eps, 20)
    torch.cuda.synchronize()
    fits_s = time.perf_counter() - t0
    for e in engines:
        e.close()
    rate = lambda sec: total_n * len(eps_list) / sec
    out = {"workload": "cfg5_64sets_x8eps", "value": rate(bms / 1e3), "unit": "point-clusterings/s",
           "form": "BF16+recheck, one CUDA graph (per set the autotuner keeps the screening or a plain tile "
                   "shape, whichever ran the set's distance stage faster)",
           "ms_per_batch": bms, "sets": len(sets), "points": total_n,
           "eps": [round(e, 2) for e in eps_list], "launches_per_batch": 1, "graph_lanes": blanes[0],
           "screened_sets": blanes[1].count(0),
           "setup_s": bsetup, "labels_identical_to_plain": bf16_identical,
           "plain_graph": {"value": rate(pms / 1e3), "ms_per_batch": pms, "graph_lanes": planes[0],
                           "tile_variants": {str(v): planes[1].count(v) for v in sorted(set(planes[1]))},
                           "setup_s": psetup},
           "plain_fits": {"value": rate(fits_s), "ms_per_batch": fits_s * 1e3, "fits": len(sets) * len(eps_list),
                          "labels_identical_to_graph": fits_identical,
                          "form": "512 separate fit_sDbscan calls on device-resident data"},
           "n_clusters_eps0.20_first4": [plabels[i][3][1] for i in range(4)]}
    if cpu:  # in a fresh process, like the reference arm
        out["cpu_baseline"] = _subprocess_json([sys.executable, os.path.abspath(__file__), "--impl", "reference",
                                                "--batched-cpu"])
    return out


def _subprocess_json(cmd):
    """Runs cmd and returns the JSON object of its last output line (None on failure)."""
    try:
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=900, env=dict(os.environ, WORLD_SIZE="1",
                                                                                      RANK="0", LOCAL_RANK="0"))
        line = [x for x in r.stdout.strip().splitlines() if x.startswith("{")][-1]
        return json.loads(line)
    except Exception:
        return None


def _cpu_batched(n_sets=6):
    """The oracle on the n_sets smallest datasets of the config-5 law (numpy
    generator), all host threads: separate fit_sDbscan calls per eps, and the
    reference's own index-once sweep (test_sDbscan).  Point-clusterings/s."""
    from oracle.oracle import Port, build_port
    from sdbscan_gb300 import datasets
    build_port()
    port = Port()
    threads = os.cpu_count() or 1
    sets = datasets.cfg5_batch(64, seed=5007)
    eps_list = [0.05 * (i + 1) for i in range(8)]
    params = dict(n_proj=1024, topK=5, topM=50, distance="Cosine", random_seed=42)
    order = sorted(range(len(sets)), key=lambda i: sets[i][0].shape[0])[:n_sets]
    Xs = [sets[i][0] for i in order]
    kw = dict(dist=params["distance"], n_proj=params["n_proj"], topK=params["topK"], topM=params["topM"],
              seed=params["random_seed"], threads=threads)
    pts = sum(X.shape[0] for X in Xs) * len(eps_list)
    port.set_timing_mode(True)  # distances at the reference's vectorised-Eigen speed
    try:
        t0 = time.perf_counter()
        for X in Xs:
            for eps in eps_list:
                port.fit_sdbscan(X, eps, 20, **kw)
        fits_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        for X in Xs:
            port.fit_sdbscan_sweep(X, eps_list, 20, **kw)
        sweep_s = time.perf_counter() - t0
    finally:
        port.set_timing_mode(False)
    return {"value": pts / sweep_s, "unit": "point-clusterings/s", "cores": threads, "kind": "port",
            "form": "index-once eps sweep (test_sDbscan pattern)", "separate_fits_value": pts / fits_s,
            "sample": f"the {n_sets} smallest datasets ({sum(X.shape[0] for X in Xs)} points) x 8 eps "
                      f"(oracle/ restatement with vectorised distances, OpenMP, {threads} threads; "
                      f"sweep {sweep_s:.1f} s, fits {fits_s:.1f} s)"}


def _cpu_sng(cfg, n_sample=20000):
    """The oracle's sngDbscan (point-by-point restatement of
    sng_findCorePoints) on n_sample points of the workload's law with the
    same number of draws per point as the full workload (ceil(0.01 n) =
    10,000 at 1M points), all host threads.  Points/s."""
    from oracle.oracle import Port, build_port
    build_port()
    port = Port()
    threads = os.cpu_count() or 1
    Xh = _host_data(cfg, n_sample)
    draws = -(-cfg["n"] * SNG_PROB // 1)
    prob = float(draws) / n_sample
    assert prob < 1.0, "the sample must stay in the sampled branch (samplingProb < 1)"
    port.set_timing_mode(True)  # distances at the reference's vectorised-Eigen speed
    try:
        t0 = time.perf_counter()
        port.fit_sngdbscan(Xh, cfg["eps"], cfg["minPts"], dist=cfg["distance"], samplingProb=prob, seed=SNG_SEED,
                           threads=threads)
        dt = time.perf_counter() - t0
    finally:
        port.set_timing_mode(False)
    return {"value": n_sample / dt, "unit": "points/s", "cores": threads, "kind": "port",
            "sample": f"fit_sngDbscan on {n_sample} points of the workload's law, samplingProb {prob:g} "
                      f"({int(draws)} draws per point, as the full workload), oracle/ restatement with vectorised "
                      f"distances (the reference's Eigen speed), OpenMP, "
                      f"{threads} threads, {dt:.1f} s"}


def run_sng(args, local, X, cfg, cpu=True):
    """sngDBSCAN on the headline data (n x d resident in HBM): one step =
    one fit_sngDbscan (transform, sample, dense distance block, degrees,
    union-find labels).  Dominant kernel: k_sng_block, n x (sampled points) x d."""
    import numpy as np
    import torch
    from sdbscan_gb300 import capi
    n, d = X.shape
    eng = capi.Engine(n, d, device=local)
    eng.set_sng_params(distance=cfg["distance"], samplingProb=SNG_PROB, random_seed=SNG_SEED)
    stream = torch.cuda.ExternalStream(eng.stream(), device=f"cuda:{local}")
    for _ in range(max(1, min(args.warmup, 2))):
        eng.fit_sngdbscan_device(X.data_ptr(), cfg["eps"], cfg["minPts"])
    torch.cuda.synchronize()
    steps = max(1, min(args.steps, 3))
    st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stages, launches = {}, 0
    st.record(stream)
    for _ in range(steps):
        eng.fit_sngdbscan_device(X.data_ptr(), cfg["eps"], cfg["minPts"])
        for k_, v_ in eng.stage_ms().items():
            stages[k_] = stages.get(k_, 0.0) + v_ / steps
        launches += eng.counters()["launches"]
    en.record(stream)
    torch.cuda.synchronize()
    ms = st.elapsed_time(en) / steps
    c = eng.counters()
    labels, ncl = eng.labels()
    core, _ = eng.core()
    flops = float(DIST_FLOPS[cfg["distance"]]) * n * c["sng_sampled"] * d
    achieved = flops / (stages["distances"] / 1e3) / 1e12
    # BF16 screening (Cosine): the block on the tensor cores, pairs near eps
    # re-decided in FP32; the labels must equal the FP32 fit's
    bf16 = None
    if cfg["distance"] == "Cosine" and not args.no_bf16:
        eng.set_precision(capi.PREC_BF16)
        for _ in range(max(1, min(args.warmup, 2))):
            eng.fit_sngdbscan_device(X.data_ptr(), cfg["eps"], cfg["minPts"])
        torch.cuda.synchronize()
        bstages = {}
        st.record(stream)
        for _ in range(steps):
            eng.fit_sngdbscan_device(X.data_ptr(), cfg["eps"], cfg["minPts"])
            for k_, v_ in eng.stage_ms().items():
                bstages[k_] = bstages.get(k_, 0.0) + v_ / steps
        en.record(stream)
        torch.cuda.synchronize()
        bms = st.elapsed_time(en) / steps
        bl, bn = eng.labels()
        bc = eng.counters()
        _, bf16_peak, src = _peaks()
        bach = 2.0 * n * c["sng_sampled"] * d / (bstages["distances"] / 1e3) / 1e12
        bf16 = {"value": n / (bms / 1e3), "unit": "points/s", "ms_per_step": bms, "stage_ms": bstages,
                "labels_identical": bool(np.array_equal(bl, labels)) and bn == ncl,
                "rechecked_pairs": bc["rechecked"], "fallbacks": bc["fallbacks"],
                "roofline": {"bound": "tensor", "kernel": "distance stage: k_sng_tc + k_sng_recheck",
                             "achieved": bach, "peak": bf16_peak, "unit": "TFLOP/s", "frac": bach / bf16_peak,
                             "traffic": None, "stage_ms": bstages["distances"],
                             "peak_source": f"{src} bf16_tflops_sustained (timed inside the fit)"}}
    eng.close()
    out = {"metric": "points/sec fit_sngDbscan (sampled-neighbourhood baseline)", "value": n / (ms / 1e3),
           "unit": "points/s", "ms_per_step": ms, "steps": steps, "gpu_launches": launches,
           "config": {"samplingProb": SNG_PROB, "random_seed": SNG_SEED, "eps": cfg["eps"], "minPts": cfg["minPts"],
                      "draws_per_point": int(-(-n * SNG_PROB // 1)), "distinct_sampled": c["sng_sampled"],
                      "extra_draws": c["sng_extra"]},
           "roofline": {"bound": "fp32", "kernel": f"k_sng_block<{cfg['distance']}>", "achieved": achieved,
                        "peak": FP32_PEAK_TFLOPS, "unit": "TFLOP/s", "frac": achieved / FP32_PEAK_TFLOPS,
                        "traffic": None, "flops_per_launch": flops, "kernel_ms": stages["distances"],
                        "peak_source": "nominal FP32 CUDA-core peak (152 SMs x 128 lanes x 2 flop x 2.07 GHz)"},
           "stage_ms": stages,
           "result": {"n_clusters": int(ncl), "cores": int(core.sum()), "noise": int((labels < 0).sum())},
           "bf16_screening": bf16,
           "cpu_baseline": None}
    if cpu:
        out["cpu_baseline"] = _subprocess_json([sys.executable, os.path.abspath(__file__), "--impl", "reference",
                                                "--config", str(args.config), "--sng-cpu"])
    return out


def run_ours(args, cfg):
    import numpy as np
    import torch
    ws, rank, local = _dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from sdbscan_gb300 import capi

    n, d = cfg["n"], cfg["d"]
    X = _make_data(cfg, f"cuda:{local}")
    torch.cuda.synchronize()
    kp = _kernel_params(cfg, X)
    optics = cfg["fit"] == "soptics"
    eng = capi.Engine(n, d, device=local)

    def params(precision=capi.PREC_FP32):
        eng.set_params(n_proj=cfg["n_proj"], topK=cfg["topK"], topM=cfg["topM"], distance=cfg["distance"],
                       random_seed=42, precision=precision, **kp)

    def fit_dev():
        (eng.fit_soptics_device if optics else eng.fit_sdbscan_device)(X.data_ptr(), cfg["eps"], cfg["minPts"])

    def result():
        return eng.optics() if optics else eng.labels()

    params()
    stream = torch.cuda.ExternalStream(eng.stream(), device=f"cuda:{local}")

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        fit_dev()
    barrier()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    stage_sum = {}
    launches = 0
    with ClockSampler(local) as clk:
        start.record(stream)
        for _ in range(args.steps):
            fit_dev()
            for k_, v_ in eng.stage_ms().items():
                stage_sum[k_] = stage_sum.get(k_, 0.0) + v_
            launches += eng.counters()["launches"]
        end.record(stream)
        barrier()
    ms = _max_over_ranks(start.elapsed_time(end), ws, f"cuda:{local}")
    value = _replica_rate(n, args.steps, ws, ms / 1e3)
    counters = eng.counters()
    res = result()
    labels = None if optics else res[0]

    # BF16 mode on the same data: Cosine distances screened on the tensor cores
    # with exact re-decision (identical labels); L1/L2 embedding GEMM on the
    # tensor cores (labels compared by ARI)
    bf16 = None
    if not args.no_bf16 and not optics and cfg["distance"] in ("Cosine", "L1", "L2"):
        params(capi.PREC_BF16)
        for _ in range(args.warmup):
            fit_dev()
        barrier()
        sb, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        bstages = {}
        sb.record(stream)
        for _ in range(args.steps):
            fit_dev()
            for k_, v_ in eng.stage_ms().items():
                bstages[k_] = bstages.get(k_, 0.0) + v_
        eb.record(stream)
        barrier()
        bms = sb.elapsed_time(eb)
        blabels, bncl = eng.labels()
        bc = eng.counters()
        from tests._metrics import adjusted_rand_score
        _, bf16_peak, src = _peaks()
        if cfg["distance"] == "Cosine":
            flops = 2.0 * (2 * cfg["topK"] * cfg["topM"]) * d * n
            stage_s = bstages["distances"] / args.steps / 1e3
            kern = "distance stage: k_to_bf16 + k_dist_tc + k_recheck"
        else:
            flops = 2.0 * n * d * (kp["ker_n_features"] // 2)
            stage_s = bstages["project"] / args.steps / 1e3
            kern = "projection stage incl. the embedding GEMM k_rff_tc (upper bound on its time)"
        broof = {"bound": "tensor", "kernel": kern,
                 "achieved": flops / stage_s / 1e12, "peak": bf16_peak, "unit": "TFLOP/s",
                 "frac": flops / stage_s / 1e12 / bf16_peak, "traffic": None,
                 "peak_source": f"{src} bf16_tflops_sustained (timed inside the fit)",
                 "flops_per_launch": flops, "stage_ms": stage_s * 1e3}
        bf16 = {"value": ws * n * args.steps / (bms / 1e3), "unit": "points/s", "ms_per_step": bms / args.steps,
                "roofline": broof,
                "ari_vs_plain": adjusted_rand_score(labels, blabels), "labels_identical": bool(np.array_equal(labels, blabels)),
                "rechecked_pairs": bc["rechecked"], "fallbacks": bc["fallbacks"],
                "stage_ms": {k_: v_ / args.steps for k_, v_ in bstages.items()}}
        params()

    # end to end through the public call: pinned host input, labels back
    Xh_t = torch.empty((n, d), dtype=torch.float32, pin_memory=True)
    Xh_t.copy_(X)
    Xh = Xh_t.numpy()
    fit_host = eng.fit_soptics if optics else eng.fit_sdbscan
    for _ in range(max(2, args.warmup)):
        fit_host(Xh, cfg["eps"], cfg["minPts"])
        result()
    barrier()
    t0 = time.perf_counter()
    e2e_stages = {}
    e2e_upload_stage = []  # per step: the projection stage, which the upload feeds
    for _ in range(args.steps):
        fit_host(Xh, cfg["eps"], cfg["minPts"])
        res_e2e = result()
        st_ = eng.stage_ms()
        e2e_upload_stage.append(round(st_["project"], 2))
        for k_, v_ in st_.items():
            e2e_stages[k_] = e2e_stages.get(k_, 0.0) + v_ / args.steps
    barrier()
    e2e_s = _max_over_ranks(time.perf_counter() - t0, ws, f"cuda:{local}")
    e2e_value = _replica_rate(n, args.steps, ws, e2e_s)
    assert all(np.array_equal(a, b) for a, b in zip(res_e2e[:1], res[:1])), "host-input and device-input fits disagree"
    d2h = n * 8 if optics else n * 4 + 4
    h2d_ms = _h2d_copy_ms(Xh_t, X)  # Xh_t holds X's own values, so X is unchanged

    sng = None
    if not args.no_sng and cfg["workload"].startswith("cfg2"):
        sng = run_sng(args, local, X, cfg, cpu=ws == 1 and not args.no_cpu)
    batched = None
    if not args.no_batched and cfg["workload"].startswith("cfg2"):
        batched = run_batched(args, local, cpu=ws == 1 and not args.no_cpu)
    if rank != 0:
        return 0
    # dominant kernel: the distance stage (one k_dist launch per fit)
    dist_ms = stage_sum["distances"] / args.steps
    flops = float(DIST_FLOPS[cfg["distance"]]) * (2 * cfg["topK"] * cfg["topM"]) * d * n
    achieved = flops / (dist_ms / 1e3) / 1e12
    hbm_peak, _, src = _peaks()
    traffic = K_DIST_TRAFFIC_1M if cfg["workload"].startswith("cfg2") else None
    alg_bytes = n * d * 4 + 2 * cfg["n_proj"] * cfg["topM"] * d * 4  # rows of X + candidate rows, once each
    sgemm = _sgemm_tflops(f"cuda:{local}")
    roofline = {"bound": "fp32", "kernel": f"k_dist<{cfg['distance']}>", "achieved": achieved, "peak": FP32_PEAK_TFLOPS,
                "unit": "TFLOP/s", "frac": achieved / FP32_PEAK_TFLOPS, "traffic": traffic,
                "measured_fp32_gemm": {"tflops": sgemm, "frac": achieved / sgemm,
                                       "source": "cuBLAS FP32 GEMM 8192^3, TF32 off, timed in this run"},
                "bound_note": "exact FP32 SIMT grouped GEMM (sequential fmaf per pair): bounded by the FP32 FMA "
                              "pipe, not by HBM or the tensor cores; the BF16 leg carries the tensor roofline",
                "peak_source": "nominal FP32 CUDA-core peak (152 SMs x 128 lanes x 2 flop x 2.07 GHz); "
                               "MEASURED_PEAKS.json has no FP32 figure",
                "traffic_source": "ncu dram__bytes_read+write of one k_dist launch on this workload",
                "hbm_view": {"algorithmic_bytes": alg_bytes, "achieved_gbs": alg_bytes / (dist_ms / 1e3) / 1e9,
                             "measured_traffic_gbs": traffic / (dist_ms / 1e3) / 1e9 if traffic else None,
                             "peak_gbs": hbm_peak, "peak_source": src},
                "flops_per_launch": flops, "kernel_ms": dist_ms}
    stages = {k_: v_ / args.steps for k_, v_ in stage_sum.items()}
    cpu = None
    if ws == 1 and not args.no_cpu:
        # the reference arm itself, in a fresh process (this one holds
        # torch's OpenMP runtime, whose spinning threads would share the cores)
        ref = _subprocess_json([sys.executable, os.path.abspath(__file__), "--impl", "reference", "--config",
                                str(args.config), "--steps", "2", "--warmup", "1", "--cpu-sample",
                                str(args.cpu_sample)])
        cpu = ref.get("cpu_baseline") if ref else None
        if cpu is not None and cfg["workload"].startswith("cfg2"):
            cpu = dict(cpu, full_fit=CPU_FULL_FIT_CFG2)  # the same config, all 1M points, recorded once
    line = {
        "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": ("synthetic (config-2 law: Bernoulli(0.2) x U(0.3,1) prototypes, 10% redraw, L2-normalised; "
                 "drawn on device, seed 2007)") if cfg["workload"].startswith("cfg2") else
                f"synthetic ({cfg['workload']} law, numpy, seed {cfg['seed']})",
        "config": {"workload": cfg["workload"], "n": n, "d": d, "distance": cfg["distance"],
                   "fit": "fit_sOptics" if optics else "fit_sDbscan", "n_proj": cfg["n_proj"], "topK": cfg["topK"],
                   "topM": cfg["topM"], "eps": cfg["eps"], "minPts": cfg["minPts"], "precision": "fp32",
                   **kp, "parallelism": f"replicas x{ws}",
                   "l2": f"inputs larger than L2 ({n * d * 4 / 1e9:.2f} GB per step)" if n * d * 4 > 129e6 else
                         "inputs smaller than L2: L2 flushed between steps is not done; small workload"},
        "clocks": clk.summary(),
        "e2e": {"value": e2e_value, "unit": "points/s", "h2d_bytes_per_step": n * d * 4,
                "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * e2e_s / args.steps,
                "stage_ms": e2e_stages, "project_stage_ms_per_step": e2e_upload_stage,
                "h2d_link": {"copy_ms": h2d_ms, "gbs": n * d * 4 / (h2d_ms / 1e3) / 1e9,
                             "note": "one plain pinned-host -> device copy of the step's input on this box "
                                     "(the upload floor of the step)"}},
        "gpu_launches": launches,
        "roofline": roofline,
        "cpu_baseline": cpu,
        "stage_ms": stages,
        "bf16_screening": bf16,
        "batched": batched,
        "sng": sng,
        "result": ({"reachable": int((res[1] >= 0).sum()), "max_reachability": float(res[1].max())} if optics else
                   {"n_clusters": res[1], "noise": int((labels < 0).sum())}) |
                  {"topk_ties": counters["topk_ties"], "topm_ties": counters["topm_ties"],
                   "pairs_within_eps": counters["pairs"]},
    }
    print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_single_fit(args):
    """One fit on the config-2 law at n = args.single_fit points, with the
    engine's per-stage CUDA-event times and counters printed as one JSON
    line: the small, self-contained case the ncu captures in profiles/ run.
    --fit sdbscan / soptics / sweep (d, distance: Cosine, or L1 / L2 / Chi2
    with ker 1024, sigma 1; --noise 1 for sDbscan-1NN), or sng / sngoptics
    (Cosine, samplingProb --prob, --sng-sampling); eps 0.25, minPts 50,
    seed 42."""
    import torch

    from sdbscan_gb300 import capi, datasets
    n, d, dist = args.single_fit, args.d, args.distance
    X, _ = datasets.cfg2_mnist_like_torch(n, d, seed=2007, device="cuda")
    torch.cuda.synchronize()
    eng = capi.Engine(n, d)
    if args.fit in ("sng", "sngoptics"):
        eng.set_sng_params(distance=dist, samplingProb=args.prob, random_seed=42)
        eng.set_precision(args.precision)
        if args.sng_sampling:
            eng.set_sng_sampling(args.sng_sampling)
        if args.fit == "sngoptics":
            eng.fit_sngoptics_device(X.data_ptr(), 0.25, 50)
        else:
            eng.fit_sngdbscan_device(X.data_ptr(), 0.25, 50)
    else:
        kw = dict(ker_n_features=1024, ker_sigma=1.0) if dist != "Cosine" else {}
        eng.set_params(n_proj=1024, topK=10, topM=50, distance=dist, random_seed=42, precision=args.precision,
                       clusterNoise=args.noise, samplingProb=0.01, **kw)
        if args.tile_variant:
            eng.set_tile_variant(args.tile_variant)
        if args.fit == "soptics":
            eng.fit_soptics_device(X.data_ptr(), 0.25, 50)
        elif args.fit == "sweep":  # test_sDbscan: 8 eps values, the index once (pinned host copy of X)
            eng.fit_sdbscan_sweep(X.cpu().numpy(), [0.1, 0.125, 0.15, 0.175, 0.2, 0.225, 0.25, 0.275], 50)
        else:
            eng.fit_sdbscan_device(X.data_ptr(), 0.25, 50)
    print(json.dumps({"single_fit": args.fit, "n": n, "d": d, "distance": dist, "precision": args.precision,
                      "stage_ms": eng.stage_ms(), "counters": eng.counters()}))
    eng.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=2, choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-sample", type=int, default=20000)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-bf16", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batched-cpu", action="store_true", help="(reference arm) time the config-5 CPU baseline only")
    ap.add_argument("--no-sng", action="store_true")
    ap.add_argument("--sng-cpu", action="store_true", help="(reference arm) time the sngDbscan CPU baseline only")
    ap.add_argument("--cpu-full-fit", action="store_true",
                    help="(reference arm) one CPU fit of the whole workload, timed (minutes at 1M points)")
    ap.add_argument("--single-fit", type=int, default=0, metavar="N",
                    help="one fit of N points of the config-2 law, stage times printed (for profilers)")
    ap.add_argument("--fit", default="sdbscan", choices=["sdbscan", "soptics", "sweep", "sng", "sngoptics"])
    ap.add_argument("--noise", type=int, default=0, help="clusterNoise (with --single-fit)")
    ap.add_argument("--sng-sampling", type=int, default=0, help="0 by seed, 1 shared, 2 blocks (with --single-fit)")
    ap.add_argument("--precision", type=int, default=0, help="0 = FP32, 1 = BF16 (with --single-fit)")
    ap.add_argument("--d", type=int, default=784, help="dimensions (with --single-fit)")
    ap.add_argument("--distance", default="Cosine", help="distance (with --single-fit)")
    ap.add_argument("--prob", type=float, default=0.01, help="sngDbscan samplingProb (with --single-fit --fit sng)")
    ap.add_argument("--tile-variant", type=int, default=0, help="plain distance tile shape (with --single-fit)")
    args = ap.parse_args()
    if args.single_fit:
        return run_single_fit(args)
    cfg = WORKLOADS[args.config]
    if args.impl == "reference" and args.batched_cpu:
        print(json.dumps(_cpu_batched()))
        return 0
    if args.impl == "reference" and args.cpu_full_fit:
        return run_cpu_full_fit(args, cfg)
    if args.impl == "reference" and args.sng_cpu:
        print(json.dumps(_cpu_sng(cfg)))
        return 0
    if args.impl == "reference":
        return run_reference(args, cfg)
    return run_ours(args, cfg)


if __name__ == "__main__":
    sys.exit(main())
