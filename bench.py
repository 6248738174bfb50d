"""Benchmark: ParaGraph GPU build path (K0..K11) on GB300.

Workload (the 1M x 200 inner-product configuration): N = Q = 1,000,000 base points, D = 200,
float32, mixture of 64 Gaussians; training queries from the shifted/rotated recipe; exact float32
inner-product top-128 ground truth; out-degree M = 32, beam L = 64.  Inputs are seeded synthetic
stand-ins for the reference's datasets, generated on the GPU before timing.

A step is one full build (projection + two link rounds).  `value` is distance evaluations per
second with inputs resident in HBM (evaluations counted as the reference's distance_between /
search distance calls; the kernels count them and the tests check the count against the oracle).
`e2e` is the same metric through pg_build_host with pinned host buffers: base + gt host->device
and graph + projection device->host inside the timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--points N] [--dim D]

--impl reference times the CPU restatement of the path (the oracle; the reference's own code for
this path is GPU-only and its CPU RoarGraph path does not build on this Arm host) on all host
cores: one whole build of the same workload per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

UNIT = "evals/s"


def metric_name(args, total: int | None = None) -> str:
    """The metric string of the workload the arguments describe (the 1M x 200 inner-product,
    M = 32, L = 64 build by default; `total` points over args.batched sub-indexes for the batched
    form)."""
    kind = "cosine" if args.cosine else "IP"
    if args.batched:
        what = f"batched build, {args.batched} sub-indexes, {total}x{args.d} {kind}"
    else:
        n = "1M" if args.n == 1_000_000 else str(args.n)
        what = f"build, {n}x{args.d} {kind}"
    return (f"distance_evals_per_s ({what}, M={args.degree}, L={args.beam}, "
            "screened vs FP32, identical edges)")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--points", dest="n", type=int, default=1_000_000)
    ap.add_argument("--dim", dest="d", type=int, default=200)
    ap.add_argument("--degree", type=int, default=32)
    ap.add_argument("--beam", type=int, default=64)
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--cpu-seconds", type=float, default=40.0,
                    help="target length of the CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--screen", default="fp16", choices=["fp16", "bf16", "none"],
                    help="path timed for `value`; the other one is timed beside it")
    ap.add_argument("--no-plain", action="store_true", help="skip timing the other path")
    ap.add_argument("--no-index", action="store_true",
                    help="skip timing the whole index (pg_build_index: build + RoarGraph path + "
                         "FusionFinal)")
    ap.add_argument("--cosine", action="store_true",
                    help="L2-normalise base and queries (cosine = inner product)")
    ap.add_argument("--centers", type=int, default=64, help="mixture components")
    ap.add_argument("--batched", type=int, default=0, metavar="S",
                    help="batched form: S sub-indexes of log-uniform sizes in "
                         "[--min-points, --max-points], one build for all against one by one")
    ap.add_argument("--min-points", type=int, default=10_000)
    ap.add_argument("--max-points", type=int, default=500_000)
    ap.add_argument("--no-gt", action="store_true",
                    help="skip timing the exact ground-truth generation (pg_ground_truth)")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the 1M x 512 cosine (M=48, L=96) and the batched (64 sub-indexes, "
                         "D=512) configurations timed beside the headline")
    ap.add_argument("--autotune", action="store_true",
                    help="run pg_autotune (launch shapes only; results unchanged) before timing")
    return ap.parse_args()


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}",
                                      f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits"],
                                     capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for name, v in zip(names, s[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.samples)}


def dist_init(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    if args.impl == "ours":
        torch.cuda.set_device(local)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# Above this many points the data generator's float32 top-k would scan a score matrix of
# terabytes; the workload's exact top-128 then comes from pg_ground_truth.
GT_ON_GPU_ABOVE = 2_000_000


def gpu_workload(args, device, queries: bool = False):
    """(base, gt[, queries]) on the device, and the ms pg_ground_truth took (None when the data
    generator's float32 top-k made the ground truth)."""
    from paragraph_gb300 import datagen
    if args.n <= GT_ON_GPU_ABOVE:
        return datagen.make_dataset_cuda(args.n, args.d, gt_k=128, seed=args.seed, device=device,
                                         return_queries=queries, cosine=args.cosine,
                                         centers=args.centers), None
    import torch
    import paragraph_gb300 as pg
    base, _, q = datagen.make_dataset_cuda(args.n, args.d, seed=args.seed, device=device,
                                           cosine=args.cosine, centers=args.centers,
                                           with_gt=False)
    gt = torch.empty((args.n, 128), dtype=torch.int32, device=device)
    stream = torch.cuda.Stream(device)
    dev_index = torch.device(device).index or 0
    with pg.Handle(dev_index, stream=stream) as h:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        h.ground_truth(base, q, gt)
        e1.record(stream)
        torch.cuda.synchronize()
    return ((base, gt, q) if queries else (base, gt)), e0.elapsed_time(e1)


# DRAM bytes (read + write) per launch of the search kernel, measured by ncu on these workloads
# (profiles/search_dram_1Mx200_1Mx512cos.md): round 1 over the projection, round 2 over the link
# graph.  Keys: (n, d, M, L, cosine).
SEARCH_DRAM_BYTES = {
    (1_000_000, 200, 32, 64, False): (1_217_476_352, 1_182_223_104),
    (1_000_000, 512, 48, 96, True): (143_634_611_456, 870_972_185_088),
}


def search_roofline(st, args, peak_gbs, peak_kind, rounds):
    """Dominant kernel = the beam search (K4/K8).  Algorithmic bytes per launch: every counted
    evaluation after the 32 seeds gathers one 4*D-byte row plus its 4-byte id, every iteration
    reads Kp*Kd = 32 graph ids, and the launch reads each query row and its 32 seed distances once
    and writes n*L ids.  The seed distances are computed once per build by the seed pre-pass
    (k_seed_dists, timed inside round 1's stage: it reads the n query rows and writes n*32
    distances), so no search launch gathers a seed row.  The reported launch is the last round's
    search, whose stage time is that one kernel."""
    n, d, L = args.n, args.d, args.beam

    def kernel_bytes(r):
        gathered = st.evals_search[r] - 32 * n
        return gathered * (4 * d + 4) + st.search_iters[r] * 32 * 4 + n * (4 * d + 32 * 4 + 4 * L)

    last = rounds - 1
    by = kernel_bytes(last)
    ms = st.ms_search[last]
    if last == 0:  # the stage also holds the seed pre-pass
        by += n * (4 * d + 32 * 4)
    achieved = by / (ms / 1e3) / 1e9
    dram = SEARCH_DRAM_BYTES.get((args.n, args.d, args.degree, args.beam, bool(args.cosine)))
    traffic = dram[last] if dram else None
    kname = "k_search_m32" if args.beam - 32 <= 32 else "k_search_mk"
    dram_frac = traffic / (ms / 1e3) / 1e9 / peak_gbs if traffic else None
    bound = ("hbm: DRAM-served row gathers (see dram_frac)" if dram_frac and dram_frac >= 0.4
             else "latency: L2-resident row gathers, not HBM (see dram_frac)")
    out = {"kernel": f"{kname} (round-{last + 1} beam search)",
           "bound": bound,
           "achieved": round(achieved, 1), "peak": peak_gbs, "peak_kind": peak_kind,
           "unit": "GB/s", "frac": round(achieved / peak_gbs, 4),
           "frac_meaning": "algorithmic gathered bytes / launch time / measured HBM copy peak",
           "traffic": traffic, "algorithmic_bytes_per_launch": int(by),
           "ms_per_launch": round(ms, 3)}
    if traffic:
        out["dram_gbs"] = round(traffic / (ms / 1e3) / 1e9, 1)
        out["dram_frac"] = round(traffic / (ms / 1e3) / 1e9 / peak_gbs, 4)
    if rounds > 1:
        b0 = kernel_bytes(0) + n * (4 * d + 32 * 4)
        out["round1_stage"] = {"algorithmic_bytes": int(b0), "ms": round(st.ms_search[0], 3),
                               "achieved": round(b0 / (st.ms_search[0] / 1e3) / 1e9, 1),
                               "traffic": dram[0] if dram else None,
                               "includes": "seed pre-pass + round-1 search"}
    return out


def screen_error_sample(base, graph, pairs: int = 1 << 20, seed: int = 7):
    """Worst relative error |s16 - s64| / (|x||y|) over up to `pairs` graph edges (x, y): s16 is
    the inner product of the FP16-rounded vectors accumulated in FP32 (what the screened prune
    computes on tensor cores, in another order), s64 the FP64 inner product of the FP32 vectors."""
    import torch
    n = base.shape[0]
    g = torch.Generator(device=base.device)
    g.manual_seed(seed)
    rows = torch.randint(0, n, (pairs,), generator=g, device=base.device)
    cols = torch.randint(0, graph.shape[1], (pairs,), generator=g, device=base.device)
    nb = graph[rows, cols].long()
    ok = (nb >= 0) & (nb < n)
    rows, nb = rows[ok], nb[ok]
    worst = 0.0
    for s in range(0, rows.numel(), 1 << 17):
        x = base[rows[s:s + (1 << 17)]]
        y = base[nb[s:s + (1 << 17)]]
        s64 = (x.double() * y.double()).sum(1)
        s16 = (x.half().float() * y.half().float()).sum(1)
        scale = x.double().norm(dim=1) * y.double().norm(dim=1)
        worst = max(worst, float(((s16.double() - s64).abs() / scale.clamp_min(1e-300)).max()))
    return worst, int(rows.numel())


def secondary_cosine(args, h, dev, stream):
    """The precision configuration, measured beside the headline in the same run: 1M x 512, base
    and queries L2-normalised (cosine), 128 centres, M = 48, L = 96, exact top-128 ground truth
    (pg_ground_truth).  The FP16-screened build and the plain FP32 build are timed with CUDA events
    on the handle's stream and their edges compared."""
    import torch
    import paragraph_gb300 as pg
    from paragraph_gb300 import datagen
    n, d, m, beam = 1_000_000, 512, 48, 96
    base, _, queries = datagen.make_dataset_cuda(n, d, cosine=True, centers=128,
                                                 seed=args.seed + 7, device=dev, with_gt=False)
    gt = torch.empty((n, 128), dtype=torch.int32, device=dev)
    h.ground_truth(base, queries, gt)
    del queries
    torch.cuda.empty_cache()
    out = {"workload": f"ParaGraph build {n}x{d} cosine (128 centres), gt top-128 "
                       f"(pg_ground_truth), M={m}, L={beam}"}
    graphs = {}
    for name, screen in (("fp16", pg.SCREEN_FP16), ("plain", pg.SCREEN_NONE)):
        params = pg.default_params(m, beam, screen=screen)
        graph = torch.empty((n, m), dtype=torch.int32, device=dev)
        proj = torch.empty((n, 16), dtype=torch.int32, device=dev)
        h.build_device(base, gt, graph, proj, params)  # warm-up
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        k = 2
        e0.record(stream)
        for _ in range(k):
            st = h.build_device(base, gt, graph, proj, params)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / k
        graphs[name] = (graph, proj)
        if screen:
            st_fp16 = st
        out[name] = {"ms_per_build": round(ms, 2), "evals": int(st.evals_total),
                     "evals_per_s": st.evals_total / (ms / 1e3),
                     "stage_ms": {"proj": round(st.ms_proj, 2),
                                  "search": [round(x, 2) for x in list(st.ms_search)[:2]],
                                  "prune": [round(x, 2) for x in list(st.ms_prune)[:2]],
                                  "merge": [round(x, 2) for x in list(st.ms_merge)[:2]]}}
        if screen:
            out[name]["rescored"] = list(st.rescored)[:2]
            out[name]["occlusion_tests"] = list(st.evals_prune)[:2]
    out["identical_edges"] = bool(torch.equal(graphs["fp16"][0], graphs["plain"][0]) and
                                  torch.equal(graphs["fp16"][1], graphs["plain"][1]))
    out["speedup_screened_vs_plain"] = round(out["plain"]["ms_per_build"] /
                                             out["fp16"]["ms_per_build"], 3)
    worst, npairs = screen_error_sample(base, graphs["plain"][0])
    out["fp16_max_rel_error_vs_fp64"] = worst
    out["error_sample"] = f"{npairs} random graph edges, |s16 - s64| / (|x||y|)"
    # the round-2 search of this build against the HBM roofline (it is the DRAM-heavy search:
    # 1M rows of 2 KB, about 43% of the gathers served by L2)
    shape = argparse.Namespace(n=n, d=d, degree=m, beam=beam, cosine=True)
    out["search_roofline"] = search_roofline(st_fp16, shape, *peaks(), 2)
    del base, gt, graphs
    torch.cuda.empty_cache()
    return out


def cpu_baseline_sample(args, base_np, gt_np, seconds):
    """The oracle (CPU restatement of K0..K11, all host threads) on the workload.  When the whole
    build fits the time budget (estimated from a 1% pilot of the search) it runs the complete build;
    otherwise phase 1 plus the round-1 search over as many queries as fit.  Returns
    (evals/s, description, threads, the full build's oracle result or None)."""
    import oracle
    t0 = time.perf_counter()
    p1 = oracle.build_graph(base_np, gt_np, degree=args.degree, beam=args.beam, link_rounds=0)
    t1 = time.perf_counter()
    km = args.beam - 32
    pilot = max(1, args.n // 100)
    _, pev, _, _ = oracle.search(base_np, p1["proj"], km=km, q_begin=0, q_end=pilot)
    t2 = time.perf_counter()
    est_full = (t1 - t0) + 100 * (t2 - t1) * 2 * 1.5  # two rounds, prune/merge ~50% extra
    if est_full <= seconds:
        t0 = time.perf_counter()
        full = oracle.build_graph(base_np, gt_np, degree=args.degree, beam=args.beam)
        dt = time.perf_counter() - t0
        ev = full["stats"]["evals_total"]
        desc = f"oracle full build (K0-K11) of all {args.n} points: {ev} evals in {dt:.1f} s"
        return ev / dt, desc, oracle.num_threads(), full
    per_q = (t2 - t1) / pilot
    q_more = int(min(args.n - pilot, max(seconds - (t2 - t0), 0.0) / max(per_q, 1e-9)))
    sev2 = 0
    if q_more > 0:
        _, sev2, _, _ = oracle.search(base_np, p1["proj"], km=km, q_begin=pilot,
                                      q_end=pilot + q_more)
    t3 = time.perf_counter()
    ev = p1["stats"]["evals_proj_prune"] + p1["stats"]["evals_proj_merge"] + pev + sev2
    desc = (f"oracle phase 1 (K0-K3) over all {args.n} points + round-1 search for "
            f"{pilot + q_more} queries: {ev} evals in {t3 - t0:.1f} s")
    return ev / (t3 - t0), desc, oracle.num_threads(), None


def workload_config(args) -> dict:
    """The `config` object of both arms: the workload, nothing measured."""
    kind = "cosine" if args.cosine else "IP"
    return {"workload": f"ParaGraph build {args.n}x{args.d} {kind}, gt top-128, "
                        f"M={args.degree}, L={args.beam}",
            "n": args.n, "d": args.d, "q": args.n, "degree": args.degree, "beam": args.beam,
            "centers": args.centers, "seed": args.seed,
            "l2": f"inputs larger than L2 (base {args.n * args.d * 4 / 1e6:.0f} MB, "
                  f"gt {args.n * 128 * 4 / 1e6:.0f} MB vs 129 MB L2)"}


def run_reference(args):
    """--impl reference: the CPU restatement of the path (the oracle, all host threads) on rank 0;
    one step = one complete build (K0..K11) of the workload."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import numpy as np
    import torch

    import oracle
    if torch.cuda.is_available():
        (base, gt), _ = gpu_workload(args, "cuda")
        base_np = base.cpu().numpy()
        gt_np = gt.cpu().numpy().view(np.uint32)
        del base, gt
        torch.cuda.empty_cache()
    else:
        from paragraph_gb300 import datagen
        base_np, gt_np = datagen.make_dataset(args.n, args.d, seed=args.seed, cosine=args.cosine,
                                              centers=args.centers)
    steps = max(args.steps, 1)
    times = []
    evals = None
    for i in range(args.warmup + steps):
        t0 = time.perf_counter()
        full = oracle.build_graph(base_np, gt_np, degree=args.degree, beam=args.beam)
        dt = time.perf_counter() - t0
        ev = full["stats"]["evals_total"]
        assert evals is None or ev == evals, "evaluation count changed between builds"
        evals = ev
        if i >= args.warmup:
            times.append(dt)
    t = statistics.mean(times)
    value = evals / t
    threads = oracle.num_threads()
    desc = (f"oracle full build (K0-K11) of all {args.n} points per step: {evals} evals, "
            f"{t:.2f} s mean over {steps} steps")
    line = {"metric": metric_name(args), "value": value, "unit": UNIT, "impl": "reference",
            "n_gpus": world, "steps": steps, "warmup": args.warmup,
            "ms_per_step": round(t * 1e3, 1), "ms_each": [round(x * 1e3, 1) for x in times],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded mixture-of-Gaussians stand-in for T2I-style data)",
            "config": workload_config(args),
            "evals_per_build": evals,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "the reference's build path is GPU-only, and its CPU RoarGraph code is x86 "
                    "AVX-512 and absent on this Arm host, so the oracle -- the CPU restatement of "
                    "the path, pinned to the reference's own kernels by the golden fixtures -- "
                    "stands in"}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import numpy as np
    import torch
    world, rank, local = dist_init(args)
    import paragraph_gb300 as pg
    dev = torch.device("cuda", local)
    want_q = not args.no_gt
    wl, gt_gen_ms = gpu_workload(args, dev, queries=want_q)
    base, gt = wl[0], wl[1]
    queries = wl[2] if want_q else None
    torch.cuda.synchronize()
    screen = {"bf16": pg.SCREEN_BF16, "fp16": pg.SCREEN_FP16, "none": pg.SCREEN_NONE}[args.screen]
    params = pg.default_params(args.degree, args.beam, screen=screen)
    other = pg.default_params(args.degree, args.beam,
                              screen=pg.SCREEN_NONE if screen else pg.SCREEN_BF16)
    n, d = base.shape
    graph = torch.empty((n, args.degree), dtype=torch.int32, device=dev)
    proj = torch.empty((n, 16), dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(dev)
    h = pg.Handle(local, stream=stream)
    # K0, K2 + CSR (5), K3 = 8; per link round search, prune + CSR (5), merge = 8; once per build
    # the seed-distance pass and, when screened, the norm pre-pass
    once = (1 if params.link_rounds > 0 else 0) + (
        1 if (screen and params.link_rounds > 0 and args.beam <= 128) else 0)
    launches_per_build = 8 + 8 * params.link_rounds + once
    tuning = None
    if args.autotune:
        t0 = time.perf_counter()
        _, tun = h.autotune(base, gt, params)
        tuning = dict(tun.as_dict(), seconds=round(time.perf_counter() - t0, 2))
    stats = []
    for _ in range(args.warmup):
        h.build_device(base, gt, graph, proj, params)
    torch.cuda.synchronize()
    barrier(world)
    peak, peak_kind = peaks()
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        barrier(world)
        start = torch.cuda.Event(enable_timing=True)
        stop = torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for _ in range(args.steps):
            stats.append(h.build_device(base, gt, graph, proj, params))
        stop.record(stream)
        torch.cuda.synchronize()
        barrier(world)
    ms_total = start.elapsed_time(stop)
    ms_total = allmax(ms_total, world)
    # the other path (plain FP32 when the screened path is timed), same inputs, and the check
    # that both give identical edges
    other_line = None
    if not args.no_plain:
        graph2 = torch.empty_like(graph)
        proj2 = torch.empty_like(proj)
        h.build_device(base, gt, graph2, proj2, other)
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        k2 = max(1, min(args.steps, 3))
        t0.record(stream)
        for _ in range(k2):
            ost = h.build_device(base, gt, graph2, proj2, other)
        t1.record(stream)
        torch.cuda.synchronize()
        oms = t0.elapsed_time(t1) / k2
        other_line = {"screen": "none" if screen else "bf16", "ms_per_step": round(oms, 3),
                      "value": ost.evals_total / (oms / 1e3),
                      "identical_edges": bool(torch.equal(graph, graph2) and torch.equal(proj, proj2)),
                      "speedup_of_timed_path": round(oms / (ms_total / args.steps), 3)}
        del graph2, proj2
    # the reference driver's whole index (tests/test_t2iend.cu): the GPU build plus the CPU
    # RoarGraph path (six MatchSup rounds, FusionNN) and FusionFinal, all on the GPU
    # (pg_build_index)
    index_line = None
    if not args.no_index:
        iout = torch.empty((n, 2 * 40 + 70), dtype=torch.int32, device=dev)
        icnt = torch.empty((n,), dtype=torch.int32, device=dev)
        h.build_index(base, gt, iout, icnt, params)
        ist = [h.build_index(base, gt, iout, icnt, params) for _ in range(max(1, min(args.steps, 3)))]
        last = ist[-1]
        kk = icnt.float()
        index_line = {"ms_per_index": round(statistics.mean(x.ms_total for x in ist), 3),
                      "ms_gpu_build": round(last.ms_total - last.ms_match_sup - last.ms_fusion_nn
                                            - last.ms_fusion_final, 3),
                      "ms_match_sup_6_rounds": round(last.ms_match_sup, 3),
                      "ms_fusion_nn": round(last.ms_fusion_nn, 3),
                      "ms_fusion_final": round(last.ms_fusion_final, 3),
                      "mean_degree": round(float(kk.mean()), 3), "max_degree": int(kk.max()),
                      "params": "match_rounds 6, M_nn 40, M_final 70 (tests/test_t2iend.cu)"}
        del iout, icnt
    # the build's input, ground truth top-128, generated exactly on the GPU (pg_ground_truth)
    gt_line = None
    if gt_gen_ms is not None:  # the workload's own ground truth came from pg_ground_truth
        gt_line = {"ms": round(gt_gen_ms, 1), "queries": int(n), "base": int(n), "k": 128,
                   "screen_gemm_tflops_equiv": round(2.0 * n * n * d / (gt_gen_ms / 1e3) / 1e12, 1),
                   "definition": "exact FP64 inner products, ties to the lower id (this is the "
                                 "build's input here: the float32 top-k is not run at this size)"}
        queries = None
    if queries is not None:
        gout = torch.empty((queries.shape[0], 128), dtype=torch.int32, device=dev)
        h.ground_truth(base, queries[:1024], gout[:1024])  # workspace set-up
        torch.cuda.synchronize()
        g0 = torch.cuda.Event(enable_timing=True)
        g1 = torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        h.ground_truth(base, queries, gout)
        g1.record(stream)
        torch.cuda.synchronize()
        gms = g0.elapsed_time(g1)
        same = (gout == gt).all(dim=1).float().mean().item()
        flop = 2.0 * queries.shape[0] * n * d
        gt_line = {"ms": round(gms, 1), "queries": int(queries.shape[0]), "base": int(n),
                   "k": 128, "screen_gemm_tflops_equiv": round(flop / (gms / 1e3) / 1e12, 1),
                   "rows_equal_to_fp32_topk": round(same, 5),
                   "definition": "exact FP64 inner products, ties to the lower id; the "
                                 "benchmark's own ground truth is a float32 top-k"}
        del gout, queries
        torch.cuda.empty_cache()
    secondary = batched = None
    if not args.no_secondary and args.n == 1_000_000 and args.d == 200 and not args.cosine:
        secondary = secondary_cosine(args, h, dev, stream)
        batched = batched_secondary(args, h, dev, stream)
    evals = stats[-1].evals_total
    assert all(s.evals_total == evals for s in stats), "evaluation count changed between builds"
    value = evals * args.steps * world / (ms_total / 1e3)
    ms_step = ms_total / args.steps

    e2e = None
    if not args.no_e2e:
        base_h = base.cpu().pin_memory()
        gt_h = gt.cpu().pin_memory()
        graph_h = torch.empty((n, args.degree), dtype=torch.int32).pin_memory()
        proj_h = torch.empty((n, 16), dtype=torch.int32).pin_memory()
        del base, gt
        torch.cuda.empty_cache()
        for _ in range(2):
            h.build_host_ptr(base_h.data_ptr(), n, d, gt_h.data_ptr(), gt_h.shape[0],
                             graph_h.data_ptr(), proj_h.data_ptr(), params)
        barrier(world)
        times, h2d, d2h, dev_ms = [], [], [], []
        est = None
        for _ in range(max(1, args.steps)):
            t0 = time.perf_counter()
            est = h.build_host_ptr(base_h.data_ptr(), n, d, gt_h.data_ptr(), gt_h.shape[0],
                                   graph_h.data_ptr(), proj_h.data_ptr(), params)
            times.append(time.perf_counter() - t0)
            h2d.append(est.ms_h2d)
            d2h.append(est.ms_d2h)
            dev_ms.append(est.ms_total)
        t = allmax(statistics.mean(times), world)
        e2e = {"value": est.evals_total * world / t, "unit": UNIT,
               "h2d_bytes_per_step": int(est.h2d_bytes), "d2h_bytes_per_step": int(est.d2h_bytes),
               "ms_per_step": round(t * 1e3, 2),
               "ms_median": round(statistics.median(times) * 1e3, 2),
               "ms_each": [round(x * 1e3, 1) for x in times],
               "ms_h2d_each": [round(x, 2) for x in h2d],
               "ms_d2h_each": [round(x, 2) for x in d2h],
               "ms_build_each": [round(x, 2) for x in dev_ms],
               "timing": "wall clock around each pg_build_host call, mean over --steps calls; "
                         "the copies and the build are also timed with CUDA events per call"}
        base_np = base_h.numpy()
        gt_np = gt_h.numpy().view(np.uint32)
    else:
        base_np = base.cpu().numpy()
        gt_np = gt.cpu().numpy().view(np.uint32)

    roof = search_roofline(stats[-1], args, peak, peak_kind, params.link_rounds)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, desc, threads, full = cpu_baseline_sample(args, base_np, gt_np, args.cpu_seconds)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc}
        if index_line is not None and full is not None:
            import oracle
            t0 = time.perf_counter()
            rounds = [oracle.match_sup(base_np, gt_np, r) for r in range(1, 7)]
            fnn = oracle.fusion_nn(base_np, rounds)
            oracle.fusion_final(base_np, full["proj"], fnn, full["graph"])
            index_line["cpu_oracle_roar_s"] = round(time.perf_counter() - t0, 2)
            index_line["cpu_oracle_cores"] = threads
    s = stats[-1]
    if rank == 0:
        line = {"metric": metric_name(args), "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32" if args.screen == "none" else "f32+" + args.screen,
                "data": "synthetic (seeded mixture-of-Gaussians stand-in for T2I-style data)",
                "config": workload_config(args),
                "parallelism": "replicas" if world > 1 else "single",
                "build_s": round(ms_step / 1e3, 4),
                "evals_per_build": evals,
                "stage_ms": {"proj": round(s.ms_proj, 2),
                             "search": [round(x, 2) for x in list(s.ms_search)[:params.link_rounds]],
                             "prune": [round(x, 2) for x in list(s.ms_prune)[:params.link_rounds]],
                             "merge": [round(x, 2) for x in list(s.ms_merge)[:params.link_rounds]]},
                "screen": args.screen,
                "tuning": tuning,
                "rescored": list(s.rescored)[:params.link_rounds],
                "other_path": other_line,
                "index": index_line,
                "ground_truth": gt_line,
                "secondary": secondary,
                "batched": batched,
                "gpu_launches": launches_per_build * args.steps,
                "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
                "clocks": clocks.summary()}
        print(json.dumps(line), flush=True)
    h.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def batched_workload(count, d, min_points, max_points, seed, cosine, centers, h, dev, stream):
    """`count` sub-indexes of seeded log-uniform sizes, each with its own training queries (Q = N)
    and exact top-128 ground truth from pg_ground_truth.  Returns (base, gt, node_off, sizes,
    ground-truth ms, generation s)."""
    import numpy as np
    import torch
    from paragraph_gb300 import datagen
    rng = np.random.Generator(np.random.PCG64(seed))
    sizes = np.exp(rng.uniform(np.log(min_points), np.log(max_points), count)).astype(np.int64)
    node_off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    total = int(node_off[-1])
    base = torch.empty((total, d), dtype=torch.float32, device=dev)
    gt = torch.empty((total, 128), dtype=torch.int32, device=dev)
    t0 = time.perf_counter()
    gt_ms = 0.0
    for i, ni in enumerate(sizes):
        lo, hi = int(node_off[i]), int(node_off[i + 1])
        b, _, q = datagen.make_dataset_cuda(int(ni), d, seed=seed + 1 + i, device=dev,
                                            cosine=cosine, centers=centers, with_gt=False)
        base[lo:hi] = b
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        h.ground_truth(b, q, gt[lo:hi])
        e1.record(stream)
        torch.cuda.synchronize()
        gt_ms += e0.elapsed_time(e1)
        del b, q
    torch.cuda.empty_cache()
    return base, gt, node_off, sizes, gt_ms, time.perf_counter() - t0


def batched_measure(h, stream, base, gt, node_off, sizes, degree, beam, screen, steps, warmup):
    """One CUDA-graph replay of pg_build_batched_device over every sub-index against building
    them one by one (same screen; and the plain FP32 path for the identical-edges check).
    Returns (dict, Stats of the last batched build, ms per batched build)."""
    import torch
    import paragraph_gb300 as pg
    params = pg.default_params(degree, beam, screen=screen, flags=pg.FLAG_CUDA_GRAPH)
    total = int(node_off[-1])
    graph = torch.empty((total, degree), dtype=torch.int32, device=base.device)
    for _ in range(warmup):
        st = h.build_batched(base, gt, node_off, node_off, graph, None, params)
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b_ = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(steps):
        st = h.build_batched(base, gt, node_off, node_off, graph, None, params)
    b_.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b_) / steps

    def one_by_one(p):
        out = torch.empty_like(graph)
        for i in range(len(sizes)):  # warm-up pass
            lo, hi = int(node_off[i]), int(node_off[i + 1])
            h.build_device(base[lo:hi], gt[lo:hi], out[lo:hi], None, p)
        torch.cuda.synchronize()
        a.record(stream)
        ev = 0
        for i in range(len(sizes)):
            lo, hi = int(node_off[i]), int(node_off[i + 1])
            ev += h.build_device(base[lo:hi], gt[lo:hi], out[lo:hi], None, p).evals_total
        b_.record(stream)
        torch.cuda.synchronize()
        return out, ev, a.elapsed_time(b_)

    alone, ev_alone, ms_alone = one_by_one(pg.default_params(degree, beam, screen=screen))
    out = {"ms_batched": round(ms, 3), "evals": int(st.evals_total),
           "evals_per_s": st.evals_total / (ms / 1e3),
           "one_by_one": {"ms": round(ms_alone, 3), "evals": int(ev_alone),
                          "identical_edges": bool(torch.equal(graph, alone)),
                          "speedup_of_batched": round(ms_alone / ms, 3)}}
    del alone
    if screen:
        plain, _, ms_plain = one_by_one(pg.default_params(degree, beam, screen=pg.SCREEN_NONE))
        out["plain_one_by_one"] = {"ms": round(ms_plain, 3),
                                   "identical_edges": bool(torch.equal(graph, plain))}
        del plain
    return out, st, ms


def batched_secondary(args, h, dev, stream):
    """The batched configuration, measured beside the headline: 64 sub-indexes of log-uniform
    sizes in [10k, 500k], D = 512, inner product, M = 32, L = 64."""
    import torch
    count, d = 64, 512
    base, gt, node_off, sizes, gt_ms, gen_s = batched_workload(
        count, d, 10_000, 500_000, args.seed, False, args.centers, h, dev, stream)
    screen = {"bf16": 1, "fp16": 3, "none": 0}[args.screen]
    res, _, _ = batched_measure(h, stream, base, gt, node_off, sizes, 32, 64, screen, 2, 1)
    res.update({"workload": f"{count} sub-indexes, sizes log-uniform in [10000, 500000] "
                            f"(total {int(node_off[-1])}), D={d}, IP, M=32, L=64, one "
                            "CUDA-graph replay",
                "sizes_min_max": [int(sizes.min()), int(sizes.max())],
                "ground_truth_ms_total": round(gt_ms, 1), "data_generation_s": round(gen_s, 1)})
    del base, gt
    torch.cuda.empty_cache()
    return res


def run_batched(args):
    """Batched form: S independent sub-indexes of uneven (seeded log-uniform) sizes, each with its
    own training queries (Q = N) and exact top-128 ground truth (pg_ground_truth), built in one
    CUDA-graph-captured pass (pg_build_batched_device) against building them one by one."""
    import torch
    import paragraph_gb300 as pg
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    h = pg.Handle(0, stream=stream)
    base, gt, node_off, sizes, gt_ms, gen_s = batched_workload(
        args.batched, args.d, args.min_points, args.max_points, args.seed, args.cosine,
        args.centers, h, dev, stream)
    total = int(node_off[-1])
    screen = {"bf16": pg.SCREEN_BF16, "fp16": pg.SCREEN_FP16, "none": pg.SCREEN_NONE}[args.screen]
    tuning = None
    if args.autotune:
        params = pg.default_params(args.degree, args.beam, screen=screen, flags=pg.FLAG_CUDA_GRAPH)
        _, tun = h.autotune(base, gt, params, node_off=node_off, query_off=node_off)
        tuning = tun.as_dict()
    with ClockSampler(0) as clocks:
        res, st, ms = batched_measure(h, stream, base, gt, node_off, sizes, args.degree,
                                      args.beam, screen, args.steps, args.warmup)
    launches = (10 + 8 * 2 + 1 + (1 if screen and args.beam <= 128 else 0)) * args.steps
    line = {"metric": metric_name(args, total), "value": st.evals_total / (ms / 1e3),
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if args.screen == "none" else "f32+" + args.screen,
            "data": "synthetic (seeded mixture-of-Gaussians, one set per sub-index)",
            "config": {"workload": f"{args.batched} sub-indexes, sizes log-uniform in "
                                   f"[{args.min_points}, {args.max_points}] (total {total}), "
                                   f"D={args.d}, {'cosine' if args.cosine else 'IP'}, "
                                   f"M={args.degree}, L={args.beam}, one CUDA-graph replay",
                       "sizes_min_max": [int(sizes.min()), int(sizes.max())], "total": total},
            "one_by_one": res["one_by_one"], "plain_one_by_one": res.get("plain_one_by_one"),
            "ground_truth": {"ms_total": round(gt_ms, 1), "k": 128,
                             "definition": "exact FP64 inner products (pg_ground_truth)"},
            "data_generation_s": round(gen_s, 1), "tuning": tuning,
            "gpu_launches": launches, "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)
    h.close()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.batched:
        return run_batched(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
