#!/usr/bin/env python3
"""Benchmark of the GB300 skycube engine: full skycube of 1,000,000 x 10
anticorrelated float32 points (all 1,023 cuboids), points per second.

One step = one full skycube of the workload through the batched persistent
form (MDMC bitmaps, one launch for every cuboid). The JSON line reports:
  value      points/s with the dataset resident in HBM (device events around
             each skycube call, L2 flushed by a 256 MiB write before each step)
  e2e        points/s through the C ABI with host buffers: pinned-host upload
             (H2D), skycube, download of every cuboid's id list (D2H)
  plain      the per-cuboid form (one launch sequence per cuboid), for the
             batched-versus-plain ratio
  roofline   of the dominant kernel (bitmap kernel): algorithmic bytes / its
             event-timed duration against measured HBM bandwidth, plus the
             issue roofline (pair-test lane operations / SM lane-op peak)
  cpu_baseline  the reference's own STSC (all host threads) on a bounded
             sample of the same workload
  reference_sweeps  capped skycubes of 500k x 16 points at the caps of the
             reference's published sweeps, beside its published milliseconds

--impl reference times the reference's CPU path, its own STSC built from its
unmodified sources (portable intrinsics on the aarch64 GPU hosts), on a
bounded sample of the same workload with every host thread, then once on
the whole workload. Under torchrun each rank computes its own
replica; N > 1 is replicas only (the path needs no collective).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "skycube-templates_gb300"))

import numpy as np  # noqa: E402

from skycube_gb300 import datagen  # noqa: E402

WORKLOAD = "anticorr-1m-10"
METRIC = "full-skycube points/s (1M x 10 anticorrelated, all 1,023 cuboids)"
UNIT = "points/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default=WORKLOAD, choices=sorted(datagen.CONFIGS))
    ap.add_argument("--no-plain", action="store_true", help="skip the per-cuboid form")
    ap.add_argument("--cpu-sample", type=int, default=0, help="points in the CPU sample (0: auto)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-ref-full", action="store_true",
                    help="reference arm: skip the one full-size run after the sample steps")
    ap.add_argument("--no-sweeps", action="store_true",
                    help="skip the reference's published sweep workloads")
    ap.add_argument("--serving-queries", type=int, default=600,
                    help="queries of the serving stream (0: skip serving)")
    ap.add_argument("--serving-rate", type=float, default=40.0, help="Poisson arrival rate, queries/s")
    ap.add_argument("--serving-slots", type=int, default=4)
    ap.add_argument("--serving-baseline", type=int, default=60,
                    help="queries served one at a time with the plain form for comparison")
    return ap.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload(name, rank):
    kind, n, d, max_d, seed = datagen.CONFIGS[name]
    x = datagen.generate(kind, n, d, seed + rank)
    return kind, n, d, max_d, seed, x


def cpu_impl():
    """The CPU implementation timed beside the GPU: the reference's own STSC
    (oracle/_ref, built from its unmodified sources by build()) when present,
    else the restated STSC oracle. Returns (run(points, max_d, threads), kind)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    if oracle.ref_available():
        return oracle.ref_stsc, "reference"
    return oracle.stsc, "port"


def cpu_sample_run(x, d, max_d, n_sample):
    """Times the CPU implementation on the first n_sample points of the
    workload with every host thread."""
    run, kind = cpu_impl()
    xs = np.ascontiguousarray(x[:n_sample])
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    run(xs, max_d, threads)
    dt = time.perf_counter() - t0
    return dt, threads, kind


def auto_cpu_sample(name):
    kind = datagen.CONFIGS[name][0]
    return 100_000 if kind == "anticorrelated" else 300_000


def cpu_kind_note(kind):
    if kind == "reference":
        import platform
        how = ("its AVX2 dominance tests" if platform.machine() == "x86_64" else
               "the portable intrinsics of oracle/ref_shim in place of its AVX2 ones")
        return f"the reference's own STSC (HybridCube<D>, unmodified sources, {how})"
    return "the restated STSC oracle (the reference's STSC was not built on this host)"


# --------------------------------------------------------------------------
class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons (every 200 ms)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = []
        for line in open(self.f.name):
            parts = [s.strip() for s in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for nm, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0}, "fallback"


def flush_l2(buf):
    buf.zero_()


def percentile(v, p):
    v = sorted(v)
    if not v:
        return None
    k = (len(v) - 1) * p / 100.0
    lo, hi = int(k), min(int(k) + 1, len(v) - 1)
    return v[lo] + (v[hi] - v[lo]) * (k - lo)


def run_serving(sk, ctx, args):
    """Serving stream: queries arrive Poisson at --serving-rate, each over its
    own seeded dataset (n log-uniform in [1e3, 1e6], d in 4..16, uniform /
    correlated / anticorrelated); half capped skycubes (<= 4 attributes), half
    skylines of one random subspace. Served by the continuous-batching server
    (host rows in, host results out). The first --serving-baseline queries
    are also served one at a time with the plain per-cuboid form on the same
    arrival times (sequential queue on a virtual clock from measured service
    times)."""
    stream = datagen.serving_stream(count=args.serving_queries, rate_qps=args.serving_rate, seed=7)
    data = [datagen.generate(q["kind"], q["n"], q["d"], q["seed"]) for q in stream]
    srv = sk.Server(ctx, slots=args.serving_slots)
    for x, q in list(zip(data, stream))[:8]:  # warm-up (kernels, pools)
        r, _ = srv.wait(srv.submit(x, max_d=q["max_d"], subspace=q["subspace"]))
        r.close()
    t0 = time.perf_counter()
    tickets = []
    for q, x in zip(stream, data):
        delay = t0 + q["arrival_s"] - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        tickets.append(srv.submit(x, max_d=q["max_d"], subspace=q["subspace"]))
    lat, queued, run = [], [], []
    for t in tickets:
        r, tm = srv.wait(t)
        lat.append(tm["total_ms"])
        queued.append(tm["queued_ms"])
        run.append(tm["run_ms"])
        r.close()
    span = max(time.perf_counter() - t0, stream[-1]["arrival_s"])
    stats = srv.stats()
    srv.close()
    out = {"queries": len(stream), "rate_qps": args.serving_rate, "slots": args.serving_slots,
           "p50_ms": round(percentile(lat, 50), 3), "p99_ms": round(percentile(lat, 99), 3),
           "mean_ms": round(sum(lat) / len(lat), 3), "max_ms": round(max(lat), 3),
           "qps": round(len(stream) / span, 2), "peak_in_flight": stats["peak_in_flight"],
           "queued_p50_ms": round(percentile(queued, 50), 3),
           "queued_p99_ms": round(percentile(queued, 99), 3),
           "run_p50_ms": round(percentile(run, 50), 3), "run_p99_ms": round(percentile(run, 99), 3),
           "form": "batched form (per-point bitmaps, or the level form for capped "
                   "skycubes on many candidates), continuous batching over CUDA-stream slots"}
    nb = min(args.serving_baseline, len(stream))
    if nb:
        def one_at_a_time(mode):
            end, lats = 0.0, []
            for q, x in list(zip(stream, data))[:nb]:
                s0 = time.perf_counter()
                ds = sk.Dataset(ctx, x)
                r = sk.skycube(ctx, ds, "sdsc" if mode == "plain" else "mdmc", mode,
                               max_d=q["max_d"], subspace=q["subspace"])
                r.download()
                r.close()
                ds.close()
                service = time.perf_counter() - s0
                start = max(q["arrival_s"], end)
                end = start + service
                lats.append((end - q["arrival_s"]) * 1000.0)
            return {"queries": nb, "p50_ms": round(percentile(lats, 50), 3),
                    "p99_ms": round(percentile(lats, 99), 3),
                    "qps": round(nb / max(end, stream[nb - 1]["arrival_s"]), 2)}
        out["one_at_a_time_plain"] = one_at_a_time("plain")
        out["one_at_a_time_batched"] = one_at_a_time("batched")
        sub = lat[:nb]
        out["first_queries_concurrent"] = {"queries": nb, "p50_ms": round(percentile(sub, 50), 3),
                                           "p99_ms": round(percentile(sub, 99), 3)}
    return out


# The reference's only published timings: its authors' sweep scripts, SDSC on
# one GPU (CUDA 8 era, GPU model not stated) over 500k-point 16-d synthetic
# files, Execute() wall ms per cap -m (Release/scaleanticorr16:29-35,
# Release/scalecorrelated16:15-21).
REFERENCE_SWEEPS = [
    ("anticorrelated", 4, 25469.0, "Release/scaleanticorr16:29"),
    ("anticorrelated", 6, 279723.0, "Release/scaleanticorr16:30"),
    ("anticorrelated", 8, 1109848.0, "Release/scaleanticorr16:31"),
    ("correlated", 4, 9487.0, "Release/scalecorrelated16:15"),
    ("correlated", 6, 74686.0, "Release/scalecorrelated16:16"),
    ("correlated", 8, 240978.0, "Release/scalecorrelated16:17"),
    ("correlated", 10, 422859.0, "Release/scalecorrelated16:18"),
]


def run_reference_sweeps(sk, ctx):
    """Capped skycubes of 500,000 x 16 points (seeded stand-ins for the
    authors' anticorrelated and correlated files, which are not shipped) at
    the caps of the reference's published sweeps, batched form. device_ms:
    CUDA events around the skycube call, dataset resident (best of two after
    a warm-up). e2e_ms: host rows in, every cuboid's ids in host memory
    (upload, skycube, download), best of two."""
    rows, cache = [], {}
    for kind, m, ref_ms, src in REFERENCE_SWEEPS:
        if kind not in cache:
            cache[kind] = datagen.generate(kind, 500000, 16, 1)
        x = cache[kind]
        ds = sk.Dataset(ctx, x)
        dev, info = [], None
        for rep in range(3):
            r = sk.skycube(ctx, ds, max_d=m)
            info = r.info()
            r.close()
            if rep:
                dev.append(ctx.last_device_ms())
        ds.close()
        e2e = []
        for _ in range(2):
            t0 = time.perf_counter()
            ds = sk.Dataset(ctx, x)
            r = sk.skycube(ctx, ds, max_d=m)
            r.download()
            r.close()
            ds.close()
            e2e.append((time.perf_counter() - t0) * 1000.0)
        rows.append({"workload": f"{kind} 500,000 x 16", "max_d": m,
                     "device_ms": round(min(dev), 3), "e2e_ms": round(min(e2e), 3),
                     "total_skyline_ids": info["total_skyline_ids"],
                     "reference_ms": ref_ms, "reference_source": src})
    return {"rows": rows,
            "note": "reference_ms: the authors' SDSC runs on one GPU of their own machine "
                    "(not a GB300) over their data files; these inputs are seeded synthetic "
                    "stand-ins with the same shape and distribution family"}


def run_ours(args, world, rank, local):
    import torch
    import skycube_gb300 as sk

    torch.cuda.set_device(local)
    kind, n, d, max_d, seed, x = workload(args.workload, rank)
    ctx = sk.Context(local)
    ds = sk.Dataset(ctx, x)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def step():
        r = sk.skycube(ctx, ds, "mdmc", "batched", max_d=max_d)
        info = r.info()
        phases = dict(ctx.last_phases())
        ms = ctx.last_device_ms()
        r.close()
        return ms, phases, info

    for _ in range(args.warmup):
        flush_l2(flush)
        torch.cuda.synchronize()
        step()

    clocks = Clocks(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    launches0 = sk.kernel_launches()
    step_ms, kern_ms = [], []
    t_wall0 = time.perf_counter()
    info = None
    for _ in range(args.steps):
        flush_l2(flush)
        torch.cuda.synchronize()
        ms, phases, info = step()
        timed_phases = phases
        step_ms.append(ms)
        kern_ms.append(phases.get("bitmap kernel", float("nan")))
    torch.cuda.synchronize()
    barrier(world)
    wall = time.perf_counter() - t_wall0
    launches = sk.kernel_launches() - launches0
    clk = clocks.stop()

    mean_ms = max_over_ranks(world, sum(step_ms) / len(step_ms))
    value = world * n / (mean_ms / 1000.0)

    # e2e through the C ABI with host buffers (pinned), every step copies the
    # points in and every cuboid's ids out.
    pinned = torch.from_numpy(x).pin_memory()
    xp = pinned.numpy()
    e2e_s, d2h = [], 0
    for i in range(args.warmup + args.steps):
        flush_l2(flush)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dse = sk.Dataset(ctx, xp)
        r = sk.skycube(ctx, dse, "mdmc", "batched", max_d=max_d)
        r.download()
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_s.append(t1 - t0)
        d2h = ((1 << d) + 1) * 8 + r.info()["total_skyline_ids"] * 4
        r.close()
        dse.close()
    e2e_mean = max_over_ranks(world, sum(e2e_s) / len(e2e_s))

    # The same skycube through a plan (one CUDA graph per step): device time
    # of the replay, and end to end with the points updated in place from
    # pinned host memory and every cuboid's ids copied out.
    plan = sk.Plan(ctx, ds, algo="mdmc", mode="batched", max_d=max_d)
    pinfo = plan.info()
    g_ms, g_e2e = [], []
    for i in range(args.warmup + args.steps):
        flush_l2(flush)
        torch.cuda.synchronize()
        r = plan.execute()
        ms = ctx.last_device_ms()
        r.close()
        flush_l2(flush)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ds.update(xp)
        r = plan.execute()
        r.download()
        t1 = time.perf_counter()
        r.close()
        if i >= args.warmup:
            g_ms.append(ms)
            g_e2e.append(t1 - t0)
    g_mean = max_over_ranks(world, sum(g_ms) / len(g_ms))
    g_e2e_mean = max_over_ranks(world, sum(g_e2e) / len(g_e2e))
    graph = {"form": "batched skycube captured as one CUDA graph (skc_plan), replayed per step",
             "ms": round(g_mean, 3), "value": round(world * n / (g_mean / 1000.0), 1), "unit": UNIT,
             "kernels_per_replay": pinfo["kernels"], "replans": plan.info()["replans"],
             "e2e": {"value": round(world * n / g_e2e_mean, 1), "unit": UNIT,
                     "ms_per_step": round(g_e2e_mean * 1000, 3),
                     "h2d_bytes_per_step": n * d * 4, "d2h_bytes_per_step": d2h,
                     "path": "skc_dataset_update (pinned host rows) + skc_plan_execute + "
                             "skc_result_download"}}
    plan.close()

    plain = None
    if not args.no_plain:
        flush_l2(flush)
        torch.cuda.synchronize()
        r = sk.skycube(ctx, ds, "sdsc", "plain", max_d=max_d)
        pms = ctx.last_device_ms()
        tot = r.info()["total_skyline_ids"]
        r.close()
        plain = {"form": "sdsc per-cuboid (one launch sequence + host sync per cuboid)",
                 "ms": round(pms, 3), "value": round(n / (pms / 1000.0), 1), "unit": UNIT,
                 "total_skyline_ids": tot,
                 "batched_speedup": round(pms / mean_ms, 3)}

    peaks, peak_kind = measured_peaks()
    m = info["n_candidates"]
    kern = statistics.median(kern_ms)
    words = max(1, (1 << d) // 32)
    # algorithmic bytes of one bitmap launch: the candidates' coordinates and
    # grid cells read once, one dominated-subspace bitmap written per candidate
    alg_bytes = m * (d * 4 + 16) + m * words * 4
    achieved_gbs = alg_bytes / (kern / 1000.0) / 1e9
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    pairs = float(m) * float(m)
    sm_mhz = clk.get("sm_mhz") or float(peaks.get("sm_max_mhz", 2070.0))
    issue_peak = 152 * 4 * sm_mhz * 1e6  # warp instructions/s: 152 SMs x 4 schedulers
    # Counters of the same kernel from one ncu capture of this workload
    # (profiles/kernel_counters_<workload>.json): DRAM bytes and warp
    # instructions per launch.
    traffic, inst = None, None
    tpath = os.path.join(REPO, "profiles", f"kernel_counters_{args.workload}.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            t = json.load(f).get("k_bitmaps", {})
        traffic = t.get("dram_bytes_per_launch")
        inst = t.get("warp_inst_per_launch")

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        ns = min(n, args.cpu_sample or auto_cpu_sample(args.workload))
        dt, threads, ckind = cpu_sample_run(x, d, max_d, ns)
        cpu = {"value": round(ns / dt, 1), "unit": UNIT, "cores": threads, "kind": ckind,
               "sample": f"first {ns:,} points of the same workload, the same cuboids, "
                         f"{dt:.2f} s, timed around the skycube computation only, with "
                         f"{cpu_kind_note(ckind)}; its cost grows faster than linearly in n, so "
                         f"the whole workload runs at a lower rate on the CPU"}

    serving = None
    if rank == 0 and world == 1 and args.serving_queries > 0:
        serving = run_serving(sk, ctx, args)
    sweeps = None
    if rank == 0 and world == 1 and not args.no_sweeps:
        sweeps = run_reference_sweeps(sk, ctx)

    out = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(mean_ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded; the suite's data files are not shipped)",
        "config": {"workload": f"{kind} n={n:,} d={d} float32, cuboids with <= {max_d} attributes "
                               f"(all {2 ** d - 1 if max_d == d else 'capped'}), batched persistent form",
                   "name": args.workload, "n": n, "d": d, "max_d": max_d, "seed": seed,
                   "algo": "mdmc", "mode": "batched",
                   "l2": "flushed before every step (256 MiB device write)",
                   "parallelism": f"{world} replica(s), no collective"},
        "e2e": {"value": round(world * n / e2e_mean, 1), "unit": UNIT,
                "h2d_bytes_per_step": n * d * 4, "d2h_bytes_per_step": d2h,
                "ms_per_step": round(e2e_mean * 1000, 3)},
        "roofline": {"kernel": "k_bitmaps", "bound": "hbm", "achieved": round(achieved_gbs, 3),
                     "peak": hbm, "unit": "GB/s", "frac": round(achieved_gbs / hbm, 6),
                     "traffic": traffic, "peak_source": peak_kind,
                     "kernel_ms": round(kern, 3), "alg_bytes": alg_bytes},
        "issue_roofline": {
            "kernel": "k_bitmaps",
            "achieved": round(inst / (kern / 1000.0) / 1e9, 2) if inst else None,
            "peak": round(issue_peak / 1e9, 2), "unit": "G warp-instructions/s",
            "frac": round(inst / (kern / 1000.0) / issue_peak, 4) if inst else None,
            "warp_inst_per_launch": inst,
            "pair_space": int(pairs),
            "note": "the kernel is bound by instruction issue, not DRAM: warp instructions "
                    "per launch from one ncu capture of this workload, divided by the live "
                    "event-timed kernel duration; peak = 152 SMs x 4 schedulers x median SM "
                    "clock under load"},
        "cpu_baseline": cpu,
        "clocks": clk,
        "gpu_launches": int(launches),
        "phases_ms": {k: round(v, 3) for k, v in timed_phases.items()},
        "n_candidates": m, "total_skyline_ids": info["total_skyline_ids"],
        "wall_s_timed_region": round(wall, 3),
    }
    out["graph"] = graph
    if plain:
        out["plain"] = plain
    if serving:
        out["serving"] = serving
    if sweeps:
        out["reference_sweeps"] = sweeps
    if rank == 0:
        print(json.dumps(out), flush=True)
    ctx.close()


def run_reference(args, world, rank):
    """The reference arm: the reference's own CPU path for this computation,
    STSC (HybridCube<D>, the suite's -c oracle) built from its unmodified
    sources, on every host thread. Each step is a bounded sample of the
    workload (its first --cpu-sample points, same cuboids); one full-size run
    follows the timed steps unless --no-ref-full."""
    if rank != 0:
        return
    kind, n, d, max_d, seed, x = workload(args.workload, 0)
    ns = min(n, args.cpu_sample or auto_cpu_sample(args.workload))
    times, threads, ckind = [], os.cpu_count() or 1, "port"
    for i in range(args.warmup + args.steps):
        dt, threads, ckind = cpu_sample_run(x, d, max_d, ns)
        if i >= args.warmup:
            times.append(dt)
    mean = sum(times) / len(times)
    value = ns / mean
    sample = (f"first {ns:,} of the {n:,} points of the workload, the same cuboids, per step; "
              f"{cpu_kind_note(ckind)}, timed around the skycube computation only")
    out = {
        "impl": "reference", "metric": METRIC, "value": round(value, 1), "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(mean * 1000, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": f"{kind} n={n:,} d={d} float32, cuboids with <= {max_d} attributes",
                   "name": args.workload, "n": n, "d": d, "max_d": max_d, "seed": seed},
        "cpu_baseline": {"value": round(value, 1), "unit": UNIT, "cores": threads, "kind": ckind,
                         "sample": sample},
        "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    if not args.no_ref_full and ns < n:
        dt, threads, ckind = cpu_sample_run(x, d, max_d, n)
        out["full_size"] = {"points": n, "seconds": round(dt, 3), "value": round(n / dt, 1),
                            "unit": UNIT, "cores": threads, "kind": ckind, "same_config": True,
                            "note": "one untimed-by-steps run of the whole workload after the "
                                    "timed sample steps"}
    print(json.dumps(out), flush=True)


def main():
    args = parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
