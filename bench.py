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
    ap.add_argument("--serving-queries", type=int, default=2000,
                    help="queries of the serving stream (0: skip serving)")
    ap.add_argument("--serving-rate", type=float, default=20.0, help="Poisson arrival rate, queries/s")
    ap.add_argument("--serving-slots", type=int, default=4)
    ap.add_argument("--serving-baseline", type=int, default=200,
                    help="queries served one at a time with the plain form for comparison")
    ap.add_argument("--record-counters", metavar="NCU_CSV",
                    help="write profiles/kernel_counters_<workload>.json from the --csv output of "
                         "ncu --print-units base --metrics smsp__inst_executed.sum,"
                         "dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum "
                         "-k regex:k_bitmaps over this benchmark, with the sha256 of the bitmap "
                         "kernel's sources, then exit")
    ap.add_argument("--record-useful", action="store_true",
                    help="build the bitmap kernel's counters library, run the workload once with "
                         "it and add its per-candidate work figures to "
                         "profiles/kernel_counters_<workload>.json, then exit")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the other benchmark configurations (100k x 6, ties, 15-d capped)")
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


def bitmap_sources_sha():
    """sha256 of the bitmap kernel's sources (mdmc.cu and the headers it
    includes): a recorded instruction count is valid only for these."""
    import hashlib
    h = hashlib.sha256()
    csrc = os.path.join(REPO, "skycube-templates_gb300", "csrc")
    for f in ("mdmc.cu", "common.cuh", "kernels.cuh"):
        with open(os.path.join(csrc, f), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()


def kernel_counts(workload):
    """Counters of the bitmap kernel from profiles/kernel_counters_<workload>.json
    (an ncu capture of the full-size workload): warp instructions and DRAM
    bytes per launch, used only when the capture's recorded source hash
    matches the sources built now."""
    path = os.path.join(REPO, "profiles", f"kernel_counters_{workload}.json")
    if not os.path.exists(path):
        return {"provenance": {"file": None, "matches": False}}
    with open(path) as f:
        t = json.load(f).get("k_bitmaps", {})
    sha = bitmap_sources_sha()
    ok = t.get("sources_sha256") == sha
    prov = {"file": os.path.relpath(path, REPO), "matches": ok,
            "sources_sha256": sha[:16], "recorded_sha256": (t.get("sources_sha256") or "")[:16]}
    if not ok:
        return {"provenance": prov}
    return {"warp_inst_per_launch": t.get("warp_inst_per_launch"),
            "dram_bytes_per_launch": t.get("dram_bytes_per_launch"),
            "useful": t.get("useful"), "provenance": prov}


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
    """Serving stream (config 5): --serving-queries queries arrive Poisson at
    --serving-rate, each over its own seeded dataset (n log-uniform in
    [1e3, 1e6], d in 4..16, uniform / correlated / anticorrelated; a seeded
    window of a per-(distribution, d) pool, datagen.ServingPools); half
    skycubes (every cuboid for d <= 10, else a cap of 2..6 attributes drawn
    per query), half skylines of one random subspace. Served by the
    continuous-batching server (host rows in, host results out). The first
    --serving-baseline queries are also served one at a time with the plain
    per-cuboid form and with the batched form, on the same arrival times
    (a sequential queue on a virtual clock from measured service times)."""
    stream = datagen.serving_stream(count=args.serving_queries, rate_qps=args.serving_rate, seed=7)
    pools = datagen.ServingPools()
    t_gen = time.perf_counter()
    data = [pools.dataset(q) for q in stream]
    gen_s = time.perf_counter() - t_gen
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
    lat, queued, run, dev = [], [], [], []
    for t in tickets:
        r, tm = srv.wait(t)
        lat.append(tm["total_ms"])
        queued.append(tm["queued_ms"])
        run.append(tm["run_ms"])
        dev.append(tm["device_ms"])
        r.close()
    span = max(time.perf_counter() - t0, stream[-1]["arrival_s"])
    stats = srv.stats()
    srv.close()
    sky = [i for i, q in enumerate(stream) if not q["subspace"]]

    def pct(idx, p):
        return round(percentile([lat[i] for i in idx], p), 3) if idx else None

    out = {"queries": len(stream), "rate_qps": args.serving_rate, "slots": args.serving_slots,
           "p50_ms": round(percentile(lat, 50), 3), "p99_ms": round(percentile(lat, 99), 3),
           "mean_ms": round(sum(lat) / len(lat), 3), "max_ms": round(max(lat), 3),
           "qps": round(len(stream) / span, 2), "peak_in_flight": stats["peak_in_flight"],
           "queued_p50_ms": round(percentile(queued, 50), 3),
           "queued_p99_ms": round(percentile(queued, 99), 3),
           "run_p50_ms": round(percentile(run, 50), 3), "run_p99_ms": round(percentile(run, 99), 3),
           "device_p50_ms": round(percentile(dev, 50), 3),
           "device_p99_ms": round(percentile(dev, 99), 3),
           "skycube_queries": len(sky), "skycube_p50_ms": pct(sky, 50), "skycube_p99_ms": pct(sky, 99),
           "skyline_p50_ms": pct([i for i in range(len(stream)) if stream[i]["subspace"]], 50),
           "skyline_p99_ms": pct([i for i in range(len(stream)) if stream[i]["subspace"]], 99),
           "datasets_host_s": round(gen_s, 2),
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


def run_configs(sk, ctx, flush):
    """The other benchmark configurations (the headline is 1M x 10
    anticorrelated): 100k x 6 uniform in the plain per-cuboid form and
    batched; 581k x 10 ties batched with the work parameters autotuned over
    grid depths 2..4; 566k x 15 correlated (quantised), cuboids of <= 6
    attributes, as a CUDA-graph plan. Device ms: CUDA events around the
    computation, L2 flushed before each run, median of 5 after a warm-up.
    e2e ms: host rows in (pinned), every cuboid's ids in host memory."""
    import torch

    def dev_ms(fn, reps=5):
        fn().close()
        ms = []
        for _ in range(reps):
            flush_l2(flush)
            torch.cuda.synchronize()
            r = fn()
            ms.append(ctx.last_device_ms())
            r.close()
        return round(statistics.median(ms), 3)

    def e2e_ms(x, reps=3, **opts):
        xp = torch.from_numpy(x).pin_memory().numpy()
        best = None
        for _ in range(reps):
            flush_l2(flush)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ds = sk.Dataset(ctx, xp)
            r = sk.skycube(ctx, ds, **opts)
            r.download()
            t = (time.perf_counter() - t0) * 1000.0
            r.close()
            ds.close()
            best = t if best is None else min(best, t)
        return round(best, 3)

    out = {}
    # 100k x 6 uniform: the plain form (one launch sequence per cuboid)
    kind, n, d, m, seed = datagen.CONFIGS["uniform-100k-6"]
    x = datagen.generate(kind, n, d, seed)
    ds = sk.Dataset(ctx, x)
    plain = dev_ms(lambda: sk.skycube(ctx, ds, "sdsc", "plain", max_d=m))
    batched = dev_ms(lambda: sk.skycube(ctx, ds, "mdmc", "batched", max_d=m))
    r = sk.skycube(ctx, ds, "sdsc", "plain", max_d=m)
    ids = r.info()["total_skyline_ids"]
    r.close()
    ds.close()
    out["uniform-100k-6"] = {
        "workload": f"uniform n={n:,} d={d}, all {2 ** d - 1} cuboids", "plain_ms": plain,
        "plain_points_per_s": round(n / (plain / 1000.0), 1), "batched_ms": batched,
        "batched_over_plain": round(plain / batched, 2),
        "plain_e2e_ms": e2e_ms(x, algo="sdsc", mode="plain", max_d=m),
        "batched_e2e_ms": e2e_ms(x, algo="mdmc", mode="batched", max_d=m),
        "total_skyline_ids": ids}

    # 581k x 10 ties: batched, work parameters autotuned over depths 2..4
    kind, n, d, m, seed = datagen.CONFIGS["ties-581k-10"]
    x = datagen.generate(kind, n, d, seed)
    ds = sk.Dataset(ctx, x)
    ctx.tuning_clear()
    default = dev_ms(lambda: sk.skycube(ctx, ds, "mdmc", "batched", max_d=m))
    tuned = []
    for depth in (2, 3, 4):
        params, ms = sk.autotune(ctx, ds, repeats=2, algo="mdmc", mode="batched", depth=depth)
        tuned.append((ms, depth, params))
    tuned.sort(key=lambda t: t[0])
    _, depth, params = tuned[0]
    opts = {k: params[k] for k in ("depth", "pq_size", "tile_points", "chunk", "blocks_per_sm")}
    batched = dev_ms(lambda: sk.skycube(ctx, ds, "mdmc", "batched", max_d=m, **opts))
    flush_l2(flush)
    torch.cuda.synchronize()
    r = sk.skycube(ctx, ds, "sdsc", "plain", max_d=m)
    plain = round(ctx.last_device_ms(), 3)
    ids = r.info()["total_skyline_ids"]
    r.close()
    ctx.tuning_clear()
    ds.close()
    out["ties-581k-10"] = {
        "workload": f"ties n={n:,} d={d} (integer-valued), all {2 ** d - 1} cuboids",
        "batched_ms": batched, "points_per_s": round(n / (batched / 1000.0), 1),
        "autotuned": {"over_depths": [2, 3, 4], "chosen": opts,
                      "tuning_ms_by_depth": {str(t[1]): round(t[0], 3) for t in tuned}},
        "default_params_ms": default, "plain_ms": plain,
        "batched_over_plain": round(plain / batched, 1),
        "batched_e2e_ms": e2e_ms(x, algo="mdmc", mode="batched", max_d=m, **opts),
        "total_skyline_ids": ids}

    # 566k x 15 correlated (quantised), -m 6: the batched form as a CUDA graph
    kind, n, d, m, seed = datagen.CONFIGS["corrq-566k-15-m6"]
    x = datagen.generate(kind, n, d, seed)
    ds = sk.Dataset(ctx, x)
    plan = sk.Plan(ctx, ds, algo="mdmc", mode="batched", max_d=m)
    graph = dev_ms(plan.execute)
    batched = dev_ms(lambda: sk.skycube(ctx, ds, "mdmc", "batched", max_d=m))
    xp = torch.from_numpy(x).pin_memory().numpy()
    g_e2e = None
    for _ in range(3):
        flush_l2(flush)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ds.update(xp)
        r = plan.execute()
        r.download()
        t = (time.perf_counter() - t0) * 1000.0
        ids = r.info()["total_skyline_ids"]
        r.close()
        g_e2e = t if g_e2e is None else min(g_e2e, t)
    pinfo = plan.info()
    plan.close()
    ds.close()
    ncub = sum(1 for c in range(1, 1 << d) if bin(c).count("1") <= m) + 1
    out["corrq-566k-15-m6"] = {
        "workload": f"correlated (quantised to 0.1/{d}) n={n:,} d={d}, {ncub:,} cuboids of <= {m} "
                    f"attributes plus the full space, capped bitmaps",
        "graph_ms": graph, "points_per_s": round(n / (graph / 1000.0), 1), "batched_ms": batched,
        "graph_e2e_ms": round(g_e2e, 3), "kernels_per_replay": pinfo["kernels"],
        "total_skyline_ids": ids,
        "plain_ms_note": "the per-cuboid form takes about 31 s here (9,949 cuboids, one launch "
                         "sequence and host round trip each); not re-run by the benchmark"}
    return out


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
    sm_mhz = clk.get("sm_mhz") or float(peaks.get("sm_max_mhz", 2070.0))
    issue_peak = 152 * 4 * sm_mhz * 1e6  # warp instructions/s: 152 SMs x 4 schedulers
    counts = kernel_counts(args.workload)
    inst = counts.get("warp_inst_per_launch")
    roofline = {
        "kernel": "k_bitmaps", "bound": "issue",
        "achieved": round(inst / (kern / 1000.0) / 1e9, 2) if inst else None,
        "peak": round(issue_peak / 1e9, 2), "unit": "G warp-instructions/s",
        "frac": round(inst / (kern / 1000.0) / issue_peak, 4) if inst else None,
        "traffic": counts.get("dram_bytes_per_launch"),
        "kernel_ms": round(kern, 3), "warp_inst_per_launch": inst,
        "counts": counts.get("provenance"),
        "peak_source": f"152 SMs x 4 schedulers x median SM clock under load ({sm_mhz:.0f} MHz)",
        "note": "the bitmap kernel is bound by instruction issue (integer ALU), not DRAM: "
                "warp instructions per launch from an ncu capture of this workload whose "
                "kernel sources match the ones built (sha256 recorded with the count; "
                "null when they differ), divided by the live event-timed kernel duration",
        "hbm": {"achieved": round(achieved_gbs, 3), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved_gbs / hbm, 6), "alg_bytes": alg_bytes,
                "peak_source": peak_kind},
    }
    if counts.get("useful"):
        roofline["useful_work"] = counts["useful"]

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        ns = min(n, args.cpu_sample or auto_cpu_sample(args.workload))
        dt, threads, ckind = cpu_sample_run(x, d, max_d, ns)
        cpu = {"value": round(ns / dt, 1), "unit": UNIT, "cores": threads, "kind": ckind,
               "sample": f"first {ns:,} points of the same workload, the same cuboids, "
                         f"{dt:.2f} s, timed around the skycube computation only, with "
                         f"{cpu_kind_note(ckind)}; its cost grows faster than linearly in n, so "
                         f"the whole workload runs at a lower rate on the CPU"}

    configs = None
    if rank == 0 and world == 1 and not args.no_configs:
        configs = run_configs(sk, ctx, flush)
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
        "roofline": roofline,
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
    if configs:
        out["configs"] = configs
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


def record_counters(csv_path, workload):
    """Per-launch counters of the bitmap kernel from an ncu --csv log (the
    last k_bitmaps launch in it) into profiles/kernel_counters_<workload>.json."""
    import csv
    rows = []
    with open(csv_path) as f:
        lines = [ln for ln in f if ln.startswith('"')]
    for r in csv.DictReader(lines):
        if "k_bitmaps" in r.get("Kernel Name", ""):
            rows.append(r)
    if not rows:
        raise SystemExit(f"no k_bitmaps launch in {csv_path}")
    last = max(int(r["ID"]) for r in rows)
    vals = {}
    for r in rows:
        if int(r["ID"]) == last:
            vals[r["Metric Name"]] = float(r["Metric Value"].replace(",", ""))
    out = {"k_bitmaps": {
        "warp_inst_per_launch": int(vals["smsp__inst_executed.sum"]),
        "dram_bytes_per_launch": int(vals["dram__bytes_read.sum"] + vals["dram__bytes_write.sum"]),
        "dram_bytes_read": int(vals["dram__bytes_read.sum"]),
        "dram_bytes_write": int(vals["dram__bytes_write.sum"]),
        "gpu_time_ms_under_ncu": round(vals["gpu__time_duration.sum"] / 1e6, 3),
        "kernel_name": next(r["Kernel Name"] for r in rows if int(r["ID"]) == last),
        "sources_sha256": bitmap_sources_sha(),
        "source": os.path.basename(csv_path)}}
    path = os.path.join(REPO, "profiles", f"kernel_counters_{workload}.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out))


def record_useful(workload):
    """Per-candidate work of the bitmap kernel from its counters build (the
    same sources with SKC_BITMAP_COUNTERS=1), into the counts file."""
    import ctypes
    import importlib
    bmod = importlib.import_module("skycube_gb300.build")
    path = bmod.build(counters=True)
    import skycube_gb300 as sk
    sk.LIB_PATH = path
    L = sk.lib()
    f = L.skc_debug_bitmap_counters
    f.argtypes = [ctypes.c_void_p, ctypes.c_int]
    f.restype = ctypes.c_int
    kind, n, d, max_d, seed = datagen.CONFIGS[workload]
    ctx = sk.Context(0)
    ds = sk.Dataset(ctx, datagen.generate(kind, n, d, seed))
    sk.skycube(ctx, ds, "mdmc", "batched", max_d=max_d).close()
    c = (ctypes.c_ulonglong * 32)()
    f(c, 1)
    sk.skycube(ctx, ds, "mdmc", "batched", max_d=max_d).close()
    f(c, 0)
    m = max(1, c[0])
    names = ["candidates", "partition_ballots", "partitions_visited", "box_test_steps",
             "block_boxes_tested", "walk_steps", "walk_steps_all_covered",
             "strict_updates", "tie_pairs", "uncovered_q_tested", "sub_boxes_tested",
             "sub_blocks_opened", "cycles_partition_ballots", "cycles_box_tests",
             "cycles_quarter_and_half_box_tests", "cycles_walks", "cycles_candidate",
             "cycles_output", "half_boxes_tested", "halves_opened"]
    useful = {"per_candidate": {nm: round(c[i] / m, 3) for i, nm in enumerate(names) if i},
              "candidates": int(c[0]),
              "useful_walk_fraction": round(1 - c[6] / max(1, c[5]), 4),
              "note": "counters build of the same sources (SKC_BITMAP_COUNTERS=1): a walk "
                      "step tests 32 q's (four 8-q sub-blocks whose minimum-cell boxes "
                      "were not strict) and is useful when at least one of them was not "
                      "already covered by STRICT"}
    cpath = os.path.join(REPO, "profiles", f"kernel_counters_{workload}.json")
    with open(cpath) as fh:
        t = json.load(fh)
    kb = t.setdefault("k_bitmaps", {})
    if kb.get("sources_sha256") != bitmap_sources_sha():
        raise SystemExit("the recorded instruction count is for other sources: record it first")
    kb["useful"] = useful
    with open(cpath, "w") as fh:
        json.dump(t, fh, indent=1)
    print(json.dumps(useful))


def main():
    args = parse_args()
    if args.record_useful:
        record_useful(args.workload)
        return
    if args.record_counters:
        record_counters(args.record_counters, args.workload)
        return
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
