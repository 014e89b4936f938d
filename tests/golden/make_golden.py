"""Generates the golden fixtures of tests/golden from the REFERENCE's own STSC.

Runs only where the reference checkout is present and oracle/build_ref.sh has
built oracle/_ref/libskycube_ref.so (the reference's HybridCube + MommyQ
compiled from its sources). For every case it stores the input points and the
reference's per-cuboid skyline and extended-skyline id sets, so the fixtures
pin both the C oracle and the CUDA path on machines without the reference.

Usage: python tests/golden/make_golden.py
       python tests/golden/make_golden.py --digests [workload ...]
       python tests/golden/make_golden.py --crosscheck-pq workload ...
The second form writes digest_<workload>.npz for the full-size benchmark
workloads (per-cuboid counts and id-list hashes, not the id lists). The
third checks existing digests' skylines against the reference's PQSkycube.
"""
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "skycube-templates_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from skycube_gb300 import datagen  # noqa: E402
import oracle  # noqa: E402

# name: (distribution, n, d, max_d, seed)
CASES = {
    "uniform_2000_6": ("uniform", 2000, 6, 6, 1),
    "ties_3000_6": ("ties", 3000, 6, 6, 2),
    "anticorr_2000_8": ("anticorrelated", 2000, 8, 8, 3),
    "corrq_2000_10_m4": ("correlated_q", 2000, 10, 4, 4),
    "ties_1500_12_m3": ("ties", 1500, 12, 3, 5),
    "uniform_400_16_m2": ("uniform", 400, 16, 2, 6),
    "anticorr_3000_5": ("anticorrelated", 3000, 5, 5, 7),
    "ties_800_2": ("ties", 800, 2, 2, 8),
}


def edge_cases():
    """Small hand-made inputs: duplicates, a single point, signed zeros."""
    rng = np.random.default_rng(99)
    dup = np.repeat(rng.random((5, 4), dtype=np.float64), 7, axis=0)
    dup = dup[rng.permutation(len(dup))].astype(np.float32)
    same = np.full((40, 3), 0.5, dtype=np.float32)
    one = np.array([[0.25, 0.75, 0.5]], dtype=np.float32)
    zeros = np.array([[0.0, 1.0], [-0.0, 1.0], [0.0, 0.5], [1.0, -0.0], [-0.0, 0.0]],
                     dtype=np.float32)
    grid = np.floor(rng.random((600, 7)) * 3).astype(np.float32)  # 3 levels: heavy ties
    return {
        "edge_duplicates_35_4": (dup, 4),
        "edge_identical_40_3": (same, 3),
        "edge_single_1_3": (one, 3),
        "edge_signed_zero_5_2": (zeros, 2),
        "edge_grid3_600_7": (grid, 7),
    }


def pack(d, sets):
    off = [0]
    ids = []
    for c in range(1, 1 << d):
        a = sets.get(c, np.empty(0, np.uint32))
        ids.append(a)
        off.append(off[-1] + len(a))
    return np.array(off, np.uint64), (np.concatenate(ids) if ids else np.empty(0, np.uint32)).astype(np.uint32)


def write(name, x, max_d):
    d = x.shape[1]
    res = oracle.ref_stsc(x, max_d, threads=8)
    if res is None:
        raise SystemExit("reference STSC not built: run oracle/build_ref.sh first")
    sky, ext = res
    so, si = pack(d, sky)
    eo, ei = pack(d, ext)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), x=x, max_d=np.int32(max_d),
                        sky_off=so, sky_ids=si, ext_off=eo, ext_ids=ei)
    print(f"{name}: n={len(x)} d={d} max_d={max_d} skyline ids={len(si)} extended ids={len(ei)}")


def id_hash(ids):
    """64-bit digest of an ascending id list (BLAKE2b of its little-endian
    uint32 bytes); the full-size GPU tests compute the same."""
    a = np.ascontiguousarray(ids, dtype="<u4")
    return int.from_bytes(hashlib.blake2b(a.tobytes(), digest_size=8).digest(), "little")


def points_hash(x):
    return id_hash(np.ascontiguousarray(x, dtype="<f4").view("<u4").ravel())


# Full-size benchmark workloads pinned by digest (datagen.CONFIGS names).
DIGEST_CASES = ("anticorr-1m-10", "corrq-566k-15-m6", "uniform-100k-6", "ties-581k-10")


# Down-scaled stand-ins of full-size workloads whose reference run takes too
# long here: (distribution, n, d, max_d, seed), same generator and seed.
SCALED = {"corrq-100k-15-m6": ("correlated_q", 100_000, 15, 6, 42)}

# Seeded stand-ins of the reference's published capped sweeps over 500k x 16
# files (the benchmark's reference_sweeps), at the cap whose reference run
# finishes here (-m 4: 36 s anticorrelated, 1,352 s correlated on 8 threads;
# a correlated -m 10 run, 26,000 cuboids, was stopped unfinished).
SWEEPS = {
    "sweep-anticorr-500k-16-m4": ("anticorrelated", 500_000, 16, 4, 1),
    "sweep-corr-500k-16-m4": ("correlated", 500_000, 16, 4, 1),
}


def write_digest(name, threads):
    """Per-cuboid digest of the reference's own STSC on one full-size
    workload (or a SCALED or SWEEPS stand-in): for every computed cuboid its skyline
    and extended-skyline counts and the 64-bit hashes of both ascending id
    lists, plus a hash of the generated points (so a generator that differs
    is reported as such)."""
    kind, n, d, max_d, seed = (SCALED.get(name) or SWEEPS.get(name) or datagen.CONFIGS[name])
    x = datagen.generate(kind, n, d, seed)
    t0 = time.time()
    res = oracle.ref_stsc(x, max_d, threads=threads)
    if res is None:
        raise SystemExit("reference STSC not built: run oracle/build_ref.sh first")
    secs = time.time() - t0
    sky, ext = res
    cub = np.array(sorted(sky), dtype=np.uint32)
    out = dict(
        points_hash=np.uint64(points_hash(x)), n=np.uint64(n), d=np.int32(d),
        max_d=np.int32(max_d), seed=np.int64(seed), kind=np.array(kind),
        cuboids=cub,
        sky_count=np.array([len(sky[c]) for c in cub], dtype=np.uint64),
        ext_count=np.array([len(ext[c]) for c in cub], dtype=np.uint64),
        sky_hash=np.array([id_hash(sky[c]) for c in cub], dtype=np.uint64),
        ext_hash=np.array([id_hash(ext[c]) for c in cub], dtype=np.uint64),
        reference_seconds=np.float64(secs), reference_threads=np.int32(threads))
    np.savez_compressed(os.path.join(HERE, f"digest_{name}.npz"), **out)
    print(f"digest {name}: {len(cub)} cuboids, {int(out['sky_count'].sum())} skyline ids, "
          f"{int(out['ext_count'].sum())} extended ids; reference STSC {secs:.1f} s on "
          f"{threads} threads", flush=True)


def crosscheck_pq(name, threads):
    """Runs the reference's PQSkycube (oracle/_ref/libskycube_ref_pq.so) on
    a digest's workload and compares its skyline of every cuboid with the
    digest (made by the reference's STSC): two independent reference
    algorithms on the same full-size input. Returns the number of cuboids
    that differ."""
    dg = dict(np.load(os.path.join(HERE, f"digest_{name}.npz")))
    kind, n, d, max_d, seed = (str(dg["kind"]), int(dg["n"]), int(dg["d"]), int(dg["max_d"]),
                               int(dg["seed"]))
    x = datagen.generate(kind, n, d, seed)
    if points_hash(x) != int(dg["points_hash"]):
        raise SystemExit(f"{name}: the generator gives other points than the digest's")
    t0 = time.time()
    res = oracle.ref_pq(x, max_d, threads=threads)
    if res is None:
        raise SystemExit("reference PQSkycube not built: run oracle/build_ref.sh --pq first")
    secs = time.time() - t0
    sky = res[0]
    bad = [int(c) for i, c in enumerate(dg["cuboids"].tolist())
           if len(sky[c]) != int(dg["sky_count"][i]) or id_hash(sky[c]) != int(dg["sky_hash"][i])]
    print(f"pq-crosscheck {name}: {len(dg['cuboids'])} cuboids, {len(bad)} differ "
          f"(first: {bad[:5]}); PQSkycube {secs:.1f} s on {threads} threads", flush=True)
    return len(bad)


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "--crosscheck-pq":
        bad = sum(crosscheck_pq(name, os.cpu_count() or 1) for name in sys.argv[2:])
        raise SystemExit(1 if bad else 0)
    if len(sys.argv) > 1 and sys.argv[1] == "--digests":
        names = sys.argv[2:] or DIGEST_CASES
        for name in names:
            write_digest(name, os.cpu_count() or 1)
        return
    for name, (kind, n, d, max_d, seed) in CASES.items():
        write(name, datagen.generate(kind, n, d, seed), max_d)
    for name, (x, d) in edge_cases().items():
        write(name, x, d)


if __name__ == "__main__":
    main()
