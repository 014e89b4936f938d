"""Work parameters never change results: the pruner prefilter (the suite's
PQFilter ahead of the full-space skyline, any pruner count) and the
autotuner's choices (grid depth, pruners, bitmap tile, queue chunk, CTAs per
SM) against the golden fixtures, the C oracle and the unfiltered run.
Comparisons are exact id-set equality per cuboid."""
import numpy as np
import pytest

import oracle
import skycube_gb300 as sk
from conftest import golden_names, load_golden
from skycube_gb300 import datagen

pytestmark = pytest.mark.gpu


def sets(r, d, max_d, ext=False):
    out = {}
    for c in range(1, 1 << d):
        if bin(c).count("1") <= max_d or c == (1 << d) - 1:
            out[c] = r.extended(c) if ext else r.cuboid(c)
    return out


def assert_same(a, b):
    assert a.keys() == b.keys()
    for c in a:
        assert np.array_equal(a[c], b[c]), f"cuboid {c}: {len(a[c])} vs {len(b[c])}"


@pytest.mark.parametrize("name", golden_names())
def test_golden_with_prefilter(gpu_ctx, name):
    x, max_d, sky, ext = load_golden(name)
    n, d = x.shape
    pq = max(1, min(16, (n - 1) // 2))  # n > 2 * pq: the filter runs (n >= 3)
    ds = sk.Dataset(gpu_ctx, x)
    for algo, mode in (("mdmc", "batched"), ("sdsc", "batched"), ("mdmc", "plain")):
        r = sk.skycube(gpu_ctx, ds, algo, mode, max_d=max_d, want_extended=True, pq_size=pq)
        assert_same(sets(r, d, max_d), {c: sky[c] for c in sets(r, d, max_d)})
        assert_same(sets(r, d, max_d, True), {c: ext[c] for c in sets(r, d, max_d, True)})


PQ_CASES = [("ties", 3000, 6, 1), ("uniform", 5000, 5, 2), ("anticorrelated", 4000, 7, 3),
            ("correlated_q", 6000, 9, 4), ("ties", 2500, 12, 5)]


@pytest.mark.parametrize("kind,n,d,seed", PQ_CASES)
def test_prefilter_against_oracle(gpu_ctx, kind, n, d, seed):
    x = datagen.generate(kind, n, d, seed)
    sky, ext = oracle.stsc(x)
    ds = sk.Dataset(gpu_ctx, x)
    for pq in (1, 5, 128, 1000, -1):
        r = sk.skycube(gpu_ctx, ds, "mdmc", "batched", want_extended=True, pq_size=pq)
        ran = any(p == "full: prefilter" for p, _ in gpu_ctx.last_phases())
        assert ran == (pq > 0 and n > 2 * pq)
        assert_same(sets(r, d, d), {c: sky[c] for c in range(1, 1 << d)})
        assert_same(sets(r, d, d, True), {c: ext[c] for c in range(1, 1 << d)})


def test_prefilter_skyline_query(gpu_ctx):
    x = datagen.generate("ties", 40000, 9, 8)
    ds = sk.Dataset(gpu_ctx, x)
    for S in (0b101, 0b110110, (1 << 9) - 1):
        a = sk.skycube(gpu_ctx, ds, subspace=S, want_extended=True, pq_size=-1)
        b = sk.skycube(gpu_ctx, ds, subspace=S, want_extended=True, pq_size=64)
        assert np.array_equal(a.cuboid(S), b.cuboid(S))
        assert np.array_equal(a.extended(S), b.extended(S))


@pytest.mark.parametrize("name", ["uniform-100k-6", "anticorr-1m-10", "ties-581k-10", "corrq-566k-15-m6"])
def test_prefilter_full_size(gpu_ctx, name):
    kind, n, d, m, seed = datagen.CONFIGS[name]
    x = datagen.generate(kind, n, d, seed)
    ds = sk.Dataset(gpu_ctx, x)
    a = sk.skycube(gpu_ctx, ds, "mdmc", "batched", max_d=m, pq_size=-1)
    b = sk.skycube(gpu_ctx, ds, "mdmc", "batched", max_d=m, pq_size=512)
    assert a.info() == b.info()
    assert_same(sets(a, d, m), sets(b, d, m))


def test_work_parameters_do_not_change_results(gpu_ctx):
    x = datagen.generate("ties", 40000, 10, 9)
    ds = sk.Dataset(gpu_ctx, x)
    ref = sk.skycube(gpu_ctx, ds, "sdsc", "batched", want_extended=True, pq_size=-1)
    rs, re = sets(ref, 10, 10), sets(ref, 10, 10, True)
    for kw in ({"tile_points": 32}, {"tile_points": 4096}, {"chunk": 7}, {"chunk": 64},
               {"blocks_per_sm": 1}, {"blocks_per_sm": 3, "chunk": 2}, {"depth": 3, "pq_size": 300}):
        r = sk.skycube(gpu_ctx, ds, "sdsc", "batched", want_extended=True, **kw)
        assert_same(sets(r, 10, 10), rs)
        assert_same(sets(r, 10, 10, True), re)
    r = sk.skycube(gpu_ctx, ds, "mdmc", "plain", chunk=5, tile_points=128)
    assert_same(sets(r, 10, 10), rs)


def test_rejects_bad_work_parameters(gpu_ctx):
    ds = sk.Dataset(gpu_ctx, datagen.generate("uniform", 100, 3, 1))
    for kw in ({"pq_size": 1025}, {"tile_points": 100}, {"tile_points": 16}, {"chunk": 65},
               {"chunk": -1}, {"blocks_per_sm": 33}, {"blocks_per_sm": -2}):
        with pytest.raises(sk.SkycubeError):
            sk.skycube(gpu_ctx, ds, **kw)


def test_signature_classes(gpu_ctx):
    sig = {k: sk.signature(sk.Dataset(gpu_ctx, datagen.generate(k, 50000, 8, 3)))
           for k in ("correlated", "uniform", "anticorrelated", "ties")}
    assert sig["correlated"]["sky_class"] < sig["uniform"]["sky_class"] < sig["anticorrelated"]["sky_class"]
    assert sig["ties"]["ties"] == 1 and sig["uniform"]["ties"] == 0
    assert all(s["size_class"] == 15 for s in sig.values())  # 2^15 <= 50000 < 2^16


def test_autotune_stores_and_applies(gpu_ctx):
    gpu_ctx.tuning_clear()
    try:
        x = datagen.generate("ties", 60000, 8, 5)
        ds = sk.Dataset(gpu_ctx, x)
        ref = sk.skycube(gpu_ctx, ds, "mdmc", "batched", want_extended=True, pq_size=-1)
        params, ms = sk.autotune(gpu_ctx, ds, repeats=1, algo="mdmc", mode="batched",
                                 want_extended=True)
        assert ms > 0
        assert 1 <= params["depth"] <= 7
        assert params["pq_size"] in (-1, 32, 128, 512)
        assert params["tile_points"] in (64, 256, 1024)
        assert params["chunk"] in (1, 4, 16)
        assert params["blocks_per_sm"] in (0, 1, 2)
        assert gpu_ctx.tuning_count() == 1
        # Another dataset with the same signature picks the tuning up: the
        # points scaled by 2 (exact in float32, so every comparison, tie and
        # the sample signature are unchanged).
        x2 = x * np.float32(2.0)
        ds2 = sk.Dataset(gpu_ctx, x2)
        assert sk.signature(ds2) == sk.signature(ds)
        sky, ext = oracle.stsc(x2)
        r2 = sk.skycube(gpu_ctx, ds2, "mdmc", "batched", want_extended=True)
        ran = any(p == "full: prefilter" for p, _ in gpu_ctx.last_phases())
        assert ran == (params["pq_size"] > 0)
        assert_same(sets(r2, 8, 8), {c: sky[c] for c in range(1, 256)})
        assert_same(sets(r2, 8, 8, True), {c: ext[c] for c in range(1, 256)})
        r = sk.skycube(gpu_ctx, ds, "mdmc", "batched", want_extended=True)
        assert_same(sets(r, 8, 8), sets(ref, 8, 8))
        # Other forms tune their own keys.
        sk.autotune(gpu_ctx, ds, repeats=1, algo="sdsc", mode="plain", max_d=2)
        sk.autotune(gpu_ctx, ds, repeats=1, subspace=0b1011)
        assert gpu_ctx.tuning_count() == 3
    finally:
        gpu_ctx.tuning_clear()
    assert gpu_ctx.tuning_count() == 0
