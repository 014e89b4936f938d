"""Full-size parity on the benchmark workloads.

Every full-size workload is pinned against the reference's own STSC through
a per-cuboid digest (counts and 64-bit hashes of the ascending skyline and
extended-skyline id lists, tests/golden/digest_*.npz, made by
tests/golden/make_golden.py --digests), for the batched form the benchmark
times, the batched form with extended skylines, and the per-cuboid form.

The two execution forms are independent GPU algorithms (per-point bitmaps in
one launch; per-cuboid median-partition skylines), so their exact agreement
on every cuboid of the full-size workloads is checked for all of them; the
CPU oracle (restated STSC, all host threads) pins the two workloads it
finishes in minutes. Size-independent properties are checked too: every
skyline is non-empty, nested under the candidate set, and the full-space
cuboid is always present."""
import numpy as np
import pytest

import oracle
import skycube_gb300 as sk
from conftest import id_hash, load_digest, points_hash
from skycube_gb300 import datagen

pytestmark = pytest.mark.gpu


def all_sets(r, d, max_d, ext=False):
    out = {}
    for c in range(1, 1 << d):
        if bin(c).count("1") <= max_d or c == (1 << d) - 1:
            out[c] = r.extended(c) if ext else r.cuboid(c)
    return out


@pytest.mark.parametrize("name", ["uniform-100k-6", "anticorr-1m-10", "ties-581k-10", "corrq-566k-15-m6"])
def test_batched_equals_plain(gpu_ctx, name):
    kind, n, d, m, seed = datagen.CONFIGS[name]
    x = datagen.generate(kind, n, d, seed)
    ds = sk.Dataset(gpu_ctx, x)
    a = sk.skycube(gpu_ctx, ds, "sdsc", "batched", max_d=m, want_extended=True)
    b = sk.skycube(gpu_ctx, ds, "sdsc", "plain", max_d=m, want_extended=True)
    sa, sb = all_sets(a, d, m), all_sets(b, d, m)
    ea, eb = all_sets(a, d, m, True), all_sets(b, d, m, True)
    cand = a.info()["n_candidates"]
    full = (1 << d) - 1
    assert len(sa[full]) + len(ea[full]) == cand
    for c in sa:
        assert np.array_equal(sa[c], sb[c]), f"skyline of cuboid {c}"
        assert np.array_equal(ea[c], eb[c]), f"extended skyline of cuboid {c}"
        assert len(sa[c]) > 0
        assert len(np.intersect1d(sa[c], ea[c])) == 0
    assert a.info()["total_skyline_ids"] == sum(len(v) for v in sa.values())


@pytest.mark.parametrize("name", ["uniform-100k-6", "ties-581k-10"])
def test_against_oracle_full_size(gpu_ctx, name):
    kind, n, d, m, seed = datagen.CONFIGS[name]
    x = datagen.generate(kind, n, d, seed)
    sky, ext = oracle.stsc(x, m)
    ds = sk.Dataset(gpu_ctx, x)
    r = sk.skycube(gpu_ctx, ds, "sdsc", "batched", max_d=m, want_extended=True)
    for c in sky:
        assert np.array_equal(r.cuboid(c), sky[c]), f"skyline of cuboid {c}"
        assert np.array_equal(r.extended(c), ext[c]), f"extended skyline of cuboid {c}"


def test_full_space_always_present_under_cap(gpu_ctx):
    x = datagen.generate("correlated_q", 20000, 9, 3)
    sky, ext = oracle.stsc(x, 2)
    ds = sk.Dataset(gpu_ctx, x)
    for algo, mode in (("mdmc", "batched"), ("sdsc", "plain")):
        r = sk.skycube(gpu_ctx, ds, algo, mode, max_d=2)
        assert np.array_equal(r.cuboid(511), sky[511])
        assert len(r.cuboid(0b111)) == 0


DIGESTS = ["uniform-100k-6", "anticorr-1m-10", "ties-581k-10", "corrq-566k-15-m6",
           "corrq-100k-15-m6"]
# Stand-ins of the reference's published capped sweeps (500k x 16, -m 4):
# the two batched forms only (the per-cuboid form would take minutes on
# their 2,516 cuboids).
SWEEP_DIGESTS = ["sweep-anticorr-500k-16-m4", "sweep-corr-500k-16-m4"]


def check_digest(gpu_ctx, name, form):
    dg = load_digest(name)
    if dg is None:
        pytest.skip(f"no reference digest for {name}")
    kind, n, d, m, seed = str(dg["kind"]), int(dg["n"]), int(dg["d"]), int(dg["max_d"]), int(dg["seed"])
    x = datagen.generate(kind, n, d, seed)
    assert points_hash(x) == int(dg["points_hash"]), "the generator gives other points than the digest's"
    algo, mode = form.split("/")
    ext = algo == "sdsc"
    ds = sk.Dataset(gpu_ctx, x)
    r = sk.skycube(gpu_ctx, ds, algo, mode, max_d=m, want_extended=ext)
    r.download()
    bad = []
    for i, c in enumerate(dg["cuboids"].tolist()):
        s_ = r.cuboid(c)
        if len(s_) != int(dg["sky_count"][i]) or id_hash(s_) != int(dg["sky_hash"][i]):
            bad.append(("skyline", c, len(s_), int(dg["sky_count"][i])))
        if ext:
            e_ = r.extended(c)
            if len(e_) != int(dg["ext_count"][i]) or id_hash(e_) != int(dg["ext_hash"][i]):
                bad.append(("extended", c, len(e_), int(dg["ext_count"][i])))
    assert not bad, f"{len(bad)} cuboids differ from the reference, first: {bad[:5]}"
    assert r.info()["total_skyline_ids"] == int(dg["sky_count"].sum())
    r.close()
    ds.close()


@pytest.mark.parametrize("form", ["mdmc/batched", "sdsc/batched", "sdsc/plain"])
@pytest.mark.parametrize("name", DIGESTS)
def test_full_size_digest(gpu_ctx, name, form):
    check_digest(gpu_ctx, name, form)


@pytest.mark.parametrize("form", ["mdmc/batched", "sdsc/batched"])
@pytest.mark.parametrize("name", SWEEP_DIGESTS)
def test_sweep_digest(gpu_ctx, name, form):
    check_digest(gpu_ctx, name, form)
