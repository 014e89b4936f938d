"""Full-size parity on the benchmark workloads.

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
