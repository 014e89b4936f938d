"""Capped skycubes (max_d below d - 1): the bitmap kernel then skips q's
that can only dominate on subspaces above the cap and takes the full-space
bits from the candidates' known full-space status. Checked against the C
oracle on seeded inputs for every bitmap storage form (registers d <= 10,
shared memory d = 11, 12, global tie slab d >= 13), and against the full
computation (per-point bitmaps requested, which disables the cap inside the
kernel) at sizes the oracle would take minutes on. Exact id-set equality."""
import numpy as np
import pytest

import oracle
import skycube_gb300 as sk
from skycube_gb300 import datagen

pytestmark = pytest.mark.gpu


def sets(r, d, max_d, ext=False):
    out = {}
    for c in range(1, 1 << d):
        if bin(c).count("1") <= max_d or c == (1 << d) - 1:
            out[c] = r.extended(c) if ext else r.cuboid(c)
    return out


CASES = [
    ("uniform", 6000, 6, 1, 71), ("ties", 8000, 6, 4, 72), ("anticorrelated", 6000, 7, 3, 73),
    ("ties", 6000, 8, 2, 74), ("anticorrelated", 5000, 9, 4, 75), ("ties", 6000, 10, 3, 76),
    ("anticorrelated", 4000, 11, 4, 77), ("ties", 5000, 11, 2, 78), ("uniform", 4000, 12, 5, 79),
    ("ties", 4000, 12, 4, 80), ("anticorrelated", 3000, 13, 4, 81), ("ties", 3000, 14, 4, 82),
    ("uniform", 2500, 15, 3, 83), ("anticorrelated", 2500, 16, 4, 84), ("ties", 2000, 16, 1, 85),
]


@pytest.mark.parametrize("kind,n,d,max_d,seed", CASES)
def test_capped_against_oracle(gpu_ctx, kind, n, d, max_d, seed):
    x = datagen.generate(kind, n, d, seed)
    sky, ext = oracle.stsc(x, max_d)
    ds = sk.Dataset(gpu_ctx, x)
    for algo in ("mdmc", "sdsc"):
        r = sk.skycube(gpu_ctx, ds, algo, "batched", max_d=max_d, want_extended=True)
        got, gext = sets(r, d, max_d), sets(r, d, max_d, True)
        for c in sky:
            assert np.array_equal(got[c], sky[c]), f"{algo} skyline of cuboid {c}"
            assert np.array_equal(gext[c], ext[c]), f"{algo} extended skyline of cuboid {c}"
        r.close()
    ds.close()


@pytest.mark.parametrize("kind,n,d,max_d,seed", [
    ("anticorrelated", 200000, 14, 4, 91), ("uniform", 300000, 16, 4, 92),
    ("anticorrelated", 400000, 10, 4, 93), ("ties", 200000, 12, 3, 94),
])
def test_capped_equals_full_computation(gpu_ctx, kind, n, d, max_d, seed):
    x = datagen.generate(kind, n, d, seed)
    ds = sk.Dataset(gpu_ctx, x)
    a = sk.skycube(gpu_ctx, ds, max_d=max_d, want_extended=True)
    b = sk.skycube(gpu_ctx, ds, max_d=max_d, want_extended=True, want_bitmaps=True)
    sa, sb = sets(a, d, max_d), sets(b, d, max_d)
    ea, eb = sets(a, d, max_d, True), sets(b, d, max_d, True)
    full = (1 << d) - 1
    assert len(sa[full]) + len(ea[full]) == a.info()["n_candidates"]
    for c in sa:
        assert np.array_equal(sa[c], sb[c]), f"skyline of cuboid {c}"
        assert np.array_equal(ea[c], eb[c]), f"extended skyline of cuboid {c}"
    assert a.info()["total_skyline_ids"] == b.info()["total_skyline_ids"]
    a.close()
    b.close()
    ds.close()


def test_capped_plan_replay(gpu_ctx):
    d, m = 13, 3
    x = datagen.generate("anticorrelated", 20000, d, 95)
    sky, ext = oracle.stsc(x, m)
    ds = sk.Dataset(gpu_ctx, x)
    plan = sk.Plan(gpu_ctx, ds, max_d=m, want_extended=True)
    for _ in range(2):
        r = plan.execute()
        got, gext = sets(r, d, m), sets(r, d, m, True)
        for c in sky:
            assert np.array_equal(got[c], sky[c]), f"skyline of cuboid {c}"
            assert np.array_equal(gext[c], ext[c]), f"extended skyline of cuboid {c}"
        r.close()
    plan.close()
    ds.close()
