"""Plans: the batched skycube captured as one CUDA graph and replayed.
Every replay must equal the direct call (exact id sets, extended skylines
and bitmaps), follow in-place dataset updates (re-sizing itself when a
capacity overflows), and report its launches."""
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


def assert_same(a, b):
    assert a.keys() == b.keys()
    for c in a:
        assert np.array_equal(a[c], b[c]), f"cuboid {c}: {len(a[c])} vs {len(b[c])}"


CASES = [("ties", 30000, 8, 8, "mdmc"), ("anticorrelated", 20000, 6, 6, "sdsc"),
         ("correlated_q", 40000, 13, 4, "sdsc"), ("uniform", 3000, 4, 4, "mdmc"),
         ("ties", 5000, 16, 2, "mdmc")]


@pytest.mark.parametrize("kind,n,d,max_d,algo", CASES)
def test_plan_equals_direct(gpu_ctx, kind, n, d, max_d, algo):
    x = datagen.generate(kind, n, d, 61)
    ds = sk.Dataset(gpu_ctx, x)
    kw = dict(algo=algo, mode="batched", max_d=max_d, want_extended=True,
              want_bitmaps=(algo == "mdmc"))
    ref = sk.skycube(gpu_ctx, ds, **kw)
    plan = sk.Plan(gpu_ctx, ds, **kw)
    info = plan.info()
    assert info["kernels"] >= 10 and info["replans"] == 0
    assert info["cand_capacity"] >= ref.info()["n_candidates"]
    for _ in range(3):
        before = sk.kernel_launches()
        r = plan.execute()
        assert sk.kernel_launches() - before == info["kernels"]
        assert r.info() == ref.info()
        assert_same(sets(r, d, max_d), sets(ref, d, max_d))
        assert_same(sets(r, d, max_d, True), sets(ref, d, max_d, True))
        if algo == "mdmc":
            b1, p1 = r.bitmaps()
            b0, p0 = ref.bitmaps()
            assert np.array_equal(p1, p0) and np.array_equal(b1, b0)
        r.close()
    plan.close()


def test_plan_follows_dataset_updates(gpu_ctx):
    n, d = 20000, 6
    ds = sk.Dataset(gpu_ctx, datagen.generate("correlated", n, d, 1))
    plan = sk.Plan(gpu_ctx, ds, want_extended=True)
    cap0 = plan.info()["cand_capacity"]
    # Anticorrelated points have far more candidates: the plan re-sizes.
    for kind, seed in (("anticorrelated", 2), ("ties", 3), ("correlated", 4)):
        x = datagen.generate(kind, n, d, seed)
        ds.update(x)
        r = plan.execute()
        sky, ext = oracle.stsc(x)
        assert_same(sets(r, d, d), {c: sky[c] for c in range(1, 1 << d)})
        assert_same(sets(r, d, d, True), {c: ext[c] for c in range(1, 1 << d)})
    info = plan.info()
    assert info["replans"] >= 1 and info["cand_capacity"] > cap0
    plan.close()


def test_dataset_update_rejects_nonfinite(gpu_ctx):
    x = datagen.generate("uniform", 2000, 5, 7)
    ds = sk.Dataset(gpu_ctx, x)
    before = sets(sk.skycube(gpu_ctx, ds), 5, 5)
    bad = x.copy()
    bad[17, 3] = np.nan
    with pytest.raises(sk.SkycubeError):
        ds.update(bad)
    with pytest.raises(sk.SkycubeError):
        ds.update(x[:100])
    assert_same(sets(sk.skycube(gpu_ctx, ds), 5, 5), before)


def test_plan_rejects_other_forms_and_freed_datasets(gpu_ctx):
    ds = sk.Dataset(gpu_ctx, datagen.generate("uniform", 3000, 5, 8))
    with pytest.raises(sk.SkycubeError):
        sk.Plan(gpu_ctx, ds, mode="plain")
    with pytest.raises(sk.SkycubeError):
        sk.Plan(gpu_ctx, ds, subspace=0b11)
    plan = sk.Plan(gpu_ctx, ds)
    ds.close()
    with pytest.raises(sk.SkycubeError):
        plan.execute()
    plan.close()


def test_plan_full_size_capped_high_d(gpu_ctx):
    """566k x 15 correlated, cuboids of <= 6 attributes: graph replay equals
    the direct batched call."""
    kind, n, d, m, seed = datagen.CONFIGS["corrq-566k-15-m6"]
    x = datagen.generate(kind, n, d, seed)
    ds = sk.Dataset(gpu_ctx, x)
    ref = sk.skycube(gpu_ctx, ds, max_d=m)
    plan = sk.Plan(gpu_ctx, ds, max_d=m)
    r = plan.execute()
    assert r.info() == ref.info()
    assert_same(sets(r, d, m), sets(ref, d, m))
    plan.close()
