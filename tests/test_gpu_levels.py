"""The level form of capped skycubes (max_d <= 4): every wanted cuboid in
one persistent lattice launch whose device queue runs the levels top down,
each cuboid from its smallest computed parent; several datasets share one
launch through skc_skycube_batch. Checked against the C oracle on seeded inputs (the form forced,
each case asserting that it ran), on a tie-heavy input whose one-attribute skylines
exceed the kernel's window (so the per-cuboid fallback runs), and against
the bitmap form at sizes the oracle would take minutes on. Exact id-set
equality per cuboid, skylines and extended skylines."""
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


def check(gpu_ctx, x, max_d, algos=("mdmc", "sdsc")):
    d = x.shape[1]
    sky, ext = oracle.stsc(x, max_d)
    ds = sk.Dataset(gpu_ctx, x)
    fallbacks = []
    for algo in algos:
        r = sk.skycube(gpu_ctx, ds, algo, "batched", max_d=max_d, want_extended=True,
                       form="levels")
        form, fb = r.form()
        assert form == "levels", form
        fallbacks.append(fb)
        got, gext = sets(r, d, max_d), sets(r, d, max_d, True)
        for c in sky:
            assert np.array_equal(got[c], sky[c]), f"{algo} skyline of cuboid {c}"
            assert np.array_equal(gext[c], ext[c]), f"{algo} extended skyline of cuboid {c}"
        r.close()
    ds.close()
    return fallbacks


@pytest.mark.parametrize("kind,n,d,max_d,seed", [
    ("anticorrelated", 12000, 6, 4, 3), ("anticorrelated", 12000, 8, 3, 3),
    ("anticorrelated", 8000, 12, 4, 3), ("uniform", 20000, 10, 2, 3),
    ("uniform", 20000, 14, 4, 3), ("anticorrelated", 6000, 16, 4, 3),
    ("uniform", 20000, 10, 1, 4),
])
def test_levels_against_oracle(gpu_ctx, kind, n, d, max_d, seed):
    check(gpu_ctx, datagen.generate(kind, n, d, seed), max_d)


def test_levels_ties_and_fallback(gpu_ctx):
    # Three values per attribute: about a third of the points share the
    # minimum of each attribute, more than a level kernel's skyline window.
    rng = np.random.default_rng(5)
    x = np.floor(rng.random((12000, 6)) * 3).astype(np.float32)
    fb = check(gpu_ctx, x, 2)
    assert min(fb) >= 1


def test_levels_give_up_to_bitmaps(gpu_ctx):
    # Two values per attribute: every 2-attribute skyline holds about a
    # quarter of the points, over the window on every top-level cuboid, so
    # the level form hands over and the bitmap form computes the result.
    rng = np.random.default_rng(7)
    x = np.floor(rng.random((20000, 8)) * 2).astype(np.float32)
    d, m = 8, 2
    sky, ext = oracle.stsc(x, m)
    ds = sk.Dataset(gpu_ctx, x)
    r = sk.skycube(gpu_ctx, ds, max_d=m, want_extended=True, form="levels")
    assert r.form()[0] == "bitmaps"
    got, gext = sets(r, d, m), sets(r, d, m, True)
    for c in sky:
        assert np.array_equal(got[c], sky[c]), f"skyline of cuboid {c}"
        assert np.array_equal(gext[c], ext[c]), f"extended skyline of cuboid {c}"
    r.close()
    ds.close()


def test_levels_duplicates_and_signed_zero(gpu_ctx):
    base = datagen.generate("anticorrelated", 5000, 7, 6)
    x = np.concatenate([base, base])
    x[:40, 2] = -0.0
    x[5000:5040, 2] = 0.0
    check(gpu_ctx, x, 3)


def auto_form(d, max_d, candidates):
    """The form skc_skycube picks for a batched capped skycube (the rule of
    api.cu's use_levels): the level form from 65,536 candidates when the
    cap is under 4, at 16 attributes, or at 14-15 attributes from 600,000
    candidates."""
    if candidates < 65536:
        return "bitmaps"
    lv = max_d <= 3 or d >= 16 or (d >= 14 and candidates >= 600000)
    return "levels" if lv else "bitmaps"


@pytest.mark.parametrize("kind,n,d,max_d,seed", [
    ("anticorrelated", 500000, 16, 4, 1), ("uniform", 300000, 14, 3, 2),
    ("anticorrelated", 400000, 10, 4, 93), ("correlated", 500000, 16, 4, 1),
])
def test_levels_equal_bitmap_form(gpu_ctx, kind, n, d, max_d, seed):
    x = datagen.generate(kind, n, d, seed)
    ds = sk.Dataset(gpu_ctx, x)
    a = sk.skycube(gpu_ctx, ds, max_d=max_d, want_extended=True, form="levels")
    b = sk.skycube(gpu_ctx, ds, max_d=max_d, want_extended=True, form="bitmaps")
    c = sk.skycube(gpu_ctx, ds, max_d=max_d, want_extended=True)
    assert b.form()[0] == "bitmaps"
    cand = b.info()["n_candidates"]
    if cand >= 65536:
        assert a.form()[0] == "levels"
    assert c.form()[0] == auto_form(d, max_d, cand)
    for ext in (False, True):
        sa, sb = sets(a, d, max_d, ext), sets(b, d, max_d, ext)
        for cub in sa:
            assert np.array_equal(sa[cub], sb[cub]), f"cuboid {cub} (extended={ext})"
    assert a.info()["total_skyline_ids"] == b.info()["total_skyline_ids"]
    assert c.info()["total_skyline_ids"] == b.info()["total_skyline_ids"]
    for r in (a, b, c):
        r.close()
    ds.close()


def test_batch_of_datasets_equals_each_alone(gpu_ctx):
    """skc_skycube_batch: three capped skycubes in one lattice launch (one of
    them tie-heavy enough to use the per-cuboid fallback), a full skycube in
    the bitmap form and a skyline query, each equal to its own skc_skycube
    and the capped ones to the oracle."""
    rng = np.random.default_rng(9)
    cases = [
        (datagen.generate("anticorrelated", 9000, 7, 21), dict(max_d=3, want_extended=True)),
        (datagen.generate("uniform", 15000, 12, 22), dict(algo="sdsc", max_d=4, want_extended=True)),
        (np.floor(rng.random((8000, 6)) * 3).astype(np.float32), dict(max_d=2, want_extended=True)),
        (datagen.generate("correlated", 20000, 8, 23), dict(want_extended=True)),
        (datagen.generate("ties", 10000, 9, 24), dict(subspace=0b101100111, want_extended=True)),
    ]
    dss = [sk.Dataset(gpu_ctx, x) for x, _ in cases]
    for o in (dict(form="levels"), {}):
        opts = [{**o, **c} if c.get("max_d", 99) <= 4 else c for _, c in cases]
        batch = sk.skycube_batch(gpu_ctx, dss, opts)
        forms = [r.form()[0] for r in batch]
        if o:
            assert forms[:3] == ["levels"] * 3, forms
        for (x, c), ds, o2, rb in zip(cases, dss, opts, batch):
            ra = sk.skycube(gpu_ctx, ds, **o2)
            d = x.shape[1]
            md = c.get("max_d", 0) or d
            if c.get("subspace"):
                S = c["subspace"]
                assert np.array_equal(rb.cuboid(S), ra.cuboid(S))
                assert np.array_equal(rb.extended(S), ra.extended(S))
            else:
                for cub in range(1, 1 << d):
                    if bin(cub).count("1") <= md or cub == (1 << d) - 1:
                        assert np.array_equal(rb.cuboid(cub), ra.cuboid(cub)), (c, cub)
                        assert np.array_equal(rb.extended(cub), ra.extended(cub)), (c, cub)
            ra.close()
        for (x, c), rb in zip(cases[:3], batch[:3]):
            sky, ext = oracle.stsc(x, c["max_d"])
            for cub in sky:
                assert np.array_equal(rb.cuboid(cub), sky[cub]) and np.array_equal(rb.extended(cub), ext[cub])
        for r in batch:
            r.close()
    for ds in dss:
        ds.close()


def test_lattice_wait_runs_out_cleanly(gpu_ctx, monkeypatch):
    """A lattice-phase wait that can never end (injected on the host: the
    first phase counts one item more than exists) runs out after its bound
    (about 2 s) and comes back as SKC_ERR_TIMEOUT; the context stays
    usable."""
    x = datagen.generate("uniform", 20000, 8, 31)
    ds = sk.Dataset(gpu_ctx, x)
    monkeypatch.setenv("SKC_FAULT_LATTICE_WAIT", "1")
    with pytest.raises(sk.SkycubeError) as e:
        sk.skycube(gpu_ctx, ds, max_d=3, form="levels")
    assert e.value.code == 4 and "wait ran out" in str(e.value)
    monkeypatch.delenv("SKC_FAULT_LATTICE_WAIT")
    r = sk.skycube(gpu_ctx, ds, max_d=3, form="levels", want_extended=True)
    sky, ext = oracle.stsc(x, 3)
    for c in sky:
        assert np.array_equal(r.cuboid(c), sky[c]) and np.array_equal(r.extended(c), ext[c])
    r.close()
    ds.close()
