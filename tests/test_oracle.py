"""The CPU oracle pinned against the reference: golden fixtures produced by
the reference's own STSC, definition-level brute force, and (where the
reference was built in this checkout) a live comparison."""
import numpy as np
import pytest

import oracle
from conftest import golden_names, id_hash, load_digest, load_golden, points_hash, wanted
from skycube_gb300 import datagen


@pytest.mark.parametrize("name", golden_names())
def test_oracle_matches_reference_golden(name):
    x, max_d, sky, ext = load_golden(name)
    d = x.shape[1]
    osky, oext = oracle.stsc(x, max_d)
    for c in range(1, 1 << d):
        if not wanted(c, d, max_d):
            continue
        assert np.array_equal(osky[c], sky[c]), f"skyline of cuboid {c}"
        assert np.array_equal(oext[c], ext[c]), f"extended skyline of cuboid {c}"


def _random_points(rng, n, d, levels):
    if levels:
        return np.floor(rng.random((n, d)) * levels).astype(np.float32)
    return rng.random((n, d), dtype=np.float64).astype(np.float32)


@pytest.mark.parametrize("seed", range(12))
def test_oracle_matches_bruteforce(seed):
    rng = np.random.default_rng(1000 + seed)
    d = int(rng.integers(2, 7))
    n = int(rng.integers(1, 70))
    levels = [0, 2, 3, 8][seed % 4]
    x = _random_points(rng, n, d, levels)
    bits = oracle.bruteforce_bitmaps(x)
    truth = oracle.skylines_from_bitmaps(bits, d)
    sky, _ = oracle.stsc(x)
    for c in range(1, 1 << d):
        assert np.array_equal(sky[c], truth[c]), f"cuboid {c}"


def test_bruteforce_definition_tiny():
    # q=(0,1) vs p=(0,2): q dominates p on {1} and {0,1}, not on {0} (tie).
    x = np.array([[0.0, 2.0], [0.0, 1.0]], dtype=np.float32)
    bits = oracle.bruteforce_bitmaps(x)
    assert bits[0, 0] == (1 << 2) | (1 << 3)
    assert bits[1, 0] == 0


@pytest.mark.skipif(not oracle.ref_available(), reason="reference STSC not built here")
@pytest.mark.parametrize("kind,n,d,max_d,seed", [
    ("uniform", 5000, 7, 7, 11), ("ties", 6000, 9, 9, 12), ("correlated_q", 4000, 13, 3, 13),
    ("anticorrelated", 4000, 6, 6, 14), ("correlated", 3000, 11, 11, 15),
    ("anticorrelated", 3000, 16, 3, 16), ("uniform", 4000, 14, 4, 17), ("ties", 5000, 12, 5, 18),
    ("anticorrelated", 2500, 10, 10, 19),
])
def test_oracle_matches_reference_live(kind, n, d, max_d, seed):
    x = datagen.generate(kind, n, d, seed)
    a = oracle.ref_stsc(x, max_d)
    b = oracle.stsc(x, max_d)
    for c in a[0]:
        assert np.array_equal(a[0][c], b[0][c])
        assert np.array_equal(a[1][c], b[1][c])


@pytest.mark.parametrize("kind,seed,K", [("ties", 41, 4), ("uniform", 42, 16), ("correlated_q", 43, 1),
                                          ("anticorrelated", 44, 64)])
def test_prefilter_keeps_full_space_statuses(kind, seed, K):
    """The exactness argument of the pruner prefilter, on the CPU: dropping
    every point that one of K pruners strictly dominates leaves the
    full-space skyline and extended skyline unchanged (the survivors'
    statuses over the survivors equal their statuses over all points)."""
    x = datagen.generate(kind, 3000, 6, seed)
    pruners = x[np.argsort(x.sum(1), kind="stable")[:K]]
    dropped = np.zeros(len(x), bool)
    for t in pruners:
        dropped |= np.all(t < x, axis=1)
    assert dropped.any()
    keep = np.nonzero(~dropped)[0].astype(np.uint32)
    full = (1 << 6) - 1
    sky, ext = oracle.stsc(x)
    fsky, fext = oracle.stsc(x[keep])
    assert np.array_equal(keep[fsky[full]], sky[full])
    assert np.array_equal(keep[fext[full]], ext[full])


@pytest.mark.skipif(not (oracle.ref_available() and oracle.ref_available(shim=True)),
                    reason="the AVX and portable builds of the reference STSC are not both built here")
@pytest.mark.parametrize("case", golden_names() + ["gen:ties:7000:10:4", "gen:anticorrelated:5000:8:8",
                                                   "gen:correlated_q:3000:15:5", "gen:uniform:2500:16:3"])
def test_reference_portable_build_matches_avx_build(case):
    """The reference STSC built with the portable intrinsics of
    oracle/ref_shim (as on the aarch64 GPU hosts) gives the same skyline and
    extended skyline of every cuboid as its AVX2 build, on every golden input
    and on larger seeded ones (ties, d = 15 and 16 included)."""
    if case.startswith("gen:"):
        _, kind, n, d, max_d = case.split(":")
        x = datagen.generate(kind, int(n), int(d), 77)
        max_d = int(max_d)
    else:
        x, max_d, _, _ = load_golden(case)
    a = oracle.ref_stsc(x, max_d)
    b = oracle.ref_stsc(x, max_d, shim=True)
    assert a[0].keys() == b[0].keys()
    for c in a[0]:
        assert np.array_equal(a[0][c], b[0][c]), f"skyline of cuboid {c}"
        assert np.array_equal(a[1][c], b[1][c]), f"extended skyline of cuboid {c}"


@pytest.mark.skipif(not oracle.ref_pq_available(), reason="the reference's PQSkycube is not built here")
@pytest.mark.parametrize("case", golden_names() + ["gen:ties:20000:8:8", "gen:anticorrelated:5000:10:10",
                                                   "gen:correlated_q:20000:14:4", "gen:uniform:5000:16:3",
                                                   "gen:correlated:8000:12:12"])
def test_reference_pqskycube_agrees(case):
    """The reference's second skycube algorithm, PQSkycube (sky-tree based,
    src/qskycube/QSkycubeG.h:223-303), gives the same skyline on every
    cuboid as the golden fixtures (the reference's STSC) and the C oracle:
    two independent algorithms of the suite behind one set of answers."""
    if case.startswith("gen:"):
        _, kind, n, d, max_d = case.split(":")
        x = datagen.generate(kind, int(n), int(d), 31)
        max_d = int(max_d)
        want = oracle.stsc(x, max_d)[0]
    else:
        x, max_d, want, _ = load_golden(case)
    d = x.shape[1]
    got = oracle.ref_pq(x, max_d)[0]
    osky = oracle.stsc(x, max_d)[0]
    for c in range(1, 1 << d):
        if not wanted(c, d, max_d):
            continue
        assert np.array_equal(got[c], want[c]), f"skyline of cuboid {c}"
        assert np.array_equal(osky[c], want[c]), f"oracle skyline of cuboid {c}"


@pytest.mark.skipif(not oracle.ref_pq_available(), reason="the reference's PQSkycube is not built here")
@pytest.mark.parametrize("name", ["uniform-100k-6", "ties-581k-10", "corrq-100k-15-m6",
                                  "corrq-566k-15-m6", "sweep-corr-500k-16-m4"])
def test_full_size_digest_matches_reference_pqskycube(name):
    """The full-size digests (made by the reference's STSC, the ones the GPU
    forms are tested against) agree with the reference's PQSkycube on the
    skyline of every cuboid: two independent reference algorithms at full
    size. These workloads take PQSkycube under a second; the 1M x 10
    anticorrelated and 500k x 16 anticorrelated -m 4 digests agree too
    (make_golden.py --crosscheck-pq, minutes each)."""
    dg = load_digest(name)
    if dg is None:
        pytest.skip(f"no digest for {name}")
    kind, n, d, m, seed = str(dg["kind"]), int(dg["n"]), int(dg["d"]), int(dg["max_d"]), int(dg["seed"])
    x = datagen.generate(kind, n, d, seed)
    assert points_hash(x) == int(dg["points_hash"])
    sky = oracle.ref_pq(x, m)[0]
    bad = [c for i, c in enumerate(dg["cuboids"].tolist())
           if len(sky[c]) != int(dg["sky_count"][i]) or id_hash(sky[c]) != int(dg["sky_hash"][i])]
    assert not bad, f"{len(bad)} cuboids differ, first: {bad[:5]}"
