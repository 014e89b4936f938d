import numpy as np
import pytest

from skycube_gb300 import datagen


@pytest.mark.parametrize("kind", datagen.KINDS)
def test_shapes_and_determinism(kind):
    a = datagen.generate(kind, 5000, 7, seed=3)
    b = datagen.generate(kind, 5000, 7, seed=3)
    assert a.shape == (5000, 7) and a.dtype == np.float32 and a.flags.c_contiguous
    assert np.array_equal(a, b)
    assert np.all(np.isfinite(a))


def test_anticorrelated_constraint():
    x = datagen.generate("anticorrelated", 20000, 10, seed=1).astype(np.float64)
    assert x.min() >= 0.0 and x.max() <= 1.0
    s = x.sum(axis=1) / 10
    assert abs(s.mean() - 0.5) < 0.01 and 0.03 < s.std() < 0.07


def test_ties_are_integer_valued():
    x = datagen.generate("ties", 20000, 10, seed=42)
    assert np.array_equal(x, np.floor(x)) and x.min() >= 0 and x.max() <= 256
    assert len(np.unique(x[:, 0])) <= 257


def test_correlated_q_quantised():
    d = 15
    x = datagen.generate("correlated_q", 20000, d, seed=42).astype(np.float64)
    step = 0.1 / d
    assert np.allclose(np.round(x / step) * step, x, atol=1e-6)


def test_unknown_kind():
    with pytest.raises(ValueError):
        datagen.generate("nope", 10, 3)


def test_serving_stream_shape():
    qs = datagen.serving_stream(count=400, rate_qps=20.0, seed=7)
    assert len(qs) == 400
    t = [q["arrival_s"] for q in qs]
    assert all(b > a for a, b in zip(t, t[1:]))
    assert 10 < t[-1] < 40  # Poisson at 20/s
    for q in qs:
        assert 1000 <= q["n"] <= 1_000_000 and 4 <= q["d"] <= 16
        if q["subspace"]:
            assert q["max_d"] == 0 and bin(q["subspace"]).count("1") >= 2
            assert q["subspace"] < (1 << q["d"])
        elif q["d"] <= 10:
            assert q["max_d"] == q["d"]
        else:
            assert 2 <= q["max_d"] <= 6
    caps = {q["max_d"] for q in qs if not q["subspace"] and q["d"] > 10}
    assert caps == {2, 3, 4, 5, 6}


def test_serving_pools_windows():
    pools = datagen.ServingPools(pool_n=50_000)
    q = {"kind": "anticorrelated", "d": 6, "n": 1234, "seed": 10_001}
    a, b = pools.dataset(q), pools.dataset(q)
    assert a.shape == (1234, 6) and a.flags.c_contiguous and np.array_equal(a, b)
    other = pools.dataset({**q, "seed": 10_002})
    assert not np.array_equal(a, other)
