"""Seeded synthetic point sets with the shapes and value distributions of the
benchmark workloads of the skycube suite (its own data files are not shipped).

Every generator returns a C-contiguous float32 array of shape (n, d), rows are
points and smaller is better on every attribute. All randomness comes from
``numpy.random.default_rng(seed)`` so the same seed gives the same points.

Distributions:
  uniform         every coordinate iid U[0,1)
  anticorrelated  v ~ N(0.5, sigma); x_i ~ U[0,1); every coordinate shifted by
                  (d*v - sum x)/d; the point is redrawn if a coordinate leaves
                  [0,1]
  correlated      v ~ N(0.5, 0.25) clipped to [0,1]; x_i = clip(v + N(0,0.05))
  ties            60% uniform, 40% correlated points, then floor(256*u) stored
                  as float32 (integer valued, many duplicates)
  correlated_q    correlated, rounded to multiples of 0.1/d of the unit range
"""
import numpy as np

KINDS = ("uniform", "anticorrelated", "correlated", "ties", "correlated_q")


def _uniform(rng, n, d):
    return rng.random((n, d), dtype=np.float64)


def _anticorrelated(rng, n, d, sigma=0.05):
    out = np.empty((n, d), dtype=np.float64)
    filled = 0
    while filled < n:
        m = max(1024, int((n - filled) * 1.3))
        v = rng.normal(0.5, sigma, size=(m, 1))
        x = rng.random((m, d))
        x += (d * v - x.sum(axis=1, keepdims=True)) / d
        ok = np.all((x >= 0.0) & (x <= 1.0), axis=1)
        x = x[ok]
        take = min(len(x), n - filled)
        out[filled:filled + take] = x[:take]
        filled += take
    return out


def _correlated(rng, n, d):
    v = np.clip(rng.normal(0.5, 0.25, size=(n, 1)), 0.0, 1.0)
    return np.clip(v + rng.normal(0.0, 0.05, size=(n, d)), 0.0, 1.0)


def generate(kind, n, d, seed=1):
    """Returns an (n, d) float32 point set of the given distribution."""
    if kind not in KINDS:
        raise ValueError(f"unknown distribution {kind!r}; expected one of {KINDS}")
    rng = np.random.default_rng(seed)
    if kind == "uniform":
        x = _uniform(rng, n, d)
    elif kind == "anticorrelated":
        x = _anticorrelated(rng, n, d)
    elif kind == "correlated":
        x = _correlated(rng, n, d)
    elif kind == "ties":
        n_corr = (n * 4) // 10
        u = _uniform(rng, n - n_corr, d)
        c = _correlated(rng, n_corr, d)
        x = np.concatenate([u, c], axis=0)
        x = x[rng.permutation(n)]
        x = np.floor(256.0 * x)
    else:  # correlated_q
        step = 0.1 / d
        x = np.round(_correlated(rng, n, d) / step) * step
    return np.ascontiguousarray(x, dtype=np.float32)


# The five benchmark workloads: (distribution, n, d, max_d, seed).
CONFIGS = {
    "uniform-100k-6": ("uniform", 100_000, 6, 6, 1),
    "anticorr-1m-10": ("anticorrelated", 1_000_000, 10, 10, 1),
    "ties-581k-10": ("ties", 581_012, 10, 10, 42),
    "corrq-566k-15-m6": ("correlated_q", 566_268, 15, 6, 42),
}


def serving_stream(count=2000, rate_qps=20.0, seed=7, n_min=1_000, n_max=1_000_000,
                   full_skycube_max_dims=10, cap_range=(2, 6)):
    """Queries of the serving workload, in arrival order.

    Each query has its own seeded dataset: n log-uniform in [n_min, n_max],
    d uniform in {4..16}, distribution uniform over uniform (independent),
    correlated and anticorrelated. Half are skycube queries, half skyline
    queries on one random subspace of at least two attributes. A skycube
    query computes every cuboid when d <= full_skycube_max_dims, else every
    cuboid of at most max_d attributes with max_d drawn uniformly from
    cap_range (a whole 16-d skycube of a million points has tens of
    billions of ids). Arrivals are Poisson with the given rate
    (exponential gaps). Returns a list of dicts with keys arrival_s, kind,
    n, d, seed, max_d, subspace.
    """
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    kinds = ("uniform", "correlated", "anticorrelated")
    for i in range(count):
        t += rng.exponential(1.0 / rate_qps)
        n = int(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        d = int(rng.integers(4, 17))
        kind = kinds[int(rng.integers(0, 3))]
        if rng.random() < 0.5:
            cap = int(rng.integers(cap_range[0], cap_range[1] + 1))
            q = {"max_d": d if d <= full_skycube_max_dims else cap, "subspace": 0}
        else:
            while True:
                sub = int(rng.integers(1, 1 << d))
                if bin(sub).count("1") >= 2:
                    break
            q = {"max_d": 0, "subspace": sub}
        out.append({"arrival_s": t, "kind": kind, "n": n, "d": d, "seed": 10_000 + i, **q})
    return out


class ServingPools:
    """Datasets of the serving stream, drawn without generating each one
    whole: for every (distribution, d) one pool of `pool_n` seeded points is
    generated once, and a query's dataset is the window of n consecutive
    pool rows at an offset drawn from the query's own seed. Points of a pool
    are independent draws of the distribution, so every window is a sample
    of it of size n. dataset(q) returns a read-only view (no copy)."""

    def __init__(self, pool_n=1_000_000, seed=4242):
        self.pool_n = pool_n
        self.seed = seed
        self.pools = {}

    def pool(self, kind, d):
        key = (kind, d)
        if key not in self.pools:
            self.pools[key] = generate(kind, self.pool_n, d, self.seed + 97 * d + KINDS.index(kind))
        return self.pools[key]

    def dataset(self, q):
        p = self.pool(q["kind"], q["d"])
        n = min(q["n"], self.pool_n)
        off = int(np.random.default_rng(q["seed"]).integers(0, self.pool_n - n + 1))
        return p[off:off + n]
