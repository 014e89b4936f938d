"""The skyline kernel's algorithm (partition.cu, k_skyline_part) restated in
Python and checked against brute-force statuses: points grouped by median
mask over B attributes, partitions processed in lattice-rank order, each
point scanning only the partitions under its mask, in 32-q tiles skipped
when the tile's minimum cells lie above the point's cell on some attribute,
and a finished partition read through its confirmed list (its points that
are not strictly dominated) instead of all its points. Which earlier
partitions count as finished is drawn at random, as the launch's timing
decides it on the device. Statuses: 0 skyline, 1 dominated but not strictly
(extended skyline), 2 strictly dominated. CPU only."""
import numpy as np
import pytest

from skycube_gb300 import datagen


def brute_status(x):
    n = len(x)
    st = np.zeros(n, dtype=np.int64)
    for p in range(n):
        le = np.all(x <= x[p], axis=1)
        lt = np.any(x < x[p], axis=1)
        strict = np.all(x < x[p], axis=1)
        if strict.any():
            st[p] = 2
        elif (le & lt).any():
            st[p] = 1
    return st


def model_status(x, depth, B, seed, tile=32):
    rng = np.random.default_rng(seed)
    n, d = x.shape
    P = (1 << depth) - 1
    cells = np.empty((n, d), dtype=np.int64)
    for k in range(d):
        s = np.sort(x[:, k])
        piv = s[[((r + 1) * n) // (P + 1) for r in range(P)]]
        cells[:, k] = np.searchsorted(piv, x[:, k], side="left")
    sh = depth - 1
    med = ((cells[:, :B] >> sh) & 1) @ (1 << np.arange(B))
    order = sorted(range(1 << B), key=lambda m: bin(m).count("1"))  # rank -> mask
    members = {m: [int(i) for i in rng.permutation(np.nonzero(med == m)[0])] for m in order}
    status = np.zeros(n, dtype=np.int64)
    confirmed, finished = {}, set()
    for m in order:
        for p in members[m]:
            st = 0
            for qm in order:  # partitions under p's mask, in rank order
                if (qm & ~m) != 0:
                    continue
                use_conf = qm != m and qm in finished and rng.random() < 0.7
                lst = confirmed[qm] if use_conf else members[qm]
                for t0 in range(0, len(lst), tile):
                    tq = lst[t0:t0 + tile]
                    if np.any(cells[tq].min(axis=0) > cells[p]):
                        continue  # no q of the tile dominates p
                    for q in tq:
                        if q == p:
                            continue
                        a, b = x[q], x[p]
                        if np.all(a <= b) and np.any(a < b):
                            if np.all(a < b):
                                st = 2
                                break
                            st = 1
                    if st == 2:
                        break
                if st == 2:
                    break
            status[p] = st
        confirmed[m] = [p for p in members[m] if status[p] != 2]
        finished.add(m)
    return status


@pytest.mark.parametrize("kind,n,d,depth,B,seed", [
    ("anticorrelated", 1500, 5, 3, 5, 1), ("uniform", 2000, 4, 3, 4, 2),
    ("ties", 1500, 5, 2, 3, 3), ("correlated_q", 2000, 6, 3, 6, 4),
    ("anticorrelated", 1200, 7, 2, 4, 5),
])
def test_skyline_model_against_bruteforce(kind, n, d, depth, B, seed):
    x = datagen.generate(kind, n, d, seed)
    if kind == "anticorrelated" and seed == 5:
        x = np.round(x * 8) / 8  # exact ties: statuses 1 appear
    want = brute_status(x)
    for rep in range(2):
        got = model_status(x, depth, B, seed * 10 + rep)
        assert np.array_equal(got, want), np.nonzero(got != want)[0][:10]
    assert (want == 0).any() and (want == 2).any()
