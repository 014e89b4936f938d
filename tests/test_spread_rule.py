"""The rule that orders the skyline kernel's partitions (partition.cu,
gray_order): the Gray order with tile boxes when the points' cell sums are
concentrated, below 0.8 of the spread of a sum of independent uniform
cells, else the strength order. It was measured on the benchmark's
workloads; this pins their classification on the CPU with quantile cells
(128 per attribute, as the device's 7-bit grid), so that a change of a data
generator that moves a workload across the limit shows here."""
import numpy as np
import pytest

from skycube_gb300 import datagen

LIMIT = 0.8  # kGraySpread


def spread_ratio(x, depth=7):
    n, d = x.shape
    c = 1 << depth
    cells = np.empty((n, d), dtype=np.int64)
    for k in range(d):
        rank = np.empty(n, dtype=np.int64)
        rank[np.argsort(x[:, k], kind="stable")] = np.arange(n)
        cells[:, k] = (rank * c) // n
    s = cells.sum(axis=1).astype(np.float64)
    independent = np.sqrt(d * (c * c - 1) / 12.0)
    return s.std() / independent


@pytest.mark.parametrize("kind,d,gray", [
    ("anticorrelated", 10, True), ("anticorrelated", 12, True), ("anticorrelated", 16, True),
    ("anticorrelated", 8, True), ("uniform", 10, False), ("uniform", 16, False),
    ("correlated", 10, False), ("correlated_q", 15, False), ("ties", 10, False),
])
def test_spread_rule_classifies_the_benchmark_workloads(kind, d, gray):
    x = datagen.generate(kind, 200_000, d, 1)
    r = spread_ratio(x)
    assert (r < LIMIT) == gray, (kind, d, r)
    # measured margins: anticorrelated 0.51-0.62, uniform 1.01, ties and
    # correlated 2.0-3.8
    assert abs(r - LIMIT) > 0.15, (kind, d, r)


def test_independent_attributes_have_ratio_one():
    rng = np.random.default_rng(3)
    x = rng.random((100_000, 9), dtype=np.float32)
    assert abs(spread_ratio(x) - 1.0) < 0.02
