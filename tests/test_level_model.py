"""The level form's algorithm (levels.cu) restated in Python and checked
against the C oracle on small tie-heavy inputs, with capacities small
enough that every case the kernels rely on occurs: pruners that drop
entries, sort-filter batches that end on cell-sum bucket boundaries or
split a bucket, entries of equal cell sum dominating each other across
batches (settled by the equal-cell pass), and cuboids computed from a
parent's skyline + extended skyline. CPU only."""
import numpy as np
import pytest

import oracle
from skycube_gb300 import datagen


def dom(x, q, p, S):
    """0: q does not dominate p on S, 1: dominates, 2: strictly."""
    a, b = x[q, S], x[p, S]
    if np.any(a > b):
        return 0
    if np.all(a < b):
        return 2
    return 1 if np.any(a < b) else 0


def cuboid(x, cells, S, lst, pruners=4, sample=16, batch=8):
    """Skyline and extended skyline of subspace S over the list `lst`, the
    way k_lv_pruners, k_lv_filter and k_lv_sfs compute them."""
    key = {p: int(cells[p, S].sum()) for p in lst}
    n = len(lst)
    ns = min(n, sample)
    samp = [lst[i * n // ns] for i in range(ns)]
    pr = sorted(samp, key=lambda p: key[p])[:pruners]
    surv = [p for p in lst if not any(dom(x, q, p, S) == 2 for q in pr)]
    surv.sort(key=lambda p: key[p])
    bounds = {i for i in range(len(surv) + 1) if i == 0 or i == len(surv) or key[surv[i]] != key[surv[i - 1]]}
    window, ext, st = [], [], {}
    base = 0
    while base < len(surv):
        target = base + batch
        if target >= len(surv):
            end = len(surv)
        else:
            cand = [b for b in bounds if base < b <= target]
            end = max(cand) if cand else target
        b_ents = []
        for p in surv[base:end]:
            s = 0
            for q in window:
                r = dom(x, q, p, S)
                if r == 2:
                    s = 2
                    break
                s = max(s, r)
            if s < 2:
                b_ents.append((p, s))
        new = []
        for p, s in b_ents:
            for q, _ in b_ents:
                if q == p or key[q] > key[p]:
                    continue
                r = dom(x, q, p, S)
                if r == 2:
                    s = 2
                    break
                s = max(s, r)
            new.append((p, s))
        for p, s in new:
            if s == 0:
                window.append(p)
            elif s == 1:
                ext.append(p)
        base = end
    for p in window:
        st[p] = 0
    for p in ext:
        st[p] = 1
    for p in window + ext:  # equal cells, any position in the bucket
        for q in surv:
            if q == p or key[q] != key[p] or not np.array_equal(cells[q, S], cells[p, S]):
                continue
            r = dom(x, q, p, S)
            if r == 2:
                st[p] = 2
                break
            st[p] = max(st[p], r)
    sky = sorted(p for p, s in st.items() if s == 0)
    ex = sorted(p for p, s in st.items() if s == 1)
    return sky, ex


def level_form(x, max_d, cell_levels=8, **kw):
    n, d = x.shape
    full = (1 << d) - 1
    # a monotone cell per attribute (equal values share a cell)
    cells = np.zeros(x.shape, dtype=np.int64)
    for k in range(d):
        order = np.argsort(x[:, k], kind="stable")
        v = x[order, k]
        first = np.searchsorted(v, v, side="left")  # rank of the first equal value
        cells[order, k] = first * cell_levels // n
    sky0, ext0 = oracle.stsc(x, max_d)
    res = {full: (list(sky0[full]), list(ext0[full]))}
    for lev in range(max_d, 0, -1):
        for c in range(1, full):
            if bin(c).count("1") != lev:
                continue
            src, best = full, None
            for j in range(d - 1, -1, -1):
                p = c | (1 << j)
                if c & (1 << j) or p == full or p not in res:
                    continue
                v = len(res[p][0]) + len(res[p][1])
                if best is None or v < best:
                    best, src = v, p
            lst = res[src][0] + res[src][1]
            S = [k for k in range(d) if c >> k & 1]
            res[c] = cuboid(x, cells, S, lst, **kw) if lst else ([], [])
    return res, sky0, ext0


@pytest.mark.parametrize("seed,n,d,levels,max_d", [
    (1, 160, 5, 3, 3), (2, 200, 6, 4, 2), (3, 150, 6, 0, 4), (4, 180, 5, 2, 3), (5, 120, 7, 5, 2),
])
def test_level_form_matches_oracle(seed, n, d, levels, max_d):
    rng = np.random.default_rng(seed)
    x = rng.random((n, d))
    if levels:
        x = np.floor(x * levels)
    x = x.astype(np.float32)
    res, sky, ext = level_form(x, max_d)
    for c in sky:
        got_sky, got_ext = res[c]
        assert np.array_equal(np.array(got_sky, dtype=np.uint32), sky[c]), f"skyline of cuboid {c}"
        assert np.array_equal(np.array(got_ext, dtype=np.uint32), ext[c]), f"extended skyline of cuboid {c}"


def test_level_form_coarse_cells():
    # Two cells per attribute: entries of equal cell sum differ in their
    # floats, so a later batch's entry can dominate an earlier one of the
    # same sum (the equal-cell pass settles it).
    x = np.random.default_rng(11).random((200, 5)).astype(np.float32)
    res, sky, ext = level_form(x, 3, cell_levels=2, pruners=2, batch=4)
    for c in sky:
        assert list(res[c][0]) == list(sky[c]), f"skyline of cuboid {c}"
        assert list(res[c][1]) == list(ext[c]), f"extended skyline of cuboid {c}"


def test_level_form_anticorrelated():
    x = datagen.generate("anticorrelated", 300, 6, 9)
    res, sky, ext = level_form(x, 3, pruners=2, batch=4)
    for c in sky:
        assert list(res[c][0]) == list(sky[c]), f"skyline of cuboid {c}"
        assert list(res[c][1]) == list(ext[c]), f"extended skyline of cuboid {c}"
