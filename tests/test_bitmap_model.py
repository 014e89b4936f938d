"""The bitmap kernel's algorithm (mdmc.cu, k_bitmaps) restated in Python and
checked against the C oracle on every cuboid: quantile grid cells, q's in
median-partition rank order (shuffled inside the partitions: the result
must not depend on the order), partitions selected 32 at a time, the blocks
of the selected partitions box-tested as one list, open blocks, 8-q
quarters and 4-q halves held in stacks until a full 32-lane step's worth
waits, walks with repeated lanes, STRICT updates in lane order and the tie
map with its superset closure. A coarse grid (8 cells per attribute) makes
equal cells, and so the exact float checks, frequent; quantised data makes
exact ties, and so the tie map, frequent. CPU only."""
import numpy as np
import pytest

import oracle
from skycube_gb300 import datagen

LANES = 32


def cells_of(x, depth):
    """cell(v) = number of pivots < v, pivots = 2^depth - 1 quantiles."""
    n, d = x.shape
    P = (1 << depth) - 1
    out = np.empty((n, d), dtype=np.int64)
    for k in range(d):
        s = np.sort(x[:, k])
        piv = s[[((r + 1) * n) // (P + 1) for r in range(P)]]
        out[:, k] = np.searchsorted(piv, x[:, k], side="left")
    return out


def level_order(B):
    """rank -> median mask: masks by popcount, ties by value (stable)."""
    return sorted(range(1 << B), key=lambda m: bin(m).count("1"))


class Model:
    def __init__(self, x, depth, B, seed):
        self.x = x
        n, d = x.shape
        self.d = d
        self.nsub = 1 << d
        self.full = self.nsub - 1
        self.cells = cells_of(x, depth)
        sky, ext = oracle.stsc(x, d)
        self.sky, self.ext = sky, ext
        self.cand = np.union1d(sky[self.full], ext[self.full])
        qs = list(sky[self.full])  # q's: the full-space skyline
        sh = depth - 1
        med = lambda i: sum((((self.cells[i, k] >> sh) & 1) << k) for k in range(B))
        unrank = level_order(B)
        rank = {m: r for r, m in enumerate(unrank)}
        rng = np.random.default_rng(seed)
        parts = [[] for _ in range(1 << B)]
        for q in qs:
            parts[rank[med(q)]].append(q)
        order, boff = [], [0]
        for p in parts:
            p = list(p)
            rng.shuffle(p)
            order += p
            boff.append(len(order))
        self.K, self.B, self.sh = 1 << B, B, sh
        self.unrank, self.boff = unrank, boff
        nq = len(order)
        padded = -(-nq // LANES) * LANES
        big = 1 << 20  # padding cells: above every real cell, never lower a minimum
        self.qid = np.array(order + [-1] * (padded - nq))
        self.qcell = np.full((padded, d), big, dtype=np.int64)
        self.qx = np.full((padded, d), np.inf, dtype=np.float32)
        if nq:
            self.qcell[:nq] = self.cells[order]
            self.qx[:nq] = x[order]
        self.bmin = self.qcell.reshape(-1, 32, d).min(axis=1)
        self.smin = self.qcell.reshape(-1, 8, d).min(axis=1)
        self.hmin = self.qcell.reshape(-1, 4, d).min(axis=1)
        self.subsets = [[s for s in range(self.nsub) if (s & ~m) == 0] for m in range(self.nsub)]

    def U(self, qcells, pc):  # attributes where q may be <= p
        le = qcells <= pc
        return (le * (1 << np.arange(self.d))).sum(axis=-1)

    def candidate(self, p):
        d, pc, px = self.d, self.cells[p], self.x[p]
        strict = np.zeros(self.nsub, dtype=bool)
        strict[0] = True
        A = np.zeros(self.nsub, dtype=np.int64)  # tie map: A[E] |= LT
        stats = dict(steps=0, skipped=0, float_checks=0, tie_writes=0, updates=0, sub_full=0,
                     sub_short=0, half_full=0, half_short=0, walk_full=0, walk_short=0,
                     walk_quarters=0)

        def test_q(qi):
            stats["steps"] += 1
            U = self.U(self.qcell[qi], pc)
            hit = strict[U]
            if hit.all():
                stats["skipped"] += 1
                return
            le = np.zeros(LANES, dtype=np.int64)
            lt = np.zeros(LANES, dtype=np.int64)
            for t in range(LANES):
                if hit[t]:
                    continue
                q = qi[t]
                for k in range(d):
                    if not (U[t] >> k) & 1:
                        continue
                    if self.qcell[q, k] < pc[k]:
                        le[t] |= 1 << k
                        lt[t] |= 1 << k
                    else:  # equal cells: the floats decide
                        stats["float_checks"] += 1
                        a, b = self.qx[q, k], px[k]
                        if a <= b:
                            le[t] |= 1 << k
                        if a < b:
                            lt[t] |= 1 << k
            t_lt, t_le = strict[lt].copy(), strict[le].copy()  # state at the step's start
            for t in range(LANES):
                if not hit[t] and le[t] != lt[t] and not t_le[t]:
                    stats["tie_writes"] += 1
                    A[le[t]] |= lt[t]
            for t in range(LANES):  # STRICT updates in lane order
                if hit[t] or t_lt[t]:
                    continue
                if strict[lt[t]]:
                    continue
                stats["updates"] += 1
                strict[self.subsets[lt[t]]] = True

        bq, wq, hq = [], [], []

        def walk(quarters, c):
            stats["walk_quarters" if quarters else ("walk_full" if c == 8 else "walk_short")] += 1
            st = wq if quarters else hq
            lg = 3 if quarters else 2
            top = st[len(st) - c:]
            del st[len(st) - c:]
            qi = np.array([(top[min(t >> lg, c - 1)] << lg) + (t & ((1 << lg) - 1)) for t in range(LANES)])
            test_q(qi)

        def half_step(c):
            stats["half_full" if c == 16 else "half_short"] += 1
            top = wq[len(wq) - c:]
            del wq[len(wq) - c:]
            for t in range(LANES):
                if (t >> 1) < c:
                    hid = top[t >> 1] * 2 + (t & 1)
                    if not strict[self.U(self.hmin[hid], pc)]:
                        hq.append(hid)
            while len(hq) >= 8:
                walk(False, 8)

        def sub_step(c):
            stats["sub_full" if c == 8 else "sub_short"] += 1
            top = bq[len(bq) - c:]
            del bq[len(bq) - c:]
            for t in range(LANES):
                if (t >> 2) < c:
                    sid = top[t >> 2] * 4 + (t & 3)
                    if not strict[self.U(self.smin[sid], pc)]:
                        wq.append(sid)
            while len(wq) >= 16:
                half_step(16)

        pmask = sum((((pc[k] >> self.sh) & 1) << k) for k in range(self.B))
        next_blk = 0
        for b0 in range(0, self.K, LANES):
            sel, rng_ = [], []
            for bl in range(b0, min(b0 + LANES, self.K)):
                qb, qe = self.boff[bl], self.boff[bl + 1]
                Sb = self.full & ~(self.unrank[bl] & ~pmask)
                if qb != qe and not strict[Sb]:
                    sel.append(bl)
                    rng_.append((qb, qe))
            if not sel:
                continue
            lst, prev_be = [], None
            for qb, qe in rng_:
                be = (qe + 31) // 32
                bf = max(qb // 32, prev_be if prev_be is not None else next_blk)
                lst += list(range(bf, be))
                prev_be = be
            next_blk = max(next_blk, (rng_[-1][1] + 31) // 32)
            for t0 in range(0, len(lst), LANES):
                for kb in lst[t0:t0 + LANES]:
                    if not strict[self.U(self.bmin[kb], pc)]:
                        bq.append(kb)
                while len(bq) >= 8:
                    sub_step(8)
        if bq:
            sub_step(len(bq))
        if len(wq) > 4:
            half_step(len(wq))
        elif wq:
            walk(True, len(wq))
        if hq:
            walk(False, len(hq))

        # TIE = {S : S meets T[S]}, T[S] = union of A[E] over E containing S
        T = A.copy()
        for k in range(d):
            bit = 1 << k
            for S in range(self.nsub):
                if not S & bit:
                    T[S] |= T[S | bit]
        S = np.arange(self.nsub)
        tie = (S & T) != 0
        dom = strict | tie
        ext = tie & ~strict
        dom[0] = ext[0] = False
        return dom, ext, stats


CASES = [
    # kind, n, d, grid depth, partition attributes, seed, quantisation steps
    ("anticorrelated", 3000, 6, 3, 4, 1, 0),
    ("anticorrelated", 4000, 7, 2, 5, 2, 16),  # exact ties on top of anticorrelation
    ("anticorrelated", 3000, 6, 2, 4, 5, 8),   # many ties: the tie map
    ("uniform", 5000, 5, 3, 5, 4, 0),
    ("ties", 3000, 6, 3, 3, 3, 0),             # a handful of q's: the short paths
]


def run_case(kind, n, d, depth, B, seed, quant, per_case=120):
    x = datagen.generate(kind, n, d, seed)
    if quant:
        x = np.round(x * quant) / quant
    M = Model(x, depth, B, seed)
    members = {c: (set(M.sky[c].tolist()), set(M.ext[c].tolist())) for c in range(1, M.nsub)}
    totals = {}
    for p in M.cand[:: max(1, len(M.cand) // per_case)]:
        dom, ext, st = M.candidate(int(p))
        for k, v in st.items():
            totals[k] = totals.get(k, 0) + v
        for c in range(1, M.nsub):
            in_sky, in_ext = members[c]
            assert dom[c] == (int(p) not in in_sky), (int(p), c)
            assert ext[c] == (int(p) in in_ext), (int(p), c)
    return totals


@pytest.mark.parametrize("case", CASES)
def test_bitmap_model_against_oracle(case):
    assert run_case(*case)["steps"] > 0


def test_bitmap_model_exercises_every_path():
    """Summed over the anticorrelated cases, every step kind runs both full
    and short, the flush walks whole quarters, equal cells go to the floats
    and exact ties reach the tie map."""
    tot = {}
    for case in CASES[:3]:
        for k, v in run_case(*case, per_case=40).items():
            tot[k] = tot.get(k, 0) + v
    for k in ("skipped", "float_checks", "tie_writes", "updates", "sub_full", "sub_short",
              "half_full", "half_short", "walk_full", "walk_short", "walk_quarters"):
        assert tot[k] > 0, (k, tot)
