"""Serving loop: each request's result is identical when served alone and in
a concurrent mix (exact id-set equality), admission rejects requests above
the memory budget, and skyline queries match the oracle."""
import threading

import numpy as np
import pytest

import oracle
import skycube_gb300 as sk
from skycube_gb300 import datagen

pytestmark = pytest.mark.gpu

MIX = [
    ("anticorrelated", 60000, 8, dict(algo="mdmc", mode="batched")),
    ("ties", 40000, 6, dict(algo="sdsc", mode="plain", want_extended=True)),
    ("correlated_q", 30000, 12, dict(algo="sdsc", mode="batched", max_d=3, want_extended=True)),
    ("uniform", 20000, 5, dict(subspace=0b10110)),
    ("anticorrelated", 5000, 16, dict(max_d=2)),
    ("correlated", 50000, 9, dict(algo="mdmc", mode="plain")),
    ("uniform", 3000, 10, dict(subspace=(1 << 10) - 1, want_extended=True)),
    ("ties", 25000, 11, dict()),
]


def snapshot(res, ext):
    out = {c: res.cuboid(c) for c in range(1, 1 << res.d)}
    if ext:
        out.update({-c: res.extended(c) for c in range(1, 1 << res.d)})
    return out


def test_results_identical_alone_and_in_the_mix(gpu_ctx):
    data = [datagen.generate(k, n, d, 100 + i) for i, (k, n, d, _) in enumerate(MIX)]
    alone = []
    for x, (_, _, _, o) in zip(data, MIX):
        ds = sk.Dataset(gpu_ctx, x)
        r = sk.skycube(gpu_ctx, ds, **o)
        alone.append(snapshot(r, o.get("want_extended", False)))
        r.close()
        ds.close()
    srv = sk.Server(gpu_ctx, slots=4)
    # submit everything at once from two threads, then wait in reverse order
    tickets = [None] * len(MIX)

    def submit(idx):
        for i in idx:
            tickets[i] = srv.submit(data[i], **MIX[i][3])

    th = [threading.Thread(target=submit, args=(range(j, len(MIX), 2),)) for j in (0, 1)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for i in reversed(range(len(MIX))):
        r, timing = srv.wait(tickets[i])
        assert timing["total_ms"] >= timing["run_ms"] >= 0
        got = snapshot(r, MIX[i][3].get("want_extended", False))
        assert got.keys() == alone[i].keys()
        for c in got:
            assert np.array_equal(got[c], alone[i][c]), f"request {i} cuboid {c}"
    st = srv.stats()
    assert st["admitted"] == len(MIX) and st["peak_in_flight"] >= 2
    srv.close()


def test_skyline_query_matches_oracle(gpu_ctx):
    x = datagen.generate("ties", 8000, 7, 7)
    sky, ext = oracle.stsc(x)
    ds = sk.Dataset(gpu_ctx, x)
    for S in (0b1, 0b1011, 0b1110001, 0b1111111):
        r = sk.skycube(gpu_ctx, ds, subspace=S, want_extended=True)
        assert np.array_equal(r.cuboid(S), sky[S])
        assert np.array_equal(r.extended(S), ext[S])
        other = 1 if S != 1 else 2
        assert len(r.cuboid(other)) == 0


def test_admission_rejects_oversized_requests(gpu_ctx):
    srv = sk.Server(gpu_ctx, slots=2, budget=1 << 20)  # 1 MiB
    with pytest.raises(sk.SkycubeError) as e:
        srv.submit(datagen.generate("uniform", 100000, 8, 1))
    assert e.value.code == 6 and "budget" in str(e.value)
    t = srv.submit(datagen.generate("uniform", 500, 3, 1))  # small enough
    r, _ = srv.wait(t)
    assert len(r.cuboid(7)) > 0
    srv.close()


def test_budget_serialises_requests(gpu_ctx):
    """With a budget that fits one request at a time, requests still all
    complete, one after another."""
    x = datagen.generate("anticorrelated", 20000, 6, 3)
    srv = sk.Server(gpu_ctx, slots=4, budget=16 << 20)  # one request is about 10.6 MiB
    ts = [srv.submit(x) for _ in range(5)]
    outs = [srv.wait(t)[0].cuboid(63) for t in ts]
    assert all(np.array_equal(o, outs[0]) for o in outs)
    assert srv.stats()["peak_in_flight"] == 1
    srv.close()


def test_one_waiter_per_ticket(gpu_ctx):
    """Two threads waiting on the same ticket: one gets the result, the other
    SKC_ERR_INVALID (never a shared or double-freed result); a wait on a
    collected ticket is refused too."""
    import ctypes
    L = sk.lib()
    srv = sk.Server(gpu_ctx, slots=1)
    x = datagen.generate("anticorrelated", 200000, 8, 11)
    t = srv.submit(x)
    codes, handles = [None, None], [None, None]

    def wait(i):
        h = ctypes.c_void_p()
        codes[i] = L.skc_server_wait(srv.handle, ctypes.c_uint64(t), ctypes.byref(h), None)
        handles[i] = h

    th = [threading.Thread(target=wait, args=(i,)) for i in (0, 1)]
    for x_ in th:
        x_.start()
    for x_ in th:
        x_.join()
    assert sorted(codes) == [0, 1], codes
    winner = codes.index(0)
    r = sk.Result(gpu_ctx, handles[winner], 8, 8)
    assert len(r.cuboid(255)) > 0
    r.close()
    h = ctypes.c_void_p()
    assert L.skc_server_wait(srv.handle, ctypes.c_uint64(t), ctypes.byref(h), None) == 1
    srv.close()


def test_capped_skycubes_batched_into_one_launch(gpu_ctx):
    """With one slot, capped skycube requests that wait behind a running
    request are taken together into one lattice launch; each result equals
    the request served alone."""
    xs = [datagen.generate(k, 30000, 10, 200 + i) for i, k in
          enumerate(("anticorrelated", "uniform", "correlated", "anticorrelated", "uniform"))]
    opts = dict(max_d=3, want_extended=True, form="levels")
    alone = []
    for x in xs:
        ds = sk.Dataset(gpu_ctx, x)
        r = sk.skycube(gpu_ctx, ds, **opts)
        alone.append(snapshot(r, True))
        r.close()
        ds.close()
    srv = sk.Server(gpu_ctx, slots=1)
    big = srv.submit(datagen.generate("anticorrelated", 300000, 10, 7))  # keeps the slot busy
    ts = [srv.submit(x, **opts) for x in xs]
    srv.wait(big)[0].close()
    for t, want in zip(ts, alone):
        r, _ = srv.wait(t)
        got = snapshot(r, True)
        assert got.keys() == want.keys()
        for c in got:
            assert np.array_equal(got[c], want[c]), c
        r.close()
    st = srv.batch_stats()
    assert st["batches"] >= 1 and st["largest"] >= 2, st
    srv.close()
