"""skc_skyline_noalloc: the entry point for callers that cannot allocate
device memory (their host process or runtime owns the GPU's memory).

The test hands it device buffers it allocated itself and compares the
per-point statuses with the ones the regular entry point (skc_skycube)
produces for the same points and subspace, exactly, on calls in a row: a
larger call followed by a smaller one with another d (the shared scratch
array keeps the larger call's leftovers), one on a non-default stream with
an explicit grid depth. The tie-heavy case is also checked against the CPU
oracle directly. This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

import oracle
import skycube_gb300 as sk
from skycube_gb300 import datagen

pytestmark = pytest.mark.gpu


def _entry():
    f = sk.lib().skc_skyline_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_uint32, ctypes.c_int,
                  ctypes.c_void_p, ctypes.c_void_p]
    return f


def _statuses_from_skycube(ctx, x, S):
    ds = sk.Dataset(ctx, x)
    r = sk.skycube(ctx, ds, "sdsc", "batched", want_extended=True)
    st = np.full(len(x), 2, dtype=np.uint8)
    st[r.extended(S)] = 1
    st[r.cuboid(S)] = 0
    r.close()
    ds.close()
    return st


def _statuses_from_oracle(x, S):
    sky, ext = oracle.stsc(x)
    st = np.full(len(x), 2, dtype=np.uint8)
    st[ext[S]] = 1
    st[sky[S]] = 0
    return st


def test_noalloc_matches_skycube_on_calls_in_a_row():
    import torch
    sk.build()
    ctx = sk.Context(0)
    f = _entry()
    side = torch.cuda.Stream()
    # (distribution, n, d, subspace, seed, depth, on the side stream)
    cases = [("ties", 20000, 8, 0b10110101, 3, 0, False),
             ("anticorrelated", 30000, 10, (1 << 10) - 1, 4, 0, False),
             ("correlated_q", 6000, 6, 0b101101, 5, 5, True),
             ("ties", 20000, 8, 0b10110101, 3, 5, True)]
    for kind, n, d, S, seed, depth, on_side in cases:
        x = datagen.generate(kind, n, d, seed)
        want = _statuses_from_skycube(ctx, x, S)
        xd = torch.from_numpy(x).cuda()
        out = torch.full((n,), 7, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        stream = side.cuda_stream if on_side else None
        rc = f(xd.data_ptr(), n, d, S, depth, out.data_ptr(), stream)
        assert rc == 0, sk.lib().skc_last_error().decode()
        got = out.cpu().numpy()
        assert np.array_equal(got, want), (kind, n, d)
        if kind == "ties" and d == 8:
            assert np.array_equal(got, _statuses_from_oracle(x, S))
    ctx.close()


def test_noalloc_rejects_inputs_beyond_its_limit_and_host_buffers():
    import torch
    sk.build()
    f = _entry()
    dummy = torch.zeros(16, dtype=torch.float32, device="cuda")
    out = torch.zeros(16, dtype=torch.uint8, device="cuda")
    rc = f(dummy.data_ptr(), 65537, 4, 3, 0, out.data_ptr(), None)
    assert rc == 5  # SKC_ERR_UNSUPPORTED
    assert b"65536" in sk.lib().skc_last_error()
    assert f(dummy.data_ptr(), 4, 17, 3, 0, out.data_ptr(), None) == 1
    # host memory passed by mistake is refused before any kernel runs
    host_rows = np.zeros((4, 4), dtype=np.float32)
    host_out = np.zeros(4, dtype=np.uint8)
    assert f(host_rows.ctypes.data, 4, 4, 3, 0, out.data_ptr(), None) == 1
    assert b"d_rows" in sk.lib().skc_last_error()
    assert f(dummy.data_ptr(), 4, 4, 3, 0, host_out.ctypes.data, None) == 1
    assert b"d_status" in sk.lib().skc_last_error()
