"""skc_skyline_noalloc: the entry point for callers that cannot allocate
device memory (their host process or runtime owns the GPU's memory).

The test hands it device buffers it allocated itself and compares the
per-point statuses with the ones the regular entry point (skc_skycube)
produces for the same points and subspace, exactly, on two calls in a row.
This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

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


def test_noalloc_matches_skycube_on_two_calls_in_a_row():
    import torch
    sk.build()
    ctx = sk.Context(0)
    f = _entry()
    cases = [("ties", 20000, 8, 0b10110101, 3), ("anticorrelated", 30000, 10, (1 << 10) - 1, 4)]
    for kind, n, d, S, seed in cases:
        x = datagen.generate(kind, n, d, seed)
        want = _statuses_from_skycube(ctx, x, S)
        xd = torch.from_numpy(x).cuda()
        out = torch.full((n,), 7, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        rc = f(xd.data_ptr(), n, d, S, 0, out.data_ptr(), None)
        assert rc == 0, sk.lib().skc_last_error().decode()
        assert np.array_equal(out.cpu().numpy(), want)
    ctx.close()


def test_noalloc_rejects_inputs_beyond_its_limit():
    import torch
    sk.build()
    f = _entry()
    dummy = torch.zeros(16, dtype=torch.float32, device="cuda")
    out = torch.zeros(16, dtype=torch.uint8, device="cuda")
    rc = f(dummy.data_ptr(), 65537, 4, 3, 0, out.data_ptr(), None)
    assert rc == 5  # SKC_ERR_UNSUPPORTED
    assert b"65536" in sk.lib().skc_last_error()
    assert f(dummy.data_ptr(), 4, 17, 3, 0, out.data_ptr(), None) == 1
