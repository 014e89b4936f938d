"""CUDA path parity: every execution form against the reference's golden
fixtures, the C oracle on seeded inputs, and definition-level bitmaps.
Comparisons are exact id-set equality per cuboid (integer/index work)."""
import numpy as np
import pytest

import oracle
import skycube_gb300 as sk
from conftest import golden_names, load_golden
from skycube_gb300 import datagen

pytestmark = pytest.mark.gpu

FORMS = [("mdmc", "batched"), ("sdsc", "batched"), ("sdsc", "plain"), ("mdmc", "plain")]


def within(c, max_d):
    return bin(c).count("1") <= max_d


def check_result(r, d, max_d, sky, ext=None):
    for c in range(1, 1 << d):
        got = r.cuboid(c)
        if not within(c, max_d) and c != (1 << d) - 1:
            assert len(got) == 0, f"cuboid {c} above max_d must be empty"
            continue
        assert np.array_equal(got, sky[c]), f"skyline of cuboid {c}: {len(got)} vs {len(sky[c])}"
        if ext is not None:
            e = r.extended(c)
            assert np.array_equal(e, ext[c]), f"extended skyline of cuboid {c}: {len(e)} vs {len(ext[c])}"


@pytest.mark.parametrize("name", golden_names())
@pytest.mark.parametrize("algo,mode", FORMS)
def test_golden_fixture(gpu_ctx, name, algo, mode):
    x, max_d, sky, ext = load_golden(name)
    ds = sk.Dataset(gpu_ctx, x)
    r = sk.skycube(gpu_ctx, ds, algo, mode, max_d=max_d, want_extended=True)
    check_result(r, x.shape[1], max_d, sky, ext)


CASES = [
    ("uniform", 20000, 3, 3, 21), ("uniform", 30000, 9, 9, 22), ("anticorrelated", 20000, 7, 7, 23),
    ("ties", 30000, 10, 10, 24), ("correlated", 20000, 11, 11, 25), ("correlated_q", 20000, 13, 4, 26),
    ("ties", 8000, 14, 3, 27), ("anticorrelated", 3000, 15, 2, 28), ("correlated_q", 5000, 16, 3, 29),
    ("uniform", 2000, 12, 12, 30),
]


@pytest.mark.parametrize("kind,n,d,max_d,seed", CASES)
def test_against_oracle(gpu_ctx, kind, n, d, max_d, seed):
    x = datagen.generate(kind, n, d, seed)
    sky, ext = oracle.stsc(x, max_d)
    ds = sk.Dataset(gpu_ctx, x)
    for algo, mode in (("mdmc", "batched"), ("sdsc", "plain")):
        r = sk.skycube(gpu_ctx, ds, algo, mode, max_d=max_d, want_extended=True)
        check_result(r, d, max_d, sky, ext)


@pytest.mark.parametrize("depth", [1, 2, 4, 7])
def test_grid_depth_does_not_change_results(gpu_ctx, depth):
    x = datagen.generate("ties", 10000, 8, 31)
    sky, ext = oracle.stsc(x)
    ds = sk.Dataset(gpu_ctx, x)
    for algo, mode in (("mdmc", "batched"), ("sdsc", "plain")):
        r = sk.skycube(gpu_ctx, ds, algo, mode, depth=depth, want_extended=True)
        check_result(r, 8, 8, sky, ext)


@pytest.mark.parametrize("seed", range(6))
def test_bitmaps_match_definition(gpu_ctx, seed):
    rng = np.random.default_rng(500 + seed)
    d = [3, 5, 6, 8, 10, 11][seed]
    levels = [0, 3, 5, 0, 4, 2][seed]
    n = 300
    x = rng.random((n, d))
    if levels:
        x = np.floor(x * levels)
    x = x.astype(np.float32)
    truth = oracle.bruteforce_bitmaps(x)
    ds = sk.Dataset(gpu_ctx, x)
    r = sk.skycube(gpu_ctx, ds, "mdmc", "batched", want_bitmaps=True)
    bits, pids = r.bitmaps()
    assert np.array_equal(pids, np.sort(pids))
    words = max(1, (1 << d) // 32)
    mask = np.full(words, 0xffffffff, np.uint32)
    if d < 5:
        mask[0] = (1 << (1 << d)) - 1
    mask[0] &= ~np.uint32(1)  # the empty subspace carries no information
    assert np.array_equal(bits & mask, truth[pids] & mask)
    # points outside the candidate set are strictly dominated in the full space
    full = (1 << d) - 1
    col = (truth[:, full // 32] >> np.uint32(full % 32)) & 1
    others = np.setdiff1d(np.arange(n), pids)
    assert np.all(col[others] == 1)


def test_rejects_bad_input(gpu_ctx):
    x = datagen.generate("uniform", 100, 4, 1)
    x[5, 2] = np.nan
    with pytest.raises(sk.SkycubeError) as e:
        sk.Dataset(gpu_ctx, x)
    assert e.value.code == 1 and "non-finite" in str(e.value)
    for bad in (np.zeros((10, 1), np.float32), np.zeros((10, 17), np.float32), np.zeros((0, 4), np.float32)):
        with pytest.raises(sk.SkycubeError):
            sk.Dataset(gpu_ctx, bad)


def test_repeat_calls_are_identical(gpu_ctx):
    x = datagen.generate("anticorrelated", 20000, 8, 33)
    ds = sk.Dataset(gpu_ctx, x)
    a = sk.skycube(gpu_ctx, ds).all_cuboids()
    for _ in range(3):
        b = sk.skycube(gpu_ctx, ds).all_cuboids()
        assert all(np.array_equal(a[c], b[c]) for c in a)


def test_context_destroy_detaches_children():
    import skycube_gb300 as sk2
    ctx = sk2.Context(0)
    ds = sk2.Dataset(ctx, datagen.generate("uniform", 1000, 4, 3))
    r = sk2.skycube(ctx, ds)
    ctx.close()  # closes the children first
    assert r.handle is None and ds.handle is None
    # the C ABI itself detaches live objects when the context goes first
    L = sk2.lib()
    import ctypes
    h = ctypes.c_void_p()
    assert L.skc_context_create(0, ctypes.byref(h)) == 0
    x = datagen.generate("uniform", 500, 3, 4)
    dh = ctypes.c_void_p()
    assert L.skc_dataset_upload(h, x.ctypes.data_as(ctypes.c_void_p), 500, 3, ctypes.byref(dh)) == 0
    rh = ctypes.c_void_p()
    assert L.skc_skycube(h, dh, None, ctypes.byref(rh)) == 0
    assert L.skc_context_destroy(h) == 0
    p = ctypes.POINTER(ctypes.c_uint32)()
    c = ctypes.c_uint64()
    assert L.skc_result_cuboid(rh, 1, ctypes.byref(p), ctypes.byref(c)) == 1
    assert L.skc_result_free(rh) == 0
    assert L.skc_dataset_free(dh) == 0


def test_device_upload_rejects_host_memory(gpu_ctx):
    """skc_dataset_upload_device checks that its pointer is device memory:
    a host buffer passed by mistake is an error, not a kernel fault."""
    host = np.zeros((8, 3), dtype=np.float32)
    with pytest.raises(sk.SkycubeError) as e:
        sk.Dataset(gpu_ctx, device_ptr=host.ctypes.data, n=8, d=3)
    assert e.value.code == 1 and "device memory" in str(e.value)
