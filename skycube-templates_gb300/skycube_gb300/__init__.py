"""Python binding of the GB300 skycube engine's C ABI (include/skycube_gb300.h).

The engine itself is CUDA + C++ (``libskycube_gb300.so``); this module is a
thin ctypes layer used by the tests and the benchmark. It never computes a
skycube in Python and raises ``SkycubeError`` if the native library is
missing or a call fails.

Vocabulary follows the skycube suite: a *cuboid* is a non-empty subspace,
given as a bitmask over the d attributes; its *skyline* holds the point ids
(row indices) no other point dominates on it, its *extended skyline* the
dominated points nobody strictly dominates. ``algo`` is "mdmc" or "sdsc"
(the suite's ``-s``), ``mode`` "plain" (one launch sequence per cuboid) or
"batched" (one persistent launch for all cuboids), ``max_d`` the suite's
``-m`` cap and ``depth`` its ``-d`` grid depth.
"""
import ctypes
import os
import weakref

import numpy as np

from .build import LIB_PATH, build  # noqa: F401

SKC_OK = 0
ERROR_NAMES = {1: "INVALID", 2: "CUDA", 3: "OOM", 4: "TIMEOUT", 5: "UNSUPPORTED", 6: "REJECTED"}
ALGOS = {"mdmc": 0, "sdsc": 1}
MODES = {"plain": 0, "batched": 1}


class SkycubeError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"skycube error {ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


class _Timing(ctypes.Structure):
    _fields_ = [("queued_ms", ctypes.c_double), ("run_ms", ctypes.c_double),
                ("total_ms", ctypes.c_double), ("device_ms", ctypes.c_float)]


class _Options(ctypes.Structure):
    _fields_ = [("algo", ctypes.c_int), ("mode", ctypes.c_int), ("max_d", ctypes.c_int),
                ("depth", ctypes.c_int), ("want_extended", ctypes.c_int),
                ("want_bitmaps", ctypes.c_int), ("subspace", ctypes.c_uint32),
                ("pq_size", ctypes.c_int), ("tile_points", ctypes.c_int),
                ("chunk", ctypes.c_int), ("blocks_per_sm", ctypes.c_int),
                ("form", ctypes.c_int)]

    def work_params(self):
        return {"depth": self.depth, "pq_size": self.pq_size, "tile_points": self.tile_points,
                "chunk": self.chunk, "blocks_per_sm": self.blocks_per_sm}


_lib = None


def lib():
    """Loads libskycube_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise SkycubeError(2, f"native library {LIB_PATH} is missing; run skycube_gb300.build()")
    L = ctypes.CDLL(LIB_PATH)
    vp, u32, u64, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
    P = ctypes.POINTER
    sig = {
        "skc_options_init": (None, [P(_Options)]),
        "skc_context_create": (i32, [i32, P(vp)]),
        "skc_context_destroy": (i32, [vp]),
        "skc_dataset_upload": (i32, [vp, vp, u64, i32, P(vp)]),
        "skc_dataset_upload_device": (i32, [vp, vp, u64, i32, P(vp)]),
        "skc_dataset_free": (i32, [vp]),
        "skc_skycube": (i32, [vp, vp, P(_Options), P(vp)]),
        "skc_skycube_batch": (i32, [vp, P(vp), P(_Options), i32, P(vp)]),
        "skc_server_batch_stats": (i32, [vp, P(u64), P(u64), P(u64)]),
        "skc_result_info": (i32, [vp, P(i32), P(u64), P(u64)]),
        "skc_result_form": (i32, [vp, P(i32), P(i32)]),
        "skc_result_cuboid": (i32, [vp, u32, P(P(u32)), P(u64)]),
        "skc_result_extended": (i32, [vp, u32, P(P(u32)), P(u64)]),
        "skc_result_device_csr": (i32, [vp, P(vp), P(vp)]),
        "skc_result_download": (i32, [vp]),
        "skc_result_bitmaps": (i32, [vp, P(P(u32)), P(P(u32)), P(u64), P(u32)]),
        "skc_result_free": (i32, [vp]),
        "skc_last_device_ms": (i32, [vp, P(ctypes.c_float)]),
        "skc_last_error": (ctypes.c_char_p, []),
        "skc_kernel_launches": (u64, []),
        "skc_last_phase": (i32, [vp, i32, P(ctypes.c_char_p), P(ctypes.c_float)]),
        "skc_server_create": (i32, [vp, i32, u64, P(vp)]),
        "skc_server_submit": (i32, [vp, vp, u64, i32, P(_Options), P(u64)]),
        "skc_server_submit_dataset": (i32, [vp, vp, P(_Options), P(u64)]),
        "skc_server_wait": (i32, [vp, u64, P(vp), P(_Timing)]),
        "skc_server_stats": (i32, [vp, P(u64), P(u64), P(u64)]),
        "skc_server_destroy": (i32, [vp]),
        "skc_autotune": (i32, [vp, vp, P(_Options), i32, P(_Options), P(ctypes.c_float)]),
        "skc_dataset_signature": (i32, [vp, P(i32), P(i32), P(i32)]),
        "skc_tuning_count": (i32, [vp, P(u64)]),
        "skc_tuning_clear": (i32, [vp]),
        "skc_plan_create": (i32, [vp, vp, P(_Options), P(vp)]),
        "skc_plan_execute": (i32, [vp, P(vp)]),
        "skc_plan_info": (i32, [vp, P(u64), P(u64), P(u64), P(u64)]),
        "skc_plan_destroy": (i32, [vp]),
        "skc_dataset_update": (i32, [vp, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(code):
    if code != SKC_OK:
        raise SkycubeError(code, lib().skc_last_error().decode())


class Context:
    """A CUDA device plus the engine's stream and memory pool (the -g value)."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        _check(lib().skc_context_create(device, ctypes.byref(h)))
        self.handle = h
        self.device = device
        self._children = weakref.WeakSet()

    def _adopt(self, child):
        self._children.add(child)

    def close(self):
        if self.handle:
            for c in list(self._children):
                c.close()
            lib().skc_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_phases(self):
        """[(phase name, device ms)] of the last skycube call."""
        out, i = [], 0
        name, ms = ctypes.c_char_p(), ctypes.c_float()
        while lib().skc_last_phase(self.handle, i, ctypes.byref(name), ctypes.byref(ms)) == SKC_OK:
            out.append((name.value.decode(), ms.value))
            i += 1
        return out

    def last_device_ms(self):
        v = ctypes.c_float()
        _check(lib().skc_last_device_ms(self.handle, ctypes.byref(v)))
        return v.value

    def tuning_count(self):
        v = ctypes.c_uint64()
        _check(lib().skc_tuning_count(self.handle, ctypes.byref(v)))
        return v.value

    def tuning_clear(self):
        _check(lib().skc_tuning_clear(self.handle))


class Dataset:
    """A point set resident on the device (MDMC<D>::Init / SDSC<D>::Init)."""

    def __init__(self, ctx, points=None, device_ptr=None, n=None, d=None):
        self.ctx = ctx
        h = ctypes.c_void_p()
        if device_ptr is not None:
            _check(lib().skc_dataset_upload_device(ctx.handle, ctypes.c_void_p(device_ptr),
                                                   n, d, ctypes.byref(h)))
            self.n, self.d = n, d
        else:
            x = np.ascontiguousarray(points, dtype=np.float32)
            if x.ndim != 2:
                raise SkycubeError(1, "points must be a 2-d array (n, d)")
            self.n, self.d = x.shape
            _check(lib().skc_dataset_upload(ctx.handle, x.ctypes.data_as(ctypes.c_void_p),
                                            self.n, self.d, ctypes.byref(h)))
        self.handle = h
        ctx._adopt(self)

    def update(self, points):
        """skc_dataset_update: new points in place (same n and d)."""
        x = np.ascontiguousarray(points, dtype=np.float32)
        if x.shape != (self.n, self.d):
            raise SkycubeError(1, f"update needs shape {(self.n, self.d)}, got {x.shape}")
        _check(lib().skc_dataset_update(self.handle, x.ctypes.data_as(ctypes.c_void_p)))

    def close(self):
        if self.handle:
            lib().skc_dataset_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Result:
    """Per-cuboid skylines (and optionally extended skylines / bitmaps)."""

    def __init__(self, ctx, handle, d, max_d):
        self.ctx = ctx  # keeps the context alive while the result is
        self.handle = handle
        self.d = d
        self.max_d = max_d
        ctx._adopt(self)

    def close(self):
        if self.handle:
            lib().skc_result_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        d, m, t = ctypes.c_int(), ctypes.c_uint64(), ctypes.c_uint64()
        _check(lib().skc_result_info(self.handle, ctypes.byref(d), ctypes.byref(m), ctypes.byref(t)))
        return {"d": d.value, "n_candidates": m.value, "total_skyline_ids": t.value}

    FORMS = {1: "bitmaps", 2: "cuboids", 3: "levels", 4: "skyline"}

    def form(self):
        """(computation that produced the result, cuboids of the level form
        that went through the per-cuboid pipeline)."""
        f, fb = ctypes.c_int(), ctypes.c_int()
        _check(lib().skc_result_form(self.handle, ctypes.byref(f), ctypes.byref(fb)))
        return self.FORMS.get(f.value, "unknown"), fb.value

    def download(self):
        _check(lib().skc_result_download(self.handle))

    def _view(self, fn, cuboid):
        p = ctypes.POINTER(ctypes.c_uint32)()
        c = ctypes.c_uint64()
        _check(fn(self.handle, cuboid, ctypes.byref(p), ctypes.byref(c)))
        if c.value == 0:
            return np.empty(0, dtype=np.uint32)
        return np.ctypeslib.as_array(p, shape=(c.value,)).copy()

    def cuboid(self, cuboid):
        """Skyline ids of one cuboid (ascending)."""
        return self._view(lib().skc_result_cuboid, cuboid)

    def extended(self, cuboid):
        """Extended-skyline ids of one cuboid (ascending)."""
        return self._view(lib().skc_result_extended, cuboid)

    def all_cuboids(self, extended=False):
        """{cuboid mask: ids} for every cuboid within max_d and the full space."""
        out = {}
        for c in range(1, 1 << self.d):
            if bin(c).count("1") <= self.max_d or c == (1 << self.d) - 1:
                out[c] = self.extended(c) if extended else self.cuboid(c)
        return out

    def device_csr(self):
        off, ids = ctypes.c_void_p(), ctypes.c_void_p()
        _check(lib().skc_result_device_csr(self.handle, ctypes.byref(off), ctypes.byref(ids)))
        return off.value, ids.value

    def bitmaps(self):
        """(bits[n_cand, words] uint32, pids[n_cand]) of the dominated subspaces."""
        b = ctypes.POINTER(ctypes.c_uint32)()
        p = ctypes.POINTER(ctypes.c_uint32)()
        n, w = ctypes.c_uint64(), ctypes.c_uint32()
        _check(lib().skc_result_bitmaps(self.handle, ctypes.byref(b), ctypes.byref(p),
                                        ctypes.byref(n), ctypes.byref(w)))
        if n.value == 0:
            return np.zeros((0, w.value), np.uint32), np.zeros(0, np.uint32)
        bits = np.ctypeslib.as_array(b, shape=(n.value * w.value,)).reshape(n.value, w.value).copy()
        pids = np.ctypeslib.as_array(p, shape=(n.value,)).copy()
        return bits, pids


def kernel_launches():
    """Kernels launched by the native library in this process so far."""
    return int(lib().skc_kernel_launches())


FORM_CODES = {"auto": 0, "bitmaps": 1, "levels": 3}


def options(algo="mdmc", mode="batched", max_d=0, depth=0, want_extended=False,
            want_bitmaps=False, subspace=0, pq_size=0, tile_points=0, chunk=0,
            blocks_per_sm=0, form="auto"):
    """skc_options. The work parameters (depth, pq_size, tile_points, chunk,
    blocks_per_sm) change the work, never the result; 0 = automatic (a stored
    tuning for datasets like this one, else the default); pq_size < 0 turns
    the prefilter off. form: "auto", "bitmaps" or "levels" (the computation
    of a batched capped skycube; never changes the result)."""
    return _Options(ALGOS[algo], MODES[mode], int(max_d), int(depth),
                    int(bool(want_extended)), int(bool(want_bitmaps)), int(subspace),
                    int(pq_size), int(tile_points), int(chunk), int(blocks_per_sm),
                    FORM_CODES[form])


def skycube(ctx, ds, algo="mdmc", mode="batched", max_d=0, depth=0,
            want_extended=False, want_bitmaps=False, subspace=0, pq_size=0,
            tile_points=0, chunk=0, blocks_per_sm=0, form="auto"):
    """Computes the skycube of a resident dataset (MDMC/SDSC ::Execute), or
    with `subspace` set, only that cuboid's skyline (a skyline query)."""
    o = options(algo, mode, max_d, depth, want_extended, want_bitmaps, subspace, pq_size,
                tile_points, chunk, blocks_per_sm, form)
    h = ctypes.c_void_p()
    _check(lib().skc_skycube(ctx.handle, ds.handle, ctypes.byref(o), ctypes.byref(h)))
    md = ds.d if max_d <= 0 or max_d > ds.d else max_d
    return Result(ctx, h, ds.d, md)


def skycube_batch(ctx, datasets, opts_list):
    """skc_skycube_batch: the skycubes of several resident datasets in one
    pass (one lattice launch shared by those that take the level form).
    opts_list holds one dict of skycube() keyword options per dataset."""
    n = len(datasets)
    arr = (ctypes.c_void_p * n)(*[ds.handle.value for ds in datasets])
    opts = (_Options * n)(*[options(**o) for o in opts_list])
    outs = (ctypes.c_void_p * n)()
    _check(lib().skc_skycube_batch(ctx.handle, arr, opts, n, outs))
    res = []
    for ds, o, h in zip(datasets, opts_list, outs):
        md = o.get("max_d", 0)
        md = ds.d if md <= 0 or md > ds.d else md
        res.append(Result(ctx, ctypes.c_void_p(h), ds.d, md))
    return res


class Plan:
    """skc_plan_*: the batched skycube of one dataset captured as a CUDA
    graph; execute() replays it on the dataset's current points."""

    def __init__(self, ctx, ds, **opts):
        self.ctx, self.ds = ctx, ds
        o = options(**opts)
        self.max_d = ds.d if o.max_d <= 0 or o.max_d > ds.d else o.max_d
        h = ctypes.c_void_p()
        _check(lib().skc_plan_create(ctx.handle, ds.handle, ctypes.byref(o), ctypes.byref(h)))
        self.handle = h
        ctx._adopt(self)

    def execute(self):
        h = ctypes.c_void_p()
        _check(lib().skc_plan_execute(self.handle, ctypes.byref(h)))
        return Result(self.ctx, h, self.ds.d, self.max_d)

    def info(self):
        k, r, c, i = (ctypes.c_uint64() for _ in range(4))
        _check(lib().skc_plan_info(self.handle, ctypes.byref(k), ctypes.byref(r), ctypes.byref(c),
                                   ctypes.byref(i)))
        return {"kernels": k.value, "replans": r.value, "cand_capacity": c.value,
                "ids_capacity": i.value}

    def close(self):
        if self.handle:
            lib().skc_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(ctx, ds, repeats=2, **opts):
    """skc_autotune: times the work parameters left at 0 in `opts` on `ds`,
    stores the winner for datasets with the same signature and returns
    (chosen work parameters as a dict, device ms)."""
    base = options(**opts)
    best = _Options()
    ms = ctypes.c_float()
    _check(lib().skc_autotune(ctx.handle, ds.handle, ctypes.byref(base), int(repeats),
                              ctypes.byref(best), ctypes.byref(ms)))
    return best.work_params(), ms.value


def signature(ds):
    """skc_dataset_signature: {size_class, sky_class, ties}."""
    a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _check(lib().skc_dataset_signature(ds.handle, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
    return {"size_class": a.value, "sky_class": b.value, "ties": c.value}


class Server:
    """Continuous-batching serving loop (skc_server_*): `slots` concurrent
    requests, admitted in order by estimated device-memory footprint."""

    def __init__(self, ctx, slots=4, budget=0):
        self.ctx = ctx
        h = ctypes.c_void_p()
        _check(lib().skc_server_create(ctx.handle, slots, budget, ctypes.byref(h)))
        self.handle = h
        self._keep = {}  # ticket -> host rows kept alive until the result is taken

    def submit(self, points, **opts):
        x = np.ascontiguousarray(points, dtype=np.float32)
        o = options(**opts)
        t = ctypes.c_uint64()
        _check(lib().skc_server_submit(self.handle, x.ctypes.data_as(ctypes.c_void_p), x.shape[0],
                                       x.shape[1], ctypes.byref(o), ctypes.byref(t)))
        self._keep[t.value] = (x, x.shape[1], o.max_d if not o.subspace else bin(o.subspace).count("1"))
        return t.value

    def wait(self, ticket):
        """(Result, timing dict) of a submitted request."""
        h = ctypes.c_void_p()
        tm = _Timing()
        x, d, md = self._keep.pop(ticket, (None, 0, 0))
        _check(lib().skc_server_wait(self.handle, ticket, ctypes.byref(h), ctypes.byref(tm)))
        md = d if md <= 0 or md > d else md
        res = Result(self.ctx, h, d, md)
        return res, {"queued_ms": tm.queued_ms, "run_ms": tm.run_ms, "total_ms": tm.total_ms,
                     "device_ms": tm.device_ms}

    def stats(self):
        a, p, b = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        _check(lib().skc_server_stats(self.handle, ctypes.byref(a), ctypes.byref(p), ctypes.byref(b)))
        return {"admitted": a.value, "peak_in_flight": p.value, "budget": b.value}

    def batch_stats(self):
        b, r, m = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        _check(lib().skc_server_batch_stats(self.handle, ctypes.byref(b), ctypes.byref(r),
                                            ctypes.byref(m)))
        return {"batches": b.value, "batched_requests": r.value, "largest": m.value}

    def close(self):
        if self.handle:
            lib().skc_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
