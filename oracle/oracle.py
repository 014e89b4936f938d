"""ctypes wrapper of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Loaded by tests/, the smoke check and the CPU-baseline leg of bench.py to
check or time the CUDA path; the product never imports it.

  stsc(points, max_d, threads)        the C restatement (skycube_oracle.c)
  ref_stsc(points, max_d, threads)    the reference's own STSC built from its
                                      unmodified sources by build_ref.sh (None
                                      when not built): with its AVX dominance
                                      tests on x86-64, with the portable
                                      intrinsics of ref_shim/ elsewhere;
                                      shim=True selects the portable build
                                      made beside the AVX one on x86-64
  ref_pq(points, max_d, threads)      the reference's PQSkycube (its parallel
                                      QSkycube, build_ref.sh --pq; None when
                                      not built): skylines only, ext empty
  bruteforce_bitmaps(points)          definition-level bitmaps for tiny inputs

Both STSC variants return (sky, ext): dicts {cuboid mask: sorted uint32 ids}.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libskycube_ref.so")
REF_SHIM_LIB = os.path.join(HERE, "_ref", "libskycube_ref_shim.so")
REF_PQ_LIB = os.path.join(HERE, "_ref", "libskycube_ref_pq.so")

_lib = None
_ref = {}
_pq = None


def build():
    """Compiles the C oracle (portable C11 + OpenMP)."""
    subprocess.run(["sh", os.path.join(HERE, "build.sh")], check=True)


def _bind(L, prefix, run_args):
    run = getattr(L, prefix + "_run")
    run.restype = ctypes.c_void_p
    run.argtypes = run_args
    cnt = getattr(L, prefix + "_count")
    cnt.restype = ctypes.c_uint64
    cnt.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int]
    ids = getattr(L, prefix + "_ids")
    ids.restype = None
    ids.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_void_p]
    free = getattr(L, prefix + "_free")
    free.restype = None
    free.argtypes = [ctypes.c_void_p]
    return run, cnt, ids, free


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        vp, u32, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
        _lib = _bind(L, "oracle_stsc", [vp, u32, i32, i32, i32])
        bf = L.oracle_bruteforce_bitmaps
        bf.restype = None
        bf.argtypes = [vp, u32, i32, vp]
        _lib = _lib + (bf,)
    return _lib


def ref_available(shim=False):
    return os.path.exists(REF_SHIM_LIB if shim else REF_LIB)


def ref_lib(shim=False):
    if shim not in _ref:
        L = ctypes.CDLL(REF_SHIM_LIB if shim else REF_LIB)
        vp, u32, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
        _ref[shim] = _bind(L, "ref_stsc", [vp, u32, i32, i32, i32, i32, i32])
    return _ref[shim]


def ref_pq_available():
    return os.path.exists(REF_PQ_LIB)


def ref_pq(points, max_d=0, threads=None):
    """Per-cuboid skylines from the reference's PQSkycube (None when not
    built); the extended-skyline dict is empty lists (QSkycube has none)."""
    global _pq
    if not ref_pq_available():
        return None
    if _pq is None:
        vp, u32, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
        _pq = _bind(ctypes.CDLL(REF_PQ_LIB), "ref_pq", [vp, u32, i32, i32, i32])
    x = np.ascontiguousarray(points, dtype=np.float32)
    n, d = x.shape
    md = d if max_d <= 0 or max_d > d else max_d
    h = _pq[0](x.ctypes.data, n, d, md, _threads(threads))
    if not h:
        raise ValueError(f"reference PQSkycube rejected n={n} d={d}")
    return _collect(_pq, h, d, md)


def build_ref(reference_root=None, shim=False):
    """Builds the reference's STSC with build_ref.sh; returns True on success."""
    cmd = ["sh", os.path.join(HERE, "build_ref.sh")]
    if shim:
        cmd.append("--shim")
    if reference_root:
        cmd.append(reference_root)
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.returncode == 0


def _collect(fns, h, d, max_d):
    _, cnt, ids, free = fns[:4]
    sky, ext = {}, {}
    try:
        for c in range(1, 1 << d):
            if bin(c).count("1") > max_d and c != (1 << d) - 1:
                continue
            for e, out in ((0, sky), (1, ext)):
                k = cnt(h, c, e)
                a = np.empty(k, dtype=np.uint32)
                if k:
                    ids(h, c, e, a.ctypes.data)
                out[c] = np.sort(a)
    finally:
        free(h)
    return sky, ext


def _threads(threads):
    return threads if threads else (os.cpu_count() or 1)


def stsc(points, max_d=0, threads=None):
    x = np.ascontiguousarray(points, dtype=np.float32)
    n, d = x.shape
    md = d if max_d <= 0 or max_d > d else max_d
    fns = lib()
    h = fns[0](x.ctypes.data, n, d, md, _threads(threads))
    if not h:
        raise ValueError(f"oracle rejected d={d}")
    return _collect(fns, h, d, md)


def ref_stsc(points, max_d=0, threads=None, shim=False):
    if not ref_available(shim):
        return None
    x = np.ascontiguousarray(points, dtype=np.float32)
    n, d = x.shape
    md = d if max_d <= 0 or max_d > d else max_d
    fns = ref_lib(shim)
    h = fns[0](x.ctypes.data, n, d, md, _threads(threads), 0, 0)
    if not h:
        raise ValueError(f"reference rejected d={d}")
    return _collect(fns, h, d, md)


def bruteforce_bitmaps(points):
    """Dominated-subspace bitmaps by definition: bits[p, s // 32] bit s % 32
    set iff point p is dominated on cuboid s."""
    x = np.ascontiguousarray(points, dtype=np.float32)
    n, d = x.shape
    words = max(1, (1 << d) // 32)
    out = np.zeros((n, words), dtype=np.uint32)
    lib()[4](x.ctypes.data, n, d, out.ctypes.data)
    return out


def skylines_from_bitmaps(bits, d, max_d=0):
    """{cuboid: sorted row ids} with a clear bit (skyline members)."""
    md = d if max_d <= 0 or max_d > d else max_d
    out = {}
    for c in range(1, 1 << d):
        if bin(c).count("1") > md:
            continue
        col = (bits[:, c // 32] >> np.uint32(c % 32)) & np.uint32(1)
        out[c] = np.nonzero(col == 0)[0].astype(np.uint32)
    return out
