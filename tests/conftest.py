import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(REPO, "skycube-templates_gb300"), os.path.join(REPO, "oracle"), REPO):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def golden_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN)
                  if f.endswith(".npz") and not f.startswith("digest_"))


def load_digest(workload):
    """The reference STSC's per-cuboid digest of a full-size workload
    (tests/golden/make_golden.py --digests), or None if not generated."""
    p = os.path.join(GOLDEN, f"digest_{workload}.npz")
    return dict(np.load(p)) if os.path.exists(p) else None


def id_hash(ids):
    """64-bit digest of an ascending id list, as make_golden.py computes it."""
    import hashlib
    a = np.ascontiguousarray(ids, dtype="<u4")
    return int.from_bytes(hashlib.blake2b(a.tobytes(), digest_size=8).digest(), "little")


def points_hash(x):
    return id_hash(np.ascontiguousarray(x, dtype="<f4").view("<u4").ravel())


def load_golden(name):
    """(x, max_d, sky, ext) with sky/ext = {cuboid: sorted ids}."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    x = z["x"]
    d = x.shape[1]
    out = []
    for off, ids in ((z["sky_off"], z["sky_ids"]), (z["ext_off"], z["ext_ids"])):
        sets = {}
        for c in range(1, 1 << d):
            sets[c] = np.sort(ids[int(off[c - 1]):int(off[c])])
        out.append(sets)
    return x, int(z["max_d"]), out[0], out[1]


def wanted(c, d, max_d):
    """Cuboids compared: every cuboid within max_d plus the full space."""
    return bin(c).count("1") <= max_d or c == (1 << d) - 1


@pytest.fixture(scope="session")
def gpu_ctx():
    import skycube_gb300 as sk
    sk.build()
    ctx = sk.Context(0)
    yield ctx
    ctx.close()
