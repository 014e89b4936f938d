"""The suite-shaped result layout on the host, without a GPU: HashCube<D>
(src/skycube/Hashcube.h:36-178) filled from definition-level bitmaps, both
per-cuboid decodes (HashCube::getSubspace and getsubspace over getMaps(),
src/utilities/utilities.h:253-267) against the skylines the bitmaps define,
and the lattice helpers (generate_lattice, get_tds_list,
src/utilities/lattice_utilities.cpp:10-79): parents and children one
attribute apart in descending mask order, cuboids top-down by level.
The C++ program compiles against host/skycube_templates.h only."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from conftest import REPO

HOST = os.path.join(REPO, "skycube-templates_gb300", "host")
INCLUDE = os.path.join(REPO, "include")


@pytest.fixture(scope="module")
def prog(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("cpp") / "hashcube_check")
    src = os.path.join(REPO, "tests", "cpp", "hashcube_check.cpp")
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", INCLUDE, "-I", HOST, src, "-o", out],
                   check=True)
    return out


def _run(prog, tmp_path, x, pids):
    n, d = x.shape
    bits = oracle.bruteforce_bitmaps(x)
    f = tmp_path / "bits.bin"
    with open(f, "wb") as fh:
        fh.write(np.ascontiguousarray(bits, dtype="<u4").tobytes())
        fh.write(np.ascontiguousarray(pids, dtype="<u4").tobytes())
    r = subprocess.run([prog, str(f), str(d), str(n)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    out = {"C": {}, "P": {}, "K": {}, "W": {}}
    tds = None
    for line in r.stdout.splitlines():
        tag, *vals = line.split()
        if tag == "T":
            tds = [int(v) for v in vals]
        else:
            out[tag][int(vals[0])] = [int(v) for v in vals[1:]]
    return bits, out, tds


@pytest.mark.parametrize("d,n,levels,seed", [(2, 40, 3, 1), (3, 60, 0, 2), (4, 80, 4, 3),
                                             (5, 120, 0, 4), (6, 150, 3, 5), (8, 200, 8, 6),
                                             (10, 160, 0, 7)])
def test_hashcube_decode_and_lattice(prog, tmp_path, d, n, levels, seed):
    rng = np.random.default_rng(seed)
    if levels:
        x = np.floor(rng.random((n, d)) * levels).astype(np.float32)
    else:
        x = rng.random((n, d), dtype=np.float64).astype(np.float32)
    pids = rng.permutation(n).astype(np.uint32) + 1000  # ids other than row numbers
    bits, out, tds = _run(prog, tmp_path, x, pids)
    truth = oracle.skylines_from_bitmaps(bits, d)
    m = 1 << d
    for c in range(1, m):
        assert out["C"][c] == sorted(pids[truth[c]].tolist()), f"cuboid {c}"
        parents = sorted((c | (1 << k) for k in range(d) if not c >> k & 1), reverse=True)
        children = sorted((c ^ (1 << k) for k in range(d) if c >> k & 1 and c ^ (1 << k)),
                          reverse=True)
        assert out["P"][c] == parents, f"parents of {c}"
        assert out["K"][c] == children, f"children of {c}"
    assert tds == sorted(range(1, m), key=lambda c: -bin(c).count("1"))


def test_hashcube_skips_all_dominated_words(prog, tmp_path):
    """A point dominated on all 32 cuboids of a bitmap word is not listed
    under that word (the suite's layout), yet every decode stays exact."""
    x = np.array([[0.0] * 6, [1.0] * 6, [0.5] * 6], dtype=np.float32)
    pids = np.array([7, 8, 9], dtype=np.uint32)
    bits, out, _ = _run(prog, tmp_path, x, pids)
    # (1, ..., 1) and (0.5, ..., 0.5) are dominated on every non-empty
    # cuboid: their word 1 (cuboids 32..63) is all ones and goes unlisted,
    # their word 0 is not (the empty cuboid's bit is clear); word 2, the
    # extra word, is zero for every point
    for p in (1, 2):
        assert bits[p][0] == 0xFFFFFFFE and bits[p][1] == 0xFFFFFFFF
    assert out["W"] == {0: [3], 1: [1], 2: [3]}
    for c in range(1, 64):
        assert out["C"][c] == [7]
