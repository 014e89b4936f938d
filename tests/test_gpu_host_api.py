"""The suite-shaped C++ interface (MDMC<D>, SDSC<D>, HashCube, getsubspace,
lattice_node) against the CPU oracle, through a small C++ program built here."""
import os
import subprocess

import numpy as np
import pytest

import oracle
import skycube_gb300 as sk
from conftest import REPO
from skycube_gb300 import datagen
from skycube_gb300.build import BUILD, HOST, INCLUDE

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def prog(tmp_path_factory):
    sk.build()
    out = str(tmp_path_factory.mktemp("cpp") / "host_api_check")
    src = os.path.join(REPO, "tests", "cpp", "host_api_check.cpp")
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", INCLUDE, "-I", HOST, src, "-o", out,
                    "-L", BUILD, "-lskycube_gb300", f"-Wl,-rpath,{BUILD}"], check=True)
    return out


@pytest.mark.parametrize("kind,n,d,max_d,seed", [
    ("ties", 3000, 4, 4, 1), ("anticorrelated", 4000, 7, 7, 2), ("correlated_q", 2000, 12, 3, 3),
])
def test_host_interface_matches_oracle(prog, tmp_path, kind, n, d, max_d, seed):
    x = datagen.generate(kind, n, d, seed)
    p = tmp_path / "x.csv"
    with open(p, "w") as f:
        for row in x:
            f.write(",".join(repr(float(v)) for v in row) + ",\n")
    xr = np.loadtxt(p, delimiter=",", usecols=range(d), dtype=np.float32, ndmin=2)
    assert np.array_equal(xr, x)
    r = subprocess.run([prog, str(p), str(max_d)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "MISMATCH" not in r.stdout
    sky, ext = oracle.stsc(x, max_d)
    seen = set()
    for line in r.stdout.splitlines():
        parts = line.split()
        tag, c, ids = parts[0], int(parts[1]), np.array(sorted(map(int, parts[2:])), dtype=np.uint32)
        want = ext[c] if tag.startswith("sdscext") else sky[c]
        assert np.array_equal(ids, want), f"{tag} cuboid {c}"
        seen.add(tag)
    assert seen == {f"{a}-{f}" for a in ("mdmc", "sdsc", "sdscext") for f in ("batched", "plain")}
