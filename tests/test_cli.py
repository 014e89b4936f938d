"""Command-line driver: argument handling on CPU, the -c cross-check on GPU."""
import os
import subprocess

import numpy as np
import pytest

import skycube_gb300 as sk
from skycube_gb300 import datagen
from skycube_gb300.build import CLI_PATH


@pytest.fixture(scope="module")
def cli():
    sk.build()
    assert os.path.exists(CLI_PATH)
    return CLI_PATH


def write_csv(path, x, trailing_comma=True):
    with open(path, "w") as f:
        for row in x:
            f.write(",".join(f"{v:.7g}" for v in row) + ("," if trailing_comma else "") + "\n")


def run(cli, *args):
    return subprocess.run([cli, *args], capture_output=True, text=True, timeout=600)


def test_usage_without_arguments(cli):
    r = run(cli)
    assert r.returncode == 1 and "USAGE" in r.stdout


def test_unknown_algorithm(cli, tmp_path):
    p = tmp_path / "x.csv"
    write_csv(p, np.eye(3, dtype=np.float32))
    r = run(cli, "-f", str(p), "-s", "stsc")
    assert r.returncode == 1 and "not provided" in r.stderr


def test_missing_file_and_bad_csv(cli, tmp_path):
    r = run(cli, "-f", str(tmp_path / "nope.csv"), "-s", "mdmc")
    assert r.returncode == 1 and "No such file" in r.stderr
    p = tmp_path / "bad.csv"
    p.write_text("0.1,0.2\n0.3,abc\n")
    r = run(cli, "-f", str(p), "-s", "mdmc")
    assert r.returncode == 1 and "PARSE FAILED" in r.stderr
    p.write_text("0.1,0.2\n0.3,0.4,0.5\n")
    r = run(cli, "-f", str(p), "-s", "sdsc")
    assert r.returncode == 1 and "attributes" in r.stderr


def test_bad_execution_form(cli, tmp_path):
    p = tmp_path / "x.csv"
    write_csv(p, np.eye(3, dtype=np.float32))
    r = run(cli, "-f", str(p), "-s", "mdmc", "-e", "fast")
    assert r.returncode == 1 and "execution form" in r.stderr


def test_without_gpu_fails_cleanly(cli, tmp_path):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    p = tmp_path / "x.csv"
    write_csv(p, np.eye(3, dtype=np.float32))
    r = run(cli, "-f", str(p), "-s", "mdmc")
    assert r.returncode == 2 and "skycube error" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("algo,form,kind,n,d,m", [
    ("mdmc", "batched", "anticorrelated", 20000, 8, 8),
    ("sdsc", "plain", "ties", 20000, 6, 6),
    ("sdsc", "batched", "correlated_q", 10000, 12, 3),
    ("mdmc", "plain", "uniform", 5000, 5, 5),
])
def test_cli_cross_check(cli, tmp_path, algo, form, kind, n, d, m):
    p = tmp_path / "data.csv"
    write_csv(p, datagen.generate(kind, n, d, 5))
    r = run(cli, "-f", str(p), "-s", algo, "-e", form, "-m", str(m), "-c", "-o")
    assert r.returncode == 0, r.stdout + r.stderr
    assert "done checking" in r.stdout and "In cuboid" not in r.stdout
    assert r.stdout.strip().split("\t")[0].split()[-1].isdigit()
