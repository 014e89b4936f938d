"""The C ABI library builds, loads and exports every entry point declared in
include/*.h; argument checks work without a GPU."""
import ctypes
import glob
import os
import re
import subprocess

import pytest

import skycube_gb300 as sk
from conftest import REPO


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(REPO, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(skc_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def built():
    return sk.build()


def test_header_declares_entry_points():
    names = declared_functions()
    assert "skc_skycube" in names and "skc_dataset_upload" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol(built):
    out = subprocess.run(["nm", "-D", "--defined-only", built], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (skc_[a-z0-9_]+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    L = ctypes.CDLL(built)
    for n in declared_functions():
        assert hasattr(L, n)


def test_options_defaults(built):
    o = sk._Options()
    sk.lib().skc_options_init(ctypes.byref(o))
    assert (o.algo, o.mode, o.max_d, o.depth) == (0, 1, 0, 0)


def test_null_arguments_are_rejected(built):
    L = sk.lib()
    assert L.skc_context_create(0, None) == 1
    assert L.skc_skycube(None, None, None, None) == 1
    assert L.skc_result_info(None, None, None, None) == 1
    assert b"NULL" in L.skc_last_error()


def test_no_gpu_context_fails_cleanly(built):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    code = sk.lib().skc_context_create(0, ctypes.byref(h))
    assert code in (1, 2)
    assert sk.lib().skc_last_error()
    with pytest.raises(sk.SkycubeError):
        sk.Context(0)
