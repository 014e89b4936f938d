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
    o.pq_size = o.chunk = 9
    sk.lib().skc_options_init(ctypes.byref(o))
    assert (o.algo, o.mode, o.max_d, o.depth) == (0, 1, 0, 0)
    assert (o.pq_size, o.tile_points, o.chunk, o.blocks_per_sm) == (0, 0, 0, 0)


def test_options_layout_matches_header(tmp_path):
    """The ctypes mirror of skc_options has the C struct's size and offsets."""
    src = tmp_path / "layout.c"
    fields = [f for f, _ in sk._Options._fields_]
    body = "".join(f'printf("%zu ", offsetof(skc_options, {f}));' for f in fields)
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "skycube_gb300.h"\n'
                   f'int main(void) {{ printf("%zu ", sizeof(skc_options)); {body} return 0; }}\n')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    want = [ctypes.sizeof(sk._Options)] + [getattr(sk._Options, f).offset for f in fields]
    assert got == want


def test_null_arguments_are_rejected(built):
    L = sk.lib()
    assert L.skc_context_create(0, None) == 1
    assert L.skc_skycube(None, None, None, None) == 1
    assert L.skc_result_info(None, None, None, None) == 1
    assert L.skc_result_form(None, None, None) == 1
    assert L.skc_autotune(None, None, None, 0, None, None) == 1
    assert L.skc_dataset_signature(None, None, None, None) == 1
    assert L.skc_tuning_count(None, None) == 1
    assert L.skc_tuning_clear(None) == 1
    assert L.skc_plan_create(None, None, None, None) == 1
    assert L.skc_plan_execute(None, None) == 1
    assert L.skc_plan_info(None, None, None, None, None) == 1
    assert L.skc_dataset_update(None, None) == 1
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
