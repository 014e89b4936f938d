"""Builds the engine's shared library and command-line tool for sm_103a.

Everything is compiled in-tree into ``skycube-templates_gb300/_build``:
  libskycube_gb300.so   the CUDA kernels and the C ABI (include/skycube_gb300.h)
  skycube               the command-line tool (host/cli.cpp)
Translation units compile in parallel; only one -gencode target is built.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
HOST = os.path.join(PKG_ROOT, "host")
INCLUDE = os.path.join(REPO_ROOT, "include")
BUILD = os.path.join(PKG_ROOT, "_build")
LIB_NAME = "libskycube_gb300.so"
LIB_PATH = os.path.join(BUILD, LIB_NAME)
# The counters build: the same library with the bitmap kernel's work
# counters compiled in (SKC_BITMAP_COUNTERS=1, skc_debug_bitmap_counters);
# used to measure the kernel's useful work, never by the product.
BUILD_COUNTERS = os.path.join(PKG_ROOT, "_build_counters")
COUNTERS_LIB_PATH = os.path.join(BUILD_COUNTERS, LIB_NAME)
CLI_PATH = os.path.join(BUILD, "skycube")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["api.cu", "prep.cu", "skyline.cu", "partition.cu", "mdmc.cu", "noalloc.cu",
              "prefilter.cu", "levels.cu"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build")
    return cand


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, flush=True)
    return r


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose=False, force=False, ptxas_verbose=False, counters=False):
    """Compiles the library and the CLI if any source is newer; returns LIB_PATH.
    counters=True builds the counters library instead (COUNTERS_LIB_PATH)."""
    out_dir = BUILD_COUNTERS if counters else BUILD
    lib_path = COUNTERS_LIB_PATH if counters else LIB_PATH
    os.makedirs(out_dir, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    headers.append(os.path.join(INCLUDE, "skycube_gb300.h"))
    common = ["-O3", "-std=c++17", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC",
              "-I", INCLUDE, "-I", CSRC]
    if ptxas_verbose:
        common += ["-Xptxas", "-v"]
    if counters:
        common += ["-DSKC_BITMAP_COUNTERS=1"]
    objs, jobs = [], []
    for src in CU_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(out_dir, src.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [path, *headers]):
            jobs.append([nvcc, *common, "-c", path, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, j, verbose) for j in jobs]:
            f.result()
    if force or jobs or _stale(lib_path, objs):
        _run([nvcc, "-shared", *ARCH, "-o", lib_path, *objs], verbose)
    if counters:
        return lib_path
    cli_src = os.path.join(HOST, "cli.cpp")
    if os.path.exists(cli_src):
        host_headers = [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")]
        if force or _stale(CLI_PATH, [cli_src, LIB_PATH, *host_headers]):
            _run(["g++", "-O2", "-std=c++17", "-I", INCLUDE, "-I", HOST, cli_src,
                  "-o", CLI_PATH, "-L", BUILD, "-lskycube_gb300",
                  f"-Wl,-rpath,{BUILD}", "-lpthread"], verbose)
    return LIB_PATH


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv, ptxas_verbose="--ptxas" in sys.argv)
    print(LIB_PATH)
