"""Build recipe for librg.so (the GB300 frontier engine).

Compiles every CUDA translation unit for sm_103a only and the host C++ with
OpenMP, in parallel, into radar-graph_gb300/_build/, links
radar-graph_gb300/librg.so, then builds the command-line apps (apps/*.cc ->
bin/PageRank, bin/BFS, bin/BC, bin/Radii) against it, and the benchmark's
measurement aid (measure/*.cu -> librg_probe.so, linked against librg.so;
not part of the product ABI).  Incremental: a unit is
rebuilt when its source or any header in csrc/ is newer than its object.

    python radar-graph_gb300/build.py [-v] [--force]
"""

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librg.so")
MEASURE = os.path.join(HERE, "measure")
PROBE_LIB = os.path.join(HERE, "librg_probe.so")
APPS = os.path.join(HERE, "apps")
BIN = os.path.join(HERE, "bin")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp",
                     "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-Wall", "-I", INCLUDE, "-I", CSRC]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_lib_dir():
    root = os.path.dirname(os.path.dirname(_nvcc()))
    for d in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"):
        p = os.path.join(root, d)
        if os.path.exists(os.path.join(p, "libcudart.so")) or os.path.exists(os.path.join(p, "libcudart_static.a")):
            return p
    return os.path.join(root, "lib64")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cc")))


def _headers_mtime():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "radar_graph.h"))
    return max(os.path.getmtime(h) for h in hs)


def _compile(src, force, verbose):
    obj = os.path.join(BUILD, src + ".o")
    path = os.path.join(CSRC, src)
    if (not force and os.path.exists(obj)
            and os.path.getmtime(obj) >= max(os.path.getmtime(path), _headers_mtime())):
        return obj
    if src.endswith(".cu"):
        cmd = [_nvcc()] + NVCC_FLAGS + ["-c", path, "-o", obj]
    else:
        cmd = [os.environ.get("CXX", "g++")] + CXX_FLAGS + ["-I", os.path.join(os.path.dirname(_nvcc()), "..", "include"),
                                                          "-c", path, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, flush=True)
    return obj


def build(force=False, verbose=False):
    """Builds librg.so if needed and returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, force, verbose), srcs))
    if (force or not os.path.exists(LIB)
            or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs)):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + [
            "-L", _cuda_lib_dir(), "-lcudart", "-Xcompiler", "-fopenmp", "-lgomp"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    build_apps(verbose)
    build_probe(force, verbose)
    return LIB


def build_probe(force=False, verbose=False):
    """librg_probe.so: measurement aids for the benchmark, linked against
    librg.so (graph handles, the thread's stream); librg.so does not export
    them."""
    srcs = sorted(f for f in os.listdir(MEASURE) if f.endswith(".cu"))
    newest = max([os.path.getmtime(os.path.join(MEASURE, f)) for f in srcs] + [_headers_mtime(), os.path.getmtime(LIB)])
    if not force and os.path.exists(PROBE_LIB) and os.path.getmtime(PROBE_LIB) >= newest:
        return PROBE_LIB
    cmd = [_nvcc()] + NVCC_FLAGS + ["-shared", "-o", PROBE_LIB] + [os.path.join(MEASURE, f) for f in srcs] + [
        "-L", HERE, "-lrg", "-L", _cuda_lib_dir(), "-lcudart", "-Xlinker", "-rpath,$ORIGIN"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"probe library build failed\n{r.stdout}\n{r.stderr}")
    return PROBE_LIB


def build_apps(verbose=False):
    """The CLI binaries: host C++ over the C ABI, found next to librg.so at run time."""
    os.makedirs(BIN, exist_ok=True)
    hdr = max(os.path.getmtime(os.path.join(APPS, "cli.h")), os.path.getmtime(os.path.join(INCLUDE, "radar_graph.h")))
    srcs = sorted(f for f in os.listdir(APPS) if f.endswith(".cc"))

    def one(src):
        exe = os.path.join(BIN, src[:-3])
        path = os.path.join(APPS, src)
        if (os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(path), hdr, os.path.getmtime(LIB))):
            return exe
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-Wall", "-I", INCLUDE, path, "-o", exe,
               "-L", HERE, "-lrg", "-Wl,-rpath,$ORIGIN/.."]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"app build failed: {src}\n{r.stdout}\n{r.stderr}")
        return exe

    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        return list(ex.map(one, srcs))


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("-v", "--verbose", action="store_true")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    try:
        print(build(force=a.force, verbose=a.verbose))
    except RuntimeError as e:
        print(e, file=sys.stderr)
        sys.exit(1)
