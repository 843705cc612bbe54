"""Build the galaexi_gb300 shared library (CUDA for sm_103a + host C++), in-tree.

One translation unit per polynomial degree (dg_np<N+1>.cu) plus the C-ABI and host files are
compiled in parallel with nvcc and linked into galaexi_gb300/_build/libgalaexi_gb300.so.
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgalaexi_gb300.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3"]


def sources():
    srcs = ["dg_api.cu", "dg_host.cpp", "dg_hdf5.cpp", "dg_hopr.cpp", "dg_noalloc.cu"] + [
        "dg_np%d.cu" % np_ for np_ in range(2, 11)]
    return [os.path.join(CSRC, s) for s in srcs]


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "galaexi_gb300.h")]


def _compile(src):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    newest_dep = max(os.path.getmtime(d) for d in _deps())
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(newest_dep, os.path.getmtime(__file__)):
        return obj, None
    if src.endswith(".cpp"):
        cmd = [NVCC, "-x", "c++", "-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-c", src, "-o", obj]
    else:
        cmd = [NVCC] + CUFLAGS + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, "compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr)
    return obj, None


def build(verbose=True, jobs=None):
    """Compile (incrementally) and link the library; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(_compile, srcs))
    errs = [e for _, e in results if e]
    if errs:
        raise RuntimeError("\n".join(errs))
    objs = [o for o, _ in results]
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build()
    sys.exit(0)
