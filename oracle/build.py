"""Build the oracle (test infrastructure): oracle/_build/liboracle.so from dgsem_oracle.cpp."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "dgsem_oracle.cpp")
LIB = os.path.join(HERE, "_build", "liboracle.so")


def build(verbose=True):
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    deps = [SRC, os.path.join(HERE, "..", "include", "galaexi_gb300.h"), __file__]
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-fno-fast-math", "-ffp-contract=off",
           SRC, "-o", LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s" % (" ".join(cmd), r.stderr))
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build()
