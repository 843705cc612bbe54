"""The mixed form's integer-pipe FP64 <-> FP32 conversions (galaexi_gb300/csrc/dg_convert.cuh).

The header is compiled for the host with g++ and its f64_to_f32_rn / f32_to_f64 are compared bit for
bit with the host's IEEE-754 conversions (round to nearest, ties to even; the GPU's conversion
instructions round the same way).  Inputs: random bit patterns (every class of double), values
across the float range, values a few ulps around float rounding ties and carries, the edge cases
(signed zeros, subnormals, FLT_MAX and the overflow boundary, infinities, NaN), and every 7th float
bit pattern for the widening conversion.
"""
import os
import shutil
import subprocess

import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "galaexi_gb300", "csrc")

HARNESS = r"""
#include "dg_convert.cuh"
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

static bool same(float a, float b) {
  unsigned x, y;
  memcpy(&x, &a, 4);
  memcpy(&y, &b, 4);
  return x == y || (std::isnan(a) && std::isnan(b));
}
static bool same(double a, double b) {
  unsigned long long x, y;
  memcpy(&x, &a, 8);
  memcpy(&y, &b, 8);
  return x == y || (std::isnan(a) && std::isnan(b));
}

int main() {
  std::mt19937_64 g(20261204);
  long bad = 0, checked = 0;
  auto chk = [&](double x) {
    ++checked;
    if (!same(gx::f64_to_f32_rn(x), (float)x)) {
      if (bad < 5) printf("narrow mismatch %a\n", x);
      ++bad;
    }
  };
  for (long i = 0; i < 4000000; ++i) {
    const uint64_t b = g();
    double x;
    memcpy(&x, &b, 8);
    chk(x);
  }
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  for (long i = 0; i < 2000000; ++i) {
    const double x = u(g) * std::ldexp(1.0, (int)(g() % 300) - 150);
    chk(x);
    // a float value plus exactly half an ulp (a tie) or just below it
    double t = (double)(float)x;
    uint64_t b;
    memcpy(&b, &t, 8);
    b += (g() & 1) ? (1ull << 28) : ((1ull << 28) - 1);
    memcpy(&t, &b, 8);
    chk(t);
    chk(-t);
  }
  const double edge[] = {0.0, -0.0, FLT_MAX, (double)FLT_MAX * (1 + 1e-8), (double)FLT_MAX * (1 + 1e-7), FLT_MIN,
                         FLT_MIN * 0.5, -FLT_MIN * 0.75, 1e-300, -1e300, INFINITY, -INFINITY, NAN, 1.0, 0.1,
                         71.42857142857143, 3.4028235677973366e38, 3.4028234663852886e38, 1.1754942807573643e-38};
  for (double x : edge) chk(x);
  long bad2 = 0;
  for (uint64_t w = 0; w < (1ull << 32); w += 7) {
    const unsigned v = (unsigned)w;
    float f;
    memcpy(&f, &v, 4);
    if (!same(gx::f32_to_f64(f), (double)f)) {
      if (bad2 < 5) printf("widen mismatch %a\n", f);
      ++bad2;
    }
  }
  printf("%ld %ld %ld\n", checked, bad, bad2);
  return 0;
}
"""


def _cuda_include():
    for root in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if root and os.path.exists(os.path.join(root, "include", "cuda_runtime.h")):
            return os.path.join(root, "include")
    nvcc = shutil.which("nvcc")
    if nvcc:
        inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
        if os.path.exists(os.path.join(inc, "cuda_runtime.h")):
            return inc
    return None


def test_integer_conversions_match_ieee_round_to_nearest(tmp_path):
    gxx = shutil.which("g++")
    inc = _cuda_include()
    if gxx is None or inc is None:
        pytest.skip("needs g++ and the CUDA headers")
    src = tmp_path / "conv.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "conv"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC, "-I", inc, str(src), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=300).stdout.split()
    checked, bad, bad2 = (int(v) for v in out[-3:])
    assert checked > 10_000_000
    assert bad == 0 and bad2 == 0, out
