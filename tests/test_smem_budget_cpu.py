"""Shared-memory budgets of the mixed form's persistent kernels (galaexi_gb300/csrc/dg_lines.cuh).

Their speed rests on how many blocks share an SM: two double-buffered blocks of k_volume_lines at
n = 8 (168 registers each: the register file holds two) and four of k_prolong_gl (512 threads each).
The layouts are constexpr structs; a host program built with nvcc from the same header prints them,
and the test checks them against GB300's shared memory (228 KB per SM, at most 227 KB per block,
1 KB reserved per block).  No GPU is needed.
"""
import os
import shutil
import subprocess

import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "galaexi_gb300", "csrc")

SM_BYTES = 228 * 1024
BLOCK_MAX = 227 * 1024
RESERVED = 1024

HARNESS = r"""
#include "dg_kernels.cuh"  // includes dg_lines.cuh after the definitions it uses
#include <cstdio>
template <int NP> void vol() {
  printf("vol %d %zu %zu\n", NP, gx::VolLinesSmem<NP>::bytes, gx::VolLinesSmem<NP>::buffer);
}
int main() {
  vol<4>(); vol<5>(); vol<6>(); vol<7>(); vol<8>();
  printf("prolong 6 %zu\n", gx::ProlongGLSmem<6>::bytes);
  printf("prolong 8 %zu\n", gx::ProlongGLSmem<8>::bytes);
  return 0;
}
"""


def _layouts(tmp_path):
    nvcc = shutil.which("nvcc")
    if not nvcc:
        pytest.skip("needs nvcc")
    src = tmp_path / "smem.cu"
    src.write_text(HARNESS)
    exe = tmp_path / "smem"
    subprocess.run([nvcc, "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-I", CSRC, str(src), "-o",
                    str(exe)], check=True, capture_output=True, timeout=600)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=60).stdout
    vol, prolong = {}, {}
    for line in out.splitlines():
        f = line.split()
        if f[0] == "vol":
            vol[int(f[1])] = (int(f[2]), int(f[3]))
        else:
            prolong[int(f[1])] = int(f[2])
    return vol, prolong


def test_persistent_kernels_fit_their_blocks_per_sm(tmp_path):
    vol, prolong = _layouts(tmp_path)
    static = 16  # the two mbarriers
    for NP, (total, buf) in vol.items():
        assert total == 2 * buf and buf % 16 == 0, NP
        assert total + static <= BLOCK_MAX, NP
    # n = 8: two blocks of k_volume_lines per SM
    assert 2 * (vol[8][0] + static + RESERVED) <= SM_BYTES, vol[8]
    # k_prolong_gl: four blocks of 512 threads (n = 8) per SM
    assert 4 * (prolong[8] + static + RESERVED) <= SM_BYTES, prolong[8]
    assert prolong[8] == 2 * (5 * 512 * 8 + 64)
