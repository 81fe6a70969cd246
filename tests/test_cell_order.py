"""The cutoff path's cell order (od_hilbert.h, the code the binning kernel runs), compiled for the
host: for every grid size the kernels use (2^1 .. 2^7 cells per axis) the key is a bijection onto
[0, G^3) and consecutive keys are face-adjacent cells (a Hilbert curve)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "opendust_gb300", "csrc")

HARNESS = r"""
#include <stdio.h>
#include <stdlib.h>
#include "od_hilbert.h"
int main(void) {
  for (int bits = 1; bits <= 7; bits++) {
    const int G = 1 << bits;
    const size_t n = (size_t)G * G * G;
    int* at = (int*)malloc(3 * n * sizeof(int));
    char* seen = (char*)calloc(n, 1);
    for (int x = 0; x < G; x++)
      for (int y = 0; y < G; y++)
        for (int z = 0; z < G; z++) {
          const uint32_t k = od_hilbert3(x, y, z, bits);
          if (k >= n || seen[k]) { printf("bits %d: not a bijection\n", bits); return 1; }
          seen[k] = 1; at[3 * k] = x; at[3 * k + 1] = y; at[3 * k + 2] = z;
        }
    for (size_t k = 1; k < n; k++) {
      const int d = abs(at[3 * k] - at[3 * k - 3]) + abs(at[3 * k + 1] - at[3 * k - 2]) +
                    abs(at[3 * k + 2] - at[3 * k - 1]);
      if (d != 1) { printf("bits %d: keys %zu and %zu not adjacent\n", bits, k - 1, k); return 1; }
    }
    free(at); free(seen);
  }
  printf("ok\n");
  return 0;
}
"""


def test_hilbert_cell_order(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "order.c"
    src.write_text(HARNESS)
    exe = tmp_path / "order"
    subprocess.run([cc, "-O2", "-std=c99", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout
