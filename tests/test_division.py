"""The horizon-slope division of VIEWSHED, checked against IEEE division.

The kernel computes s = RN(a/k) for an integer elevation difference a and a
step k as q0 = RN(a*y), s = RN(q0 + RN(a - k*q0)*y), with y = RN(1/k) from a
table and both corrections fused (fmaf).  One fused correction of a quotient
within an ulp, given a correctly rounded reciprocal, yields the correctly
rounded quotient (Markstein's theorem); this test runs the same operations on
the host (C fmaf and float division are IEEE round-to-nearest, as are the
device's __fmaf_rn and __fmul_rn) over every |a| <= 2^21 and k <= 2048, the
range the library sends to the table path (heights up to 10^6 over 16-bit
elevations, roi up to 2048), and requires bit-identical results.
"""
import os
import shutil
import subprocess
import tempfile

import pytest

SRC = r"""
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>
int main(int argc, char **argv) {
  const int amax = 1 << 21, kmax = 2048;
  long bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(dynamic)
  for (int k = 1; k <= kmax; k++) {
    volatile float fk = (float)k;
    volatile float y = 1.0f / fk;  /* RN(1/k), the table entry */
    for (int ia = -amax; ia <= amax; ia++) {
      const float a = (float)ia;
      volatile float q0 = a * y;
      const float s = fmaf(fmaf(-q0, fk, a), y, q0);
      volatile float want = a / fk;
      float w = want;
      uint32_t u1, u2;
      memcpy(&u1, &s, 4);
      memcpy(&u2, &w, 4);
      if (u1 != u2) bad++;
    }
  }
  printf("%ld\n", bad);
  return 0;
}
"""


def test_reciprocal_table_division_equals_ieee_division():
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "divchk.c")
        exe = os.path.join(d, "divchk")
        with open(src, "w") as f:
            f.write(SRC)
        # -ffp-contract=off: no contraction beyond the explicit fmaf calls
        subprocess.run([cc, "-O2", "-fopenmp", "-ffp-contract=off", src, "-o", exe, "-lm"],
                       check=True, capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=600)
    assert int(out.stdout.strip()) == 0
