"""The serial step's draws u = x / (2^32 - 1) without a division and its
Metropolis test (plum_gb300/csrc/unit_draw.h): the header's C build against
the IEEE division (double)x / 4294967295.0 for every 32-bit x, and
metropolis(u, x) against u < exp(-x) on the draws at the edges of its
shortcuts. The device build is the same arithmetic with the CUDA intrinsics
(count of leading zeros, round-to-nearest conversion, bit casts) and the
device exp; the GPU replay tests check both against the oracle's decision
sequences."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(os.path.dirname(HERE), "plum_gb300", "csrc", "unit_draw.h")

DRIVER = r"""
#include <stdio.h>
#include "unit_draw.h"
int main(void) {
  unsigned long long bad = 0;
  for (unsigned long long x = 0; x <= 0xFFFFFFFFull; x++) {
    const double a = (double)(uint32_t)x / 4294967295.0;
    if (unit_draw((uint32_t)x) != a) bad++;
  }
  printf("%llu\n", bad);
  return bad != 0;
}
"""


def test_unit_draw_equals_the_division_for_every_word(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "chk.c"
    src.write_text(DRIVER)
    exe = tmp_path / "chk"
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-I", os.path.dirname(HEADER), str(src),
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0 and out.stdout.strip() == "0", out.stdout


METRO = r"""
#include <stdio.h>
#include <math.h>
#include "unit_draw.h"
static unsigned long long bad = 0, n = 0;
static void check(uint32_t w, double x) {
  const double u = unit_draw(w);
  n++;
  if (metropolis(u, x) != (u < exp(-x))) bad++;
}
int main(void) {
  const double xs[] = {-INFINITY, -1e3, -1.0, -1e-300, -0.0, 0.0, 4.9e-324, 1e-300, 1e-17,
                       1.1e-16, 1e-10, 0.5, 1.0, 5.0, 22.18, 22.9, 23.0, 23.0000000001, 23.5,
                       30.0, 100.0, 700.0, 745.0, 745.13, 745.2, 746.0, 800.0, INFINITY, NAN};
  uint64_t s = 88172645463325252ull;  /* xorshift words */
  for (unsigned i = 0; i < sizeof xs / sizeof xs[0]; i++) {
    const double x = xs[i];
    const uint32_t fixed[] = {0u, 1u, 2u, 3u, 0xFFFFFFFEu, 0xFFFFFFFFu, 0x80000000u};
    for (unsigned k = 0; k < sizeof fixed / sizeof fixed[0]; k++) check(fixed[k], x);
    if (x == x && x > -1e9 && x < 1e9) {  /* the words around the threshold exp(-x) M */
      const double t = exp(-x) * 4294967295.0;
      if (t >= 0.0 && t < 4294967295.0)
        for (long long d = -3; d <= 3; d++) {
          const long long w = (long long)t + d;
          if (w >= 0 && w <= 0xFFFFFFFFll) check((uint32_t)w, x);
        }
    }
    for (int k = 0; k < 200000; k++) {
      s ^= s << 13; s ^= s >> 7; s ^= s << 17;
      check((uint32_t)(s >> 32), x);
    }
  }
  printf("%llu %llu\n", bad, n);
  return bad != 0;
}
"""


def test_metropolis_equals_the_exponential_test(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "metro.c"
    src.write_text(METRO)
    exe = tmp_path / "metro"
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-I", os.path.dirname(HEADER), str(src),
                    "-o", str(exe), "-lm"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    bad, n = (int(v) for v in out.stdout.split())
    assert out.returncode == 0 and bad == 0 and n > 5_000_000, out.stdout
