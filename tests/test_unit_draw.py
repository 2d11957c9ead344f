"""The serial step's draws u = x / (2^32 - 1) without a division
(plum_gb300/csrc/unit_draw.h): the header's C build against the IEEE
division (double)x / 4294967295.0 for every 32-bit x. The device build is
the same arithmetic with the CUDA intrinsics (count of leading zeros,
round-to-nearest conversion, bit casts); the GPU replay tests check it
against the oracle's draw sequences."""
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
