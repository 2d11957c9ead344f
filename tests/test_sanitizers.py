"""The CPU restatement (oracle/plum_oracle.c) built with AddressSanitizer and
UndefinedBehaviorSanitizer and driven through tests/slit_pressure_harness.cc:
reading each case, 120 steps of its Monte Carlo loop (exchange moves in the
grand-canonical cases) and two wall-force pressure evaluations end without a
sanitizer report, so the checker's own memory and arithmetic are sound where
it is used."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CASES = ["slab_charged_sites", "slab_lj", "slab_hardwall", "stat_slab", "bulk_small", "hs_bulk",
         "gcx_charged", "muvt_charged"]


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    d = tmp_path_factory.mktemp("san")
    flags = ["-O1", "-g", "-fsanitize=address,undefined", "-fno-omit-frame-pointer",
             "-ffp-contract=off"]
    obj, exe = str(d / "plum_oracle.o"), str(d / "harness")
    r = subprocess.run(["gcc", "-std=c11", *flags, "-c", os.path.join(ROOT, "oracle",
                                                                       "plum_oracle.c"),
                        "-o", obj], capture_output=True, text=True)
    if r.returncode == 0:
        r = subprocess.run(["g++", "-std=c++17", *flags, "-o", exe,
                            os.path.join(HERE, "slit_pressure_harness.cc"), obj, "-lm"],
                           capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("no sanitizer runtime: " + r.stderr[-200:])
    return exe


@pytest.mark.parametrize("case", CASES)
def test_oracle_is_clean_under_sanitizers(harness, case):
    out = subprocess.run([harness, os.path.join(HERE, "golden", case), "7", "60", "60"],
                         capture_output=True, text=True, timeout=600,
                         env=dict(os.environ, ASAN_OPTIONS="detect_leaks=1"))
    assert out.returncode == 0, out.stderr[-2000:]
    assert "Sanitizer" not in out.stderr and "runtime error" not in out.stderr, out.stderr[-2000:]
    assert len(out.stdout.splitlines()) == 2
