"""The library's readers of run.in and the coordinate / topology files
(plum_gb300/csrc/host/input.cc; the C ABI builds every device context from
them) and its Ewald set-up (host/ewald_setup.cc: Ewald box, cut-offs, cells,
the k-set and its weights) against the oracle's on every case directory:
everything must be identical (tests/input_reader_harness.cc). Malformed
input is an error with a message, where the reference would exit or read
forever (potential_truncated_lj.cc:31-35)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(HERE, "golden")
DIRS = sorted(d for d in os.listdir(GOLDEN)
              if os.path.isfile(os.path.join(GOLDEN, d, "input_crd.dat")))


@pytest.fixture(scope="module")
def harness(built, tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("reader") / "input_reader_harness")
    lib = os.path.join(ROOT, "oracle", "_ref")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-o", exe,
                        os.path.join(HERE, "input_reader_harness.cc"),
                        os.path.join(ROOT, "plum_gb300", "csrc", "host", "input.cc"),
                        os.path.join(ROOT, "plum_gb300", "csrc", "host", "ewald_setup.cc"),
                        "-L" + lib, "-loracle", "-Wl,-rpath," + lib], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_every_case_directory_is_covered():
    assert len(DIRS) >= 14
    assert {"bulk_small", "slab_lj", "muvt_charged", "slab_charged_sites"} <= set(DIRS)


@pytest.mark.parametrize("case", DIRS)
def test_library_reader_matches_oracle(harness, case):
    out = subprocess.run([harness, os.path.join(GOLDEN, case)], capture_output=True, text=True,
                         timeout=120)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr
    assert int(out.stdout.split()[3]) > 0  # every case has Ewald: its k-set was compared


@pytest.mark.parametrize("workload", ["bulk_1000", "bulk_20000_pinned", "brush"])
def test_library_reader_matches_oracle_on_generated_workloads(harness, tmp_path, workload):
    """The generators' workloads at full size: the measured 20,000-bead
    system (with the trailing plum_* Ewald items), the 1,000-bead one, and a
    confined brush replica of the batched workload."""
    from plum_gb300 import systems
    d = str(tmp_path / workload)
    if workload == "brush":
        systems.write_brush(d, systems.brush_ensemble(1, seed=20261203)[0], seed=20261203)
    else:
        systems.write_bulk(d, systems.CONFIGS[workload], seed=20261203)
    out = subprocess.run([harness, d], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr
    assert int(out.stdout.split()[3]) > 0


def _copy_case(case, dst):
    for f in ("run.in", "input_crd.dat", "input_top.dat"):
        shutil.copy(os.path.join(GOLDEN, case, f), dst / f)
    return (dst / "run.in").read_text().splitlines()


def test_table_without_end_is_an_error(harness, tmp_path):
    lines = _copy_case("bulk_small", tmp_path)
    ends = [i for i, ln in enumerate(lines) if ln.split()[-1:] == ["end"]]
    assert ends
    (tmp_path / "run.in").write_text("\n".join(lines[:ends[0]]) + "\n")
    out = subprocess.run([harness, str(tmp_path), "library"], capture_output=True, text=True,
                         timeout=60)
    assert out.returncode == 1 and "library reader:" in out.stdout, out.stdout


def test_missing_coordinate_file_is_an_error(harness, tmp_path):
    _copy_case("bulk_small", tmp_path)
    os.remove(tmp_path / "input_crd.dat")
    out = subprocess.run([harness, str(tmp_path), "library"], capture_output=True, text=True,
                         timeout=60)
    assert out.returncode == 1 and "input_crd.dat" in out.stdout, out.stdout


def test_truncated_coordinates_are_an_error(harness, tmp_path):
    _copy_case("bulk_small", tmp_path)
    rows = (tmp_path / "input_crd.dat").read_text().splitlines()
    (tmp_path / "input_crd.dat").write_text("\n".join(rows[:len(rows) // 2]) + "\n")
    out = subprocess.run([harness, str(tmp_path), "library"], capture_output=True, text=True,
                         timeout=60)
    assert out.returncode == 1, out.stdout


def test_readers_are_clean_under_sanitizers(built, tmp_path):
    """The readers and the Ewald set-up built with AddressSanitizer and
    UndefinedBehaviorSanitizer: well-formed cases and cut-off or corrupted
    files end without a sanitizer report (malformed input is an error)."""
    exe = str(tmp_path / "reader_asan")
    lib = os.path.join(ROOT, "oracle", "_ref")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined",
                        "-fno-omit-frame-pointer", "-o", exe,
                        os.path.join(HERE, "input_reader_harness.cc"),
                        os.path.join(ROOT, "plum_gb300", "csrc", "host", "input.cc"),
                        os.path.join(ROOT, "plum_gb300", "csrc", "host", "ewald_setup.cc"),
                        "-L" + lib, "-loracle", "-Wl,-rpath," + lib], capture_output=True,
                       text=True)
    if r.returncode != 0:
        pytest.skip("no sanitizer runtime: " + r.stderr[-200:])
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1", UBSAN_OPTIONS="print_stacktrace=1")

    def run(d, *extra):
        out = subprocess.run([exe, d, *extra], capture_output=True, text=True, timeout=300,
                             env=env)
        assert "Sanitizer" not in out.stderr and "runtime error" not in out.stderr, out.stderr
        return out

    for case in ("bulk_small", "slab_lj", "muvt_charged"):
        assert run(os.path.join(GOLDEN, case)).returncode == 0
    lines = _copy_case("bulk_small", tmp_path)
    for cut in (3, 20, len(lines) - 3):
        (tmp_path / "run.in").write_text("\n".join(lines[:cut]) + "\n")
        assert run(str(tmp_path), "library").returncode == 1
    (tmp_path / "run.in").write_text("\n".join(lines) + "\n")
    rows = (tmp_path / "input_crd.dat").read_text().splitlines()
    (tmp_path / "input_crd.dat").write_text("\n".join(rows[:2] + ["x y z"] + rows[3:]) + "\n")
    assert run(str(tmp_path), "library").returncode == 1
