"""Widom's chemical potential (ForceField::CalcChemicalPotentialF,
cbmc.cc:444-531) in the CPU restatement against the reference itself: three
successive evaluations from the same seed (50 configurational-bias test
insertions each) give the same averages, so both also consumed the same
draws.

Each case runs in a fresh process: the reference keeps gasdev's cached
deviate in function statics shared by the whole process (misc.cc:112-113),
so an earlier run in the same process would change its draws; the
restatement keeps it per context."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = ["gcx_neutral", "gcx_charged", "muvt_neutral", "muvt_charged"]

CODE = r"""
import json, sys
sys.path.insert(0, %r)
from oracle import bindings as ob
R = ob.Ref(%r, seed=9)
O = ob.Oracle(%r, seed=9)
print(json.dumps([[R.chem_pot(), O.chem_pot()] for _ in range(3)]))
"""


@pytest.mark.parametrize("case", CASES)
def test_widom_average_matches_reference(built, case):
    from oracle import bindings as ob
    if not ob.have_ref():
        pytest.skip("reference library not built")
    d = os.path.join(ROOT, "tests", "golden", case)
    out = subprocess.run([sys.executable, "-c", CODE % (ROOT, d, d)], capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    vals = json.loads(out.stdout.strip().splitlines()[-1])
    for ref, mine in vals:
        assert abs(mine - ref) <= 1e-9 * abs(ref), (case, vals)
    assert any(ref > 0 for ref, _ in vals)
