"""Reasons for the plugin's bound changes (scip_gb300/plugin/gpulinear_reason.c): the row that implies a change and
the bounds cons_linear's addConflictBounds would add for it (cons_linear.c:4799-4970), on hand-checkable rows."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

EXPECTED = {
    # x0 + x1 + x2 + x3 <= 1, x0 = 1 => x3 <= 0: the integral reason stops once x0 used up the capacity
    "packing": "row 0 adds L0",
    # x0 + x2 <= 5 cannot imply x2 <= 0; x1 + x2 <= 1 with x1 = 1 can
    "second_row": "row 1 adds L1",
    # continuous column: every responsible bound
    "continuous": "row 0 adds L0 U1",
    # -x2 + x0 + x1 >= 1 with x0 = x1 = 0 => x2 <= -1 needs both upper bounds
    "lhs_negative": "row 0 adds U0 U1",
    "none": "row -1 adds",
    # x0 + x1 - y <= 1 with x0 = x1 = 1 => y >= 1
    "indicator": "row 0 adds L0 L1",
}


def test_reasons(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "reason_driver")
    subprocess.run([cc, "-std=c99", "-O1", "-I" + os.path.join(ROOT, "scip_gb300", "plugin"),
                    os.path.join(ROOT, "tests", "plugin", "reason_driver.c"),
                    os.path.join(ROOT, "scip_gb300", "plugin", "gpulinear_reason.c"), "-lm", "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.strip().splitlines()
    got = {line.split(" ", 1)[0]: line.split(" ", 1)[1].strip() for line in out}
    assert got == EXPECTED
