"""The search epilogue's division-free rad -> deg (k_finish_outputs,
div_pi_rn: Markstein's correction of RN(v * RN(1/pi))) gives the IEEE
quotient v / pi bit for bit: checked on the host with the same IEEE
operations (tests/c_checks/div_pi_check.c) over 54M values, lattice sums as
the search forms them with their ulp neighbours, sector sums and random
doubles."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_checks", "div_pi_check.c")


def test_division_free_quotient_is_correctly_rounded(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "div_pi_check")
    r = subprocess.run([cc, "-std=c99", "-O2", "-ffp-contract=off", "-Wall", "-Wextra",
                        "-Werror", SRC, "-o", exe, "-lm"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout and "checked 54027960" in r.stdout
