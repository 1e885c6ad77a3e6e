"""The exact-rounding helpers the kernels use (gm_exact_math.h), compiled on
the CPU as C and checked against the rounding they must reproduce: the
integer-only fixed-point conversion against nearbyint(v * 2^40), and the
Markstein-corrected division by dt against the division (CPU only)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "geodesic-m_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("gcc not found")
    exe = str(tmp_path_factory.mktemp("exact") / "exact_arith_check")
    subprocess.run([cc, "-std=c11", "-O2", "-ffp-contract=off", "-I", CSRC, "-o", exe,
                    os.path.join(HERE, "exact_arith_check.c"), "-lm"], check=True)
    return exe


def test_fixed_point_conversion_and_resync_division_are_exact(checker):
    out = subprocess.run([checker, "4000000"], capture_output=True, text=True)
    counts = {line.split()[0]: (int(line.split()[1]), int(line.split()[2])) for line in out.stdout.splitlines()}
    assert counts["f2fix"][0] > 3_000_000 and counts["div"][0] == 4_000_000, counts
    assert counts["f2fix"][1] == 0 and counts["div"][1] == 0, counts
    assert out.returncode == 0
