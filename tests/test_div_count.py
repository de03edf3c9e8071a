"""The red-black pressure solve divides by a cell's non-solid neighbour count with one multiply and
two FMAs instead of an IEEE division (pressure_stream.cu, div_count). The claim that this is the
correctly rounded quotient rests on an exhaustive comparison with IEEE division over every 32-bit
float and every count 1 .. 6 (tests/div_count_check.c), run here on the host's cores."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_div_count_equals_ieee_division_for_every_float(tmp_path):
    cc = shutil.which(os.environ.get("CC", "gcc"))
    if not cc:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "div_count_check")
    subprocess.run([cc, "-O2", "-fopenmp", "-ffp-contract=off", "-o", exe, os.path.join(HERE, "div_count_check.c"),
                    "-lm"], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count(": 0 mismatches") == 6, r.stdout
