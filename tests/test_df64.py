"""CPU check of the double-float arithmetic that the plain path's pair gates
use in the double-float mode (quantumlab_gb300/csrc/df64.cuh): conversions
between double and two floats by integer field operations, and the
compensated four-term dot product.  Compiled with g++, no GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_df64_bounds(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "df64_check"
    res = subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "quantumlab_gb300", "csrc"),
                          os.path.join(ROOT, "tests", "native", "df64_check.cpp"), "-o", str(exe)],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    v = {k: float(x) for k, x in (line.split() for line in out.stdout.strip().splitlines())}
    print(v)
    assert v["in_rel"] <= 2.0 ** -48                 # hi and the signed remainder each rounded to 24 bits
    assert v["in_abs_small"] <= 2.0 ** -97           # below 2^-73 the low part is dropped
    assert v["lo_not_below_ulp"] == 0
    assert v["out_rel"] <= 2.0 ** -53                # rounded to the nearest double
    assert v["pow2_rel"] <= 2.0 ** -53               # subtraction across a power of two
    assert v["dot4_rel_to_largest_term"] <= 2.0 ** -42       # four inputs at 2^-47 each, sums compensated
    assert v["exact_cases"] == 1
