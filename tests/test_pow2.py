"""half()/twice() (pyhype_gb300/csrc/e2d_pow2.cuh) replace the FP64 kernels' scalings
by 0.5 and 2 with exponent arithmetic on the integer pipe.  This CPU test compiles
them for the host and compares them with the IEEE multiplications for every exponent
field (zeros, subnormals, the subnormal boundary, overflow, infinities, NaN) with
random and boundary significands of both signs."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_half_twice_equal_ieee_multiplication(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "pow2")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "pow2_check.cpp"), "-o", exe],
                   check=True)
    r = subprocess.run([exe, "1000", "3"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches=0" in r.stdout
