"""The FP64 reconstruction kernel evaluates the limiter only at the faces that decide
phi (pyhype_gb300/csrc/e2d_slope_pick.cuh).  These CPU tests compile the pick for the
host and check, over millions of random and adversarial cells with four candidates
(one point per face) and with 8 and 12 (2 and 3 face quadrature points) (linear profiles, exact
and one-ulp ties, uniform regions, slopes at the limiters' special points and on the
falling branch, zeros of both signs, subnormals, infinities, NaN), that phi from the
picked faces equals phi from all four faces bit for bit, for all four limiters.  The
second test weakens each safeguard of the pick in a copy and checks that the harness
then finds mismatches, so a pass means something."""
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
HEADER = os.path.join(ROOT, "pyhype_gb300", "csrc", "e2d_slope_pick.cuh")
SOURCE = os.path.join(HERE, "slope_pick_check.cpp")


def _compile(tmp, header_text=None):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    os.makedirs(os.path.join(tmp, "pyhype_gb300", "csrc"), exist_ok=True)
    os.makedirs(os.path.join(tmp, "tests"), exist_ok=True)
    with open(HEADER) as f:
        text = f.read()
    with open(os.path.join(tmp, "pyhype_gb300", "csrc", "e2d_slope_pick.cuh"), "w") as f:
        f.write(text if header_text is None else header_text(text))
    shutil.copy(SOURCE, os.path.join(tmp, "tests", "slope_pick_check.cpp"))
    exe = os.path.join(tmp, "check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-Wno-unknown-pragmas",
                    os.path.join(tmp, "tests", "slope_pick_check.cpp"), "-o", exe], check=True)
    return exe


def _run(exe, cases, seed):
    r = subprocess.run([exe, str(cases), str(seed)], capture_output=True, text=True)
    out = {}
    for line in r.stdout.splitlines():  # "<lim> ..." four candidates, "<lim>+ ..." 8 or 12
        lim, rest = line.split(" ", 1)
        out[lim] = {k: int(v) for k, v in re.findall(r"(\w+)=(\d+)", rest)}
    return r.returncode, out


def test_pick_equals_all_faces(tmp_path):
    exe = _compile(str(tmp_path))
    for seed in (1, 2):
        rc, out = _run(exe, 1_500_000, seed)
        assert set(out) == {"0", "1", "2", "3", "0+", "1+", "2+", "3+"}
        for lim, c in out.items():
            assert c["mismatches"] == 0, (lim, seed, c)
            assert c["fallback"] < 0.3 * c["cases"], (lim, c)  # the pick mostly applies
        assert rc == 0


@pytest.mark.parametrize("mutation,limiters", [
    (("kTau = 1e-5f", "kTau = 1e-8f"), (0, 1, 2, 3)),                 # ties too narrow
    (("kPsiSep = 1e-5f", "kPsiSep = 2e-7f"), (0, 2)),                # psi ordering too tight
    (("kFallingLimit = 1e8f", "kFallingLimit = 1e30f"), (0, 2)),     # falling branch unguarded
    (("1.99f : 0.99f", "2.01f : 1.01f"), (0, 2)),                    # psi = 1 threshold wrong
    (("if (LIM == 1 && zpos && zneg) ok = false;", ""), (1,)),       # signed zero slopes
])
def test_harness_detects_weakened_pick(tmp_path, mutation, limiters):
    old, new = mutation

    def weaken(text):
        assert text.count(old) == 1
        return text.replace(old, new)

    exe = _compile(str(tmp_path), weaken)
    rc, out = _run(exe, 1_500_000, 5)
    assert rc != 0
    for lim in limiters:
        assert out[str(lim)]["mismatches"] > 0, (mutation, lim, out[str(lim)])
