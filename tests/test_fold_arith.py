"""The fold's `float += double` without FP64 instructions (neurocorrelation_gb300/csrc/
nc_fold.h): its host build against (float)((double)p + T) on constructed ties, real fold
sequences and random bit patterns (tests/cpp/fold_check.cpp).  The device kernels use the
same header; the GPU parity tests check them bit for bit against the oracle."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_fold_arithmetic_matches_double_add(tmp_path):
    exe = str(tmp_path / "fold_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I" + os.path.join(ROOT, "neurocorrelation_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "cpp", "fold_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe, "4"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    line = r.stdout.strip().splitlines()[-1]
    words = line.split()
    assert words[0] == "cases" and int(words[1]) > 20_000_000
    assert words[3] == "0", line
