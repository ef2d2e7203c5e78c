"""Host-side facts the step kernels rely on (no GPU): the per-net flag that lets the
neuron passes stop a fold once the neuron is certain to fire (it must be false whenever
a term can be negative) and the id range that input requests test first.  Compiles
tests/cpp/host_flags.cpp against neurocorrelation_gb300/csrc/nc_host.cpp with g++."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "neurocorrelation_gb300", "csrc")
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


def test_host_flags(tmp_path):
    if not os.path.exists(os.path.join(CUDA_INC, "vector_types.h")):
        pytest.skip("CUDA headers not found")
    exe = str(tmp_path / "host_flags")
    subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-I" + CSRC, "-I" + CUDA_INC,
                    os.path.join(ROOT, "tests", "cpp", "host_flags.cpp"), os.path.join(CSRC, "nc_host.cpp"),
                    "-o", exe, "-lpthread"], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("OK")
