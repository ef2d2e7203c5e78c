"""The C++ class interface (include/neucor_gb300.hpp) used the way the reference's
presets use NeuCor."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "few_neurons.cpp")
PRESET = os.path.join(ROOT, "tests", "cpp", "few_neurons_preset.cpp")


def compile_demo(out_path, nc, src=SRC):
    libdir = os.path.dirname(nc.library_path())
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I" + os.path.join(ROOT, "include"), src, "-o", out_path,
                    "-L" + libdir, "-lneucor_gb300", "-Wl,-rpath," + libdir], check=True)


def test_shim_compiles_and_links(nc, tmp_path):
    compile_demo(str(tmp_path / "few"), nc)
    compile_demo(str(tmp_path / "preset"), nc, PRESET)


@pytest.mark.gpu
def test_shim_few_neurons_preset_with_periodic_inputs(nc, oracle_mod, tmp_path):
    """The reference's FEW_NEURONS preset as src/main.cpp:162-189 sets it up (periodic
    inputs through setInputRateArray / addInputOffset, runSpeed 0.02 ms): the GPU matches
    the oracle's InputFirer restatement bit for bit and reaches the essay's result,
    w(0->1) = 1 and w(0->2) = 0."""
    exe = str(tmp_path / "preset")
    compile_demo(exe, nc, PRESET)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {int(l.split()[0]): (float(l.split()[1]), float(l.split()[2])) for l in out if l and l[0].isdigit()}
    O = oracle_mod
    xyz = np.array([[0, 0, 0], [0.3, 0.3, 0], [0.3, -0.3, 0]], np.float32)
    o = O.OracleS(xyz, [0, 0], [1, 2], [0.5, 0.5], params=O.default_params(seed=1, run_speed=0.02))
    o.set_firers([50.0, 50.0, 50.0], xyz, [0.1, 0.1, 0.1])
    o.add_firer_offset(1, 2.0)
    o.add_firer_offset(2, -2.0)
    done = 0
    for mark in (2500, 5000, 7500, 12500):
        o.run(mark - done)
        done = mark
        w = o.weights()
        assert np.float32(got[mark][0]) == w[0] and np.float32(got[mark][1]) == w[1], (mark, got[mark], w)
    assert got[12500] == (1.0, 0.0)


@pytest.mark.gpu
def test_shim_few_neurons_matches_oracle(nc, oracle_mod, tmp_path):
    exe = str(tmp_path / "few")
    compile_demo(exe, nc)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {int(l.split()[0]): (float(l.split()[1]), float(l.split()[2])) for l in out if l and l[0].isdigit()}
    O = oracle_mod
    xyz = np.array([[0, 0, 0], [0.3, 0.3, 0], [0.3, -0.3, 0]], np.float32)
    o = O.OracleS(xyz, [0, 0], [1, 2], [0.5, 0.5], params=O.default_params(seed=1))
    for t in range(1, 251):
        due = [i for i, off in enumerate((0, 2, -2)) if (t - off) % 20 == 0 and t - off > 0]
        if due:
            o.schedule_fire(due)
        o.run(1)
        if t in got:
            w = o.weights()
            assert np.float32(got[t][0]) == w[0] and np.float32(got[t][1]) == w[1], (t, got[t], w)
    assert got[250] == (1.0, 0.0)
