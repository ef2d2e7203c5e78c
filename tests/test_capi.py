"""The C-ABI library without a GPU: exports, builders, failure without a device."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from scenario import load

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "neucor_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nc_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(nc):
    lib = nc.load_library()
    names = declared_functions()
    assert len(names) >= 30
    out = subprocess.run(["nm", "-D", "--defined-only", nc.library_path()], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT\s+(nc_[a-z0-9_]+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        getattr(lib, n)


def test_philox_known_answers(nc):
    assert [hex(x) for x in nc.philox4x32_10([0, 0, 0, 0], [0, 0])] == \
        ["0x6627e8d5", "0xe169c58d", "0xbc57ac4c", "0x9b00dbd8"]
    assert [hex(x) for x in nc.philox4x32_10([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                                             [0xa4093822, 0x299f31d0])] == \
        ["0xd16cfe09", "0x94fdcceb", "0x5001e420", "0x24126ea1"]


def test_reference_constructor_reproduced(nc):
    """nc_build_reference_random after srand(3) == the reference's NeuCor(60) after srand(3)."""
    fx = load("construct_n60_seed3")
    xyz, pre, post, w = nc.build_reference_random(60, 3)
    np.testing.assert_array_equal(xyz.view(np.uint32), fx["xyz"].view(np.uint32))
    np.testing.assert_array_equal(pre, fx["pre"])
    np.testing.assert_array_equal(post, fx["post"])
    np.testing.assert_array_equal(w.view(np.uint32), fx["w"].view(np.uint32))


def test_reference_lengths_match_oracle_delays(oracle_mod):
    """coord3::getDist lengths recorded from the reference give the oracle's delays."""
    O = oracle_mod
    fx = load("construct_n60_seed3")
    o = O.OracleS(fx["xyz"], fx["pre"], fx["post"], fx["w"], params=O.default_params())
    want = np.array([O.lib().ncs_delay_steps(float(x), 1.0) for x in fx["length"]], dtype=np.int32)
    np.testing.assert_array_equal(o.delays(), want)


def test_knn_builder_matches_brute_force(nc):
    n, k = 400, 12
    xyz, pre, post, w = nc.build_knn(n, k, 8.0, seed=5)
    assert xyz.min() >= 0 and xyz.max() <= (n / 8.0) ** (1 / 3) + 1e-5
    d = np.sqrt(((xyz[:, None, :] - xyz[None, :, :]) ** 2).sum(-1, dtype=np.float32)).astype(np.float32)
    np.fill_diagonal(d, np.inf)
    for i in range(0, n, 7):
        want = np.lexsort((np.arange(n), d[i]))[:k]
        got = post[i * k:(i + 1) * k]
        np.testing.assert_array_equal(np.sort(got), np.sort(want))
    assert np.all(pre == np.repeat(np.arange(n), k))
    assert w.min() >= 0 and w.max() < 1


def test_knn_builder_deterministic(nc):
    a = nc.build_knn(300, 10, 8.0, seed=9)
    b = nc.build_knn(300, 10, 8.0, seed=9)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_create_without_device_fails_loudly(nc):
    if nc.device_count() > 0:
        pytest.skip("a CUDA device is present")
    xyz, pre, post, w = nc.build_knn(64, 4, 8.0, seed=1)
    with pytest.raises(nc.NeuCorError) as e:
        nc.NeuCor.from_arrays(xyz, pre, post, w)
    assert e.value.code == -5


def test_unsupported_operations_are_reported(nc):
    lib = nc.load_library()
    assert lib.nc_delete_synapse(None, 0, 1) == -4
    assert lib.nc_delete_neuron(None, 0) == -4


@pytest.mark.parametrize("n,k,seed", [(300, 299, 1), (2000, 30, 5), (1000, 50, 1), (20000, 100, 7)])
def test_oracle_knn_builder_equals_library_builder(nc, oracle_mod, n, k, seed):
    """The oracle's own kNN restatement (oracle/nc_knn.c, used where the library must not
    be loaded) and the library's host builder make the same network, bit for bit."""
    a = oracle_mod.build_knn(n, k, 8.0, seed)
    b = nc.build_knn(n, k, 8.0, seed=seed)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.view(np.uint32) if x.dtype == np.float32 else x,
                                      y.view(np.uint32) if y.dtype == np.float32 else y)


def test_oracle_knn_builder_matches_brute_force(oracle_mod):
    n, k = 500, 20
    xyz, pre, post, w = oracle_mod.build_knn(n, k, 8.0, 3)
    d = np.sqrt(((xyz[:, None, :] - xyz[None, :, :]) ** 2).sum(-1, dtype=np.float32)).astype(np.float32)
    np.fill_diagonal(d, np.inf)
    for i in range(n):
        np.testing.assert_array_equal(post[i * k:(i + 1) * k], np.lexsort((np.arange(n), d[i]))[:k])
