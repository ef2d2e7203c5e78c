"""The GPU step on the two large workloads against the oracle, bit for bit, through
SHA-256 digests of the oracle's outputs (tests/golden/make_digests.py ran the oracle
once on the CPU; at these sizes it is too slow to run beside the GPU).

* 100,000 neurons x 100 nearest targets (10M synapses), 200 inputs in 10 correlated
  groups at 5-40 Hz: the first 1,000 steps in both forms of the step kernels — every
  100-step block of the spike raster, and the potentials, weights and counters after
  steps 300 and 1,000.
* 2,000,000 neurons x 200 nearest targets (400M synapses) built on the GPU
  (nc_create_knn), 2,000 inputs in 20 correlated groups at 10-40 Hz: the first 20
  steps — every step's raster row, and the potentials, weights and counters after
  step 20.

A digest says only that something differs.  To localise a mismatch, rerun the same
workload at the first mismatching block step by step on the GPU and on the oracle
(OracleS over the network from oracle.build_knn) and compare the rows of that block,
then the potentials of its steps, as tests/test_gpu_parity.py does on small networks."""
import hashlib

import numpy as np
import pytest

from scenario import load

pytestmark = pytest.mark.gpu

MODES = {"dense": 0, "event": 1}


def sha(a) -> bytes:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest()


def groups_of(fx):
    return [dict(first=int(g[0]), count=int(g[1]), rate_hz=float(g[2]), correlated=int(g[3]), jitter=int(g[4]))
            for g in fx["groups"]]


def check(net, fx, label):
    """Runs the fixture's steps block by block and compares every digest."""
    steps, block = int(fx["steps"]), int(fx["block"])
    cks = [int(c) for c in fx["checkpoints"]]
    done, b = 0, 0
    while done < steps:
        m = min(block, steps - done)
        net.record_raster(m)
        net.run(m)
        r = net.raster()
        fires = np.unpackbits(r, axis=1, bitorder="little")[:, :net.n].sum(1)
        if sha(r) != fx["raster_sha"][b].tobytes():
            bad = np.nonzero(fires != fx["fires"][done:done + m])[0]
            at = done + 1 + int(bad[0]) if bad.size else None
            raise AssertionError(f"{label}: raster of steps {done + 1}-{done + m} differs "
                                 f"(first step with another fire count: {at})")
        done += m
        b += 1
        if done in cks:
            q = cks.index(done)
            assert sha(net.potentials()) == fx["pot_sha"][q].tobytes(), f"{label}: potentials after step {done}"
            assert sha(net.weights()) == fx["w_sha"][q].tobytes(), f"{label}: weights after step {done}"
            st = net.stats()
            assert [st["fires"], st["launched"], st["dropped"]] == list(fx["counts"][q]), \
                f"{label}: counters after step {done}"


@pytest.mark.parametrize("mode", MODES)
def test_gpu_c2_1000_bit_exact(nc, mode):
    G = nc
    fx = load("c2_digests")
    xyz, pre, post, w = G.build_knn(int(fx["n"]), int(fx["k"]), 8.0, seed=int(fx["net_seed"]))
    net = G.NeuCor.from_arrays(xyz, pre, post, w,
                               params=G.default_params(seed=int(fx["sim_seed"]), step_mode=MODES[mode]))
    net.set_input_groups(groups_of(fx))
    check(net, fx, f"100k x 100, {mode} form")
    net.close()


def test_gpu_c5_prefix_bit_exact(nc):
    G = nc
    fx = load("c5_digests")
    net = G.NeuCor.knn(int(fx["n"]), int(fx["k"]), 8.0, seed=int(fx["net_seed"]),
                       params=G.default_params(seed=int(fx["sim_seed"])))
    net.set_input_groups(groups_of(fx))
    check(net, fx, "2M x 200, built on the GPU")
    net.close()
