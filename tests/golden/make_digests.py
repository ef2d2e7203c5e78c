"""Digests of the oracle on the two large GPU workloads (test fixtures).

The oracle (oracle/nc_oracle.c, the stepped CPU restatement pinned to the reference's
own code by the fixtures of make_golden.py) is too slow to run beside the GPU in a
test at these sizes, so it runs here once and the GPU tests compare SHA-256 digests:

* c2_digests.npz — 100,000 neurons x 100 nearest targets (10M synapses), 200 inputs in
  10 correlated groups at 5-40 Hz, seed 7 / 99, 1,000 steps: a digest of every
  100-step block of the spike raster, per-step fire counts, and digests of the
  potentials and weights (with the counters) after steps 300 and 1,000.
* c5_digests.npz — 2,000,000 neurons x 200 nearest targets (400M synapses), 2,000
  inputs in 20 correlated groups at 10-40 Hz, seed 5 / 5, 20 steps: a digest of every
  step's raster row, per-step fire counts, and digests of the potentials and weights
  (with the counters) after step 20.

Networks come from the oracle's own kNN restatement (oracle/nc_knn.c), which is the
network the library's host and device builders make.  Needs no reference tree and no
GPU; the C5 run needs about 25 GB of host memory.

    python tests/golden/make_digests.py [c2] [c5]
"""
import hashlib
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402


def sha(a) -> bytes:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest()


def c2_workload():
    rates = np.linspace(5.0, 40.0, 10)
    groups = [dict(first=20 * g, count=20, rate_hz=float(rates[g]), correlated=1, jitter=2) for g in range(10)]
    return dict(n=100_000, k=100, net_seed=7, sim_seed=99, groups=groups)


def c5_workload():
    rates = np.linspace(10.0, 40.0, 20)
    groups = [dict(first=100 * g, count=100, rate_hz=float(rates[g]), correlated=1, jitter=2) for g in range(20)]
    return dict(n=2_000_000, k=200, net_seed=5, sim_seed=5, groups=groups)


def run(wl, steps, block, checkpoints, name):
    t0 = time.time()
    xyz, pre, post, w = O.build_knn(wl["n"], wl["k"], 8.0, wl["net_seed"])
    print(name, "network built", round(time.time() - t0, 1), "s", flush=True)
    o = O.OracleS(xyz, pre, post, w, params=O.default_params(seed=wl["sim_seed"]), groups=wl["groups"])
    del xyz, pre, post, w
    raster_digests, fires, ck = [], [], {}
    done = 0
    while done < steps:
        m = min(block, steps - done)
        r, _ = o.run(m, raster=True)
        raster_digests.append(sha(r))
        fires.extend(int(x) for x in np.unpackbits(r, axis=1, bitorder="little")[:, :wl["n"]].sum(1))
        done += m
        if done in checkpoints:
            st = o.stats()
            ck[done] = dict(pot=sha(o.potentials()), w=sha(o.weights()),
                            counts=np.array([st["fires"], st["launched"], st["dropped"]], np.int64))
        print(name, "step", done, round(time.time() - t0, 1), "s", flush=True)
    out = dict(n=np.asarray(wl["n"]), k=np.asarray(wl["k"]), net_seed=np.asarray(wl["net_seed"]),
               sim_seed=np.asarray(wl["sim_seed"]), steps=np.asarray(steps), block=np.asarray(block),
               groups=np.array([[g["first"], g["count"], g["rate_hz"], g["correlated"], g["jitter"]]
                                for g in wl["groups"]], np.float64),
               raster_sha=np.frombuffer(b"".join(raster_digests), np.uint8).reshape(-1, 32),
               fires=np.asarray(fires, np.int32), checkpoints=np.asarray(sorted(ck), np.int32),
               pot_sha=np.stack([np.frombuffer(ck[c]["pot"], np.uint8) for c in sorted(ck)]),
               w_sha=np.stack([np.frombuffer(ck[c]["w"], np.uint8) for c in sorted(ck)]),
               counts=np.stack([ck[c]["counts"] for c in sorted(ck)]))
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print(name, "written", path, os.path.getsize(path), "bytes", flush=True)


def main(argv):
    which = argv or ["c2", "c5"]
    if "c2" in which:
        run(c2_workload(), 1000, 100, {300, 1000}, "c2_digests")
    if "c5" in which:
        run(c5_workload(), 20, 1, {20}, "c5_digests")


if __name__ == "__main__":
    main(sys.argv[1:])
