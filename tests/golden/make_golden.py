"""Generates the golden fixtures in this directory from the REFERENCE's own code.

Runs oracle/_ref/neucor_ref — the reference's src/NeuCor.cpp compiled unmodified from
its sources by oracle/Makefile — on small seeded scenarios and stores inputs and
outputs.  Needs the reference tree (this script does not run on the GPU machines;
its outputs are committed).

    python tests/golden/make_golden.py [base] [c1_stats] [snapshots]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import oracle as O  # noqa: E402
from netgen import knn_net, random_net  # noqa: E402


def params_dict(p):
    return {f: np.asarray(getattr(p, f)) for f, _ in O.Params._fields_}


def groups_arr(groups):
    return np.array([[g["first"], g["count"], g["rate_hz"], g.get("correlated", 1), g.get("jitter", 2)]
                     for g in groups], dtype=np.float64).reshape(-1, 5)


def save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    print(name, os.path.getsize(path), "bytes")


def scenario(name, mode, net, params, groups, steps, extra=(), record_pot=True, checkpoints=()):
    xyz, pre, post, w = net
    r = O.run_reference(mode, xyz, pre, post, w, params, groups=groups, steps=steps, record_pot=record_pot,
                        extra_fires=list(extra), checkpoints=list(checkpoints) or [steps])
    ex = np.asarray(list(extra), dtype=np.int32).reshape(-1, 2)
    save(name, mode=np.asarray(mode), xyz=xyz, pre=pre, post=post, w=w, groups=groups_arr(groups), extra=ex,
         steps=np.asarray(steps), checkpoints=np.asarray(list(checkpoints) or [steps], dtype=np.int32),
         raster=r["raster"], pots=r["pots"] if record_pot else np.zeros(0, np.float32), weights=r["weights"],
         pot=r["pot"], activity=r["activity"], last_fire=r["last_fire"], inhibitory=r["inhibitory"],
         **{"p_" + k: v for k, v in params_dict(params).items()})


C1_SEEDS = (2024, 7, 99)


def c1_workload():
    """1,000 neurons uniform in a cube, 50 nearest targets each, U[0,1) weights (the
    oracle's kNN restatement, seed 1); 20 inputs at 20 Hz: a correlated group of 10
    (shared source, +-2-step jitter) and an uncorrelated control group of 10."""
    xyz, pre, post, w = O.build_knn(1000, 50, 8.0, 1)
    groups = [dict(first=0, count=10, rate_hz=20.0, correlated=1, jitter=2),
              dict(first=10, count=10, rate_hz=20.0, correlated=0, jitter=0)]
    return xyz, pre, post, w, groups


def c1_stats(mode, seed, steps=10000, window=1000):
    """Population statistics of the reference's own NeuCor::run on the C1 workload:
    the population rate per 1,000-step window, per-neuron fire counts, and the final
    weights (all excitatory, so in [0, 1]) quantised to 16 bits."""
    xyz, pre, post, w, groups = c1_workload()
    r = O.run_reference(mode, xyz, pre, post, w, O.default_params(seed=seed), groups=groups, steps=steps,
                        checkpoints=[steps])
    ras = O.unpack_raster(r["raster"], xyz.shape[0])
    pop = ras.reshape(steps // window, window, -1).sum((1, 2)) / (xyz.shape[0] * window / 1000.0)
    wq = np.rint(np.clip(r["weights"][-1], 0.0, 1.0) * 65535.0).astype(np.uint16)
    return dict(pop_rate_hz=pop.astype(np.float64), counts=ras.sum(0).astype(np.int32), weights_u16=wq)


def c1_statistics():
    """F. C1 for its 10,000 steps through the reference's own NeuCor::run.
    native: runAll, synapse lengths on the step grid (whole-step delays, as in the
    stepped model), background fire times on the step grid; three simulation seeds.
    continuous: the unmodified timing (lengths as built, glibc rand() background at
    random times inside the step); one seed.
    continuous_grid: as continuous with the lengths on the step grid (only the
    background fire times off it); one seed."""
    import concurrent.futures as cf
    runs = [("native", s) for s in C1_SEEDS] + [("continuous", C1_SEEDS[0]), ("continuous_grid", C1_SEEDS[0])]
    out = {}
    with cf.ThreadPoolExecutor(len(runs)) as ex:  # each run is its own reference process
        for (mode, seed), res in zip(runs, ex.map(lambda ms: c1_stats(*ms), runs)):
            for k, v in res.items():
                out[f"{mode}_{seed}_{k}"] = v
    save("c1_reference_stats", seeds=np.asarray(C1_SEEDS), steps=np.asarray(10000), window=np.asarray(1000), **out)


def snapshots():
    """G. The renderer's read-backs through the reference's own code at checkpoints:
    NeuCor::getSynapseSnapshots (weights and the pre/post render potentials of spikes in
    flight, src/NeuCor.cpp:115-134, 547-570) and NeuCor::getDetectorVoltages
    (src/NeuCor.cpp:79-87, 359-366), canonical step order, at dt 1 and dt 0.5."""
    cases = [
        ("snapshots_knn64", knn_net(64, 6, 11, inhibitory=0.2), O.default_params(seed=5),
         [dict(first=0, count=8, rate_hz=40.0, correlated=1, jitter=2)], 120, [1, 2, 3, 17, 60, 119, 120]),
        ("snapshots_random40_dt05", random_net(40, 300, 3), O.default_params(seed=9, run_speed=0.5),
         [dict(first=0, count=6, rate_hz=60.0, correlated=1, jitter=3)], 90, [4, 5, 31, 90]),
        ("snapshots_knn200_busy", knn_net(200, 20, 13), O.default_params(seed=21),
         [dict(first=0, count=20, rate_hz=40.0, correlated=1, jitter=2)], 60, [10, 11, 12, 40, 60]),
    ]
    for name, net, params, groups, steps, ck in cases:
        xyz, pre, post, w = net
        lo, hi = xyz.min(0), xyz.max(0)
        det = [(float(lo[0] + (hi[0] - lo[0]) * f), float(lo[1] + (hi[1] - lo[1]) * f), float(lo[2] + (hi[2] - lo[2]) * f),
                r) for f, r in [(0.5, 1.0), (0.25, 0.7), (0.8, 1.6)]]
        r = O.run_reference("canonical", xyz, pre, post, w, params, groups=groups, steps=steps, checkpoints=ck,
                            detectors=det)
        sn = np.stack([np.stack([s[f].astype(np.float64) for f in ("from_id", "to_id", "weight", "pre_potential",
                                                                   "post_potential", "inhibitory")], 1)
                       for s in r["snapshots"]])
        save(name, xyz=xyz, pre=pre, post=post, w=w, groups=groups_arr(groups), steps=np.asarray(steps),
             checkpoints=np.asarray(ck, np.int32), detectors=np.asarray(det, np.float32),
             snap_from=sn[:, :, 0].astype(np.int32), snap_to=sn[:, :, 1].astype(np.int32),
             snap_weight=sn[:, :, 2].astype(np.float32), snap_pre=sn[:, :, 3].astype(np.float32),
             snap_post=sn[:, :, 4].astype(np.float32), snap_inh=sn[:, :, 5].astype(np.uint8),
             voltages=r["voltages"], **{"p_" + k: v for k, v in params_dict(params).items()})
        nz = int((sn[:, :, 3] != 0).sum())
        print(name, "spikes in flight over the checkpoints:", nz)


def input_snapshots():
    """H. NeuCor::getInputSnapshots after srand(4); NeuCor(0); 30 neurons;
    setInputRateArray(rates, 5, NULL, NULL): firer positions drawn from the C library's
    rand() in the reference's order (src/NeuCor.cpp:46-64, 309-313)."""
    xyz = (np.random.default_rng(8).random((30, 3)) * 3.0 - 1.5).astype(np.float32)
    rates = np.array([20.0, 0.0, 55.5, 13.0, 100.0], np.float32)
    r = O.reference_input_snapshots(xyz, rates, 4)
    save("input_snapshots_seed4", xyz=xyz, rates=rates, seed=np.asarray(4), snap=r["v"].copy(),
         enabled=r["enabled"].copy())


def main(sections):
    if not O.reference_available():
        O.build()
    assert O.reference_available(), "needs the reference tree to build oracle/_ref"
    if "c1_stats" in sections:
        c1_statistics()
    if "snapshots" in sections:
        snapshots()
        input_snapshots()
    if "base" not in sections:
        return

    # A. FEW_NEURONS preset through the reference's own API (src/main.cpp:162-189):
    # 3 neurons, synapses 0->1, 0->2 at 0.5, periodic inputs at 50 Hz offset 0/+2/-2 ms,
    # runAll, runSpeed 0.02, seed 1.  Weights at 50, 100, 150, 250 ms.
    xyz = np.array([[0, 0, 0], [0.3, 0.3, 0], [0.3, -0.3, 0]], np.float32)
    pre, post, w = np.array([0, 0], np.int32), np.array([1, 2], np.int32), np.array([0.5, 0.5], np.float32)
    p = O.default_params(run_speed=0.02, seed=1)
    firers = [dict(pos=tuple(map(float, xyz[i])), radius=0.1, rate_hz=50.0, offset_ms=[0.0, 2.0, -2.0][i])
              for i in range(3)]
    ck = [2500, 5000, 7500, 12500]
    r = O.run_reference("continuous", xyz, pre, post, w, p, steps=12500, checkpoints=ck, firers=firers)
    save("few_neurons_preset", checkpoints_ms=np.asarray(ck, np.float32) * np.float32(0.02), weights=r["weights"])

    # B. canonical order: the reference's Neuron/Synapse code under a stepped scheduler
    g1 = [dict(first=0, count=8, rate_hz=40.0, correlated=1, jitter=2),
          dict(first=8, count=8, rate_hz=40.0, correlated=0)]
    scenario("canonical_knn64", "canonical", knn_net(64, 6, 11, inhibitory=0.2), O.default_params(seed=5), g1, 400)
    g2 = [dict(first=0, count=6, rate_hz=60.0, correlated=1, jitter=3)]
    extra2 = [(t, (7 * t) % 40) for t in range(1, 300, 9)]
    scenario("canonical_random40_dt05", "canonical", random_net(40, 300, 3),
             O.default_params(seed=9, run_speed=0.5, learning_rate=0.7), g2, 300, extra=extra2)
    extra3 = [(t, (13 * t) % 100) for t in range(1, 500, 4)]
    scenario("canonical_knn100_nobg", "canonical", knn_net(100, 8, 12, weight_scale=0.6),
             O.default_params(seed=2, background_firing=0), [], 500, extra=extra3, checkpoints=[100, 500])

    # C. native order: the reference's own NeuCor::run with runAll (bit-exact until the
    # first same-step coincidence whose order the reference leaves to its heap)
    g4 = [dict(first=0, count=10, rate_hz=10.0, correlated=1, jitter=2),
          dict(first=10, count=10, rate_hz=10.0, correlated=0)]
    net = knn_net(200, 6, 0, weight_scale=0.25)
    xyz, pre, post, w = net
    p4 = O.default_params(seed=77)
    r = O.run_reference("native", xyz, pre, post, w, p4, groups=g4, steps=1000, record_pot=True)
    save("native_knn200", xyz=xyz, pre=pre, post=post, w=w, groups=groups_arr(g4), steps=np.asarray(1000),
         raster=r["raster"], inhibitory=r["inhibitory"], pots_every50=r["pots"][49::50], **{"p_" + k: v for k, v in params_dict(p4).items()})

    # E. InputFirer's schedule through the reference's own run calls: lastFire of every
    # firer after each call, at steps that are and are not exactly representable
    rates = np.array([50.0, 33.3, 125.0, 700.0, 2500.0, 0.0, 20.0], np.float32)
    offsets = [0.0, 2.0, -2.0, 0.37, 0.0, 1.0, 0.25]
    xyz = np.array([[0, 0, 0], [0.3, 0.3, 0], [0.3, -0.3, 0]], np.float32)
    pre, post, w = np.array([0, 0], np.int32), np.array([1, 2], np.int32), np.array([0.5, 0.5], np.float32)
    fdts, flasts = [], []
    for dt in (0.02, 0.1, 0.25, 0.3, 1.0, 2.0):
        fr = [dict(pos=(0.0, 0.0, 0.0), radius=0.1, rate_hz=float(rates[i]), offset_ms=offsets[i])
              for i in range(len(rates))]
        steps = int(round(60.0 / dt))
        r = O.run_reference("continuous", xyz, pre, post, w, O.default_params(run_speed=dt, seed=1), steps=steps,
                            firers=fr)
        fdts.append(dt)
        flasts.append(r["firer_last"])
    save("firer_schedule", dts=np.asarray(fdts, np.float32), rates=rates, offsets=np.asarray(offsets, np.float32),
         steps=np.asarray([x.shape[0] for x in flasts], np.int32), last=np.concatenate(flasts))

    # D. the reference constructor NeuCor(60) after srand(3)
    xyz, fr, to, w, ln = O.reference_construct(60, 3)
    save("construct_n60_seed3", xyz=xyz, pre=fr, post=to, w=w, length=ln)


if __name__ == "__main__":
    main(sys.argv[1:] or ["base", "c1_stats", "snapshots"])
