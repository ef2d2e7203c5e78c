"""The stepped CPU restatement (oracle/nc_oracle.c) against fixtures made by the
REFERENCE's own src/NeuCor.cpp (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from scenario import extra_by_step, groups_list, load, params_kw

CANONICAL = ["canonical_knn64", "canonical_random40_dt05", "canonical_knn100_nobg"]


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def test_philox_known_answers(oracle_mod):
    # Random123 known-answer vectors for Philox4x32-10
    O = oracle_mod
    assert [hex(x) for x in O.philox([0, 0, 0, 0], [0, 0])] == ["0x6627e8d5", "0xe169c58d", "0xbc57ac4c", "0x9b00dbd8"]
    assert [hex(x) for x in O.philox([0xffffffff] * 4, [0xffffffff] * 2)] == \
        ["0x408f276d", "0x41c83b0e", "0xa20bc7c6", "0x6d5451fd"]
    assert [hex(x) for x in O.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0])] == \
        ["0xd16cfe09", "0x94fdcceb", "0x5001e420", "0x24126ea1"]


@pytest.mark.parametrize("name", CANONICAL)
def test_oracle_matches_reference_canonical(oracle_mod, name):
    """Every step's raster and potentials, and the weights and activities, bit-equal to
    the reference's own Neuron/Synapse code run in ascending-id order."""
    O = oracle_mod
    fx = load(name)
    p = O.default_params(**params_kw(fx))
    o = O.OracleS(fx["xyz"], fx["pre"], fx["post"], fx["w"], params=p, groups=groups_list(fx))
    extras = extra_by_step(fx)
    steps = int(fx["steps"])
    ck = list(fx["checkpoints"])
    raster, pots, weights = [], [], []
    for t in range(1, steps + 1):
        if t in extras:
            o.schedule_fire(extras[t])
        r, pt = o.run(1, raster=True, pots=True)
        raster.append(r[0])
        pots.append(pt[0])
        if t in ck:
            weights.append(o.weights())
    np.testing.assert_array_equal(np.asarray(raster), fx["raster"])
    np.testing.assert_array_equal(bits(np.asarray(pots)), bits(fx["pots"]))
    np.testing.assert_array_equal(bits(np.asarray(weights)), bits(fx["weights"]))
    np.testing.assert_array_equal(bits(o.activity()), bits(fx["activity"]))
    lf = o.last_fire_step()
    lf_ms = np.where(lf == O.NEVER, np.nan, lf.astype(np.float32) * np.float32(p.run_speed)).astype(np.float32)
    np.testing.assert_array_equal(np.isnan(lf_ms), np.isnan(fx["last_fire"]))
    np.testing.assert_array_equal(lf_ms[~np.isnan(lf_ms)], fx["last_fire"][~np.isnan(fx["last_fire"])])
    assert o.stats()["fires"] > 0


def test_oracle_matches_reference_native_until_first_coincidence(oracle_mod):
    """The reference's own NeuCor::run (runAll) agrees with the oracle bit for bit until
    the first step where the reference's heap order decides an outcome."""
    O = oracle_mod
    fx = load("native_knn200")
    p = O.default_params(**params_kw(fx))
    o = O.OracleS(fx["xyz"], fx["pre"], fx["post"], fx["w"], params=p, groups=groups_list(fx))
    steps = int(fx["steps"])
    r, pots = o.run(steps, raster=True, pots=True)
    first = o.stats()["first_conflict_step"]
    assert first > 20
    limit = steps if first < 0 else first - 1
    np.testing.assert_array_equal(r[:limit], fx["raster"][:limit])
    sel = np.arange(49, steps, 50)
    sel = sel[sel < limit]
    np.testing.assert_array_equal(bits(pots[sel]), bits(fx["pots_every50"][: len(sel)]))


def test_few_neurons_preset_known_answer(oracle_mod):
    """The essay's 3-neuron result (w(0->1) -> 1, w(0->2) -> 0 in about 120 ms),
    recorded from the reference's own FEW_NEURONS preset, and the same network on the
    stepped oracle with inputs forced on the preset's schedule."""
    O = oracle_mod
    fx = load("few_neurons_preset")
    np.testing.assert_allclose(fx["weights"], [[0.6861805, 0.32505023], [0.8726871, 0.15197149],
                                               [1.0, 0.00962104], [1.0, 0.0]], rtol=0, atol=1e-7)
    xyz = np.array([[0, 0, 0], [0.3, 0.3, 0], [0.3, -0.3, 0]], np.float32)
    o = O.OracleS(xyz, [0, 0], [1, 2], [0.5, 0.5], params=O.default_params(seed=1))
    w = {}
    for t in range(1, 251):
        due = [i for i, off in enumerate((0, 2, -2)) if (t - off) % 20 == 0 and t - off > 0]
        if due:
            o.schedule_fire(due)
        o.run(1)
        if t in (50, 100, 150, 250):
            w[t] = o.weights()
    assert w[50][0] > 0.5 and w[50][1] < 0.5
    assert w[150][0] == 1.0 and w[150][1] < 0.05
    assert w[250][0] == 1.0 and w[250][1] == 0.0


def test_firer_schedule_matches_reference(oracle_mod):
    """InputFirer::schedule (src/NeuCor.cpp:333-345) as the reference's own run calls
    drive it: lastFire of every firer after each call, recorded from the reference at
    steps that are (0.25, 1, 2 ms) and are not (0.02, 0.1, 0.3 ms) exact in float.  The
    oracle's step t runs the call at time T_t (and step 1 also the one at time 0), so
    after its step t it holds the reference's lastFire after call t."""
    O = oracle_mod
    fx = load("firer_schedule")
    xyz = np.array([[0, 0, 0], [0.3, 0.3, 0], [0.3, -0.3, 0]], np.float32)
    rates = fx["rates"]
    nf = len(rates)
    base = 0
    for dt, steps in zip(fx["dts"], fx["steps"]):
        rows = fx["last"][base: base + steps]
        base += steps
        o = O.OracleS(xyz, [0, 0], [1, 2], [0.5, 0.5], params=O.default_params(run_speed=float(dt), seed=1))
        o.set_firers(rates, np.zeros((nf, 3), np.float32), np.full(nf, 0.1, np.float32))
        for i, off in enumerate(fx["offsets"]):
            o.add_firer_offset(i, float(off))
        got = np.zeros((steps - 1, nf), np.float32)
        for t in range(1, steps):
            o.run(1)
            got[t - 1] = o.firer_last()
        np.testing.assert_array_equal(bits(got), bits(rows[1:]), err_msg=f"dt {dt}")
        assert len(np.unique(rows[:, 3])) > 20  # the 700 Hz firer advanced


def test_oracle_input_groups_rates(oracle_mod):
    """Poisson groups fire at their rate; correlated members share jittered events."""
    O = oracle_mod
    groups = [dict(first=0, count=10, rate_hz=20.0, correlated=1, jitter=2),
              dict(first=10, count=10, rate_hz=20.0, correlated=0)]
    counts = np.zeros(20)
    lag0 = 0
    for t in range(1, 20001):
        ids = O.input_fires(groups, 123, 1.0, t)
        counts[ids] += 1
        lag0 += int(np.sum(ids < 10) >= 3)
    rate = counts / 20.0
    assert np.all(np.abs(rate - 20.0) < 4.0), rate
    assert lag0 > 50  # correlated members often fire within the same step


def test_background_draw_rate(oracle_mod):
    O = oracle_mod
    hits = 0
    for c in range(200):
        h, tgt = O.background_draws(5, 3000, 1.0, c)
        hits += int(h.sum())
        assert tgt.min() >= 0 and tgt.max() < 3000
    assert abs(hits / (200 * 3000) - 1 / 600) < 0.0005


def _ks(a, b):
    a, b = np.sort(np.asarray(a)), np.sort(np.asarray(b))
    v = np.union1d(a, b)
    return float(np.max(np.abs(np.searchsorted(a, v, "right") / a.size - np.searchsorted(b, v, "right") / b.size)))


def test_oracle_c1_statistics_match_reference_run(oracle_mod):
    """The oracle (bit-identical to the GPU) against the reference's own NeuCor::run with
    every event on the step grid, 1,000-neuron / 50k-synapse workload, 10,000 steps, one
    seed: every 1,000-step window's population rate within 1%, final-weight KS distance no
    larger than the reference's own between two seeds (tests/test_gpu_c1_statistics.py
    runs all seeds on the GPU)."""
    O = oracle_mod
    fx = load("c1_reference_stats")
    seed = int(fx["seeds"][0])
    xyz, pre, post, w = O.build_knn(1000, 50, 8.0, 1)
    groups = [dict(first=0, count=10, rate_hz=20.0, correlated=1, jitter=2),
              dict(first=10, count=10, rate_hz=20.0, correlated=0, jitter=0)]
    o = O.OracleS(xyz, pre, post, w, params=O.default_params(seed=seed), groups=groups)
    rates = []
    for _ in range(10):
        f0 = o.stats()["fires"]
        o.run(1000)
        rates.append((o.stats()["fires"] - f0) / 1000.0)
    ref = fx[f"native_{seed}_pop_rate_hz"]
    assert np.max(np.abs(np.asarray(rates) - ref) / ref) <= 0.01
    wq = np.rint(np.clip(o.weights(), 0.0, 1.0) * 65535.0).astype(np.uint16)
    s = [int(x) for x in fx["seeds"]]
    bound = min(_ks(fx[f"native_{a}_weights_u16"], fx[f"native_{b}_weights_u16"])
                for i, a in enumerate(s) for b in s[i + 1:])
    assert _ks(wq, fx[f"native_{seed}_weights_u16"]) <= bound
