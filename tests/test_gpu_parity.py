"""GPU step (libneucor_gb300.so through the C ABI) against the reference's own outputs
(golden fixtures) and against the stepped CPU restatement (oracle), bit for bit:
spike rasters, potentials, weights, activities, last-fire times and counters.  Every
case runs in both forms of the step kernels (dense: a synapse pass walking the
in-rows; event: fired-list compaction and spike launch)."""
import numpy as np
import pytest

from netgen import knn_net, random_net
from scenario import extra_by_step, groups_list, load, params_kw

pytestmark = pytest.mark.gpu

MODES = {"dense": 0, "event": 1}


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def assert_bits_equal(a, b, what):
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    bad = bits(a) != bits(b)
    if bad.any():
        idx = np.argwhere(bad)[0]
        raise AssertionError(f"{what}: {int(bad.sum())} differ; first at {tuple(idx)}: "
                             f"gpu={a[tuple(idx)]!r} ref={b[tuple(idx)]!r}")


def gpu_net(G, xyz, pre, post, w, pkw, groups=(), inhibitory=None):
    net = G.NeuCor.from_arrays(xyz, pre, post, w, params=G.default_params(**pkw), inhibitory=inhibitory)
    if groups:
        net.set_input_groups(groups)
    return net


def run_gpu_stepwise(net, steps, extras=None, checkpoints=(), pots=True):
    extras = extras or {}
    net.record_raster(steps)
    pot_rows, weights = [], []
    for t in range(1, steps + 1):
        if t in extras:
            net.schedule_fire(extras[t])
        net.run(1)
        if pots:
            pot_rows.append(net.potentials())
        if t in checkpoints:
            weights.append(net.weights())
    return net.raster(), np.asarray(pot_rows), weights


def run_oracle_stepwise(o, steps, extras=None, checkpoints=()):
    extras = extras or {}
    ras, pot_rows, weights = [], [], []
    for t in range(1, steps + 1):
        if t in extras:
            o.schedule_fire(extras[t])
        r, p = o.run(1, raster=True, pots=True)
        ras.append(r[0])
        pot_rows.append(p[0])
        if t in checkpoints:
            weights.append(o.weights())
    return np.asarray(ras), np.asarray(pot_rows), weights


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("name", ["canonical_knn64", "canonical_random40_dt05", "canonical_knn100_nobg"])
def test_gpu_matches_reference_fixture(nc, name, mode):
    """The GPU reproduces what the reference's own code computed, every step."""
    G = nc
    fx = load(name)
    net = gpu_net(G, fx["xyz"], fx["pre"], fx["post"], fx["w"], dict(params_kw(fx), step_mode=MODES[mode]),
                  groups_list(fx))
    np.testing.assert_array_equal(net.inhibitory(), fx["inhibitory"])
    steps = int(fx["steps"])
    ck = [int(c) for c in fx["checkpoints"]]
    raster, pots, weights = run_gpu_stepwise(net, steps, extra_by_step(fx), ck)
    np.testing.assert_array_equal(raster, fx["raster"])
    assert_bits_equal(pots, fx["pots"], "potentials")
    assert_bits_equal(np.asarray(weights), fx["weights"], "weights")
    pa = net.potAct
    assert_bits_equal(pa[1::2], fx["activity"], "activity")
    lf = net.lastFire()
    np.testing.assert_array_equal(np.isnan(lf), np.isnan(fx["last_fire"]))
    assert_bits_equal(lf[~np.isnan(lf)], fx["last_fire"][~np.isnan(fx["last_fire"])], "lastFire")
    assert abs(net.getTime() - steps * float(fx["p_run_speed"])) < 1e-3


def edited_weights(net, edit):
    xyz, pre, post, w = net
    w = np.array(w, np.float32)
    edit(w)
    return xyz, pre, post, w


def zero_weights(w):
    """Exact zeros and negative zeros among non-negative weights: every term is still >= 0,
    so the neuron passes may stop a fold once the neuron is certain to fire."""
    w[::5] = 0.0
    w[1::10] = -0.0


def one_negative(w):
    """One negative weight among non-negative ones: the net's terms may be negative, so
    every fold runs to its last term."""
    w[17] = -0.25


SCENARIOS = [
    # (label, network, params, groups, steps)
    ("knn300_inh", lambda: knn_net(300, 10, 21, inhibitory=0.2), dict(seed=31),
     [dict(first=0, count=20, rate_hz=30.0, correlated=1, jitter=2)], 600),
    ("random150_dups_dt05", lambda: random_net(150, 2000, 22), dict(seed=32, run_speed=0.5, learning_rate=0.5),
     [dict(first=5, count=10, rate_hz=50.0, correlated=0)], 500),
    ("knn500_dt025", lambda: knn_net(500, 20, 23, weight_scale=0.5), dict(seed=33, run_speed=0.25),
     [dict(first=100, count=30, rate_hz=40.0, correlated=1, jitter=4)], 400),
    ("random90_dt2", lambda: random_net(90, 900, 24, self_loops=True), dict(seed=34, run_speed=2.0), [], 400),
    ("knn257_sign_rule", lambda: knn_net(257, 7, 25, inhibitory=0.3), dict(seed=35, inhibitory_rule=1),
     [dict(first=250, count=7, rate_hz=80.0, correlated=1, jitter=1)], 500),
    ("random64_dt4", lambda: random_net(64, 700, 26), dict(seed=36, run_speed=4.0), [], 300),
    ("knn300_id_order", lambda: knn_net(300, 10, 28, inhibitory=0.2), dict(seed=38, storage_order=1),
     [dict(first=40, count=20, rate_hz=30.0, correlated=1, jitter=2)], 400),
    ("knn200_nobg_lr", lambda: knn_net(200, 16, 27), dict(seed=37, background_firing=0, learning_rate=2.0,
                                                          presynaptic_factor=0.2, postsynaptic_factor=0.1),
     [dict(first=0, count=40, rate_hz=25.0, correlated=1, jitter=2)], 600),
    ("knn400_zero_weights", lambda: edited_weights(knn_net(400, 24, 29), zero_weights), dict(seed=39),
     [dict(first=0, count=30, rate_hz=40.0, correlated=1, jitter=2)], 500),
    ("knn300_one_negative", lambda: edited_weights(knn_net(300, 12, 30), one_negative), dict(seed=40),
     [dict(first=10, count=20, rate_hz=40.0, correlated=1, jitter=2)], 400),
]


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("label,make,pkw,groups,steps", SCENARIOS, ids=[s[0] for s in SCENARIOS])
def test_gpu_matches_oracle_stepwise(nc, oracle_mod, label, make, pkw, groups, steps, mode):
    G, O = nc, oracle_mod
    xyz, pre, post, w = make()
    extras = {t: [(t * 37 + k * 11) % len(xyz) for k in range(3)] for t in range(2, steps, 13)}
    ck = (steps // 3, steps)
    net = gpu_net(G, xyz, pre, post, w, dict(pkw, step_mode=MODES[mode]), groups)
    o = O.OracleS(xyz, pre, post, w, params=O.default_params(**pkw), groups=groups)
    np.testing.assert_array_equal(net.inhibitory(), o.inhibitory())
    np.testing.assert_array_equal(net.delays(), o.delays())
    rg, pg, wg = run_gpu_stepwise(net, steps, extras, ck)
    ro, po, wo = run_oracle_stepwise(o, steps, extras, ck)
    np.testing.assert_array_equal(rg, ro)
    assert_bits_equal(pg, po, "potentials")
    for a, b in zip(wg, wo):
        assert_bits_equal(a, b, "weights")
    assert_bits_equal(net.potAct[1::2], o.activity(), "activity")
    st, so = net.stats(), o.stats()
    assert (st["fires"], st["launched"], st["dropped"]) == (so["fires"], so["launched"], so["dropped"])
    assert st["steps"] == steps
    assert so["fires"] > 0 and so["launched"] > 0


@pytest.mark.parametrize("mode", MODES)
def test_gpu_rate_changes_and_activity_reset(nc, oracle_mod, mode):
    """learningRate / factors changed between runs and resetActivities, as the renderer's
    sliders do (src/NeuCor_Renderer.cpp:1696-1712)."""
    G, O = nc, oracle_mod
    xyz, pre, post, w = knn_net(160, 12, 41)
    groups = [dict(first=0, count=16, rate_hz=40.0, correlated=1, jitter=2)]
    pkw = dict(seed=42)
    net = gpu_net(G, xyz, pre, post, w, dict(pkw, step_mode=MODES[mode]), groups)
    o = O.OracleS(xyz, pre, post, w, params=O.default_params(**pkw), groups=groups)
    for lr, a, b in [(1.0, 0.13, 0.30), (0.0, 0.13, 0.30), (3.0, 0.05, 0.6), (1.0, 0.13, 0.30)]:
        net.learningRate, net.presynapticFactor, net.postsynapticFactor = lr, a, b
        o.set_rates(lr, a, b)
        net.run(150)
        o.run(150)
        assert_bits_equal(net.weights(), o.weights(), f"weights lr={lr}")
        assert_bits_equal(net.potentials(), o.potentials(), "potentials")
        net.resetActivities()
        o.reset_activities()
        net.run(7)
        o.run(7)
        assert_bits_equal(net.potAct[1::2], o.activity(), "activity")


def c1_network(G, seed=1):
    """1,000 neurons uniform in a cube, 50 nearest targets each, U[0,1) weights; 20 input
    neurons at 20 Hz: a correlated group (shared source, +-2-step jitter) and an
    uncorrelated control group."""
    xyz, pre, post, w = G.build_knn(1000, 50, 8.0, seed=seed)
    groups = [dict(first=0, count=10, rate_hz=20.0, correlated=1, jitter=2),
              dict(first=10, count=10, rate_hz=20.0, correlated=0, jitter=0)]
    return xyz, pre, post, w, groups


@pytest.mark.parametrize("mode", MODES)
def test_gpu_c1_full_horizon_bit_exact(nc, oracle_mod, mode):
    """The 1k-neuron / 50k-synapse workload for its full 10,000 steps: every step's
    raster, and the final potentials, weights, activities and counters."""
    G, O = nc, oracle_mod
    xyz, pre, post, w, groups = c1_network(G)
    pkw = dict(seed=2024)
    steps = 10000
    net = gpu_net(G, xyz, pre, post, w, dict(pkw, step_mode=MODES[mode]), groups)
    net.record_raster(steps)
    net.run(steps)
    o = O.OracleS(xyz, pre, post, w, params=O.default_params(**pkw), groups=groups)
    ro, _ = o.run(steps, raster=True)
    np.testing.assert_array_equal(net.raster(), ro)
    assert_bits_equal(net.potentials(), o.potentials(), "potentials")
    assert_bits_equal(net.weights(), o.weights(), "weights")
    assert_bits_equal(net.potAct[1::2], o.activity(), "activity")
    st, so = net.stats(), o.stats()
    assert (st["fires"], st["launched"], st["dropped"]) == (so["fires"], so["launched"], so["dropped"])
