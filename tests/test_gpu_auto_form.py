"""NC_STEP_AUTO: one network holding the tables of both forms of the step kernels,
switched between them at run-call boundaries — by the caller (nc_set_step_form) or by
nc_run from the fire share of the last window.  A switch flushes the current form's
deferred plasticity and converts the per-synapse arrival state (nc_form.cu); the results
stay bit-identical to the oracle whatever the switches."""
import numpy as np
import pytest

from netgen import knn_net, random_net

pytestmark = pytest.mark.gpu

DENSE, EVENT, AUTO = 0, 1, 2


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


@pytest.mark.parametrize("label,make,pkw,groups", [
    ("knn300", lambda: knn_net(300, 12, 61, inhibitory=0.15), dict(seed=71),
     [dict(first=0, count=20, rate_hz=40.0, correlated=1, jitter=2)]),
    ("random120_dt05", lambda: random_net(120, 1500, 62), dict(seed=72, run_speed=0.5),
     [dict(first=3, count=10, rate_hz=60.0, correlated=0)]),
    ("knn500_id_order", lambda: knn_net(500, 25, 63, weight_scale=0.4), dict(seed=73, storage_order=1),
     [dict(first=100, count=30, rate_hz=30.0, correlated=1, jitter=3)]),
])
def test_forced_switches_match_oracle(nc, oracle_mod, label, make, pkw, groups):
    G, O = nc, oracle_mod
    xyz, pre, post, w = make()
    net = G.NeuCor.from_arrays(xyz, pre, post, w, params=G.default_params(**pkw, step_mode=AUTO))
    net.set_input_groups(groups)
    o = O.OracleS(xyz, pre, post, w, params=O.default_params(**pkw), groups=groups)
    plan = [(DENSE, 37), (EVENT, 1), (DENSE, 1), (EVENT, 53), (EVENT, 20), (DENSE, 64), (EVENT, 2), (DENSE, 90),
            (EVENT, 33)]
    total = sum(m for _, m in plan)
    net.record_raster(total)
    for form, m in plan:
        net.set_step_form(form)
        assert net.step_form == form
        net.run(m)
        o.run(m)
        np.testing.assert_array_equal(bits(net.potentials()), bits(o.potentials()), f"potentials {label}")
        np.testing.assert_array_equal(bits(net.weights()), bits(o.weights()), f"weights {label}")
    o2 = O.OracleS(xyz, pre, post, w, params=O.default_params(**pkw), groups=groups)
    ro, _ = o2.run(total, raster=True)
    np.testing.assert_array_equal(net.raster(), ro)
    st, so = net.stats(), o.stats()
    assert (st["fires"], st["launched"], st["dropped"]) == (so["fires"], so["launched"], so["dropped"])
    np.testing.assert_array_equal(bits(net.potAct[1::2]), bits(o.activity()))


def test_forced_switches_with_firers_and_detectors(nc, oracle_mod):
    """Periodic input firers (their fires land in the next step's input bits, shared by
    both forms) and detectors across form switches: raster and potentials every step
    equal the oracle's."""
    G, O = nc, oracle_mod
    xyz, pre, post, w = knn_net(250, 10, 64, inhibitory=0.1)
    pkw = dict(seed=81, run_speed=0.5)
    net = G.NeuCor.from_arrays(xyz, pre, post, w, params=G.default_params(**pkw, step_mode=AUTO))
    o = O.OracleS(xyz, pre, post, w, params=O.default_params(**pkw))
    rates = np.array([40.0, 125.0, 70.0], np.float32)
    fxyz = xyz[[3, 80, 170]]
    frad = np.array([0.6, 0.9, 0.5], np.float32)
    net.setInputRateArray(rates, inputPositions=fxyz, inputRadius=frad)
    o.set_firers(rates, fxyz, frad)
    net.setDetectors(2, xyz[[10, 200]], np.array([0.8, 1.1], np.float32))
    plan = [(EVENT, 23), (DENSE, 5), (EVENT, 1), (DENSE, 40), (EVENT, 31)]
    total = sum(m for _, m in plan)
    net.record_raster(total)
    rows = []
    for form, m in plan:
        net.set_step_form(form)
        for _ in range(m):
            net.run(1)
            r, p = o.run(1, raster=True, pots=True)
            rows.append(r[0])
            np.testing.assert_array_equal(bits(net.potentials()), bits(p[0]))
        assert len(net.getDetectorVoltages()) == 2
    np.testing.assert_array_equal(net.raster(), np.asarray(rows))
    np.testing.assert_array_equal(bits(net.weights()), bits(o.weights()))


def test_auto_policy_picks_the_form_by_activity(nc, oracle_mod):
    """A saturated network stays dense; the same network with weak synapses (quiet)
    moves to the event form on its own; both stay equal to the oracle."""
    G, O = nc, oracle_mod
    xyz, pre, post, w = G.build_knn(4000, 40, 8.0, seed=9)
    groups = [dict(first=0, count=20, rate_hz=20.0, correlated=1, jitter=2)]
    for scale, want in ((1.0, DENSE), (0.02, EVENT)):
        ws = (w * scale).astype(np.float32)
        net = G.NeuCor.from_arrays(xyz, pre, post, ws, params=G.default_params(seed=5, step_mode=AUTO))
        net.set_input_groups(groups)
        net.run(1500)
        assert net.step_form == want, (scale, net.step_form)
        o = O.OracleS(xyz, pre, post, ws, params=O.default_params(seed=5), groups=groups)
        o.run(1500)
        np.testing.assert_array_equal(bits(net.weights()), bits(o.weights()))
        np.testing.assert_array_equal(bits(net.potentials()), bits(o.potentials()))
        st, so = net.stats(), o.stats()
        assert (st["fires"], st["launched"], st["dropped"]) == (so["fires"], so["launched"], so["dropped"])


def test_auto_window_spans_single_step_calls(nc, oracle_mod):
    """A caller stepping one step per run call (as the renderer does) still gets the
    automatic choice: the windows span the calls."""
    G, O = nc, oracle_mod
    xyz, pre, post, w = G.build_knn(2000, 30, 8.0, seed=4)
    ws = (w * np.float32(0.02)).astype(np.float32)
    net = G.NeuCor.from_arrays(xyz, pre, post, ws, params=G.default_params(seed=6, step_mode=AUTO))
    for _ in range(600):
        net.run(1)
    assert net.step_form == EVENT
    o = O.OracleS(xyz, pre, post, ws, params=O.default_params(seed=6))
    o.run(600)
    np.testing.assert_array_equal(bits(net.potentials()), bits(o.potentials()))
    np.testing.assert_array_equal(bits(net.weights()), bits(o.weights()))


def test_single_form_networks_refuse_a_switch(nc):
    G = nc
    xyz, pre, post, w = knn_net(64, 4, 3)
    net = G.NeuCor.from_arrays(xyz, pre, post, w, params=G.default_params(step_mode=DENSE))
    net.set_step_form(DENSE)  # its own form: accepted
    with pytest.raises(G.NeuCorError) as e:
        net.set_step_form(EVENT)
    assert e.value.code == -4
    with pytest.raises(G.NeuCorError):
        net.set_step_form(AUTO)
