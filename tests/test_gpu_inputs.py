"""Periodic input firers (NeuCor::setInputRateArray / InputFirer / addInputOffset) and
voltage detectors (NeuCor::setDetectors / getDetectorVoltage) through the C ABI.

Firers: the GPU against the oracle's restatement of InputFirer::schedule (the reference's
float/double arithmetic on its accumulated currentTime T_t; a fire time in
(T_t, T_t + dt) fires the near neurons at step t+1 without threshold or refractory test),
bit for bit, in both forms of the step, with changes between runs: offsets, rates, firers
appended and popped, and offsets set before the first step (the FEW_NEURONS pattern).
Detectors: the mean potential of the neurons within the radius, summed in id order in
float, against the same sum over the potentials read back."""
import numpy as np
import pytest

from netgen import knn_net

pytestmark = pytest.mark.gpu

MODES = {"dense": 0, "event": 1}


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("dt,scale", [(1.0, 1.0), (0.02, 25.0), (0.3, 4.0)])
def test_periodic_firers_match_oracle(nc, oracle_mod, mode, dt, scale):
    G, O = nc, oracle_mod
    xyz, pre, post, w = knn_net(400, 10, 61, inhibitory=0.1)
    pkw = dict(seed=77, background_firing=0, run_speed=dt)
    net = G.NeuCor.from_arrays(xyz, pre, post, w, params=G.default_params(**pkw, step_mode=MODES[mode]))
    o = O.OracleS(xyz, pre, post, w, params=O.default_params(**pkw))
    fxyz = np.asarray(xyz[[3, 120, 250, 399, 77]], dtype=np.float32)
    radius = np.asarray([0.5, 0.7, 0.4, 0.6, 0.8], dtype=np.float32)
    # at 1 ms, 20 Hz is a whole number of steps: it fires only once shifted (as the reference)
    rates = np.asarray([20.0, 30.0, 47.3, 0.0], dtype=np.float32) * np.float32(scale)
    net.setInputRateArray(rates, inputPositions=fxyz[:4], inputRadius=radius[:4])
    o.set_firers(rates, fxyz[:4], radius[:4])
    # offsets before the first step, seen by its time-0 run call
    net.addInputOffset(1, 2.0 / scale)
    o.add_firer_offset(1, 2.0 / scale)
    net.record_raster(750)
    ro = []
    for action in ["none", "offset", "rates", "append", "pop"]:
        if action == "offset":
            net.addInputOffset(0, 0.25)
            o.add_firer_offset(0, 0.25)
        elif action == "rates":
            rates = np.asarray([20.0, 12.5, 90.0, 33.0], dtype=np.float32) * np.float32(scale)
            net.set_input_rates(rates)
            o.set_firer_rates(rates)
            net.addInputOffset(3, -0.75)
            o.add_firer_offset(3, -0.75)
        elif action == "append":
            rates = np.append(rates, np.float32(61.0 * scale))
            net.setInputRateArray(rates, inputPositions=fxyz[4:], inputRadius=radius[4:])
            o.set_firers(rates, fxyz, radius)
        elif action == "pop":
            rates = rates[[0, 1, 2]]
            net.setInputRateArray(rates)
            o.set_firers(rates, fxyz[:3], radius[:3])
        net.run(150)
        r, _ = o.run(150, raster=True)
        ro.append(r)
    rg = net.raster()
    np.testing.assert_array_equal(rg, np.concatenate(ro))
    np.testing.assert_array_equal(bits(net.potentials()), bits(o.potentials()))
    np.testing.assert_array_equal(bits(net.weights()), bits(o.weights()))
    st, so = net.stats(), o.stats()
    assert (st["fires"], st["launched"], st["dropped"]) == (so["fires"], so["launched"], so["dropped"])
    assert so["fires"] > 100


def test_whole_step_period_never_fires(nc, oracle_mod):
    """InputFirer::schedule's `currentT < fireTime` excludes a fire time on a step
    boundary, so a period of a whole number of steps never fires (src/NeuCor.cpp:338-343)."""
    G = nc
    xyz, pre, post, w = knn_net(200, 6, 62)
    net = G.NeuCor.from_arrays(xyz, pre, post, w, params=G.default_params(seed=5, background_firing=0))
    net.setInputRateArray([50.0, 25.0], inputPositions=xyz[[0, 100]], inputRadius=[1.5, 1.5])
    net.run(400)
    assert net.stats()["fires"] == 0


def near_ids(xyz, a, r):
    d = np.asarray(xyz, np.float32) - np.asarray(a, np.float32)
    dist = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2])
    return np.nonzero(dist < np.float32(r))[0]


def test_detector_voltages(nc):
    G = nc
    xyz, pre, post, w = knn_net(500, 12, 63)
    net = G.NeuCor.from_arrays(xyz, pre, post, w, params=G.default_params(seed=9))
    net.set_input_groups([dict(first=0, count=30, rate_hz=40.0, correlated=1, jitter=2)])
    dxyz = np.asarray([xyz[10], xyz[200], [50.0, 50.0, 50.0]], dtype=np.float32)
    drad = np.asarray([0.8, 0.5, 0.3], dtype=np.float32)
    net.setDetectors(3, dxyz, drad)
    for _ in range(3):
        net.run(97)
        v = net.getDetectorVoltages()
        pot = net.potentials()
        for d in range(3):
            ids = near_ids(xyz, dxyz[d], drad[d])
            acc = np.float32(0.0)
            for i in ids:
                acc = np.float32(acc + pot[i])
            with np.errstate(invalid="ignore", divide="ignore"):
                expect = np.float32(acc / np.float32(len(ids)))
            if len(ids) == 0:
                assert np.isnan(v[d])
            else:
                assert bits(v[d]) == bits(expect), (d, v[d], expect)
            if not np.isnan(expect):
                assert bits(net.getDetectorVoltage(d)) == bits(v[d])
    # detectors are appended by each call, as NeuCor::setDetectors does
    net.setDetectors(1, dxyz[:1], drad[:1])
    assert len(net.getDetectorVoltages()) == 4
