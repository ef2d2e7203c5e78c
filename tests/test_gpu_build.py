"""Network construction on the device (nc_create_knn): the network nc_build_knn + nc_create
build on the host, identical bit for bit — positions, weights and delays in creation
order, inhibitory flags, synapse snapshots, and what the step then computes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def pair(G, n, k, knn_seed, **pkw):
    dev = G.NeuCor.knn(n, k, 8.0, seed=knn_seed, params=G.default_params(**pkw))
    xyz, pre, post, w = G.build_knn(n, k, 8.0, seed=knn_seed)
    host = G.NeuCor.from_arrays(xyz, pre, post, w, params=G.default_params(**pkw))
    return dev, host, xyz


@pytest.mark.parametrize("n,k,seed", [(3000, 20, 1), (300, 40, 2), (20000, 100, 3), (64, 63, 4)])
def test_device_build_equals_host_build(nc, n, k, seed):
    G = nc
    dev, host, xyz = pair(G, n, k, seed, seed=100 + seed)
    np.testing.assert_array_equal(bits(dev._xyz), bits(xyz))
    np.testing.assert_array_equal(bits(dev.weights()), bits(host.weights()))
    np.testing.assert_array_equal(dev.delays(), host.delays())
    np.testing.assert_array_equal(dev.inhibitory(), host.inhibitory())
    groups = [dict(first=0, count=min(20, n), rate_hz=40.0, correlated=1, jitter=2)]
    for net in (dev, host):
        net.set_input_groups(groups)
        net.record_raster(150)
        net.run(150)
    np.testing.assert_array_equal(dev.raster(), host.raster())
    np.testing.assert_array_equal(bits(dev.potentials()), bits(host.potentials()))
    np.testing.assert_array_equal(bits(dev.weights()), bits(host.weights()))
    sd, sh = dev.stats(), host.stats()
    assert (sd["fires"], sd["launched"], sd["dropped"]) == (sh["fires"], sh["launched"], sh["dropped"])
    snap_d, snap_h = dev.getSynapseSnapshots(), host.getSynapseSnapshots()
    assert len(snap_d) == len(snap_h) == n * k
    for a, b in zip(snap_d[:: max(1, len(snap_d) // 500)], snap_h[:: max(1, len(snap_h) // 500)]):
        assert a == b


def test_device_build_falls_back_past_its_capacity(nc):
    """k above the device builder's 512: built on the host, the same network."""
    G = nc
    dev, host, _ = pair(G, 1200, 600, 5)
    np.testing.assert_array_equal(bits(dev.weights()), bits(host.weights()))
    np.testing.assert_array_equal(dev.delays(), host.delays())


def test_device_build_event_form_request_builds_on_host(nc):
    G = nc
    dev, host, _ = pair(G, 2000, 16, 6, step_mode=1)
    np.testing.assert_array_equal(bits(dev.weights()), bits(host.weights()))
    dev.run(50)
    host.run(50)
    np.testing.assert_array_equal(bits(dev.potentials()), bits(host.potentials()))
