"""Batched form: many independent networks of uneven size packed in one engine.  Each
network must compute the same bits as alone (the oracle), whatever the launch shape."""
import numpy as np
import pytest

from netgen import knn_net, random_net

pytestmark = pytest.mark.gpu

MODES = {"dense": 0, "event": 1}


def mixed_nets(O=None, G=None):
    specs = []
    shapes = [(100, 8, 1.0, 150), (333, 20, 0.5, 260), (700, 12, 1.0, 400), (64, 5, 2.0, 90), (515, 30, 1.0, 333),
              (200, 16, 0.25, 220)]
    for q, (n, k, dt, horizon) in enumerate(shapes):
        if q == 3:
            xyz, pre, post, w = random_net(n, 600, 50 + q)
        else:
            xyz, pre, post, w = knn_net(n, k, 50 + q, inhibitory=0.1 * (q % 2))
        pkw = dict(seed=1000 + q, run_speed=dt, background_firing=int(q != 4), learning_rate=1.0 + 0.25 * q)
        groups = [dict(first=0, count=min(10, n), rate_hz=10.0 + 7 * q, correlated=1, jitter=2),
                  dict(first=10, count=min(8, n - 10), rate_hz=15.0, correlated=q % 2, jitter=1)]
        specs.append(dict(xyz=xyz, pre=pre, post=post, weight=w, pkw=pkw, groups=groups, horizon=horizon))
    return specs


def batch_of(G, specs, mode="dense"):
    return G.Batch([dict(xyz=s["xyz"], pre=s["pre"], post=s["post"], weight=s["weight"],
                         params=G.default_params(**s["pkw"], step_mode=MODES[mode]), groups=s["groups"],
                         horizon=s["horizon"])
                    for s in specs])


def oracle_of(O, s):
    o = O.OracleS(s["xyz"], s["pre"], s["post"], s["weight"], params=O.default_params(**s["pkw"]), groups=s["groups"])
    o.run(s["horizon"])
    return o


def check_equal(b, q, o):
    np.testing.assert_array_equal(b.weights(q).view(np.uint32), o.weights().view(np.uint32))
    np.testing.assert_array_equal(b.potentials(q).view(np.uint32), o.potentials().view(np.uint32))
    st, so = b.stats(q), o.stats()
    assert (st["fires"], st["launched"], st["dropped"]) == (so["fires"], so["launched"], so["dropped"]), q
    assert st["steps"] == so["step"]


@pytest.mark.parametrize("mode", MODES)
def test_batch_each_net_as_alone(nc, oracle_mod, mode):
    specs = mixed_nets()
    b = batch_of(nc, specs, mode)
    b.run_to_end()
    for q, s in enumerate(specs):
        assert b.step(q) == s["horizon"]
        check_equal(b, q, oracle_of(oracle_mod, s))


@pytest.mark.parametrize("mode", MODES)
def test_batch_results_do_not_depend_on_launch_shape(nc, oracle_mod, mode):
    specs = mixed_nets()
    b = batch_of(nc, specs, mode)
    shapes = [dict(neuron_block=128, launch_blocks=152, launch_block=128, graph_steps=0, dense_blocks=0,
                   steps_per_launch=0),
              dict(neuron_block=256, launch_blocks=1216, launch_block=256, graph_steps=7, dense_blocks=3,
                   steps_per_launch=5),
              dict(neuron_block=64, launch_blocks=3, launch_block=32, graph_steps=16, dense_blocks=304,
                   steps_per_launch=0),
              dict(neuron_block=128, launch_blocks=152, launch_block=128, graph_steps=16, dense_blocks=0,
                   steps_per_launch=64)]
    done = 0
    for k, sh in enumerate(shapes * 10):
        b.set_launch(**sh)
        b.run(37)
        done += 37
        if done > 420:
            break
    b.run_to_end()
    for q, s in enumerate(specs):
        check_equal(b, q, oracle_of(oracle_mod, s))


def test_batch_persistent_launch_each_net_as_alone(nc, oracle_mod):
    """Dense form, several whole steps per cooperative launch (grid barriers between the
    passes): every network still equals the oracle, at every launch length."""
    specs = mixed_nets()
    for k in (1, 16, 400):
        b = batch_of(nc, specs, "dense")
        b.set_launch(steps_per_launch=k)
        b.run_to_end()
        for q, s in enumerate(specs):
            assert b.step(q) == s["horizon"]
            check_equal(b, q, oracle_of(oracle_mod, s))
        b.close()


def test_batch_rejects_oversized_blocks(nc):
    specs = mixed_nets()[:1]
    b = batch_of(nc, specs)
    with pytest.raises(nc.NeuCorError):
        b.set_launch(neuron_block=512)
    with pytest.raises(nc.NeuCorError):
        b.set_launch(launch_block=48)


@pytest.mark.parametrize("mode", MODES)
def test_batch_autotune_keeps_results(nc, oracle_mod, mode):
    specs = mixed_nets()
    b = batch_of(nc, specs, mode)
    cfg = b.autotune(steps_per_trial=2)
    assert cfg["neuron_block"] % 32 == 0 and cfg["launch_blocks"] > 0 and cfg["steps_per_launch"] >= 0
    b.run_to_end()
    for q, s in enumerate(specs):
        check_equal(b, q, oracle_of(oracle_mod, s))
