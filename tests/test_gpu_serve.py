"""Served form: requests arrive while others run, are admitted by device footprint and
slot, share launches with the resident networks, and leave at their horizon.  Each
result must be what the same network computes alone (the oracle), bit for bit."""
import time

import numpy as np
import pytest

from netgen import knn_net, random_net

pytestmark = pytest.mark.gpu


def requests():
    out = []
    shapes = [(400, 10, 1.0, 300), (150, 6, 0.5, 180), (900, 16, 1.0, 420), (64, 4, 2.0, 90), (333, 25, 1.0, 260),
              (520, 8, 1.0, 333), (200, 12, 0.25, 150)]
    for q, (n, k, dt, horizon) in enumerate(shapes):
        xyz, pre, post, w = (random_net(n, n * k, 90 + q) if q % 3 == 2 else knn_net(n, k, 90 + q, inhibitory=0.1))
        pkw = dict(seed=7000 + q, run_speed=dt, background_firing=int(q != 1), learning_rate=0.5 + 0.3 * q)
        groups = [dict(first=0, count=min(12, n), rate_hz=15.0 + 5 * q, correlated=1, jitter=2),
                  dict(first=12, count=min(10, n - 12), rate_hz=20.0, correlated=q % 2, jitter=1)]
        out.append(dict(xyz=xyz, pre=pre, post=post, weight=w, pkw=pkw, groups=groups, horizon=horizon))
    return out


@pytest.mark.parametrize("mode", [0, 1], ids=["dense", "event"])
def test_served_results_equal_alone(nc, oracle_mod, mode):
    G, O = nc, oracle_mod
    reqs = requests()
    srv = G.Server(budget_bytes=256 << 20, max_networks=3, steps_per_batch=16, build_threads=4, keep_results=True,
                   step_mode=mode)
    ids = []
    for q, r in enumerate(reqs):
        ids.append(srv.submit(dict(xyz=r["xyz"], pre=r["pre"], post=r["post"], weight=r["weight"],
                                   params=G.default_params(**r["pkw"]), groups=r["groups"], horizon=r["horizon"])))
        time.sleep(0.01 * (q % 3))
    srv.drain()
    done = {d["request_id"]: d for d in srv.poll()}
    assert sorted(done) == sorted(ids)
    st = srv.stats()
    assert st["finished"] == len(reqs) and st["rejected"] == 0
    assert 1 <= st["peak_resident_networks"] <= 3
    for rid, r in zip(ids, reqs):
        d = done[rid]
        assert d["status"] == 0 and d["steps"] == r["horizon"]
        assert d["submit_s"] <= d["admit_s"] <= d["done_s"]
        w, pot = srv.fetch(rid)
        o = O.OracleS(r["xyz"], r["pre"], r["post"], r["weight"], params=O.default_params(**r["pkw"]),
                      groups=r["groups"])
        o.run(r["horizon"])
        np.testing.assert_array_equal(w.view(np.uint32), o.weights().view(np.uint32))
        np.testing.assert_array_equal(pot.view(np.uint32), o.potentials().view(np.uint32))
        so = o.stats()
        assert (d["fires"], d["launched"], d["dropped"]) == (so["fires"], so["launched"], so["dropped"])
    srv.close()


def test_served_rejects_request_over_budget(nc):
    G = nc
    srv = G.Server(budget_bytes=4 << 20, max_networks=2, steps_per_batch=8, build_threads=1)
    xyz, pre, post, w = G.build_knn(20000, 20, 8.0, seed=1)
    rid = srv.submit(dict(xyz=xyz, pre=pre, post=post, weight=w, horizon=10))
    srv.drain()
    done = srv.poll()
    assert len(done) == 1 and done[0]["request_id"] == rid and done[0]["status"] == -7
    srv.close()


def test_served_knn_requests_equal_alone(nc, oracle_mod):
    """Requests sent as kNN parameters (nc_server_submit_knn), built on the server's
    builder threads, mixed with requests sent as arrays: each equals the oracle run on the
    network the oracle's own kNN restatement builds."""
    G, O = nc, oracle_mod
    srv = G.Server(budget_bytes=512 << 20, max_networks=4, steps_per_batch=16, build_threads=3, keep_results=True)
    knn = [(1500, 20, 11, 240), (700, 40, 12, 180), (3000, 12, 13, 300), (900, 30, 14, 150)]
    groups = [dict(first=0, count=10, rate_hz=30.0, correlated=1, jitter=2)]
    ids = []
    for q, (n, k, seed, horizon) in enumerate(knn):
        p = G.default_params(seed=500 + q)
        ids.append(srv.submit_knn(n, k, 8.0, seed, horizon, params=p, groups=groups))
        if q == 1:
            xyz, pre, post, w = knn_net(300, 10, 77)
            ids.append(srv.submit(dict(xyz=xyz, pre=pre, post=post, weight=w, params=G.default_params(seed=99),
                                       groups=groups, horizon=200)))
    srv.drain()
    done = {d["request_id"]: d for d in srv.poll()}
    assert sorted(done) == sorted(ids)
    k_ids = [i for q, i in enumerate(ids) if q != 2]
    for rid, (n, k, seed, horizon), q in zip(k_ids, knn, range(len(knn))):
        d = done[rid]
        assert d["status"] == 0 and d["steps"] == horizon and d["n_synapses"] == n * k
        w, pot = srv.fetch(rid)
        xyz, pre, post, wk = O.build_knn(n, k, 8.0, seed)
        o = O.OracleS(xyz, pre, post, wk, params=O.default_params(seed=500 + q), groups=groups)
        o.run(horizon)
        np.testing.assert_array_equal(w.view(np.uint32), o.weights().view(np.uint32))
        np.testing.assert_array_equal(pot.view(np.uint32), o.potentials().view(np.uint32))
    srv.close()
