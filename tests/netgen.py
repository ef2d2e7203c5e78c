"""Seeded test networks (numpy only; shared by the parity tests and the fixture script)."""
import numpy as np


def knn_net(n, k, seed, density=8.0, weight_scale=1.0, inhibitory=0.0):
    """n neurons uniform in a cube at the reference's density, k nearest targets each
    (brute force, ties by index), weights U[0,1)*scale with a fraction negated."""
    rng = np.random.default_rng(seed)
    side = (n / density) ** (1.0 / 3.0)
    xyz = (rng.random((n, 3)) * side).astype(np.float32)
    d = np.sqrt(((xyz[:, None, :].astype(np.float64) - xyz[None, :, :]) ** 2).sum(-1))
    np.fill_diagonal(d, np.inf)
    nb = np.argsort(d, axis=1, kind="stable")[:, :k]
    pre = np.repeat(np.arange(n), k).astype(np.int32)
    post = nb.reshape(-1).astype(np.int32)
    w = (rng.random(pre.shape[0]) * weight_scale).astype(np.float32)
    if inhibitory > 0:
        neg = rng.random(pre.shape[0]) < inhibitory
        w[neg] = -w[neg]
    return xyz, pre, post, w


def random_net(n, s, seed, side=3.0, inhibitory=0.2, duplicates=True, self_loops=True):
    """Random directed synapses, optionally with repeated pairs and self loops."""
    rng = np.random.default_rng(seed)
    xyz = (rng.random((n, 3)) * side).astype(np.float32)
    pre = rng.integers(0, n, s).astype(np.int32)
    post = rng.integers(0, n, s).astype(np.int32)
    if not self_loops:
        post = np.where(post == pre, (post + 1) % n, post).astype(np.int32)
    if duplicates and s > 4:
        pre[-2:] = pre[:2]
        post[-2:] = post[:2]
    w = (rng.random(s) * 0.8 + 0.2).astype(np.float32)
    neg = rng.random(s) < inhibitory
    w[neg] = -w[neg]
    return xyz, pre, post, w
