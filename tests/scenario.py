"""Loads the golden fixtures and replays them on the oracle or the GPU library."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def params_kw(fx):
    return {k[2:]: fx[k].item() for k in fx if k.startswith("p_")}


def groups_list(fx):
    return [dict(first=int(g[0]), count=int(g[1]), rate_hz=float(g[2]), correlated=int(g[3]), jitter=int(g[4]))
            for g in fx["groups"]]


def extra_by_step(fx):
    out = {}
    for t, i in fx.get("extra", np.zeros((0, 2), np.int32)):
        out.setdefault(int(t), []).append(int(i))
    return out


def run_stepwise(sim, steps, extras, schedule, step1, read_pot, read_raster_row=None):
    """Runs `steps` single steps, injecting forced fires; returns per-step potentials."""
    pots = []
    for t in range(1, steps + 1):
        if t in extras:
            schedule(extras[t])
        step1()
        pots.append(read_pot())
    return np.asarray(pots)
