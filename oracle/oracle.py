"""Python access to the oracles (TEST INFRASTRUCTURE ONLY).

* ``OracleS``  — ctypes wrapper of ``liboracle_s.so`` (nc_oracle.c), the stepped CPU
  restatement of the NeuCor step.  Used by tests/, ``__graft_entry__.smoke()`` and
  bench.py's CPU baseline as the oracle; never by the product.
* ``run_reference`` — runs ``_ref/neucor_ref`` (the reference's own src/NeuCor.cpp
  compiled from its sources by oracle/Makefile) on a scenario.  Only available where
  the reference tree was present at build time.
"""
from __future__ import annotations

import ctypes
import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle_s.so")
REF_BIN = os.path.join(HERE, "_ref", "neucor_ref")
NEVER = np.iinfo(np.int32).min


class Params(ctypes.Structure):
    _fields_ = [
        ("run_speed", ctypes.c_float),
        ("learning_rate", ctypes.c_float),
        ("presynaptic_trace_decay", ctypes.c_float),
        ("postsynaptic_trace_decay", ctypes.c_float),
        ("presynaptic_factor", ctypes.c_float),
        ("postsynaptic_factor", ctypes.c_float),
        ("background_firing", ctypes.c_int32),
        ("inhibitory_rule", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
    ]


INHIBITORY_COPY_LOSS = 0
INHIBITORY_SIGN = 1


class Group(ctypes.Structure):
    _fields_ = [
        ("first", ctypes.c_int32),
        ("count", ctypes.c_int32),
        ("rate_hz", ctypes.c_float),
        ("correlated", ctypes.c_int32),
        ("jitter", ctypes.c_int32),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("fires", ctypes.c_int64),
        ("launched", ctypes.c_int64),
        ("dropped", ctypes.c_int64),
        ("arrivals", ctypes.c_int64),
        ("order_conflicts", ctypes.c_int64),
        ("first_conflict_step", ctypes.c_int32),
        ("step", ctypes.c_int32),
    ]


_lib = None


def reference_dir() -> str:
    """The reference's source tree: $NEUCOR_REF_DIR when set, else a `reference`
    directory beside this repository's root (absent on machines without it)."""
    return os.environ.get("NEUCOR_REF_DIR") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def build(quiet: bool = True) -> None:
    """Compile liboracle_s.so (and _ref/neucor_ref when the reference tree exists)."""
    args = ["make", "-s", "-C", HERE, "all"]
    subprocess.run(args, check=True, capture_output=quiet)
    if os.path.isdir(os.path.join(reference_dir(), "src")):
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True, capture_output=quiet)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        L.ncs_create.restype = P
        L.ncs_create.argtypes = [ctypes.c_int32, P, ctypes.c_int64, P, P, P, P, P, ctypes.POINTER(Params)]
        L.ncs_read_inhibitory.argtypes = [P, P]
        L.ncs_destroy.argtypes = [P]
        L.ncs_set_groups.argtypes = [P, ctypes.c_int32, P]
        L.ncs_set_rates.argtypes = [P, ctypes.c_float, ctypes.c_float, ctypes.c_float]
        L.ncs_schedule_fire.argtypes = [P, ctypes.c_int32, P]
        L.ncs_set_firers.argtypes = [P, ctypes.c_int32, P, P, P]
        L.ncs_set_firer_rates.argtypes = [P, ctypes.c_int32, P]
        L.ncs_add_firer_offset.argtypes = [P, ctypes.c_int32, ctypes.c_float]
        L.ncs_n_firers.restype = ctypes.c_int32
        L.ncs_n_firers.argtypes = [P]
        L.ncs_read_firer_last.argtypes = [P, P]
        L.ncs_run.argtypes = [P, ctypes.c_int32, P, P]
        L.ncs_step.restype = ctypes.c_int32
        L.ncs_step.argtypes = [P]
        L.ncs_n_synapses.restype = ctypes.c_int64
        L.ncs_n_synapses.argtypes = [P]
        for name in ("ncs_read_potentials", "ncs_read_activity", "ncs_read_last_fire_step",
                     "ncs_read_weights", "ncs_read_delays"):
            getattr(L, name).argtypes = [P, P]
        L.ncs_reset_activities.argtypes = [P]
        L.ncs_get_stats.argtypes = [P, ctypes.POINTER(Stats)]
        L.ncs_default_params.argtypes = [ctypes.POINTER(Params)]
        L.ncs_philox4x32_10.argtypes = [P, P, P]
        L.ncs_input_fires.restype = ctypes.c_int32
        L.ncs_input_fires.argtypes = [P, ctypes.c_int32, ctypes.c_uint64, ctypes.c_float, ctypes.c_int32, P,
                                      ctypes.c_int32]
        L.ncs_background_draws.argtypes = [ctypes.c_uint64, ctypes.c_int32, ctypes.c_float, ctypes.c_int32, P, P]
        L.ncs_build_knn.restype = ctypes.c_int32
        L.ncs_build_knn.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_float, ctypes.c_uint64, ctypes.c_int32,
                                    P, P, P, P]
        L.ncs_delay_steps.restype = ctypes.c_int32
        L.ncs_delay_steps.argtypes = [ctypes.c_float, ctypes.c_float]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def default_params(**kw) -> Params:
    p = Params()
    lib().ncs_default_params(ctypes.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def groups_array(groups):
    arr = (Group * max(1, len(groups)))()
    for i, g in enumerate(groups):
        arr[i] = Group(int(g["first"]), int(g["count"]), float(g["rate_hz"]), int(g.get("correlated", 1)),
                       int(g.get("jitter", 2)))
    return arr


def philox(ctr, key):
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    lib().ncs_philox4x32_10(_ptr(c), _ptr(k), _ptr(o))
    return o


class OracleS:
    """The stepped CPU restatement of NeuCor::run (runAll=true, fixed dt)."""

    def __init__(self, xyz, pre, post, weight, length=None, params: Params | None = None, groups=(),
                 inhibitory=None):
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
        self.n = int(self.xyz.shape[0])
        self.pre = np.ascontiguousarray(pre, dtype=np.int32)
        self.post = np.ascontiguousarray(post, dtype=np.int32)
        self.weight = np.ascontiguousarray(weight, dtype=np.float32)
        self.length = None if length is None else np.ascontiguousarray(length, dtype=np.float32)
        self.params = params if params is not None else default_params()
        self.n_input = int(self.pre.shape[0])
        self.inh_in = None if inhibitory is None else np.ascontiguousarray(inhibitory, dtype=np.uint8)
        self.h = lib().ncs_create(self.n, _ptr(self.xyz), self.n_input, _ptr(self.pre), _ptr(self.post),
                                  _ptr(self.weight), _ptr(self.length), _ptr(self.inh_in), ctypes.byref(self.params))
        if not self.h:
            raise ValueError("oracle rejected the network")
        if groups:
            g = groups_array(groups)
            if lib().ncs_set_groups(self.h, len(groups), ctypes.cast(g, ctypes.c_void_p)) != 0:
                raise ValueError("bad input groups")

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().ncs_destroy(h)
            self.h = None

    def schedule_fire(self, ids):
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        if lib().ncs_schedule_fire(self.h, int(ids.size), _ptr(ids)) != 0:
            raise ValueError("bad neuron id")

    def set_firers(self, rates, xyz, radius):
        """Periodic input firers (NeuCor::setInputRateArray + InputFirer)."""
        r = np.ascontiguousarray(rates, dtype=np.float32)
        x = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
        rad = np.ascontiguousarray(radius, dtype=np.float32)
        assert lib().ncs_set_firers(self.h, len(r), _ptr(r), _ptr(x), _ptr(rad)) == 0

    def set_firer_rates(self, rates):
        r = np.ascontiguousarray(rates, dtype=np.float32)
        assert lib().ncs_set_firer_rates(self.h, len(r), _ptr(r)) == 0

    def add_firer_offset(self, firer: int, t_ms: float):
        """NeuCor::addInputOffset."""
        assert lib().ncs_add_firer_offset(self.h, int(firer), float(t_ms)) == 0

    def firer_last(self):
        """InputFirer::lastFire of every firer."""
        out = np.zeros(lib().ncs_n_firers(self.h), dtype=np.float32)
        lib().ncs_read_firer_last(self.h, _ptr(out))
        return out

    def set_rates(self, learning_rate, pre_factor, post_factor):
        lib().ncs_set_rates(self.h, learning_rate, pre_factor, post_factor)

    def run(self, steps: int, raster: bool = False, pots: bool = False):
        row = (self.n + 7) // 8
        r = np.zeros((steps, row), dtype=np.uint8) if raster else None
        p = np.zeros((steps, self.n), dtype=np.float32) if pots else None
        if lib().ncs_run(self.h, int(steps), _ptr(r), _ptr(p)) != 0:
            raise ValueError("run failed")
        return r, p

    @property
    def step(self) -> int:
        return int(lib().ncs_step(self.h))

    def potentials(self):
        o = np.zeros(self.n, dtype=np.float32)
        lib().ncs_read_potentials(self.h, _ptr(o))
        return o

    def activity(self):
        o = np.zeros(self.n, dtype=np.float32)
        lib().ncs_read_activity(self.h, _ptr(o))
        return o

    def last_fire_step(self):
        o = np.zeros(self.n, dtype=np.int32)
        lib().ncs_read_last_fire_step(self.h, _ptr(o))
        return o

    def weights(self):
        o = np.zeros(self.n_input, dtype=np.float32)
        lib().ncs_read_weights(self.h, _ptr(o))
        return o

    def inhibitory(self):
        o = np.zeros(self.n_input, dtype=np.uint8)
        lib().ncs_read_inhibitory(self.h, _ptr(o))
        return o

    def delays(self):
        o = np.zeros(self.n_input, dtype=np.int32)
        lib().ncs_read_delays(self.h, _ptr(o))
        return o

    def reset_activities(self):
        lib().ncs_reset_activities(self.h)

    def stats(self) -> dict:
        s = Stats()
        lib().ncs_get_stats(self.h, ctypes.byref(s))
        return {f: getattr(s, f) for f, _ in Stats._fields_}


def build_knn(n: int, k: int, density: float = 8.0, seed: int = 0, threads: int = 0):
    """The workloads' kNN network (nc_knn.c): xyz (n, 3), and per synapse (source, then
    rank) pre, post, weight — the network the library's nc_build_knn makes."""
    threads = threads or (os.cpu_count() or 1)
    xyz = np.zeros((n, 3), dtype=np.float32)
    pre = np.zeros(n * k, dtype=np.int32)
    post = np.zeros(n * k, dtype=np.int32)
    w = np.zeros(n * k, dtype=np.float32)
    rc = lib().ncs_build_knn(int(n), int(k), float(density), int(seed), int(threads), _ptr(xyz), _ptr(pre),
                             _ptr(post), _ptr(w))
    if rc != 0:
        raise ValueError(f"ncs_build_knn failed ({rc})")
    return xyz, pre, post, w


def input_fires(groups, seed: int, dt: float, t: int):
    g = groups_array(groups)
    cap = sum(int(x["count"]) for x in groups) + 1
    ids = np.zeros(cap, dtype=np.int32)
    n = lib().ncs_input_fires(ctypes.cast(g, ctypes.c_void_p), len(groups), seed, dt, t, _ptr(ids), cap)
    return ids[:n]


def background_draws(seed: int, n: int, dt: float, counter: int):
    hit = np.zeros(n, dtype=np.uint8)
    tgt = np.zeros(n, dtype=np.int32)
    lib().ncs_background_draws(seed, n, dt, counter, _ptr(hit), _ptr(tgt))
    return hit.astype(bool), tgt


# ------------------------------------------------------------- Oracle-R runner
MODES = {"canonical": 0, "native": 1, "continuous": 2, "continuous_grid": 3, "construct": 4, "inputs": 5}


def reference_available() -> bool:
    return os.path.exists(REF_BIN) and os.access(REF_BIN, os.X_OK)


def run_reference(mode, xyz, pre, post, weight, params: Params, groups=(), steps=100, record_pot=False,
                  extra_fires=(), checkpoints=(), firers=(), detectors=()):
    """Run the reference's own simulator on a scenario.  extra_fires: (step, id) pairs
    requesting a forced fire at that step.  firers: the reference's periodic input
    firers as dicts (pos, radius, rate_hz, offset_ms), continuous mode only.
    Returns dict(raster, pots, weights, pot, activity, last_fire)."""
    if not reference_available():
        raise RuntimeError("reference harness not built (needs the reference tree)")
    xyz = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
    n = xyz.shape[0]
    pre = np.ascontiguousarray(pre, dtype=np.int32)
    post = np.ascontiguousarray(post, dtype=np.int32)
    weight = np.ascontiguousarray(weight, dtype=np.float32)
    s = pre.shape[0]
    checkpoints = sorted(int(c) for c in checkpoints)
    with tempfile.TemporaryDirectory() as td:
        scen = os.path.join(td, "s.bin")
        outp = os.path.join(td, "o.bin")
        with open(scen, "wb") as f:
            f.write(b"NCRF")
            f.write(struct.pack("<iiq", MODES[mode], n, s))
            f.write(xyz.tobytes())
            f.write(pre.tobytes())
            f.write(post.tobytes())
            f.write(weight.tobytes())
            f.write(struct.pack("<6f", params.run_speed, params.learning_rate, params.presynaptic_trace_decay,
                                params.postsynaptic_trace_decay, params.presynaptic_factor,
                                params.postsynaptic_factor))
            f.write(struct.pack("<iQ", params.background_firing, params.seed))
            f.write(struct.pack("<i", len(groups)))
            for g in groups:
                f.write(struct.pack("<iifii", int(g["first"]), int(g["count"]), float(g["rate_hz"]),
                                    int(g.get("correlated", 1)), int(g.get("jitter", 2))))
            f.write(struct.pack("<ii", steps, int(bool(record_pot))))
            f.write(struct.pack("<i", len(extra_fires)))
            for st, i in extra_fires:
                f.write(struct.pack("<ii", int(st), int(i)))
            f.write(struct.pack("<i", len(checkpoints)))
            f.write(np.asarray(checkpoints, dtype=np.int32).tobytes())
            f.write(struct.pack("<i", len(firers)))
            for fr in firers:
                x, y, z = fr["pos"]
                f.write(struct.pack("<6f", x, y, z, fr["radius"], fr["rate_hz"], fr.get("offset_ms", 0.0)))
            f.write(struct.pack("<i", len(detectors)))
            for d in detectors:
                f.write(struct.pack("<4f", *[float(v) for v in d]))
        subprocess.run([REF_BIN, scen, outp], check=True)
        data = open(outp, "rb").read()
    row = (n + 7) // 8
    off = 0
    raster = np.frombuffer(data, dtype=np.uint8, count=row * steps, offset=off).reshape(steps, row)
    off += row * steps
    pots = None
    if record_pot:
        pots = np.frombuffer(data, dtype=np.float32, count=n * steps, offset=off).reshape(steps, n)
        off += 4 * n * steps
    ckw = np.frombuffer(data, dtype=np.float32, count=s * len(checkpoints), offset=off).reshape(len(checkpoints), s)
    off += 4 * s * len(checkpoints)
    fin = np.frombuffer(data, dtype=np.float32, count=3 * n, offset=off)
    off += 12 * n
    inh = np.frombuffer(data, dtype=np.uint8, count=s, offset=off)
    off += s
    nf = len(firers)
    flast = np.frombuffer(data, dtype=np.float32, count=nf * steps, offset=off).reshape(steps, nf)
    off += 4 * nf * steps
    rec = np.dtype([("from_id", "<i4"), ("to_id", "<i4"), ("weight", "<f4"), ("pre_potential", "<f4"),
                    ("post_potential", "<f4"), ("inhibitory", "u1")])
    snaps = []
    for _ in checkpoints:
        c = struct.unpack_from("<q", data, off)[0]
        off += 8
        snaps.append(np.frombuffer(data, dtype=rec, count=c, offset=off).copy())
        off += rec.itemsize * c
    nd = len(detectors)
    volts = np.frombuffer(data, dtype=np.float32, count=nd * len(checkpoints), offset=off).reshape(len(checkpoints), nd)
    return {"raster": raster.copy(), "pots": None if pots is None else pots.copy(), "weights": ckw.copy(),
            "pot": fin[:n].copy(), "activity": fin[n:2 * n].copy(), "last_fire": fin[2 * n:].copy(),
            "inhibitory": inh.copy(), "firer_last": flast.copy(), "snapshots": snaps, "voltages": volts.copy()}


def reference_construct(n: int, seed: int):
    """srand(seed); NeuCor(n) in the reference: positions and synapses (from, to,
    weight, length) in the reference's own order."""
    p = default_params(seed=seed)
    with tempfile.TemporaryDirectory() as td:
        scen = os.path.join(td, "s.bin")
        outp = os.path.join(td, "o.bin")
        with open(scen, "wb") as f:
            f.write(b"NCRF")
            f.write(struct.pack("<iiq", MODES["construct"], n, 0))
            f.write(np.zeros(3 * n, np.float32).tobytes())
            f.write(struct.pack("<6f", p.run_speed, p.learning_rate, p.presynaptic_trace_decay,
                                p.postsynaptic_trace_decay, p.presynaptic_factor, p.postsynaptic_factor))
            f.write(struct.pack("<iQ", p.background_firing, p.seed))
            f.write(struct.pack("<i", 0))
            f.write(struct.pack("<ii", 0, 0))
            f.write(struct.pack("<i", 0))
            f.write(struct.pack("<i", 0))
            f.write(struct.pack("<i", 0))
            f.write(struct.pack("<i", 0))
        subprocess.run([REF_BIN, scen, outp], check=True)
        data = open(outp, "rb").read()
    s = struct.unpack_from("<q", data, 0)[0]
    off = 8
    xyz = np.frombuffer(data, np.float32, 3 * n, off).reshape(n, 3).copy()
    off += 12 * n
    fr = np.frombuffer(data, np.int32, s, off).copy()
    off += 4 * s
    to = np.frombuffer(data, np.int32, s, off).copy()
    off += 4 * s
    w = np.frombuffer(data, np.float32, s, off).copy()
    off += 4 * s
    ln = np.frombuffer(data, np.float32, s, off).copy()
    return xyz, fr, to, w, ln


def reference_input_snapshots(xyz, rates, seed: int):
    """srand(seed); NeuCor(0) with neurons at xyz; setInputRateArray(rates, n, NULL, NULL)
    in the reference: its getInputSnapshots as (id, x, y, z, radius, frequency, enabled)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
    firers = [dict(pos=(0.0, 0.0, 0.0), radius=1.0, rate_hz=float(r)) for r in rates]
    p = default_params(seed=seed)
    with tempfile.TemporaryDirectory() as td:
        scen = os.path.join(td, "s.bin")
        outp = os.path.join(td, "o.bin")
        with open(scen, "wb") as f:
            f.write(b"NCRF")
            f.write(struct.pack("<iiq", MODES["inputs"], xyz.shape[0], 0))
            f.write(xyz.tobytes())
            f.write(struct.pack("<6f", p.run_speed, p.learning_rate, p.presynaptic_trace_decay,
                                p.postsynaptic_trace_decay, p.presynaptic_factor, p.postsynaptic_factor))
            f.write(struct.pack("<iQ", p.background_firing, p.seed))
            f.write(struct.pack("<i", 0))
            f.write(struct.pack("<ii", 0, 0))
            f.write(struct.pack("<i", 0))
            f.write(struct.pack("<i", 0))
            f.write(struct.pack("<i", len(firers)))
            for fr in firers:
                f.write(struct.pack("<6f", 0.0, 0.0, 0.0, 1.0, fr["rate_hz"], 0.0))
            f.write(struct.pack("<i", 0))
        subprocess.run([REF_BIN, scen, outp], check=True)
        data = open(outp, "rb").read()
    rec = np.dtype([("v", "<f4", 6), ("enabled", "u1")])
    return np.frombuffer(data, dtype=rec)


def unpack_raster(raster, n):
    """(steps, ceil(n/8)) bit rows -> (steps, n) bool."""
    return np.unpackbits(raster, axis=1, bitorder="little")[:, :n].astype(bool)
