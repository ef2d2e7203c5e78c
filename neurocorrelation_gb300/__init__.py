"""NeuroCorrelation simulation step on GB300 — Python binding of the C ABI.

``NeuCor`` mirrors the reference's C++ class (src/NeuCor.h:36-138): construct a
network from neuron positions and synapses (or with ``createNeuron`` /
``createSynapse`` before the first ``run``), set inputs, ``run()`` it, read back
potentials, spikes and weights.  Every call goes through ``libneucor_gb300.so``
(include/neucor_gb300.h); there is no CPU fallback — without the library or a CUDA
device, construction raises.
"""
from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass

import numpy as np

__all__ = ["NeuCor", "Params", "Group", "NeuCorError", "load_library", "library_path", "build_knn",
           "build_reference_random", "philox4x32_10", "device_count"]

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_lib", "libneucor_gb300.so")

NC_OK = 0
NC_STEP_DENSE = 0  # step_mode: a synapse pass walking the in-rows in order, then a neuron pass
NC_STEP_EVENT = 1  # step_mode: fired-list compaction and spike launch (sparse activity)
NC_STEP_AUTO = 2   # step_mode: both forms' tables; nc_run switches by the fire share
_ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "out of memory", -4: "unsupported", -5: "no CUDA device",
           -6: "device wait timed out", -7: "over memory budget"}


class NeuCorError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{_ERRORS.get(code, 'error')} ({code}): {message}")
        self.code = code


class Params(ctypes.Structure):
    """nc_params: NeuCor's public simulation members (src/NeuCor.h:68-73)."""
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
        ("storage_order", ctypes.c_int32),
        ("step_mode", ctypes.c_int32),
    ]


class Group(ctypes.Structure):
    _fields_ = [("first", ctypes.c_int32), ("count", ctypes.c_int32), ("rate_hz", ctypes.c_float),
                ("correlated", ctypes.c_int32), ("jitter", ctypes.c_int32)]


class _Stats(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int64), ("fires", ctypes.c_int64), ("launched", ctypes.c_int64),
                ("dropped", ctypes.c_int64)]


class SynapseSnapshotC(ctypes.Structure):
    _fields_ = [("from_id", ctypes.c_int32), ("to_id", ctypes.c_int32), ("weight", ctypes.c_float),
                ("pre_potential", ctypes.c_float), ("post_potential", ctypes.c_float), ("inhibitory", ctypes.c_int32)]


class InputSnapshotC(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int32), ("x", ctypes.c_float), ("y", ctypes.c_float), ("z", ctypes.c_float),
                ("radius", ctypes.c_float), ("frequency", ctypes.c_float), ("enabled", ctypes.c_int32)]


class NetSpec(ctypes.Structure):
    _fields_ = [("n_neurons", ctypes.c_int32), ("xyz", ctypes.c_void_p), ("n_synapses", ctypes.c_int64),
                ("syn_from", ctypes.c_void_p), ("syn_to", ctypes.c_void_p), ("syn_weight", ctypes.c_void_p),
                ("syn_length", ctypes.c_void_p), ("syn_inhibitory", ctypes.c_void_p), ("params", Params),
                ("n_groups", ctypes.c_int32), ("groups", ctypes.c_void_p), ("horizon", ctypes.c_int32)]


class LaunchConfig(ctypes.Structure):
    _fields_ = [("neuron_block", ctypes.c_int32), ("launch_blocks", ctypes.c_int32), ("launch_block", ctypes.c_int32),
                ("graph_steps", ctypes.c_int32), ("dense_blocks", ctypes.c_int32),
                ("steps_per_launch", ctypes.c_int32)]

    def as_dict(self):
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


_lib = None


def library_path() -> str:
    return _LIB


def load_library() -> ctypes.CDLL:
    """Loads libneucor_gb300.so (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB):
        from . import build as _build
        _build.build()
    L = ctypes.CDLL(_LIB)
    P, I32, I64, F = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_float
    sigs = {
        "nc_last_error": ([], ctypes.c_char_p), "nc_version": ([], ctypes.c_char_p),
        "nc_device_count": ([P], I32), "nc_default_params": ([P], I32), "nc_set_device": ([I32], I32),
        "nc_create": ([I32, P, I64, P, P, P, P, P, P, P], I32), "nc_destroy": ([P], I32),
        "nc_set_input_groups": ([P, I32, P], I32), "nc_set_input_rate_array": ([P, P, ctypes.c_uint32, P, P], I32),
        "nc_set_rates": ([P, F, F, F], I32), "nc_schedule_fire": ([P, I32, P], I32),
        "nc_run": ([P, I32], I32), "nc_sync": ([P], I32), "nc_get_time": ([P, P], I32),
        "nc_get_step": ([P, P], I32), "nc_get_counts": ([P, P, P], I32), "nc_record_raster": ([P, I32], I32),
        "nc_read_raster": ([P, P, I64, P], I32), "nc_read_potact": ([P, P], I32),
        "nc_read_potentials": ([P, P], I32), "nc_read_positions": ([P, P], I32),
        "nc_read_last_fire": ([P, P], I32), "nc_read_weights": ([P, P], I32), "nc_read_delays": ([P, P], I32),
        "nc_read_inhibitory": ([P, P], I32),
        "nc_read_synapse_snapshots": ([P, P, I64, P], I32), "nc_reset_activities": ([P], I32),
        "nc_read_input_snapshots": ([P, P, I32, P], I32),
        "nc_get_step_form": ([P, P], I32), "nc_set_step_form": ([P, I32], I32),
        "nc_get_stats": ([P, P], I32), "nc_delete_synapse": ([P, I32, I32], I32),
        "nc_delete_neuron": ([P, I32], I32),
        "nc_build_knn": ([I32, I32, F, ctypes.c_uint64, P, P, P, P], I32),
        "nc_reference_positions": ([I32, P], I32), "nc_reference_connection_count": ([I32, P, P], I32),
        "nc_reference_connections": ([I32, P, P, P, P, I64], I32),
        "nc_philox4x32_10": ([P, P, P], I32), "nc_time_steps": ([P, I32, P, P], I32),
        "nc_batch_create": ([I32, P, P], I32), "nc_batch_destroy": ([P], I32), "nc_batch_run": ([P, I32], I32),
        "nc_batch_time": ([P, I32, P], I32), "nc_batch_run_to_end": ([P], I32),
        "nc_batch_get_launch": ([P, P], I32), "nc_batch_set_launch": ([P, P], I32),
        "nc_batch_autotune": ([P, I32, P], I32), "nc_batch_get_stats": ([P, I32, P], I32),
        "nc_batch_get_step": ([P, I32, P], I32), "nc_batch_read_potentials": ([P, I32, P], I32),
        "nc_batch_read_weights": ([P, I32, P], I32), "nc_batch_read_last_fire": ([P, I32, P], I32),
        "nc_server_create": ([P, P], I32), "nc_server_submit": ([P, P, P], I32),
        "nc_server_poll": ([P, P, I32, P], I32), "nc_server_drain": ([P], I32),
        "nc_server_fetch": ([P, I64, P, P], I32), "nc_server_get_stats": ([P, P], I32),
        "nc_server_destroy": ([P], I32), "nc_run_noalloc": ([P, I32, P], I32),
        "nc_server_submit_knn": ([P, I32, I32, F, ctypes.c_uint64, P, I32, P, I32, P], I32),
        "nc_set_input_rates": ([P, I32, P], I32), "nc_add_input_offset": ([P, I32, F], I32),
        "nc_set_detectors": ([P, I32, P, P], I32), "nc_get_detector_voltages": ([P, P, I32, P], I32),
        "nc_get_detector_voltage": ([P, I32, P], I32),
        "nc_create_knn": ([I32, I32, F, ctypes.c_uint64, P, P, P], I32),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def _check(rc: int):
    if rc != NC_OK:
        raise NeuCorError(rc, load_library().nc_last_error().decode(errors="replace"))


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def device_count() -> int:
    c = ctypes.c_int32(0)
    _check(load_library().nc_device_count(ctypes.byref(c)))
    return int(c.value)


def set_device(device: int) -> None:
    _check(load_library().nc_set_device(int(device)))


def default_params(**kw) -> Params:
    p = Params()
    _check(load_library().nc_default_params(ctypes.byref(p)))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def philox4x32_10(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    _check(load_library().nc_philox4x32_10(_p(c), _p(k), _p(o)))
    return o


def build_knn(n: int, k: int, density: float = 8.0, seed: int = 0):
    """n neurons uniform in a cube at the reference's spawn density (src/NeuCor.cpp:155),
    each connected to its k nearest neighbours; weights uniform [0, 1)."""
    xyz = np.zeros((n, 3), dtype=np.float32)
    pre = np.zeros(n * k, dtype=np.int32)
    post = np.zeros(n * k, dtype=np.int32)
    w = np.zeros(n * k, dtype=np.float32)
    _check(load_library().nc_build_knn(n, k, density, seed, _p(xyz), _p(pre), _p(post), _p(w)))
    return xyz, pre, post, w


def build_reference_random(n: int, seed: int):
    """The network NeuCor(n) builds after srand(seed) (src/NeuCor.cpp:17-42)."""
    libc = ctypes.CDLL(None)
    libc.srand(ctypes.c_uint(seed))
    L = load_library()
    xyz = np.zeros((n, 3), dtype=np.float32)
    _check(L.nc_reference_positions(n, _p(xyz)))
    cnt = ctypes.c_int64(0)
    _check(L.nc_reference_connection_count(n, _p(xyz), ctypes.byref(cnt)))
    s = cnt.value
    pre = np.zeros(s, dtype=np.int32)
    post = np.zeros(s, dtype=np.int32)
    w = np.zeros(s, dtype=np.float32)
    _check(L.nc_reference_connections(n, _p(xyz), _p(pre), _p(post), _p(w), s))
    return xyz, pre, post, w


@dataclass
class NeuronSnapshot:       # NeuCor::NeuronSnapshot (src/NeuCor.h:38-43)
    id: int
    position: tuple
    potential: float
    activity: float


@dataclass
class SynapseSnapshot:      # NeuCor::SynapseSnapshot (src/NeuCor.h:45-54)
    fromID: int
    toID: int
    from_: tuple
    to: tuple
    weight: float
    prePotential: float
    postPotential: float
    inhibitory: bool


@dataclass
class InputSnapshot:        # NeuCor::InputSnapshot (src/NeuCor.h:56-62)
    id: int
    position: tuple
    radius: float
    frequency: float
    enabled: bool


class NeuCor:
    """GPU-resident NeuroCorrelation network with the reference's method names.

    ``NeuCor(0)`` followed by ``createNeuron`` / ``createSynapse`` builds a network the
    way the reference's presets do (src/main.cpp:162-189); the network is uploaded at
    the first ``run``.  ``NeuCor.from_arrays`` builds it from positions and synapse
    arrays in one call.
    """

    def __init__(self, n_neurons: int = 0, params: Params | None = None, seed: int | None = None):
        self._lib = load_library()
        self._h = None
        self._params = params if params is not None else default_params()
        if seed is not None:
            self._params.seed = seed
        self._pos: list = []
        self._syn: list = []
        self._groups: list = []
        self._pending_fires: list = []
        if n_neurons:
            xyz, pre, post, w = build_reference_random(n_neurons, int(self._params.seed) & 0xffffffff)
            self._pos = [tuple(map(float, p)) for p in xyz]
            self._syn = list(zip(pre.tolist(), post.tolist(), w.tolist()))

    # ------------------------------------------------------------ construction
    @classmethod
    def from_arrays(cls, xyz, pre, post, weight, length=None, params: Params | None = None, inhibitory=None, **kw):
        self = cls(0, params=params)
        for k, v in kw.items():
            setattr(self._params, k, v)
        self._materialize(xyz, pre, post, weight, length, inhibitory)
        return self

    @classmethod
    def knn(cls, n: int, k: int, density: float = 8.0, seed: int = 1, params: Params | None = None, **kw):
        """The network build_knn(n, k, density, seed) describes, built on the GPU
        (nc_create_knn): identical to from_arrays(*build_knn(...)).  The kNN seed draws
        the positions and weights; params.seed keys the simulation's own draws."""
        self = cls(0, params=params)
        for key, v in kw.items():
            setattr(self._params, key, v)
        xyz = np.zeros((int(n), 3), dtype=np.float32)
        h = ctypes.c_void_p()
        _check(self._lib.nc_create_knn(int(n), int(k), float(density), int(seed), ctypes.byref(self._params),
                                       _p(xyz), ctypes.byref(h)))
        self._h = h
        self._xyz = xyz
        self.n = int(n)
        self.n_input_synapses = int(n) * int(k)
        return self

    def createNeuron(self, position):
        """NeuCor::createNeuron (src/NeuCor.cpp:154-186), before the first run."""
        if self._h is not None:
            raise NeuCorError(-4, "the network is on the GPU; topology is fixed after the first run")
        self._pos.append(tuple(float(v) for v in position))

    def createSynapse(self, toID: int, fromID: int, weight: float):
        """NeuCor::createSynapse (src/NeuCor.cpp:187-195), before the first run."""
        if self._h is not None:
            raise NeuCorError(-4, "the network is on the GPU; topology is fixed after the first run")
        self._syn.append((int(fromID), int(toID), float(weight)))

    def _materialize(self, xyz=None, pre=None, post=None, weight=None, length=None, inhibitory=None):
        if xyz is None:
            xyz = np.asarray(self._pos, dtype=np.float32).reshape(-1, 3)
            if self._syn:
                pre, post, weight = (np.asarray(c) for c in zip(*self._syn))
            else:
                pre = post = np.zeros(0, np.int32)
                weight = np.zeros(0, np.float32)
        self._xyz = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
        self._pre = np.ascontiguousarray(pre, dtype=np.int32)
        self._post = np.ascontiguousarray(post, dtype=np.int32)
        self._w0 = np.ascontiguousarray(weight, dtype=np.float32)
        ln = None if length is None else np.ascontiguousarray(length, dtype=np.float32)
        inh = None if inhibitory is None else np.ascontiguousarray(inhibitory, dtype=np.uint8)
        h = ctypes.c_void_p()
        _check(self._lib.nc_create(self._xyz.shape[0], _p(self._xyz), self._pre.shape[0], _p(self._pre),
                                   _p(self._post), _p(self._w0), _p(ln), _p(inh), ctypes.byref(self._params),
                                   ctypes.byref(h)))
        self._h = h
        self.n = int(self._xyz.shape[0])
        self.n_input_synapses = int(self._pre.shape[0])
        if self._groups:
            self._apply_groups()
        if self._pending_fires:
            self.schedule_fire(self._pending_fires)
            self._pending_fires = []

    def _handle(self):
        if self._h is None:
            self._materialize()
        return self._h

    def close(self):
        if self._h is not None:
            self._lib.nc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------ inputs
    def set_input_groups(self, groups):
        """Poisson input groups: dicts with first, count, rate_hz, correlated, jitter."""
        self._groups = list(groups)
        if self._h is not None:
            self._apply_groups()

    def _apply_groups(self):
        arr = (Group * max(1, len(self._groups)))()
        for i, g in enumerate(self._groups):
            arr[i] = Group(int(g["first"]), int(g["count"]), float(g["rate_hz"]), int(g.get("correlated", 1)),
                           int(g.get("jitter", 2)))
        _check(self._lib.nc_set_input_groups(self._h, len(self._groups), ctypes.cast(arr, ctypes.c_void_p)))

    def setInputRateArray(self, inputs, inputCount=None, inputPositions=None, inputRadius=None):
        """NeuCor::setInputRateArray (src/NeuCor.cpp:46-64): periodic input firers at the
        given rates (Hz); positions (n x 3) and radii for the firers appended by this call
        (None: random positions from the C library's rand() and radius 1)."""
        rates = np.ascontiguousarray(inputs, dtype=np.float32).ravel()
        n = rates.size if inputCount is None else int(inputCount)
        xyz = rad = None
        if inputPositions is not None:
            xyz = np.ascontiguousarray(inputPositions, dtype=np.float32).reshape(-1, 3)
            rad = np.ascontiguousarray(inputRadius if inputRadius is not None else np.ones(len(xyz)),
                                       dtype=np.float32)
        _check(self._lib.nc_set_input_rate_array(self._handle(), _p(rates), n,
                                                 _p(xyz) if xyz is not None else None,
                                                 _p(rad) if rad is not None else None))

    def set_input_rates(self, rates):
        """New frequencies of the first len(rates) firers (the reference's borrowed array)."""
        r = np.ascontiguousarray(rates, dtype=np.float32).ravel()
        _check(self._lib.nc_set_input_rates(self._handle(), r.size, _p(r)))

    def addInputOffset(self, inputID, t):
        """NeuCor::addInputOffset (src/NeuCor.cpp:66-68)."""
        _check(self._lib.nc_add_input_offset(self._handle(), int(inputID), float(t)))

    def setDetectors(self, detectorNumber, detectorPositions=None, detectorRadius=None):
        """NeuCor::setDetectors (src/NeuCor.cpp:70-77)."""
        xyz = rad = None
        if detectorPositions is not None:
            xyz = np.ascontiguousarray(detectorPositions, dtype=np.float32).reshape(-1, 3)
            rad = np.ascontiguousarray(detectorRadius if detectorRadius is not None else np.ones(len(xyz)),
                                       dtype=np.float32)
        _check(self._lib.nc_set_detectors(self._handle(), int(detectorNumber), _p(xyz) if xyz is not None else None,
                                          _p(rad) if rad is not None else None))

    def getDetectorVoltages(self):
        """NeuCor::getDetectorVoltages (src/NeuCor.cpp:79-83)."""
        cnt = ctypes.c_int32()
        _check(self._lib.nc_get_detector_voltages(self._handle(), None, 0, ctypes.byref(cnt)))
        out = np.zeros(cnt.value, dtype=np.float32)
        if cnt.value:
            _check(self._lib.nc_get_detector_voltages(self._handle(), _p(out), cnt.value, ctypes.byref(cnt)))
        return out

    def getDetectorVoltage(self, ID):
        """NeuCor::getDetectorVoltage (src/NeuCor.cpp:75-77)."""
        v = ctypes.c_float()
        _check(self._lib.nc_get_detector_voltage(self._handle(), int(ID), ctypes.byref(v)))
        return float(v.value)

    def schedule_fire(self, ids):
        """Neuron::scheduleFire for the next step (src/NeuCor.cpp:658-661)."""
        if self._h is None:
            self._pending_fires.extend(int(i) for i in np.atleast_1d(ids))
            return
        ids = np.ascontiguousarray(np.atleast_1d(ids), dtype=np.int32)
        _check(self._lib.nc_schedule_fire(self._h, ids.size, _p(ids)))

    # -------------------------------------------------------------- parameters
    @property
    def runSpeed(self) -> float:
        return float(self._params.run_speed)

    @runSpeed.setter
    def runSpeed(self, v: float):
        if self._h is not None and float(v) != self.runSpeed:
            raise NeuCorError(-4, "runSpeed is fixed once the network is on the GPU")
        self._params.run_speed = float(v)

    @property
    def runAll(self) -> bool:
        return True  # every neuron is updated every step

    @runAll.setter
    def runAll(self, v: bool):
        if not v:
            raise NeuCorError(-4, "the GPU step updates every neuron every step (runAll=true)")

    def _rate(self, name, v=None):
        if v is None:
            return float(getattr(self._params, name))
        setattr(self._params, name, float(v))
        if self._h is not None:
            p = self._params
            _check(self._lib.nc_set_rates(self._h, p.learning_rate, p.presynaptic_factor, p.postsynaptic_factor))

    learningRate = property(lambda s: s._rate("learning_rate"), lambda s, v: s._rate("learning_rate", v))
    presynapticFactor = property(lambda s: s._rate("presynaptic_factor"),
                                 lambda s, v: s._rate("presynaptic_factor", v))
    postsynapticFactor = property(lambda s: s._rate("postsynaptic_factor"),
                                  lambda s, v: s._rate("postsynaptic_factor", v))

    @property
    def presynapticTraceDecay(self) -> float:
        return float(self._params.presynaptic_trace_decay)

    @presynapticTraceDecay.setter
    def presynapticTraceDecay(self, v):
        if self._h is not None:
            raise NeuCorError(-4, "trace decays are copied into synapses at construction")
        self._params.presynaptic_trace_decay = float(v)

    @property
    def postsynapticTraceDecay(self) -> float:
        return float(self._params.postsynaptic_trace_decay)

    @postsynapticTraceDecay.setter
    def postsynapticTraceDecay(self, v):
        if self._h is not None:
            raise NeuCorError(-4, "trace decays are copied into neurons at construction")
        self._params.postsynaptic_trace_decay = float(v)

    # --------------------------------------------------------------------- run
    def run(self, steps: int = 1):
        """NeuCor::run (src/NeuCor.cpp:583-617), `steps` times."""
        _check(self._lib.nc_run(self._handle(), int(steps)))

    def sync(self):
        _check(self._lib.nc_sync(self._handle()))

    @property
    def step_form(self) -> int:
        """The form the next steps run in: NC_STEP_DENSE or NC_STEP_EVENT."""
        v = ctypes.c_int32()
        _check(self._lib.nc_get_step_form(self._handle(), ctypes.byref(v)))
        return int(v.value)

    def set_step_form(self, form: int):
        """Pin a network created with NC_STEP_AUTO to a form, or hand the choice back (NC_STEP_AUTO)."""
        _check(self._lib.nc_set_step_form(self._handle(), int(form)))

    def getTime(self) -> float:
        v = ctypes.c_float()
        _check(self._lib.nc_get_time(self._handle(), ctypes.byref(v)))
        return float(v.value)

    @property
    def step(self) -> int:
        v = ctypes.c_int64()
        _check(self._lib.nc_get_step(self._handle(), ctypes.byref(v)))
        return int(v.value)

    def getNeuronCount(self) -> int:
        if self._h is None:
            return len(self._pos)
        n = ctypes.c_int32()
        _check(self._lib.nc_get_counts(self._h, ctypes.byref(n), None))
        return int(n.value)

    def record_raster(self, max_steps: int):
        _check(self._lib.nc_record_raster(self._handle(), int(max_steps)))

    def raster(self):
        """Recorded spike rows: (steps, ceil(N/8)) bytes, bit j = neuron j fired."""
        h = self._handle()
        steps = ctypes.c_int32()
        _check(self._lib.nc_read_raster(h, None, 0, ctypes.byref(steps)))
        out = np.zeros((steps.value, (self.n + 7) // 8), dtype=np.uint8)
        _check(self._lib.nc_read_raster(h, _p(out), out.size, ctypes.byref(steps)))
        return out

    # --------------------------------------------------------------- read-back
    @property
    def potAct(self):
        """NeuCor::potAct (src/NeuCor.h:105): [potential, activity] per neuron."""
        out = np.zeros(2 * self.getNeuronCount(), dtype=np.float32)
        _check(self._lib.nc_read_potact(self._handle(), _p(out)))
        return out

    def potentials(self):
        out = np.zeros(self.getNeuronCount(), dtype=np.float32)
        _check(self._lib.nc_read_potentials(self._handle(), _p(out)))
        return out

    @property
    def positions(self):
        out = np.zeros((self.getNeuronCount(), 3), dtype=np.float32)
        _check(self._lib.nc_read_positions(self._handle(), _p(out)))
        return out

    def lastFire(self):
        out = np.zeros(self.getNeuronCount(), dtype=np.float32)
        _check(self._lib.nc_read_last_fire(self._handle(), _p(out)))
        return out

    def weights(self):
        h = self._handle()
        out = np.zeros(self.n_input_synapses, dtype=np.float32)
        _check(self._lib.nc_read_weights(h, _p(out)))
        return out

    def inhibitory(self):
        h = self._handle()
        out = np.zeros(self.n_input_synapses, dtype=np.uint8)
        _check(self._lib.nc_read_inhibitory(h, _p(out)))
        return out

    def delays(self):
        h = self._handle()
        out = np.zeros(self.n_input_synapses, dtype=np.int32)
        _check(self._lib.nc_read_delays(h, _p(out)))
        return out

    def synapse_snapshot_array(self):
        h = self._handle()
        cnt = ctypes.c_int64()
        _check(self._lib.nc_read_synapse_snapshots(h, None, 0, ctypes.byref(cnt)))
        arr = (SynapseSnapshotC * max(1, cnt.value))()
        _check(self._lib.nc_read_synapse_snapshots(h, ctypes.cast(arr, ctypes.c_void_p), cnt.value,
                                                   ctypes.byref(cnt)))
        return arr[:cnt.value]

    def getNeuronSnapshots(self):
        """NeuCor::getNeuronSnapshots (src/NeuCor.cpp:99-113)."""
        pa = self.potAct
        pos = self.positions
        return [NeuronSnapshot(i, tuple(map(float, pos[i])), float(pa[2 * i]), float(pa[2 * i + 1]))
                for i in range(self.getNeuronCount())]

    def getSynapseSnapshots(self):
        """NeuCor::getSynapseSnapshots (src/NeuCor.cpp:115-134)."""
        pos = self.positions
        return [SynapseSnapshot(s.from_id, s.to_id, tuple(map(float, pos[s.from_id])), tuple(map(float, pos[s.to_id])),
                                float(s.weight), float(s.pre_potential), float(s.post_potential), bool(s.inhibitory))
                for s in self.synapse_snapshot_array()]

    def getInputSnapshots(self):
        """NeuCor::getInputSnapshots (src/NeuCor.cpp:136-152)."""
        h = self._handle()
        cnt = ctypes.c_int32()
        _check(self._lib.nc_read_input_snapshots(h, None, 0, ctypes.byref(cnt)))
        arr = (InputSnapshotC * max(1, cnt.value))()
        if cnt.value:
            _check(self._lib.nc_read_input_snapshots(h, ctypes.cast(arr, ctypes.c_void_p), cnt.value,
                                                     ctypes.byref(cnt)))
        return [InputSnapshot(int(r.id), (float(r.x), float(r.y), float(r.z)), float(r.radius), float(r.frequency),
                              bool(r.enabled)) for r in arr[:cnt.value]]

    def resetActivities(self):
        _check(self._lib.nc_reset_activities(self._handle()))

    def stats(self) -> dict:
        s = _Stats()
        _check(self._lib.nc_get_stats(self._handle(), ctypes.byref(s)))
        return {f: int(getattr(s, f)) for f, _ in _Stats._fields_}

    def time_steps(self, steps: int, per_kernel: bool = False):
        """Runs `steps` steps timed with CUDA events; returns (ms, [neuron_ms, launch_ms] or None)."""
        ms = ctypes.c_float()
        km = (ctypes.c_float * 2)() if per_kernel else None
        _check(self._lib.nc_time_steps(self._handle(), int(steps), ctypes.byref(ms),
                                       ctypes.cast(km, ctypes.c_void_p) if km is not None else None))
        return float(ms.value), (list(km) if km is not None else None)

    def deleteSynapse(self, fromID, toID):
        _check(self._lib.nc_delete_synapse(self._handle(), int(fromID), int(toID)))

    def deleteNeuron(self, ID):
        _check(self._lib.nc_delete_neuron(self._handle(), int(ID)))


def _nan_to_none(v):
    return None if (isinstance(v, float) and math.isnan(v)) else v


class Batch:
    """Many independent networks advanced together in one device engine (nc_batch_*).

    ``nets`` is a list of dicts: xyz, pre, post, weight (arrays), and optionally length,
    inhibitory, params (Params), groups (list of dicts), horizon (steps)."""

    def __init__(self, nets):
        self._lib = load_library()
        self._keep = []
        specs = (NetSpec * len(nets))()
        self.n_input = []
        for q, d in enumerate(nets):
            xyz = np.ascontiguousarray(d["xyz"], dtype=np.float32).reshape(-1, 3)
            pre = np.ascontiguousarray(d["pre"], dtype=np.int32)
            post = np.ascontiguousarray(d["post"], dtype=np.int32)
            w = np.ascontiguousarray(d["weight"], dtype=np.float32)
            ln = d.get("length")
            ln = None if ln is None else np.ascontiguousarray(ln, dtype=np.float32)
            inh = d.get("inhibitory")
            inh = None if inh is None else np.ascontiguousarray(inh, dtype=np.uint8)
            groups = d.get("groups", [])
            garr = (Group * max(1, len(groups)))()
            for i, g in enumerate(groups):
                garr[i] = Group(int(g["first"]), int(g["count"]), float(g["rate_hz"]), int(g.get("correlated", 1)),
                                int(g.get("jitter", 2)))
            self._keep += [xyz, pre, post, w, ln, inh, garr]
            specs[q] = NetSpec(xyz.shape[0], _p(xyz), pre.shape[0], _p(pre), _p(post), _p(w), _p(ln), _p(inh),
                               d.get("params") or default_params(), len(groups), ctypes.cast(garr, ctypes.c_void_p),
                               int(d.get("horizon", 1 << 30)))
            self.n_input.append(pre.shape[0])
        self.sizes = [int(np.asarray(d["xyz"]).reshape(-1, 3).shape[0]) for d in nets]
        h = ctypes.c_void_p()
        _check(self._lib.nc_batch_create(len(nets), ctypes.cast(specs, ctypes.c_void_p), ctypes.byref(h)))
        self._h = h
        self._keep = []

    def close(self):
        if getattr(self, "_h", None):
            self._lib.nc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, steps: int):
        _check(self._lib.nc_batch_run(self._h, int(steps)))

    def time(self, steps: int) -> float:
        ms = ctypes.c_float()
        _check(self._lib.nc_batch_time(self._h, int(steps), ctypes.byref(ms)))
        return float(ms.value)

    def run_to_end(self):
        _check(self._lib.nc_batch_run_to_end(self._h))

    def launch(self) -> dict:
        c = LaunchConfig()
        _check(self._lib.nc_batch_get_launch(self._h, ctypes.byref(c)))
        return c.as_dict()

    def set_launch(self, **kw):
        c = LaunchConfig()
        _check(self._lib.nc_batch_get_launch(self._h, ctypes.byref(c)))
        for k, v in kw.items():
            setattr(c, k, int(v))
        _check(self._lib.nc_batch_set_launch(self._h, ctypes.byref(c)))

    def autotune(self, steps_per_trial: int = 50) -> dict:
        c = LaunchConfig()
        _check(self._lib.nc_batch_autotune(self._h, int(steps_per_trial), ctypes.byref(c)))
        return c.as_dict()

    def stats(self, net: int) -> dict:
        s = _Stats()
        _check(self._lib.nc_batch_get_stats(self._h, int(net), ctypes.byref(s)))
        return {f: int(getattr(s, f)) for f, _ in _Stats._fields_}

    def step(self, net: int) -> int:
        v = ctypes.c_int64()
        _check(self._lib.nc_batch_get_step(self._h, int(net), ctypes.byref(v)))
        return int(v.value)

    def potentials(self, net: int):
        out = np.zeros(self.sizes[net], dtype=np.float32)
        _check(self._lib.nc_batch_read_potentials(self._h, int(net), _p(out)))
        return out

    def weights(self, net: int):
        out = np.zeros(self.n_input[net], dtype=np.float32)
        _check(self._lib.nc_batch_read_weights(self._h, int(net), _p(out)))
        return out

    def lastFire(self, net: int):
        out = np.zeros(self.sizes[net], dtype=np.float32)
        _check(self._lib.nc_batch_read_last_fire(self._h, int(net), _p(out)))
        return out


class ServerConfig(ctypes.Structure):
    _fields_ = [("memory_budget_bytes", ctypes.c_int64), ("max_networks", ctypes.c_int32),
                ("steps_per_batch", ctypes.c_int32), ("build_threads", ctypes.c_int32),
                ("keep_results", ctypes.c_int32), ("step_mode", ctypes.c_int32)]


class RequestDone(ctypes.Structure):
    _fields_ = [("request_id", ctypes.c_int64), ("status", ctypes.c_int32), ("n_neurons", ctypes.c_int32),
                ("horizon", ctypes.c_int32), ("reserved", ctypes.c_int32), ("n_synapses", ctypes.c_int64),
                ("submit_s", ctypes.c_double), ("admit_s", ctypes.c_double), ("done_s", ctypes.c_double),
                ("stats", _Stats)]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_ if f != "stats"}
        d.update({f: int(getattr(self.stats, f)) for f, _ in _Stats._fields_})
        return d


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("admitted", ctypes.c_int64), ("finished", ctypes.c_int64),
                ("rejected", ctypes.c_int64), ("resident_bytes", ctypes.c_int64),
                ("peak_resident_bytes", ctypes.c_int64), ("peak_resident_networks", ctypes.c_int64),
                ("steps_run", ctypes.c_int64), ("device_busy_s", ctypes.c_double)]


class Server:
    """Request server (nc_server_*): networks submitted while others run are admitted by
    device footprint, advance together in shared launches and leave at their horizon."""

    def __init__(self, budget_bytes: int, max_networks: int = 256, steps_per_batch: int = 64,
                 build_threads: int = 8, keep_results: bool = False, step_mode: int = 0):
        self._lib = load_library()
        cfg = ServerConfig(int(budget_bytes), int(max_networks), int(steps_per_batch), int(build_threads),
                           int(bool(keep_results)), int(step_mode))
        h = ctypes.c_void_p()
        _check(self._lib.nc_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self.sizes = {}

    def submit(self, d) -> int:
        xyz = np.ascontiguousarray(d["xyz"], dtype=np.float32).reshape(-1, 3)
        pre = np.ascontiguousarray(d["pre"], dtype=np.int32)
        post = np.ascontiguousarray(d["post"], dtype=np.int32)
        w = np.ascontiguousarray(d["weight"], dtype=np.float32)
        groups = d.get("groups", [])
        garr = (Group * max(1, len(groups)))()
        for i, g in enumerate(groups):
            garr[i] = Group(int(g["first"]), int(g["count"]), float(g["rate_hz"]), int(g.get("correlated", 1)),
                            int(g.get("jitter", 2)))
        spec = NetSpec(xyz.shape[0], _p(xyz), pre.shape[0], _p(pre), _p(post), _p(w), None, None,
                       d.get("params") or default_params(), len(groups), ctypes.cast(garr, ctypes.c_void_p),
                       int(d["horizon"]))
        rid = ctypes.c_int64()
        _check(self._lib.nc_server_submit(self._h, ctypes.byref(spec), ctypes.byref(rid)))
        self.sizes[rid.value] = (xyz.shape[0], pre.shape[0])
        return int(rid.value)

    def submit_knn(self, n: int, k: int, density: float, knn_seed: int, horizon: int, params=None, groups=()) -> int:
        """A request for the network build_knn(n, k, density, knn_seed) describes, built by
        one of the server's builder threads (no arrays cross the call)."""
        groups = list(groups)
        garr = (Group * max(1, len(groups)))()
        for i, g in enumerate(groups):
            garr[i] = Group(int(g["first"]), int(g["count"]), float(g["rate_hz"]), int(g.get("correlated", 1)),
                            int(g.get("jitter", 2)))
        p = params or default_params()
        rid = ctypes.c_int64()
        _check(self._lib.nc_server_submit_knn(self._h, int(n), int(k), float(density), int(knn_seed), ctypes.byref(p),
                                              len(groups), ctypes.cast(garr, ctypes.c_void_p), int(horizon),
                                              ctypes.byref(rid)))
        self.sizes[rid.value] = (int(n), int(n) * int(k))
        return int(rid.value)

    def poll(self, capacity: int = 4096):
        arr = (RequestDone * capacity)()
        n = ctypes.c_int32()
        _check(self._lib.nc_server_poll(self._h, ctypes.cast(arr, ctypes.c_void_p), capacity, ctypes.byref(n)))
        return [arr[i].as_dict() for i in range(n.value)]

    def drain(self):
        _check(self._lib.nc_server_drain(self._h))

    def fetch(self, rid: int):
        n, s = self.sizes[rid]
        w = np.zeros(s, dtype=np.float32)
        pot = np.zeros(n, dtype=np.float32)
        _check(self._lib.nc_server_fetch(self._h, int(rid), _p(w), _p(pot)))
        return w, pot

    def stats(self) -> dict:
        st = ServerStats()
        _check(self._lib.nc_server_get_stats(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.nc_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
