"""The renderer's read-backs against the reference's own code (golden fixtures made by
tests/golden/make_golden.py from the reference's src/NeuCor.cpp), bit for bit, through
the C ABI:

* NeuCor::getSynapseSnapshots (src/NeuCor.cpp:115-134): weights and the pre/post render
  potentials of spikes in flight (Synapse::getPrePot/getPostPot, :547-570), at
  checkpoints of three networks at dt 1 and 0.5, both forms of the step kernels;
* NeuCor::getDetectorVoltages (:79-87, 359-366) at the same checkpoints;
* NeuCor::getInputSnapshots (:136-152) with firer positions drawn from the C library's
  rand() in the reference's order;

and the device-side failure path of the input firers: a schedule that would need more
passes than the kernel's cap in one step sets the handle's device error, which the next
synchronisation reports as NC_ERR_TIMEOUT."""
import ctypes

import numpy as np
import pytest

from scenario import groups_list, load, params_kw

pytestmark = pytest.mark.gpu

MODES = {"dense": 0, "event": 1}


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("name", ["snapshots_knn64", "snapshots_random40_dt05", "snapshots_knn200_busy"])
def test_gpu_synapse_snapshots_and_detectors_match_reference(nc, name, mode):
    G = nc
    fx = load(name)
    net = G.NeuCor.from_arrays(fx["xyz"], fx["pre"], fx["post"], fx["w"],
                               params=G.default_params(**dict(params_kw(fx), step_mode=MODES[mode])))
    net.set_input_groups(groups_list(fx))
    det = fx["detectors"]
    net.setDetectors(len(det), det[:, :3], det[:, 3])
    done = 0
    for q, ck in enumerate(int(c) for c in fx["checkpoints"]):
        net.run(ck - done)
        done = ck
        snap = net.synapse_snapshot_array()
        got_from = np.array([s.from_id for s in snap], np.int32)
        got_to = np.array([s.to_id for s in snap], np.int32)
        np.testing.assert_array_equal(got_from, fx["snap_from"][q], f"fromID at step {ck}")
        np.testing.assert_array_equal(got_to, fx["snap_to"][q], f"toID at step {ck}")
        for field, key in (("weight", "snap_weight"), ("pre_potential", "snap_pre"), ("post_potential", "snap_post")):
            got = np.array([getattr(s, field) for s in snap], np.float32)
            bad = bits(got) != bits(fx[key][q])
            assert not bad.any(), (f"{field} at step {ck}: {int(bad.sum())} differ, first synapse "
                                   f"{int(np.argmax(bad))}: gpu {got[bad][0]!r} reference {fx[key][q][bad][0]!r}")
        np.testing.assert_array_equal(np.array([s.inhibitory for s in snap], np.uint8), fx["snap_inh"][q])
        np.testing.assert_array_equal(bits(net.getDetectorVoltages()), bits(fx["voltages"][q]),
                                      f"detector voltages at step {ck}")
    assert (fx["snap_pre"] != 0).any(), "the fixture has spikes in flight"


def test_gpu_input_snapshots_match_reference(nc):
    """setInputRateArray with no positions draws each firer's position from rand();
    after the same srand the GPU handle reports the reference's getInputSnapshots."""
    G = nc
    fx = load("input_snapshots_seed4")
    libc = ctypes.CDLL(None)
    net = G.NeuCor.from_arrays(fx["xyz"], np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32))
    libc.srand(int(fx["seed"]))
    net.setInputRateArray(fx["rates"])
    snaps = net.getInputSnapshots()
    assert len(snaps) == len(fx["snap"])
    for s, ref, en in zip(snaps, fx["snap"], fx["enabled"]):
        assert s.id == int(ref[0])
        got = np.array([*s.position, s.radius, s.frequency], np.float32)
        np.testing.assert_array_equal(bits(got), bits(ref[1:]))
        assert s.enabled == bool(en)
    # the rates stay live: a later rate change shows in the snapshot, as inputArray does
    rates = fx["rates"].copy()
    rates[1] = 7.5
    net._lib.nc_set_input_rates(net._handle(), len(rates), rates.ctypes.data_as(ctypes.c_void_p))
    assert net.getInputSnapshots()[1].frequency == np.float32(7.5)


def test_gpu_firer_loop_cap_reports_device_error(nc):
    """A 1 GHz firer at dt 2 ms would need two million schedule passes in one step; the
    kernel stops at its cap, sets the device error, and the handle reports
    NC_ERR_TIMEOUT at the next synchronisation (no fault, no hang)."""
    G = nc
    xyz, pre, post, w = G.build_knn(64, 4, 8.0, seed=2)
    net = G.NeuCor.from_arrays(xyz, pre, post, w, params=G.default_params(run_speed=2.0))
    net.setInputRateArray(np.array([1e9], np.float32), inputPositions=xyz[:1], inputRadius=np.ones(1, np.float32))
    net.run(1)
    with pytest.raises(G.NeuCorError) as e:
        net.sync()
    assert e.value.code == -6
