"""nc_run_noalloc — the step for callers that cannot let the library allocate device
memory once the network is set up: a service that reserves a fixed device budget up
front and admits work against it, or a host program whose own allocator owns the GPU's
memory (an engine embedding the simulator), where an allocation behind its back can
fail or break its accounting.

It launches the same kernels as nc_run (the event form with its per-step scratch in a
static device array; the dense form needs none), so it must compute exactly what nc_run
computes; checked on two calls in a row in both forms, bit for bit (the tolerance of
every parity test here), through the C ABI, on the handle's stream and on a stream the
caller owns."""
import ctypes

import numpy as np
import pytest

from netgen import knn_net

pytestmark = pytest.mark.gpu


def noalloc_fn(G):
    L = G.load_library()
    fn = L.nc_run_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]
    fn.restype = ctypes.c_int32
    return fn, L


def make_pair(G, mode):
    xyz, pre, post, w = knn_net(2500, 12, 77, inhibitory=0.1)
    groups = [dict(first=0, count=25, rate_hz=30.0, correlated=1, jitter=2),
              dict(first=25, count=25, rate_hz=30.0, correlated=0)]
    nets = []
    for _ in range(2):
        net = G.NeuCor.from_arrays(xyz, pre, post, w, params=G.default_params(seed=4242, step_mode=mode))
        net.set_input_groups(groups)
        nets.append(net)
    return nets


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def caller_stream():
    """A CUDA stream the caller owns (created outside the library)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch has no CUDA device")
    return torch, torch.cuda.Stream(device=0)


@pytest.mark.parametrize("mode", [0, 1], ids=["dense", "event"])
def test_noalloc_on_a_caller_stream(nc, mode):
    """Two calls on a stream the caller created; the caller synchronises it before
    reading, and the handle's step and time follow the device."""
    run_noalloc, L = noalloc_fn(nc)
    torch, stream = caller_stream()
    ref, na = make_pair(nc, mode)
    for call in range(2):
        ref.record_raster(90)
        na.record_raster(90)
        ref.run(90)
        na.sync()  # the handle's earlier work (the raster set-up) before the caller's stream
        rc = run_noalloc(na._handle(), 90, ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, L.nc_last_error().decode()
        stream.synchronize()
        np.testing.assert_array_equal(na.raster(), ref.raster())
        np.testing.assert_array_equal(bits(na.potentials()), bits(ref.potentials()))
        np.testing.assert_array_equal(bits(na.weights()), bits(ref.weights()))
        np.testing.assert_array_equal(bits(na.potAct), bits(ref.potAct))
        sa, sr = na.stats(), ref.stats()
        assert (sa["fires"], sa["launched"], sa["dropped"], sa["steps"]) == \
            (sr["fires"], sr["launched"], sr["dropped"], sr["steps"])
        assert na.step == ref.step == 90 * (call + 1)
        assert np.float32(na.getTime()).view(np.uint32) == np.float32(ref.getTime()).view(np.uint32)


@pytest.mark.parametrize("mode", [0, 1], ids=["dense", "event"])
def test_noalloc_matches_run_on_two_calls(nc, mode):
    run_noalloc, L = noalloc_fn(nc)
    ref, na = make_pair(nc, mode)
    for call in range(2):
        ref.record_raster(120)
        na.record_raster(120)
        ref.run(120)
        rc = run_noalloc(na._handle(), 120, None)  # NULL stream: the handle's own stream
        assert rc == 0, L.nc_last_error().decode()
        np.testing.assert_array_equal(na.raster(), ref.raster())
        np.testing.assert_array_equal(bits(na.potentials()), bits(ref.potentials()))
        np.testing.assert_array_equal(bits(na.weights()), bits(ref.weights()))
        np.testing.assert_array_equal(bits(na.potAct), bits(ref.potAct))
        sa, sr = na.stats(), ref.stats()
        assert (sa["fires"], sa["launched"], sa["dropped"], sa["steps"]) == \
            (sr["fires"], sr["launched"], sr["dropped"], sr["steps"])
        assert sr["fires"] > 0
        assert na.step == ref.step == 120 * (call + 1)


def test_noalloc_refuses_event_networks_above_its_limit(nc):
    run_noalloc, L = noalloc_fn(nc)
    limit = 262144
    xyz, pre, post, w = nc.build_knn(limit + 1, 2, 8.0, seed=3)
    big = nc.NeuCor.from_arrays(xyz, pre, post, w, params=nc.default_params(step_mode=1))
    rc = run_noalloc(big._handle(), 1, None)
    assert rc == -1
    assert str(limit) in L.nc_last_error().decode()
    assert big.step == 0
