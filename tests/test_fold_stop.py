"""The neuron passes stop a fold once the neuron is certain to fire, on networks whose
terms are all >= 0 (no inhibitory synapse, no negative weight).  The argument: each
`float += double` step (src/NeuCor.cpp:695) rounds a value no smaller than the last and
rounding keeps the order, so the running sum never decreases; charge_passive
((pot + 70) * leak - 70, src/NeuCor.cpp:677-680) keeps the order too, so once the
threshold test (src/NeuCor.cpp:682-686) holds for a partial sum it holds for the full one,
and the potential of a neuron that fires is replaced by the AP table.

These tests check the arithmetic of that argument on the CPU, with the same IEEE
operations the kernels use (binary64 add, round to binary32, binary32 passive charge):
for every sequence of non-negative terms, a threshold crossing at any batch boundary is
also a crossing of the full sum.  The GPU tests check the kernels themselves against the
oracle, which always folds every term."""
import numpy as np

C52 = np.float32(np.float64(np.float32(0.2)) * 52.0)


def make_terms(w, dt):
    """The launch term of each weight: RN(RN((double)x * 0.9943) * exp(0.3702*dt)),
    x = dt * (c52 * w) in binary32."""
    x = np.float32(dt) * (C52 * w.astype(np.float32))
    return (x.astype(np.float64) * 0.9943) * np.exp(0.3702 * dt)


def fires_at(pot, leak):
    pot = pot.astype(np.float32)
    return np.float32(-55.0) < (pot - np.float32(-70.0)) * leak + np.float32(-70.0)


def check(pot0, terms, leak, batch=8):
    """Folds terms (rows x k) into pot0 term by term; returns whether a crossing at a batch
    boundary was ever followed by a full sum that does not cross, and how many rows could
    stop early."""
    pot = pot0.astype(np.float32)
    crossed = fires_at(pot, leak)
    stopped = crossed.copy()
    for k in range(terms.shape[1]):
        pot = (pot.astype(np.float64) + terms[:, k]).astype(np.float32)
        if (k + 1) % batch == 0:
            c = fires_at(pot, leak)
            stopped |= c
            crossed |= c
    final = fires_at(pot, leak)
    return bool(np.any(crossed & ~final)), int(stopped.sum())


def test_fold_stop_matches_full_fold_random():
    rng = np.random.default_rng(7)
    for dt in (1.0, 0.5, 0.25, 0.1, 2.0):
        leak = np.float32(np.power(np.float32(0.5), np.float32(dt)))
        rows, k = 20000, 64
        pot0 = rng.uniform(-90.0, -20.0, rows).astype(np.float32)
        w = rng.random((rows, k)).astype(np.float32)
        w[rng.random((rows, k)) < 0.2] = 0.0
        w[rng.random((rows, k)) < 0.05] = -0.0
        bad, stopped = check(pot0, make_terms(w, dt), leak)
        assert not bad, dt
        assert stopped > 0


def test_fold_stop_matches_full_fold_near_threshold():
    """Starting potentials packed around the threshold of the passive charge and terms
    down to the smallest normal values, where the roundings decide."""
    rng = np.random.default_rng(11)
    leak = np.float32(0.5)
    # (pot + 70) * 0.5 - 70 > -55  <=>  pot > -40 (up to rounding)
    base = np.float32(-40.0)
    ulps = rng.integers(-64, 64, 50000).astype(np.int32)
    pot0 = (base.view(np.int32) + ulps).view(np.float32)
    terms = rng.choice(np.array([0.0, -0.0, 1e-30, 5e-8, 1e-6, 3e-6, 1e-3], np.float64), size=(50000, 24))
    bad, _ = check(pot0, terms, leak)
    assert not bad


def test_negative_term_breaks_the_argument():
    """Why the stop is limited to networks with no negative term: with one, a crossing at
    a batch boundary can be undone by the terms after it."""
    leak = np.float32(0.5)
    pot0 = np.array([-39.0], np.float32)
    terms = np.zeros((1, 16), np.float64)
    terms[0, :8] = 0.5
    terms[0, 8] = -20.0
    bad, _ = check(pot0, terms, leak)
    assert bad
