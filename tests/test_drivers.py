"""CPU tests of the host-side drivers: problem generators and the band
minimum used as the network's Fourier input (no GPU calls)."""
import numpy as np

from ed_gb300 import capi, learned, sweep


def test_band_minimum():
    # cos q + J2 cos 2q: minimum at pi up to J2 = 1/4, then cos q0 = -1/(4 J2)
    assert capi.band_minimum(1.0, 0.0) == np.pi
    assert capi.band_minimum(1.0, 0.25) == np.pi
    assert abs(capi.band_minimum(1.0, 0.5) - 2 * np.pi / 3) < 1e-15
    for j2 in (0.3, 0.4, 0.5):
        q = np.linspace(0, 2 * np.pi, 200001)
        e = np.cos(q) + j2 * np.cos(2 * q)
        qmin = q[np.argmin(e)]
        q0 = capi.band_minimum(1.0, j2)
        assert min(abs(qmin - q0), abs(qmin - (2 * np.pi - q0))) < 1e-4


def test_random_chains_follow_the_workload_ranges():
    a = sweep.random_chains(seed=1, n=256)
    b = sweep.random_chains(seed=1, n=256)
    assert a == b
    assert len(a) == 256
    for p in a:
        assert 48 <= p["L"] <= 128 and p["nod"] in (3, 4, 5) and 0 <= p["K"] < p["L"]
        assert 0.0 <= p["delta"] <= 2.0 and 0.0 <= p["j2"] <= 0.5
    assert {p["nod"] for p in a} == {3, 4, 5}


def test_training_problems_grid():
    probs = learned.training_problems(seed=1)
    assert probs == learned.training_problems(seed=1)
    assert sorted({L for L, _, _ in probs}) == [48, 64, 80, 96, 112, 128]
    assert len(probs) == 24
    assert all(0.0 <= d <= 2.0 and 0.0 <= j <= 0.5 for _, d, j in probs)
    d, j, q0 = learned.cond(0.7, 0.25)
    assert (d, j) == (0.7, 0.25) and q0 == np.pi
