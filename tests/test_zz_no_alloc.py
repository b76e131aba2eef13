"""qs3g_cfrac_noalloc: the continued fraction for callers that cannot allocate.

Some host codes cannot call cudaMalloc: their own allocator has already
reserved the GPU's memory, or they run inside a time-stepping loop where the
device-wide synchronisation of cudaMalloc/cudaFree is not acceptable.  The
entry point stages its inputs and output in a fixed static device array
instead, so it must give the same spectra as qs3g_cfrac, call after call, and
refuse inputs larger than that array.  This file runs last so that a run that
stops at the first failure has already run every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _spectra(seed, nq, N, nomega):
    rng = np.random.default_rng(seed)
    alpha = rng.uniform(-1.0, 3.0, (nq, N))
    beta2 = rng.uniform(0.1, 2.0, (nq, N))
    beta2[:, 0] = 0.0
    nlev = rng.integers(1, N + 1, nq).astype(np.int32)
    norm1 = rng.uniform(0.5, 2.0, nq)
    E0 = rng.uniform(-5.0, -1.0, nq)
    omega = np.linspace(0.0, 6.0, nomega)
    return alpha, beta2, nlev, norm1, E0, omega


def test_noalloc_matches_cfrac_on_two_calls_in_a_row(qs3g):
    from ed_gb300 import capi
    # two different problems back to back: the second must not see the first's data
    for seed, nq, N, nomega, compat in ((1, 200, 150, 2000, True), (2, 7, 40, 333, False)):
        a, b, nl, n1, e0, om = _spectra(seed, nq, N, nomega)
        ref = capi.cfrac(a, b, nl, n1, e0, 0.05, om, compat)
        got = capi.cfrac_noalloc(a, b, nl, n1, e0, 0.05, om, compat)
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-14)


def test_noalloc_rejects_sizes_beyond_its_static_area(qs3g):
    from ed_gb300 import capi
    a, b, nl, n1, e0, om = _spectra(3, 300, 10, 2000)  # S alone needs 600000 doubles > 524288
    with pytest.raises(capi.QS3GError) as ei:
        capi.cfrac_noalloc(a, b, nl, n1, e0, 0.05, om)
    assert ei.value.code == capi.ERANGE
    assert "static area" in str(ei.value)
