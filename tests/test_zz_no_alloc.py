"""qs3g_cfrac_noalloc: the continued fraction for callers that cannot allocate.

Some host codes cannot call cudaMalloc: their own allocator has already
reserved the GPU's memory, or they run inside a time-stepping loop where the
device-wide synchronisation of cudaMalloc/cudaFree is not acceptable.  The
entry point stages its inputs and output in a fixed static device array
instead, so it must give the same spectra as qs3g_cfrac, call after call, and
refuse inputs larger than that array.  Both entry points run the same kernel
on the same inputs, so the spectra must agree bit for bit; the sizes include
odd nq and nq, ldab, nomega that are not multiples of 32, so that every
padded region of the static area and the int32 pairs of nlev are exercised.
This file runs last so that a run that stops at the first failure has already
run every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATIC_DOUBLES = 524288


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
    # different problems back to back: a later call must not see an earlier call's data
    cases = ((1, 200, 150, 2000, True), (2, 7, 40, 333, False), (4, 33, 17, 65, True), (5, 1, 3, 1, False))
    for seed, nq, N, nomega, compat in cases:
        a, b, nl, n1, e0, om = _spectra(seed, nq, N, nomega)
        ref = capi.cfrac(a, b, nl, n1, e0, 0.05, om, compat)
        got = capi.cfrac_noalloc(a, b, nl, n1, e0, 0.05, om, compat)
        np.testing.assert_array_equal(got, ref)


def test_noalloc_at_the_size_limit(qs3g):
    """The largest accepted problem of a shape fills the area exactly; one more
    spectrum is refused."""
    from ed_gb300 import capi
    ldab, nomega = 31, 2000
    nq = 1
    while capi.cfrac_noalloc_doubles(nq + 1, ldab, nomega) <= STATIC_DOUBLES:
        nq += 1
    assert capi.cfrac_noalloc_doubles(nq, ldab, nomega) <= STATIC_DOUBLES
    a, b, nl, n1, e0, om = _spectra(6, nq, ldab, nomega)
    np.testing.assert_array_equal(capi.cfrac_noalloc(a, b, nl, n1, e0, 0.05, om),
                                  capi.cfrac(a, b, nl, n1, e0, 0.05, om))
    a, b, nl, n1, e0, om = _spectra(7, nq + 1, ldab, nomega)
    with pytest.raises(capi.QS3GError) as ei:
        capi.cfrac_noalloc(a, b, nl, n1, e0, 0.05, om)
    assert ei.value.code == capi.ERANGE


def test_noalloc_rejects_sizes_beyond_its_static_area(qs3g):
    from ed_gb300 import capi
    a, b, nl, n1, e0, om = _spectra(3, 300, 10, 2000)  # S alone needs 600000 doubles > 524288
    with pytest.raises(capi.QS3GError) as ei:
        capi.cfrac_noalloc(a, b, nl, n1, e0, 0.05, om)
    assert ei.value.code == capi.ERANGE
    assert "static area" in str(ei.value)


def test_cfrac_bindings_check_array_lengths(qs3g):
    """Short nlev / norm1 / E0 or a beta2 of another shape would make the C side read past
    the numpy buffers; the binding refuses them before the call."""
    from ed_gb300 import capi
    a, b, nl, n1, e0, om = _spectra(8, 5, 10, 50)
    for fn in (capi.cfrac, capi.cfrac_noalloc):
        with pytest.raises(ValueError):
            fn(a, b, nl[:4], n1, e0, 0.05, om)
        with pytest.raises(ValueError):
            fn(a, b, nl, n1[:3], e0, 0.05, om)
        with pytest.raises(ValueError):
            fn(a, b, nl, n1, e0[:1], 0.05, om)
        with pytest.raises(ValueError):
            fn(a, b[:, :9], nl, n1, e0, 0.05, om)
