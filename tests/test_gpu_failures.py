"""Failure detection without a GPU fault: every failure is made on the host
(an impossible size, a NaN in the start vector, an exhausted iteration cap,
a bad argument, a call out of order) and must come back as the documented
status code with the context still usable afterwards."""
import numpy as np
import pytest

from ed_gb300 import inputs

pytestmark = pytest.mark.gpu


def _chain(L, nod=None, K=0):
    from ed_gb300 import capi
    b, jxy, jz = inputs.chain_bonds(L, (1.0, 0.5), (0.3, 0.3))
    h = capi.Handle(L, L, 1, 1, b, jxy, jz)
    if nod is not None:
        h.build_sector(nod, (K, 0, 0))
    return h


def _code(fn):
    from ed_gb300 import capi
    with pytest.raises(capi.QS3GError) as e:
        fn()
    return e.value.code


def test_status_codes_and_recovery(qs3g):
    from ed_gb300 import capi
    h = _chain(1000)
    # sizes beyond what the kernels index: the reference's THS overflow stop
    assert _code(lambda: h.build_sector(8, (0, 0, 0))) == capi.ERANGE       # C(999, 7) anchored candidates
    assert _code(lambda: h.build_sector_u1(4)) == capi.ERANGE              # C(1000, 4) rows
    assert _code(lambda: h.build_sector(9, (0, 0, 0))) == capi.ENOTSUP
    # call out of order: no sector was built by the refused calls
    assert _code(lambda: h.connection_table_count()) == capi.ESTATE
    h.close()
    h = _chain(16, 4)
    D = h.D
    # the context is still usable after the refusals above
    y = h.hv(np.ones(D, complex))
    assert np.isfinite(y).all()
    # bad arguments (the reference's size checks, eigen_solver.f90:19-22)
    assert _code(lambda: h.trlan(1, 4, D + 8, maxitr=10)) == capi.EINVAL
    assert _code(lambda: h.trlan(5, 4, 12, maxitr=10)) == capi.EINVAL
    assert _code(lambda: h.trlan(1, 4, 12, maxitr=10, precision=3)) == capi.EINVAL
    # a NaN in the start vector: breakdown reported, not propagated as a result
    bad = np.ones(D, complex)
    bad[3] = np.nan
    assert _code(lambda: h.trlan(1, 4, 12, maxitr=50, start=bad)) == capi.EBREAKDOWN
    # an exhausted iteration cap: ENOTCONV with the best estimate returned
    r = h.trlan(1, 4, 12, maxitr=1, tol=1e-14, conv_mode=1, allow_unconverged=True)
    assert not r["converged"] and np.isfinite(r["ene"][0])
    assert _code(lambda: h.trlan(1, 4, 12, maxitr=1, tol=1e-14, conv_mode=1)) == capi.ENOTCONV
    # DSF: bad operator, S- from the sztot = 0 sector
    Spos = inputs.chain_positions(16)
    psi = np.ones(D, complex) / np.sqrt(D)
    assert _code(lambda: h.dsf(psi, 0.0, 4, [(0.0, 0.0, 0.0)], Spos, 5)) == capi.EINVAL
    h.close()
    h = _chain(16, 8)
    psi = np.ones(h.D, complex) / np.sqrt(h.D)
    assert _code(lambda: h.dsf(psi, 0.0, 2, [(0.0, 0.0, 0.0)], Spos, 5)) == capi.EINVAL
    # and a normal solve still works on the same process
    r = h.trlan(1, 4, 12, maxitr=500, tol=1e-10, conv_mode=1)
    assert r["converged"]
    h.close()
