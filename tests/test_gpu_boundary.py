"""Boundary forms for the reference's Fortran caller, through the C ABI.

* qs3g_build_sector_i32 / qs3g_get_sector_i32: THS and list_s as default-kind
  integers (source/main.f90:28-34, source/ham2vec_v3.f90:45), refused with
  QS3G_ERANGE where the codes do not fit (the L=1000, N_down=4 chain, whose
  C(1000,4) ~ 4.1e10 overflows the reference's own integer);
* qs3g_load_sector(_i32): a sector the caller enumerated itself (the oracle's
  allocate_lists_omp_SQ restatement here) is adopted when it is the
  (NOD, K) sector, refused row by row otherwise, the previous sector kept;
* qs3g_set_time_limit / qs3g_trlan_stats.
"""
import numpy as np
import pytest

from ed_gb300 import inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _chain(L, J1=(1.0, 0.5), J2=(0.3, 0.3)):
    from ed_gb300 import capi
    b, jxy, jz = inputs.chain_bonds(L, J1, J2)
    return capi.Handle(L, L, 1, 1, b, jxy, jz), O.Model(L, L, 1, 1, b, jxy, jz, kmax=8), b, jxy, jz


def test_i32_build_and_get(qs3g):
    h, om, *_ = _chain(20)
    D64 = h.build_sector(4, (3, 0, 0))
    ls, lr = h.get_sector()
    D32 = h.build_sector_i32(4, (3, 0, 0))
    assert D32 == D64
    ls32, lr32 = h.get_sector_i32()
    assert ls32.dtype == np.int32
    np.testing.assert_array_equal(ls32, ls)
    np.testing.assert_array_equal(lr32, lr)
    h.close()


def test_i32_refuses_codes_beyond_default_integer(qs3g):
    from ed_gb300 import capi
    h, *_ = _chain(1000)
    with pytest.raises(capi.QS3GError) as ei:
        h.build_sector_i32(4, (0, 0, 0))
    assert ei.value.code == capi.ERANGE
    h.build_sector(4, (0, 0, 0))
    with pytest.raises(capi.QS3GError) as ei:
        h.get_sector_i32()
    assert ei.value.code == capi.ERANGE
    h.close()


@pytest.mark.parametrize("i32", [False, True])
def test_load_sector_adopts_the_callers_lists(qs3g, i32):
    from ed_gb300 import capi
    h, om, b, jxy, jz = _chain(18)
    osec = om.build_sector(5, (4, 0, 0))
    D = h.load_sector(5, (4, 0, 0), osec.list_s, osec.list_r, i32=i32)
    assert D == osec.D
    rng = np.random.default_rng(1)
    x = rng.standard_normal(D) + 1j * rng.standard_normal(D)
    y0 = osec.hv(x)
    assert np.abs(h.hv(x) - y0).max() <= 1e-13 * np.abs(y0).max()
    # a list that is not the (NOD, K) sector is refused and the loaded sector stays
    bad = osec.list_s.copy()
    bad[7] += 1
    with pytest.raises(capi.QS3GError) as ei:
        h.load_sector(5, (4, 0, 0), bad, osec.list_r, i32=i32)
    assert ei.value.code == capi.EINVAL and "list_s(8)" in str(ei.value)
    with pytest.raises(capi.QS3GError) as ei:
        h.load_sector(5, (4, 0, 0), osec.list_s[:-1], osec.list_r[:-1], i32=i32)
    assert ei.value.code == capi.EINVAL
    h.D = D
    assert np.abs(h.hv(x) - y0).max() <= 1e-13 * np.abs(y0).max()
    with pytest.raises(ValueError):
        h.load_sector(5, (4, 0, 0), osec.list_s, osec.list_r[:-1], i32=i32)
    h.close()


def test_time_limit_and_stats(qs3g):
    h, *_ = _chain(24)
    h.build_sector(4, (0, 0, 0))
    r = h.trlan(1, 4, 12, maxitr=500, tol=1e-10, precision=1, conv_mode=1, seed=3)
    st = h.trlan_stats()
    assert r["converged"] and not st["timed_out"]
    assert st["hv_fp32"] > 0 and st["hv_fp64"] > 0 and st["hv_fp32"] + st["hv_fp64"] == r["iters"]
    assert st["restarts"] > 0 and st["seconds"] > 0
    r0 = h.trlan(1, 4, 12, maxitr=500, tol=1e-10, precision=0, conv_mode=1, seed=3)
    st0 = h.trlan_stats()
    assert st0["hv_fp32"] == 0 and st0["hv_fp64"] == r0["iters"]
    # a limit far below one restart stops the solve at its first restart, not converged
    h.set_time_limit(1e-6)
    rt = h.trlan(1, 4, 12, maxitr=500, tol=1e-14, precision=0, conv_mode=1, seed=3, allow_unconverged=True)
    stt = h.trlan_stats()
    assert not rt["converged"] and stt["timed_out"] and stt["restarts"] == 1
    assert np.isfinite(rt["ene"][0])
    h.set_time_limit(0.0)
    r2 = h.trlan(1, 4, 12, maxitr=500, tol=1e-10, precision=0, conv_mode=1, seed=3)
    assert r2["converged"] and not h.trlan_stats()["timed_out"]
    h.close()
