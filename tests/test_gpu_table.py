"""qs3g_hv_cache: the cached connection table.

With the table cached, complex(8) and real FP64 products equal the
matrix-free ones bit for bit (same terms, same order); complex(4) / real FP32
products match the oracle to FP32 rounding; solvers reach the same
eigenvalues; the lock-step batch can run on tables.
"""
import numpy as np
import pytest

from ed_gb300 import inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CHAINS = [
    # (L, NOD, K, J1, J2): packed (k = 0, uniform), wide (k != 0), a non-uniform chain
    (20, 4, 0, (1.0, 0.5), (0.3, 0.3)),
    (20, 4, 3, (1.0, 0.5), (0.3, 0.3)),
    (23, 5, 0, (1.0, 1.3), (0.2, 0.4)),
    (23, 5, 7, (1.0, 1.3), (0.2, 0.4)),
    (16, 3, 0, (1.0, 0.5), None),
    (18, 2, 5, (1.0, 0.8), (0.4, 0.1)),
]


def _handle(L, nod, K, J1, J2, bonds=None):
    from ed_gb300 import capi
    b, jxy, jz = bonds if bonds else inputs.chain_bonds(L, J1, J2)
    h = capi.Handle(L, L, 1, 1, b, jxy, jz)
    D = h.build_sector(nod, (K, 0, 0))
    return h, D, (b, jxy, jz)


@pytest.mark.parametrize("L,nod,K,J1,J2", CHAINS)
def test_table_products_equal_matrix_free(qs3g, L, nod, K, J1, J2):
    h, D, (b, jxy, jz) = _handle(L, nod, K, J1, J2)
    rng = np.random.default_rng(L + K)
    x = rng.standard_normal(D) + 1j * rng.standard_normal(D)
    y0 = h.hv(x)
    xr = rng.standard_normal(D)
    yr0 = h.hv_real(xr) if K == 0 else None
    nb = h.hv_cache(True)
    deg = 4 if J2 is not None else 2
    per = 4 if (K == 0) else 8
    assert nb == nod * deg * D * per
    assert np.array_equal(h.hv(x), y0)
    if K == 0:
        assert np.array_equal(h.hv_real(xr), yr0)
        om = O.Model(L, L, 1, 1, b, jxy, jz, kmax=nod + 2)
        osec = om.build_sector(nod, (K, 0, 0))
        x32 = xr.astype(np.float32)
        ref = osec.hv(x32.astype(np.complex128)).real
        assert np.abs(h.hv32_real(x32) - ref).max() <= 2e-6 * np.abs(ref).max()
    assert h.hv_cache(False) == 0
    assert np.array_equal(h.hv(x), y0)
    h.close()


def test_table_on_a_general_chain(qs3g):
    """Bonds of unequal couplings (no uniform form): the wide table, k = 0."""
    L, nod = 14, 4
    rng = np.random.default_rng(3)
    b = np.array([(i, i % L + 1) for i in range(1, L + 1)] + [(i, (i + 1) % L + 1) for i in range(1, L + 1)])
    jxy = rng.uniform(0.5, 1.5, len(b))
    jz = rng.uniform(0.2, 1.0, len(b))
    h, D, _ = _handle(L, nod, 0, None, None, bonds=(b, jxy, jz))
    x = rng.standard_normal(D) + 1j * rng.standard_normal(D)
    y0 = h.hv(x)
    assert h.hv_cache(True) == nod * 4 * D * 8
    assert np.array_equal(h.hv(x), y0)
    h.close()


def test_trlan_with_table(qs3g):
    L, nod = 24, 4
    h, D, (b, jxy, jz) = _handle(L, nod, 0, (1.0, 0.5), (0.3, 0.3))
    r0 = h.trlan(2, 4, 12, maxitr=5000, tol=1e-10, precision=0, conv_mode=1, seed=3)
    a0 = h.trlan(1, 8, 24, maxitr=5000, tol=1e-10, precision=1, conv_mode=1, seed=3, real=True)
    h.hv_cache(True)
    r1 = h.trlan(2, 4, 12, maxitr=5000, tol=1e-10, precision=0, conv_mode=1, seed=3)
    a1 = h.trlan(1, 8, 24, maxitr=5000, tol=1e-10, precision=1, conv_mode=1, seed=3, real=True)
    assert np.array_equal(r0["ene"], r1["ene"]) and r0["iters"] == r1["iters"]
    # the double-float modes read the table in double-float arithmetic
    for prec, real in ((2, False), (2, True), (1, False)):
        d = h.trlan(2, 4, 12, maxitr=5000, tol=1e-10, precision=prec, conv_mode=1, seed=3, real=real)
        assert d["converged"] and d["resid"].max() <= 1e-10
        np.testing.assert_allclose(d["ene"], r0["ene"], rtol=0, atol=1e-10 * abs(r0["ene"][0]))
    assert a1["converged"] and abs(a1["ene"][0] - a0["ene"][0]) <= 1e-10 * abs(a0["ene"][0])
    w = np.linalg.eigvalsh(O.Model(L, L, 1, 1, b, jxy, jz, kmax=nod + 2).build_sector(nod, (0, 0, 0)).dense())
    assert abs(a1["ene"][0] - w[0]) <= 1e-10 * abs(w[0])
    h.close()


def test_table_refused_for_u1(qs3g):
    from ed_gb300 import capi
    b, jxy, jz = inputs.chain_bonds(12, (1.0, 0.7), None)
    h = capi.Handle(12, 12, 1, 1, b, jxy, jz)
    h.build_sector_u1(3)
    with pytest.raises(capi.QS3GError) as e:
        h.hv_cache(True)
    assert e.value.code == capi.ENOTSUP
    h.close()


@pytest.mark.parametrize("form", ["table", "deferred", "uniform"])
def test_lockstep_row_forms_match_dense(qs3g, monkeypatch, form):
    from ed_gb300 import sweep
    monkeypatch.setenv("QS3G_SEG_FORM", form)
    probs = sweep.random_chains(seed=9, n=8, L_range=(14, 20), nods=(3, 4, 5))
    recs, _, _ = sweep.solve(probs, NOE=2, NOK=4, NOM=12, tol=1e-10, precision=1, lockstep=True)
    for p, r in zip(probs, recs):
        assert r["status"] == 0, r
        b, jxy, jz = inputs.chain_bonds(p["L"], (1.0, p["delta"]), (p["j2"], p["j2"]))
        om = O.Model(p["L"], p["L"], 1, 1, b, jxy, jz, kmax=p["nod"] + 2)
        w = np.linalg.eigvalsh(om.build_sector(p["nod"], (p["K"], 0, 0)).dense())
        assert abs(r["ene"][0] - w[0]) <= 1e-9 * max(1.0, abs(w[0])), (form, r["ene"], w[:3])
        assert max(r["resid"]) <= 1e-10


@pytest.mark.parametrize("L,nod,K,J1,J2", CHAINS[:4])
def test_double_float_table_product(qs3g, L, nod, K, J1, J2):
    """qs3g_hv_df: the table product in double-float arithmetic stays within
    a few 2^-46 of the FP64 product; it needs the cached table."""
    from ed_gb300 import capi
    h, D, _ = _handle(L, nod, K, J1, J2)
    rng = np.random.default_rng(7 + K)
    x = rng.standard_normal(D) + 1j * rng.standard_normal(D)
    with pytest.raises(capi.QS3GError) as e:
        h.hv_df(x)
    assert e.value.code == capi.ESTATE
    y = h.hv(x)
    h.hv_cache(True)
    yd = h.hv_df(x)
    assert np.abs(yd - y).max() <= 1e-13 * np.abs(y).max()
    h.close()
