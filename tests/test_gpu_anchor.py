"""The anchored FP32 thick-restart Lanczos (qs3g_trlan precision 1, NOE = 1).

The approximation is kept in FP64 and every Krylov vector in FP32 (complex(4),
or real FP32 for k = 0 chains) to the end; the convergence test is the FP64
residual ||H x - E x|| of the FP64 vector itself.  Checked here: the lowest
eigenvalue against the oracle's sparse H to 1e-10, the returned residual at
the target, FP32 vectors carrying at least 85 % of the H*v products, and an
H*v count close to the all-FP64 solve (precision 0) from the same start.
"""
import numpy as np
import pytest
import scipy.sparse.linalg as sla

from ed_gb300 import inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = [
    # (L, NOD, K, J1, J2, real)
    (16, 4, 0, (1.0, 0.5), (0.3, 0.3), True),
    (16, 4, 0, (1.0, 0.5), (0.3, 0.3), False),
    (20, 4, 3, (1.0, 0.7), (0.2, 0.1), False),
    (24, 5, 0, (1.0, 1.0), None, True),
    (48, 4, 0, (1.0, 0.5), (0.3, 0.3), True),
    (40, 4, 7, (1.0, 2.0), (0.5, 0.5), False),
]


def _lowest(osec):
    Hs = osec.sparse()
    if osec.D <= 3000:
        return np.linalg.eigvalsh(Hs.toarray())[0]
    return sla.eigsh(Hs, k=1, which="SA", tol=1e-14, return_eigenvectors=False)[0]


@pytest.mark.parametrize("L,nod,K,J1,J2,real", CASES)
def test_anchored_lowest_eigenpair(qs3g, L, nod, K, J1, J2, real):
    from ed_gb300 import capi
    b, jxy, jz = inputs.chain_bonds(L, J1, J2)
    om = O.Model(L, L, 1, 1, b, jxy, jz, kmax=nod + 2)
    osec = om.build_sector(nod, (K, 0, 0))
    w0 = _lowest(osec)
    h = capi.Handle(L, L, 1, 1, b, jxy, jz)
    D = h.build_sector(nod, (K, 0, 0))
    assert D == osec.D
    NOK, NOM = (4, 12) if D < 200 else (8, 24)
    r = h.trlan(1, NOK, NOM, maxitr=5000, tol=1e-10, precision=1, conv_mode=1, seed=5, real=real)
    st = h.trlan_stats()
    assert r["converged"]
    assert abs(r["ene"][0] - w0) <= 1e-10 * max(1.0, abs(w0))
    assert r["resid"][0] <= 1e-10
    psi = r["psi"][0]
    res = np.linalg.norm(osec.hv(psi) - r["ene"][0] * psi) / np.linalg.norm(psi)
    assert res <= 1.5e-10
    assert st["hv_fp32"] >= 0.85 * (st["hv_fp32"] + st["hv_fp64"])
    # the all-FP64 solve from the same start needs about as many products
    r0 = h.trlan(1, NOK, NOM, maxitr=5000, tol=1e-10, precision=0, conv_mode=1, seed=5, real=real)
    assert r0["converged"]
    assert abs(r0["ene"][0] - r["ene"][0]) <= 1e-10 * max(1.0, abs(w0))
    assert r["iters"] <= 1.5 * r0["iters"] + 4 * NOM
    h.close()


def test_anchored_from_a_start_vector(qs3g):
    """A start vector near the ground state (another coupling's ground state)
    converges in fewer products than a random start."""
    from ed_gb300 import capi
    L, nod = 48, 4
    b, jxy, jz = inputs.chain_bonds(L, (1.0, 0.5), (0.3, 0.3))
    b2, jxy2, jz2 = inputs.chain_bonds(L, (1.0, 0.6), (0.25, 0.25))
    h2 = capi.Handle(L, L, 1, 1, b2, jxy2, jz2)
    h2.build_sector(nod, (0, 0, 0))
    near = h2.trlan(1, 8, 24, maxitr=5000, tol=1e-8, precision=1, conv_mode=1, seed=2, real=True)["psi"][0]
    h2.close()
    h = capi.Handle(L, L, 1, 1, b, jxy, jz)
    h.build_sector(nod, (0, 0, 0))
    rr = h.trlan(1, 8, 24, maxitr=5000, tol=1e-10, precision=1, conv_mode=1, seed=5, real=True)
    rs = h.trlan(1, 8, 24, maxitr=5000, tol=1e-10, precision=1, conv_mode=1, start=near, real=True)
    assert rr["converged"] and rs["converged"]
    assert abs(rr["ene"][0] - rs["ene"][0]) <= 1e-10 * abs(rr["ene"][0])
    assert rs["iters"] < rr["iters"]
    h.close()


def test_hv32_real_matches_oracle(qs3g):
    """qs3g_hv32_real: (H - shift) x in FP32 for real x, shift applied in FP64."""
    from ed_gb300 import capi
    L, nod = 20, 4
    b, jxy, jz = inputs.chain_bonds(L, (1.0, 0.5), (0.3, 0.3))
    om = O.Model(L, L, 1, 1, b, jxy, jz, kmax=nod + 2)
    osec = om.build_sector(nod, (0, 0, 0))
    h = capi.Handle(L, L, 1, 1, b, jxy, jz)
    D = h.build_sector(nod, (0, 0, 0))
    rng = np.random.default_rng(4)
    x = rng.standard_normal(D).astype(np.float32)
    sigma = 0.25 * jz.sum()
    y0 = osec.hv(x.astype(np.complex128)).real - sigma * x.astype(np.float64)
    y = h.hv32_real(x, shift=sigma)
    assert np.abs(y - y0).max() <= 2e-6 * np.abs(y0).max()
    assert np.abs(h.hv32_real(x) - osec.hv(x.astype(np.complex128)).real).max() <= 2e-6 * np.abs(y0).max() * 10
    h.close()
