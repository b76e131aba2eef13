"""Real Krylov vectors for sectors whose H is real symmetric (QS3G_REAL).

At k = 0 every hop phase of a chain is 1, and a U(1) sector has no phases, so
H is real symmetric and its eigenvectors can be taken real.  The real mode
stores the Lanczos vectors as real vectors (two rows per complex slot) and
keeps every scalar of the recurrence real.  Checks, through the C ABI:
  * real H*v = the real part of the complex H*v of (x, 0), bit for bit;
  * eigenvalues in all three precisions are eigenvalues of the dense H
    (1e-10 relative), the lowest is its ground state, and where the lowest
    NOE + 1 levels are nondegenerate they equal the complex solve's; FP64
    residuals <= tol; eigenvectors real, of unit norm (1e-9: one Gram-Schmidt
    pass per step, as in the reference) and equal to the complex ones up to a
    sign, for even and odd D (the odd case has a zero pad row).  A real start
    vector has one component in each eigenspace, so the second copy of a
    degenerate eigenvalue (the L = 12 Heisenberg case) is not expected;
  * a given start vector is used through its real part;
  * sectors with complex phases, and the lock-step batch, refuse the flag.
"""
import numpy as np
import pytest

from oracle import oracle as O
from ed_gb300 import capi, inputs

pytestmark = pytest.mark.gpu

CHAINS = [
    # (L, NOD, J1, J2): D = 19 (odd), 1038 (even), 245 (odd), 70 (even)
    (12, 3, (1.0, 1.0), None),
    (18, 6, (1.0, 0.5), (0.3, 0.3)),
    (20, 4, (1.0, 0.5), (0.3, 0.3)),
    (22, 3, (1.0, 0.5), (0.3, 0.3)),
]


def chain(L, nod, J1, J2, K=0):
    b, jxy, jz = inputs.chain_bonds(L, J1, J2)
    om = O.Model(L, L, 1, 1, b, jxy, jz, kmax=min(L, nod + 2))
    osec = om.build_sector(nod, (K, 0, 0))
    h = capi.Handle(L, L, 1, 1, b, jxy, jz)
    D = h.build_sector(nod, (K, 0, 0))
    assert D == osec.D
    return osec, h, D


@pytest.mark.parametrize("L,nod,J1,J2", CHAINS)
def test_real_hv_is_real_part_of_complex(qs3g, L, nod, J1, J2):
    _, h, D = chain(L, nod, J1, J2)
    x = np.random.default_rng(L).standard_normal(D)
    y = h.hv_real(x)
    yc = h.hv(x.astype(np.complex128))
    assert np.array_equal(y, yc.real)
    assert not np.any(yc.imag)
    h.close()


def test_real_hv_u1(qs3g):
    b, jxy, jz = inputs.chain_bonds(13, (1.0, 0.7), (0.25, 0.1))
    h = capi.Handle(13, 13, 1, 1, b, jxy, jz)
    D = h.build_sector_u1(4)  # C(13, 4) = 715, odd
    x = np.random.default_rng(5).standard_normal(D)
    assert np.array_equal(h.hv_real(x), h.hv(x.astype(np.complex128)).real)
    w = np.linalg.eigvalsh(np.array([h.hv_real(e) for e in np.eye(D)]).T)
    for prec in (0, 1, 2):
        r = h.trlan(2, 4, 12, maxitr=2000, tol=1e-10, precision=prec, conv_mode=1, seed=3, real=True)
        np.testing.assert_allclose(r["ene"], w[:2], rtol=1e-10, atol=1e-10)
        assert r["resid"].max() <= 1e-10
    h.close()


@pytest.mark.parametrize("L,nod,J1,J2", CHAINS)
@pytest.mark.parametrize("prec", [0, 1, 2])
def test_real_trlan_matches_complex(qs3g, L, nod, J1, J2, prec):
    osec, h, D = chain(L, nod, J1, J2)
    w = np.linalg.eigvalsh(osec.dense())
    NOE, NOK, NOM = (2, 4, 12) if D >= 12 else (1, 2, 4)
    r = h.trlan(NOE, NOK, NOM, maxitr=2000, tol=1e-10, precision=prec, conv_mode=1, seed=7, real=True)
    c = h.trlan(NOE, NOK, NOM, maxitr=2000, tol=1e-10, precision=prec, conv_mode=1, seed=7)
    assert r["converged"] and c["converged"]
    tol = 1e-10 * max(1.0, abs(w[0]))
    assert abs(r["ene"][0] - w[0]) <= tol
    assert all(np.min(np.abs(w - e)) <= tol for e in r["ene"])
    if np.all(np.diff(w[:NOE + 1]) > 1e-6):
        np.testing.assert_allclose(r["ene"], w[:NOE], rtol=1e-10, atol=1e-10)
        np.testing.assert_allclose(r["ene"], c["ene"], rtol=1e-10, atol=1e-10)
    assert r["resid"].max() <= 1e-10
    psi = r["psi"][0]
    assert not np.any(psi.imag)
    assert abs(np.linalg.norm(psi) - 1.0) < 1e-9
    # H psi = E psi from the complex(8) product
    assert np.linalg.norm(h.hv(psi) - r["ene"][0] * psi) <= 2e-10
    if w[1] - w[0] > 1e-6:  # nondegenerate ground state: the same vector up to a phase
        assert abs(abs(np.vdot(c["psi"][0], psi)) - 1.0) < 1e-9
    h.close()


def test_real_trlan_start_vector(qs3g):
    """A given start vector enters through its real part."""
    osec, h, D = chain(20, 4, (1.0, 0.5), (0.3, 0.3))
    w = np.linalg.eigvalsh(osec.dense())
    rng = np.random.default_rng(1)
    v = rng.standard_normal(D) + 1j * rng.standard_normal(D)
    a = h.trlan(1, 4, 12, maxitr=2000, tol=1e-10, precision=1, conv_mode=1, start=v, real=True)
    b = h.trlan(1, 4, 12, maxitr=2000, tol=1e-10, precision=1, conv_mode=1, start=v.real.copy(), real=True)
    assert a["ene"][0] == b["ene"][0] and a["iters"] == b["iters"]
    assert abs(a["ene"][0] - w[0]) <= 1e-10 * max(1.0, abs(w[0]))
    h.close()


def test_real_flag_refused_where_h_is_complex(qs3g):
    _, h, D = chain(12, 4, (1.0, 0.5), (0.3, 0.3), K=3)
    with pytest.raises(capi.QS3GError) as e:
        h.hv_real(np.ones(D))
    assert e.value.code == capi.ENOTSUP
    with pytest.raises(capi.QS3GError) as e:
        h.trlan(1, 2, 4, maxitr=10, tol=1e-10, real=True)
    assert e.value.code == capi.ENOTSUP
    h.close()
    _, h0, _ = chain(12, 3, (1.0, 1.0), None)
    with pytest.raises(capi.QS3GError) as e:
        capi.trlan_lockstep([h0], 1, 2, 4, maxitr=10, precision=1 | capi.REAL)
    assert e.value.code == capi.EINVAL
    h0.close()
