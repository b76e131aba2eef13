"""ALG = 3 on the GPU: the dense sector H (make_full_hamiltonian) and its full
eigen-decomposition (Full_diag_routines / zheev('V','U') -> cuSOLVER zheevd).

Tolerances: dense H entries 1e-14 absolute (entries are O(1)); eigenvalues
1e-11 absolute against numpy's eigvalsh of the oracle's H; eigenvectors by
their residual ||H psi - psi diag(ene)|| <= 1e-10 and orthonormality 1e-12
(eigenvectors are unique only up to phase and within degenerate levels).
"""
import numpy as np
import pytest

from oracle import oracle as O
from ed_gb300 import inputs

pytestmark = pytest.mark.gpu


def _lattice(LX, LY):
    """Square lattice with uniform couplings: the k-sector H is Hermitian
    only for translation-invariant bonds."""
    bonds = []
    for y in range(LY):
        for x in range(LX):
            s = 1 + x + LX * y
            bonds.append((s, 1 + (x + 1) % LX + LX * y))
            bonds.append((s, 1 + x + LX * ((y + 1) % LY)))
    n = len(bonds)
    return np.array(bonds, np.int32), np.full(n, 1.0), np.full(n, 0.45)


CASES = [
    # (NOS, LX, LY, NOD, K)
    (14, 14, 1, 4, (0, 0, 0)),
    (16, 16, 1, 5, (3, 0, 0)),
    (12, 4, 3, 4, (1, 2, 0)),
    (18, 18, 1, 6, (9, 0, 0)),
]


def _check_eig(H, ene, psi):
    # zheev('V', 'U') reads the upper triangle
    w = np.linalg.eigvalsh(H, UPLO="U")
    np.testing.assert_allclose(ene, w, rtol=0, atol=1e-11 * max(1.0, np.abs(w).max()))
    r = H @ psi - psi * ene[None, :]
    assert np.linalg.norm(r, axis=0).max() <= 1e-10 * max(1.0, np.abs(w).max())
    np.testing.assert_allclose(psi.conj().T @ psi, np.eye(len(ene)), rtol=0, atol=1e-12)


@pytest.mark.parametrize("case", CASES)
def test_full_hamiltonian_and_diag(qs3g, case):
    from ed_gb300 import capi
    NOS, LX, LY, nod, K = case
    if LY == 1:
        b, jxy, jz = inputs.chain_bonds(NOS, (1.0, 0.6), (0.3, 0.25))
    else:
        b, jxy, jz = _lattice(LX, LY)
    om = O.Model(NOS, LX, LY, 1, b, jxy, jz, kmax=min(NOS, nod + 2))
    osec = om.build_sector(nod, K)
    h = capi.Handle(NOS, LX, LY, 1, b, jxy, jz)
    D = h.build_sector(nod, K)
    assert D == osec.D
    H0 = osec.dense()
    H1 = h.full_hamiltonian()
    np.testing.assert_allclose(H1, H0, rtol=0, atol=1e-14)
    ene, psi = h.full_diag()
    _check_eig(H0, ene, psi)
    ene2, _ = h.full_diag(want_psi=False)
    np.testing.assert_allclose(ene2, ene, rtol=0, atol=1e-12)
    h.close()


def test_full_diag_u1(qs3g):
    """The U(1)-only dense H (source_only_u1/ham2vec_v3.f90:5-33) and its spectrum."""
    from ed_gb300 import capi
    NOS, nod = 12, 5
    b, jxy, jz = inputs.chain_bonds(NOS, (1.0, 0.8), (0.4, 0.1))
    om = O.Model(NOS, NOS, 1, 1, b, jxy, jz, kmax=nod + 2)
    h = capi.Handle(NOS, NOS, 1, 1, b, jxy, jz)
    D = h.build_sector_u1(nod)
    H0 = O.u1_dense(om, nod)
    H1 = h.full_hamiltonian()
    np.testing.assert_allclose(H1, H0, rtol=0, atol=1e-14)
    ene, psi = h.full_diag()
    assert len(ene) == D
    _check_eig(H0, ene, psi)
    h.close()
