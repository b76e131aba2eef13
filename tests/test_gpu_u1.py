"""GPU parity of the U(1)-only basis (qs3g_build_sector_u1) against the oracle.

The U(1)-only variant of the reference (source_only_u1/) keeps every
configuration of NOD down spins in colex order and uses no translations.
Tolerances as in test_gpu_parity: H*v 1e-13 of max |y| (complex(8)), 2e-6
(complex(4)); eigenvalues 1e-10; correlations 1e-12; start vectors 1e-13;
DSF alpha/beta^2 1e-8.  The cross-check of the two bases: the union over k of
the (NOD, k) spectra equals the U(1) spectrum.
"""
import numpy as np
import pytest

from oracle import oracle as O
from oracle import solvers as S
from ed_gb300 import inputs

pytestmark = pytest.mark.gpu

CASES = [
    # (NOS, LX, LY, LZ, NOD, kind)
    (12, 12, 1, 1, 4, "chain"),
    (16, 16, 1, 1, 3, "chain"),
    (12, 4, 3, 1, 5, "square"),
    (18, 3, 3, 2, 2, "cubic"),
    (20, 20, 1, 1, 1, "chain"),
]


def _bonds(NOS, LX, LY, LZ, kind, rng, uniform=False):
    if kind == "chain":
        return inputs.chain_bonds(NOS, (1.0, 0.6), (0.35, 0.2))
    bonds = []
    site = lambda x, y, z: 1 + (x % LX) + LX * ((y % LY) + LY * (z % LZ))
    for z in range(LZ):
        for y in range(LY):
            for x in range(LX):
                s = site(x, y, z)
                bonds.append((s, site(x + 1, y, z)))
                if LY > 1:
                    bonds.append((s, site(x, y + 1, z)))
                if LZ > 1:
                    bonds.append((s, site(x, y, z + 1)))
    n = len(bonds)
    if uniform:  # translation-invariant couplings (the k sectors need them)
        return np.array(bonds, np.int32), np.full(n, 1.0), np.full(n, 0.7)
    return np.array(bonds, np.int32), rng.uniform(0.5, 1.5, n), rng.uniform(-1.0, 1.0, n)


def _setup(case, seed=0, uniform=False):
    from ed_gb300 import capi
    NOS, LX, LY, LZ, nod, kind = case
    b, jxy, jz = _bonds(NOS, LX, LY, LZ, kind, np.random.default_rng(seed), uniform)
    om = O.Model(NOS, LX, LY, LZ, b, jxy, jz, kmax=min(NOS, nod + 2))
    h = capi.Handle(NOS, LX, LY, LZ, b, jxy, jz)
    D = h.build_sector_u1(nod)
    return om, h, D, nod


@pytest.mark.parametrize("case", CASES)
def test_u1_sector_hv_table(qs3g, case):
    om, h, D, nod = _setup(case)
    NOS = case[0]
    assert D == om.binom(NOS, nod)
    ls, lr = h.get_sector()
    np.testing.assert_array_equal(ls, np.arange(1, D + 1))
    np.testing.assert_array_equal(lr, np.ones(D))
    rng = np.random.default_rng(1)
    x = rng.standard_normal(D) + 1j * rng.standard_normal(D)
    y0 = O.u1_hv(om, nod, x)
    y1 = h.hv(x)
    assert np.abs(y1 - y0).max() <= 1e-13 * np.abs(y0).max()
    x32 = x.astype(np.complex64)
    y2 = h.hv32(x32)
    y0b = O.u1_hv(om, nod, x32.astype(np.complex128))
    assert np.abs(y2 - y0b).max() <= 2e-6 * np.abs(y0b).max()
    # connection table: row i, column inv_list(j_flip_ni(...)), ell = 0, bond
    r, c, e, bnd = h.connection_table()
    assert np.all(e == 0)
    H = np.zeros((D, D), np.complex128)
    np.add.at(H, (r - 1, c - 1), 1.0)
    off = O.u1_dense(om, nod)
    np.fill_diagonal(off, 0)
    assert np.array_equal(H != 0, off != 0)
    assert np.all(np.diff(r) >= 0)
    h.close()


@pytest.mark.parametrize("case", CASES[:3])
def test_u1_spectrum_is_union_of_k_sectors(qs3g, case):
    """The U(1) spectrum is the union of all (NOD, k) spectra; TRLan finds its ground state."""
    om, h, D, nod = _setup(case, uniform=True)
    NOS, LX, LY, LZ = case[:4]
    w_u1 = np.linalg.eigvalsh(O.u1_dense(om, nod))
    ks = [(kx, ky, kz) for kz in range(LZ) for ky in range(LY) for kx in range(LX)]
    w_k = np.sort(np.concatenate([np.linalg.eigvalsh(om.build_sector(nod, k).dense()) for k in ks]))
    np.testing.assert_allclose(w_u1, w_k, rtol=0, atol=1e-11 * max(1.0, np.abs(w_u1).max()))
    # one eigenpair: a single-vector Krylov space holds one vector per eigenspace,
    # so degenerate (k, -k) copies above the ground state are not all found
    r = h.trlan(1, 6, 16, maxitr=2000, tol=1e-12, seed=7)
    np.testing.assert_allclose(r["ene"][0], w_u1[0], rtol=1e-10, atol=1e-10)
    ene, _, _, _ = S.trlan(lambda v: O.u1_hv(om, nod, v), D, 1, 6, 16, 2000, 1e-12, S.start_vector(D, 7))
    np.testing.assert_allclose(r["ene"][0], ene[0], rtol=1e-10, atol=1e-10)
    h.close()


@pytest.mark.parametrize("case", CASES)
def test_u1_correlations(qs3g, case):
    """calcu_cf / calcu_lm of the U(1) variant for all ordered pairs and sites."""
    om, h, D, nod = _setup(case)
    rng = np.random.default_rng(3)
    psi = rng.standard_normal(D) + 1j * rng.standard_normal(D)  # not translation invariant
    psi /= np.linalg.norm(psi)
    zz0, pm0, lm0 = O.u1_corr(om, nod, psi)
    zz1, pm1, lm1 = h.correlations(psi)
    np.testing.assert_allclose(zz1, zz0, rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(pm1, pm0, rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(lm1, lm0, rtol=1e-12, atol=1e-13)
    h.close()


@pytest.mark.parametrize("spsmsz", [1, 2, 3])
def test_u1_sq_a_and_dsf(qs3g, spsmsz):
    """calcu_Sq_a and the DSF recursion of the U(1) variant."""
    case = (12, 12, 1, 1, 4, "chain")
    om, h, D, nod = _setup(case)
    NOS = case[0]
    w, V = np.linalg.eigh(O.u1_dense(om, nod))
    psi = np.ascontiguousarray(V[:, 0])
    Spos = inputs.chain_positions(NOS)
    nod_new = {1: nod - 1, 2: nod + 1, 3: nod}[spsmsz]
    qs = [2 * np.pi * m / NOS for m in (1, 3, 6)]
    for q in qs:
        fo = O.u1_sq_a(om, spsmsz, nod, (q, 0, 0), Spos, psi)
        ls, fg = h.sq_a(psi, spsmsz, (q, 0, 0), Spos)
        np.testing.assert_array_equal(ls, np.arange(1, len(fo) + 1))
        assert np.abs(fg - fo).max() <= 1e-13 * max(1.0, np.abs(fo).max())
    itr, rfield = 10, 0.05
    g = h.dsf(psi, w[0], spsmsz, [(q, 0, 0) for q in qs], Spos, itr, rfield)
    for iq, q in enumerate(qs):
        fo = O.u1_sq_a(om, spsmsz, nod, (q, 0, 0), Spos, psi)
        a, b2, n1, nl = S.dsf_recursion(lambda v: O.u1_hv(om, nod_new, v), fo, itr, rfield, NOS, nod_new)
        assert g["nlev"][iq] == nl
        np.testing.assert_allclose(g["norm1"][iq], n1, rtol=1e-12)
        np.testing.assert_allclose(g["alpha"][iq, :nl], a, rtol=1e-8, atol=1e-10)
        np.testing.assert_allclose(g["beta2"][iq, :nl], b2, rtol=1e-8, atol=1e-10)
    h.close()
