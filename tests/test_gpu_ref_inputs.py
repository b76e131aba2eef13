"""The reference's own example inputs through the GPU library, against the oracle.

QS-Cube/ED ships input sets (input_ex1, input_ex2, input_ex3, input_ex5; copied
byte for byte into tests/golden/ref_inputs/ by make_ref_inputs.py) but no
outputs.  Each is read here as QS3 reads it -- input.dat namelists
(input_param.f90:58-117), list_xxz_term (input_param.f90:91-103),
list_cf_ss and list_site_position (get_expectation_values.f90:11-37) -- through
ed_gb300.inputs, and the GPU library (through the C ABI) is compared with the
oracle restatement on the same inputs:

  * input_ex1: 6x6 lattice, 72 ferromagnetic bonds, NOD=3, K=0, ALG=2 (TRLan
    NOE=10, NOK=15, NOM=30, lnc_ene_conv=1e-14), cal_cf with the 1296 pairs of
    list_cf_ss, cal_dsf with spsmsz=3, rfield=0.495;
  * input_ex2: the same lattice with ALG=3 (full diagonalisation);
  * input_ex3: 10x10x10 cubic lattice, 3000 bonds, NOD=2, K=0, ALG=1 (plain
    Lanczos), DSF at q=(0,0,1.5708) with the site positions of the file;
  * input_ex5: 6x6 triangular lattice, 108 bonds, NOD=3, K=0, ALG=1.

Tolerances: list_s and the connection table bit-exact, list_r 1e-15,
H*v 1e-13 * max|y|, eigenvalues 1e-10 relative, correlations 1e-12, DSF
alpha/beta^2 1e-8.
"""
import os

import numpy as np
import pytest

from ed_gb300 import inputs
from oracle import oracle as O
from oracle import solvers as S

pytestmark = pytest.mark.gpu

REF = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_inputs")


def load_case(name):
    with open(os.path.join(REF, name, "input.dat")) as f:
        inp = inputs.read_input(f.read())
    p = inp.params
    nos, nod, noxxz = int(p["NOS"]), int(p["NOD"]), int(p["NOXXZ"])
    bonds, jxy, jz = inputs.read_bonds(os.path.join(REF, p["FILEXXZ"]), noxxz)
    return inp, nos, nod, bonds, jxy, jz


def build_both(name):
    from ed_gb300 import capi
    inp, nos, nod, bonds, jxy, jz = load_case(name)
    LX, LY, LZ = inp.Ls
    om = O.Model(nos, LX, LY, LZ, bonds, jxy, jz, kmax=min(nos, nod + 2))
    osec = om.build_sector(nod, inp.K, nthreads=0)
    h = capi.Handle(nos, LX, LY, LZ, bonds, jxy, jz)
    D = h.build_sector(nod, inp.K)
    return inp, om, osec, h, D


def check_sector_table_hv(osec, h, D, seed):
    assert D == osec.D and D > 0
    ls, lr = h.get_sector()
    np.testing.assert_array_equal(ls, osec.list_s)
    np.testing.assert_allclose(lr, osec.list_r, rtol=1e-15, atol=0)
    r0, c0, e0, b0 = osec.connection_table()
    r1, c1, e1, b1 = h.connection_table()
    np.testing.assert_array_equal(r1, r0 + 1)
    np.testing.assert_array_equal(c1, c0 + 1)
    np.testing.assert_array_equal(e1, e0)
    np.testing.assert_array_equal(b1, b0 + 1)
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(D) + 1j * rng.standard_normal(D)
    y0 = osec.hv(x)
    y1 = h.hv(x)
    assert np.abs(y1 - y0).max() <= 1e-13 * np.abs(y0).max()


def test_input_ex1_trlan_correlations_dsf(qs3g):
    inp, om, osec, h, D = build_both("input_ex1")
    assert inp.params["ALG"] == 2
    check_sector_table_hv(osec, h, D, 1)
    w = np.linalg.eigvalsh(osec.sparse().toarray())
    t = inp.trlan
    NOE, NOK, NOM = int(t["NOE"]), int(t["NOK"]), int(t["NOM"])
    r = h.trlan(NOE, NOK, NOM, maxitr=int(t["MAXITR"]), tol=float(t["LNC_ENE_CONV"]), seed=5)
    np.testing.assert_allclose(r["ene"], w[:NOE], rtol=1e-10, atol=1e-10)
    ene, _, _, conv = S.trlan(osec.hv, D, NOE, NOK, NOM, int(t["MAXITR"]), float(t["LNC_ENE_CONV"]),
                              S.start_vector(D, 5))
    assert conv
    np.testing.assert_allclose(r["ene"], ene[:NOE], rtol=1e-10, atol=1e-10)
    # cal_cf: the pairs of list_cf_ss, read as the reference reads them
    # (line 'a b' -> list_expe_ss(2) = a, list_expe_ss(1) = b)
    st = inp.static
    pairs = inputs.read_pairs(os.path.join(REF, st["FILECF"]), int(st["NOCF"]))
    psi = r["psi"][0]
    zz1, pm1, lm1 = h.correlations(psi)
    ss = np.stack([pairs[:, 1], pairs[:, 0]], axis=1)
    zz0, pm0 = osec.corr(psi, ss=ss)
    a, b = pairs[:, 0] - 1, pairs[:, 1] - 1
    np.testing.assert_allclose(zz1.T[a, b], zz0[a, b], rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(pm1.T[a, b], pm0[a, b], rtol=1e-12, atol=1e-13)
    # cal_dsf: spsmsz = 3 (S^z) with the file's rfield, at the file's q = 0 and at two other q.
    # The ground state is the ferromagnetic multiplet's member, and S^z(q) maps it onto an
    # eigenstate: the recursion ends after one level (beta^2(2) is rounding noise, after which the
    # reference divides by it), so only level 1 and the vanishing beta^2(2) are comparable.
    dy = inp.dynamic
    spsmsz, rfield = int(dy["SPSMSZ"]), float(dy["RFIELD"])
    Spos = inputs.read_positions(os.path.join(REF, dy["FILEPOS"]), om.NOS)
    itr = 40
    qs = [(float(dy["QX"]), float(dy["QY"]), float(dy["QZ"])), (2 * np.pi / 6, 0.0, 0.0),
          (2 * np.pi / 6, 2 * np.pi / 6, 0.0)]
    g = h.dsf(psi, r["ene"][0], spsmsz, qs, Spos, itr, rfield)
    for iq, q in enumerate(qs):
        ns = oracle_new_sector(om, osec, q)
        fn = O.sq_a(spsmsz, osec, ns, q, Spos, psi)
        al, b2, n1, nl = S.dsf_recursion(ns.hv, fn, itr, rfield, om.NOS, osec.nod)
        assert g["nlev"][iq] == nl
        np.testing.assert_allclose(g["norm1"][iq], n1, rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(g["E0"][iq], r["ene"][0] - rfield * (om.NOS / 2 - osec.nod), rtol=1e-14)
        np.testing.assert_allclose(g["alpha"][iq, 0], al[0], rtol=1e-12)
        assert g["beta2"][iq, 0] == 0.0 and b2[0] == 0.0
        assert abs(g["beta2"][iq, 1]) <= 1e-20 and abs(b2[1]) <= 1e-20
    h.close()


def oracle_new_sector(om, osec, q):
    """The (NOD, k + q) sector of a DSF start vector (calcu_Sq_a with spsmsz = 3)."""
    rk = osec.rk + np.asarray(q, np.float64)
    D2 = O.lib().ora_build_sector(om.h, osec.nod, rk, None, None, 0, 0)
    ls2 = np.zeros(D2, np.int64)
    lr2 = np.zeros(D2)
    O.lib().ora_build_sector(om.h, osec.nod, rk, ls2.ctypes.data, lr2.ctypes.data, D2, 0)
    return O.Sector(om, osec.nod, (0, 0, 0), ls2, lr2, rk=rk)


def test_input_ex2_full_diag(qs3g):
    inp, om, osec, h, D = build_both("input_ex2")
    assert inp.params["ALG"] == 3
    w = np.linalg.eigvalsh(osec.sparse().toarray())
    ene, psi = h.full_diag()
    np.testing.assert_allclose(ene, w, rtol=1e-10, atol=1e-10)
    h.close()


def test_input_ex3_cubic_lanczos_dsf(qs3g):
    inp, om, osec, h, D = build_both("input_ex3")
    assert inp.params["ALG"] == 1 and (om.LX, om.LY, om.LZ) == (10, 10, 10)
    check_sector_table_hv(osec, h, D, 3)
    w = np.linalg.eigvalsh(osec.sparse().toarray())
    lz = inp.lancz
    r = h.lanczos(maxitr=int(lz["MAXITR"]), minitr=int(lz["MINITR"]), itrint=int(lz["ITRINT"]),
                  tol=float(lz["LNC_ENE_CONV"]), seed=9)
    assert abs(r["ene"] - w[0]) <= 1e-10 * abs(w[0])
    e2, _, _ = S.lanczos(osec.hv, D, int(lz["MAXITR"]), int(lz["MINITR"]), int(lz["ITRINT"]),
                         float(lz["LNC_ENE_CONV"]), S.start_vector(D, 9))
    assert abs(r["ene"] - e2) <= 1e-10 * abs(e2)
    # the file's DSF: spsmsz = 3 at q = (0, 0, 1.5708) with the file's site positions
    dy = inp.dynamic
    Spos = inputs.read_positions(os.path.join(REF, dy["FILEPOS"]), om.NOS)
    q = (float(dy["QX"]), float(dy["QY"]), float(dy["QZ"]))
    psi = r["psi"] / np.linalg.norm(r["psi"])
    itr = 30
    g = h.dsf(psi, r["ene"], int(dy["SPSMSZ"]), [q], Spos, itr, float(dy["RFIELD"]))
    # q_z = 1.5708 is not a multiple of 2 pi / LZ; the sector k + q is built as the reference
    # builds it (checkstate_SQ keeps every orbit whose norm stays above 1e-15)
    ns = oracle_new_sector(om, osec, q)
    fn = O.sq_a(int(dy["SPSMSZ"]), osec, ns, q, Spos, psi)
    al, b2, n1, nl = S.dsf_recursion(ns.hv, fn, itr, float(dy["RFIELD"]), om.NOS, osec.nod)
    assert g["nlev"][0] == nl
    np.testing.assert_allclose(g["norm1"][0], n1, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(g["alpha"][0, :nl], al, rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(g["beta2"][0, :nl], b2, rtol=1e-8, atol=1e-10)
    h.close()


def test_input_ex5_triangular_lanczos(qs3g):
    inp, om, osec, h, D = build_both("input_ex5")
    assert inp.params["ALG"] == 1 and om.NOxxz == 108
    check_sector_table_hv(osec, h, D, 5)
    w = np.linalg.eigvalsh(osec.sparse().toarray())
    lz = inp.lancz
    r = h.lanczos(maxitr=int(lz["MAXITR"]), minitr=int(lz["MINITR"]), itrint=int(lz["ITRINT"]),
                  tol=float(lz["LNC_ENE_CONV"]), seed=13)
    assert abs(r["ene"] - w[0]) <= 1e-10 * abs(w[0])
    # the same sector's lowest levels by TRLan with the file's NOE/NOK/NOM
    t = inp.trlan
    NOE, NOK, NOM = int(t["NOE"]), int(t["NOK"]), int(t["NOM"])
    rt = h.trlan(NOE, NOK, NOM, maxitr=int(t["MAXITR"]), tol=float(t["LNC_ENE_CONV"]), seed=13)
    np.testing.assert_allclose(rt["ene"], w[:NOE], rtol=1e-10, atol=1e-10)
    h.close()
