"""CPU tests: the oracle pinned against golden fixtures and known answers.

The reference (Fortran) ships no tests or outputs and cannot be compiled
here, so the restatement is pinned by physics: spectra of the independent
dense diagonalisation (tests/golden/golden.json), free fermions, magnons, the
ferromagnetic multiplet, sector sum rules and Hermiticity.
"""
import json
import os
from math import comb

import numpy as np
import pytest

from oracle import dense_ed as E
from oracle import oracle as O
from oracle import solvers as S
from ed_gb300 import inputs

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def model_of(c):
    return O.Model(c["NOS"], c["LX"], c["LY"], c["LZ"], np.array(c["bonds"], np.int32),
                   np.array(c["Jxy"]), np.array(c["Jz"]), kmax=c["NOD"] + 2)


@pytest.mark.parametrize("case", GOLDEN["cases"], ids=lambda c: c["name"])
def test_oracle_sector_spectra_match_golden(case):
    m = model_of(case)
    union = []
    for key, ref in case["sectors"].items():
        K = tuple(int(v) for v in key.split(","))
        s = m.build_sector(case["NOD"], K)
        assert s.D == len(ref)
        if s.D == 0:
            continue
        H = s.dense()
        assert np.abs(H - H.conj().T).max() < 1e-13
        w = np.linalg.eigvalsh(H)
        np.testing.assert_allclose(w, ref, atol=1e-12)
        union += list(w)
    np.testing.assert_allclose(np.sort(union), case["u1_spectrum"], atol=1e-12)


def test_xx_chain_free_fermions():
    g = GOLDEN["xx_chain"]
    L, N = g["L"], g["N"]
    b, jxy, jz = inputs.chain_bonds(L, (g["Jxy"], 0.0))
    m = O.Model(L, L, 1, 1, b, jxy, jz, kmax=N + 2)
    for K, ref in g["sector_energies"].items():
        s = m.build_sector(N, (int(K), 0, 0))
        w = np.linalg.eigvalsh(s.dense()) if s.D else np.zeros(0)
        np.testing.assert_allclose(w, np.sort(ref), atol=1e-12)


def test_single_magnon_dispersion():
    g = GOLDEN["magnon"]
    L = g["L"]
    b, jxy, jz = inputs.chain_bonds(L, (g["Jxy"], g["Jz"]))
    m = O.Model(L, L, 1, 1, b, jxy, jz, kmax=3)
    for K in range(L):
        s = m.build_sector(1, (K, 0, 0))
        assert s.D == 1
        e = s.hv(np.ones(1, complex))[0]
        assert abs(e.imag) < 1e-13
        assert abs(e.real - g["energies"][K]) < 1e-12


def test_ferromagnet_multiplet():
    """FM Heisenberg (J < 0): every sector's ground state is sum_b J_b/4 (calcu_FM_energy)."""
    b, jxy, jz = E.square_bonds(4, 3, (-1.0, -1.0))
    m = O.Model(12, 4, 3, 1, b, jxy, jz, kmax=5)
    efm = jz.sum() / 4.0
    for nod in (1, 2, 3):
        s = m.build_sector(nod, (0, 0, 0))
        w = np.linalg.eigvalsh(s.dense())
        assert abs(w[0] - efm) < 1e-12


@pytest.mark.parametrize("L,nod", [(10, 3), (12, 4), (15, 5), (16, 8)])
def test_sector_sum_rule(L, nod):
    b, jxy, jz = inputs.chain_bonds(L)
    m = O.Model(L, L, 1, 1, b, jxy, jz, kmax=nod + 2)
    assert sum(m.build_sector(nod, (K, 0, 0)).D for K in range(L)) == comb(L, nod)


@pytest.mark.parametrize("L,nod,K", [(12, 3, 0), (16, 4, 3), (20, 5, 4), (18, 6, 0), (24, 1, 6),
                                     (21, 7, 7)])
def test_chain_enumeration_equals_faithful_build(L, nod, K):
    b, jxy, jz = inputs.chain_bonds(L)
    m = O.Model(L, L, 1, 1, b, jxy, jz, kmax=nod + 2)
    s = m.build_sector(nod, (K, 0, 0))
    ls, lr = O.chain_sector_lists(L, nod, K)
    np.testing.assert_array_equal(ls, s.list_s)
    np.testing.assert_array_equal(lr, s.list_r)


def test_list_fly_inv_list_roundtrip():
    b, jxy, jz = inputs.chain_bonds(15)
    m = O.Model(15, 15, 1, 1, b, jxy, jz, kmax=6)
    for t in range(1, comb(15, 4) + 1, 7):
        n = m.list_fly(t, 4)
        assert list(n) == sorted(n) and n[0] >= 1 and n[-1] <= 15
        assert m.inv_list(n) == t


@pytest.mark.parametrize("LX,LY,nod", [(10, 1, 3), (4, 3, 4)])
def test_u1_oracle_against_dense_and_k_union(LX, LY, nod):
    """U(1)-only H*v (source_only_u1/ham2vec_v3.f90:35-65) equals an independent
    dense H in colex order, its spectrum is the union of the (NOD, k) spectra,
    and calcu_cf / calcu_lm satisfy the Sz_tot sum rules."""
    NOS = LX * LY
    if LY == 1:
        b, jxy, jz = E.chain_bonds(NOS, (1.0, 0.7), (0.4, 0.2))
    else:
        b, jxy, jz = E.square_bonds(LX, LY, (1.0, 0.6))
    m = O.Model(NOS, LX, LY, 1, b, jxy, jz, kmax=nod + 2)
    H = O.u1_dense(m, nod)
    Hd, confs, index = E.u1_hamiltonian(NOS, nod, b, jxy, jz)
    perm = [index[tuple(m.list_fly(t, nod))] for t in range(1, comb(NOS, nod) + 1)]
    np.testing.assert_allclose(H, Hd[np.ix_(perm, perm)], rtol=0, atol=1e-14)
    w = np.linalg.eigvalsh(H)
    ks = [(kx, ky, 0) for ky in range(LY) for kx in range(LX)]
    wk = np.sort(np.concatenate([np.linalg.eigvalsh(m.build_sector(nod, k).dense()) for k in ks]))
    np.testing.assert_allclose(w, wk, rtol=0, atol=1e-12)
    psi = np.linalg.eigh(H)[1][:, 0]
    zz, pm, lm = O.u1_corr(m, nod, psi)
    sz = NOS / 2 - nod
    # sum_b <Sz_a Sz_b> = <Sz_a Sz_tot> = sz <Sz_a> (psi need not be translation invariant)
    np.testing.assert_allclose(zz.sum(axis=1), sz * lm, atol=1e-12)
    np.testing.assert_allclose(lm.sum(), sz, atol=1e-12)
    # <S+_a S-_a> = P(a up) = 1/2 + <Sz_a>
    np.testing.assert_allclose(np.diag(pm).real, 0.5 + lm, atol=1e-12)
    # S^z(q=0)|psi> = Sz_tot |psi> / sqrt(NOS)
    Spos = np.array([[i % LX, i // LX, 0] for i in range(NOS)], float)
    fz = O.u1_sq_a(m, 3, nod, (0.0, 0.0, 0.0), Spos, psi)
    np.testing.assert_allclose(fz, sz * psi / np.sqrt(NOS), atol=1e-13)


def test_representative_ell_rule():
    """ell is the first translation (loop order) reaching the minimum, 0 if minimal."""
    L = 12
    b, jxy, jz = inputs.chain_bonds(L)
    m = O.Model(L, L, 1, 1, b, jxy, jz, kmax=6)
    t, n, ell = m.representative([1, 5, 9])  # period 4, already minimal
    assert list(n) == [1, 5, 9] and list(ell) == [0, 0, 0]
    t, n, ell = m.representative([2, 6, 10])  # i = 3, 7, 11 all give [1,5,9]; 3 comes first
    assert list(n) == [1, 5, 9] and list(ell) == [3, 1, 1]


def test_trlan_and_lanczos_oracle():
    L, nod = 14, 4
    b, jxy, jz = inputs.chain_bonds(L, (1.0, 0.5), (0.3, 0.3))
    m = O.Model(L, L, 1, 1, b, jxy, jz, kmax=nod + 2)
    s = m.build_sector(nod, (0, 0, 0))
    w = np.linalg.eigvalsh(s.dense())
    ene, psi, tr, conv = S.trlan(s.hv, s.D, 3, 5, 10, 500, 1e-13, S.start_vector(s.D, 1))
    assert conv
    np.testing.assert_allclose(ene[:3], w[:3], rtol=1e-11)
    e1, p1, ite = S.lanczos(s.hv, s.D, 2000, 20, 5, 1e-14, S.start_vector(s.D, 2))
    assert abs(e1 - w[0]) < 1e-11
    assert np.linalg.norm(s.hv(p1) - e1 * p1) < 1e-6


def test_trlan_stop_999_on_small_dimension():
    b, jxy, jz = inputs.chain_bonds(6)
    m = O.Model(6, 6, 1, 1, b, jxy, jz, kmax=4)
    s = m.build_sector(2, (0, 0, 0))
    with pytest.raises(ValueError):
        S.trlan(s.hv, s.D, 2, 4, 8, 10, 1e-12, S.start_vector(s.D, 1))


def test_start_vector_is_seeded_and_uniform():
    a = S.start_vector(1000, 5)
    b = S.start_vector(1000, 5)
    np.testing.assert_array_equal(a, b)
    assert np.all(np.abs(a.real) <= 0.5) and np.all(np.abs(a.imag) <= 0.5)
    assert abs(a.real.mean()) < 0.05 and abs(a.imag.mean()) < 0.05


def test_dsf_sum_rule_and_cfrac_against_resolvent():
    """norm1 = <GS| S+(-q) S-(q) |GS> and, at full Krylov depth, the continued
    fraction (without the reference's deepest-level quirk) equals the resolvent."""
    L, nod = 10, 2
    b, jxy, jz = inputs.chain_bonds(L, (1.0, 1.0))
    m = O.Model(L, L, 1, 1, b, jxy, jz, kmax=5)
    gs = m.build_sector(nod, (0, 0, 0))
    w, V = np.linalg.eigh(gs.dense())
    psi = V[:, 0]
    q = 2 * np.pi * 3 / L
    rk = O.wavevector((0, 0, 0), m.Ls) + np.array([q, 0, 0])
    D2 = O.lib().ora_build_sector(m.h, nod + 1, rk, None, None, 0, 0)
    ls = np.zeros(D2, np.int64)
    lr = np.zeros(D2)
    O.lib().ora_build_sector(m.h, nod + 1, rk, ls.ctypes.data, lr.ctypes.data, D2, 0)
    ns = O.Sector(m, nod + 1, (0, 0, 0), ls, lr, rk=rk)
    fn = O.sq_a(2, gs, ns, (q, 0, 0), inputs.chain_positions(L), psi)
    # norm1 from the U(1) basis directly: |S^-(q)|GS>|^2 / NOS with S^-(q) = sum_i e^{-iqR_i} S^-_i
    Hn = ns.dense()
    a, b2, n1, nl = S.dsf_recursion(ns.hv, fn, D2, 0.0, L, nod + 1)
    assert nl == D2
    eta = 0.05
    om = np.linspace(0, 6, 301)
    Sc = O.cfrac(a, b2, n1, w[0], eta, om, compat=False)
    f = fn / np.sqrt(n1)
    ev, U = np.linalg.eigh(Hn)
    amp = np.abs(U.conj().T @ f) ** 2
    G = np.array([np.sum(amp / (o + w[0] + 1j * eta - ev)) for o in om]) * n1
    np.testing.assert_allclose(Sc, -G.imag / np.pi, rtol=1e-9, atol=1e-12)
    Sq = O.cfrac(a, b2, n1, w[0], eta, om, compat=True)
    assert np.all(np.isfinite(Sq))


def test_input_dat_parser():
    text = """&input_parameters
NOS = 36, NOD = 3, LX = 6, LY = 6, LZ = 1, KX = 0, KY = 0, KZ = 0, NOxxz = 72, ALG = 2,
cal_lm = 1, cal_cf = 1, cal_dsf= 1, wr_wf = 1, re_wf = 0,
FILExxz= "input_ex1/list_xxz_term_36.dat", FILEwf = "work/", OUTDIR = "output_ex1/",
&end
&input_static
NOV = 2, NOLM = 36, NOCF = 1296, FILElm = "a", FILECF = "b",
&end
&input_dynamic
spsmsz = 3, itr_dsf= 200, QX = 0.0d0, QY = 0.0d0, QZ = 1.57079632679d0, rfield = 0.495d0, FILEpos= "p",
&end
&input_TRLan
NOE = 10, NOK = 15, NOM = 30, maxitr=10000, lnc_ene_conv=1.0d-14, i_vec_min = 1, i_vec_max = 1,
&end
"""
    q = inputs.read_input(text)
    assert q.params["NOS"] == 36 and q.params["NOXXZ"] == 72 and q.params["FILEXXZ"].endswith(".dat")
    assert q.Ls == (6, 6, 1) and q.K == (0, 0, 0)
    assert q.dynamic["QZ"] == pytest.approx(1.57079632679) and q.dynamic["RFIELD"] == 0.495
    assert q.trlan["LNC_ENE_CONV"] == 1e-14 and q.trlan["NOM"] == 30
    # a malformed file is refused, not half-read
    with pytest.raises(ValueError):
        inputs.read_input("&input_static\nNOV = 2,\n&end\n")


def test_bond_file_roundtrip(tmp_path):
    b, jxy, jz = inputs.chain_bonds(20, (1.0, 0.5), (0.3, 0.3))
    p = tmp_path / "list_xxz_term_20.dat"
    inputs.write_bonds(str(p), b, jxy, jz)
    b2, x2, z2 = inputs.read_bonds(str(p), len(b))
    np.testing.assert_array_equal(b, b2)
    np.testing.assert_array_equal(jxy, x2)
    np.testing.assert_array_equal(jz, z2)
    p2 = tmp_path / "fortran_d.dat"
    p2.write_text("1\t2\t1.0d0\t-0.5d0\n")
    b3, x3, z3 = inputs.read_bonds(str(p2), 1)
    assert tuple(b3[0]) == (1, 2) and x3[0] == 1.0 and z3[0] == -0.5
