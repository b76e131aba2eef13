"""GPU parity of libqs3g.so against the CPU oracle (small and medium sectors).

Every call goes through the C ABI (ed_gb300.capi).  Tolerances:
  * list_s, connection table (row, col, ell, bond): bit-exact;
  * list_r: 1e-15 relative (both sides use the host libm for the phases);
  * H*v (complex(8)): max |y_gpu - y_oracle| <= 1e-13 * max |y_oracle|;
  * H*v (complex(4)): 2e-6 relative in the same norm;
  * eigenvalues: 1e-10 relative; DSF alpha/beta^2: 1e-8 relative.
"""
import numpy as np
import pytest

from oracle import dense_ed as E
from oracle import oracle as O
from oracle import solvers as S
from ed_gb300 import inputs

pytestmark = pytest.mark.gpu

CHAINS = [
    # (L, NOD, K, J1, J2)
    (12, 3, 0, (1.0, 1.0), None),
    (12, 4, 3, (1.0, 0.5), (0.3, 0.3)),
    (14, 4, 7, (1.0, 0.7), (0.25, 0.1)),
    (16, 2, 5, (-1.0, -1.0), None),
    (18, 6, 0, (1.0, 0.5), (0.3, 0.3)),
    (20, 5, 4, (1.0, 1.0), (0.2, 0.2)),
    (24, 1, 6, (1.0, 0.3), None),
    (24, 4, 12, (1.0, 2.0), (0.5, 0.5)),
    (30, 3, 10, (1.0, 1.0), None),
]

LATTICES = [
    # (LX, LY, LZ, NOD, K, bonds-kind)
    (4, 3, 1, 3, (1, 2, 0), "square"),
    (4, 4, 1, 2, (0, 0, 0), "square"),
    (3, 3, 2, 3, (1, 0, 1), "cubic"),
    (6, 6, 1, 3, (0, 0, 0), "square"),
    (4, 4, 1, 4, (2, 1, 0), "triangular"),
]


def lattice_bonds(LX, LY, LZ, kind, rng):
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
                if kind == "triangular":
                    bonds.append((s, site(x + 1, y + 1, z)))
    n = len(bonds)
    jxy = rng.uniform(0.5, 1.5, n)
    jz = rng.uniform(-1.0, 1.0, n)
    return np.array(bonds, np.int32), jxy, jz


def make_chain(L, J1, J2):
    b, jxy, jz = inputs.chain_bonds(L, J1, J2)
    return (L, L, 1, 1, b, jxy, jz)


def both(args, nod, K):
    from ed_gb300 import capi
    NOS, LX, LY, LZ, b, jxy, jz = args
    om = O.Model(NOS, LX, LY, LZ, b, jxy, jz, kmax=min(NOS, nod + 2))
    osec = om.build_sector(nod, K)
    h = capi.Handle(NOS, LX, LY, LZ, b, jxy, jz)
    D = h.build_sector(nod, K)
    return om, osec, h, D


def check_sector(osec, h, D):
    assert D == osec.D
    ls, lr = h.get_sector()
    np.testing.assert_array_equal(ls, osec.list_s)
    np.testing.assert_allclose(lr, osec.list_r, rtol=1e-15, atol=0)


def check_table(osec, h):
    r0, c0, e0, b0 = osec.connection_table()
    r1, c1, e1, b1 = h.connection_table()
    np.testing.assert_array_equal(r1, r0 + 1)
    np.testing.assert_array_equal(c1, c0 + 1)
    np.testing.assert_array_equal(e1, e0)
    np.testing.assert_array_equal(b1, b0 + 1)
    return len(r0)


def check_hv(osec, h, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(osec.D) + 1j * rng.standard_normal(osec.D)
    y0 = osec.hv(x)
    y1 = h.hv(x)
    scale = np.abs(y0).max()
    assert np.abs(y1 - y0).max() <= 1e-13 * scale
    x32 = x.astype(np.complex64)
    y2 = h.hv32(x32)
    y0b = osec.hv(x32.astype(np.complex128))
    assert np.abs(y2 - y0b).max() <= 2e-6 * np.abs(y0b).max()


@pytest.mark.parametrize("L,nod,K,J1,J2", CHAINS)
def test_chain_sector_table_hv(qs3g, L, nod, K, J1, J2):
    args = make_chain(L, J1, J2)
    om, osec, h, D = both(args, nod, (K, 0, 0))
    check_sector(osec, h, D)
    if D:
        check_table(osec, h)
        check_hv(osec, h)
    h.close()


@pytest.mark.parametrize("LX,LY,LZ,nod,K,kind", LATTICES)
def test_lattice_sector_table_hv(qs3g, LX, LY, LZ, nod, K, kind):
    rng = np.random.default_rng(LX * 100 + LY * 10 + LZ)
    b, jxy, jz = lattice_bonds(LX, LY, LZ, kind, rng)
    args = (LX * LY * LZ, LX, LY, LZ, b, jxy, jz)
    om, osec, h, D = both(args, nod, K)
    check_sector(osec, h, D)
    if D:
        check_table(osec, h)
        check_hv(osec, h)
    h.close()


def test_sector_sum_rule(qs3g):
    """Every orbit of period p is a row of exactly p momentum sectors, so the
    sector dimensions add up to C(L, NOD); the K = 0 sector holds every orbit,
    so its orbit sizes p = L^2 / list_r^2 add up to C(L, NOD) as well."""
    from ed_gb300 import capi
    from math import comb
    L, nod = 20, 4
    b, jxy, jz = inputs.chain_bonds(L)
    h = capi.Handle(L, L, 1, 1, b, jxy, jz)
    total = 0
    for K in range(L):
        total += h.build_sector(nod, (K, 0, 0))
    assert total == comb(L, nod)
    h.build_sector(nod, (0, 0, 0))
    ls, lr = h.get_sector()
    assert int(np.rint(L * L / lr ** 2).sum()) == comb(L, nod)
    h.close()


@pytest.mark.parametrize("L,nod,K,J1,J2", [(14, 4, 0, (1.0, 0.5), (0.3, 0.3)),
                                           (16, 3, 5, (1.0, 1.0), None),
                                           (12, 6, 0, (1.0, 1.0), None)])
def test_trlan_eigenvalues(qs3g, L, nod, K, J1, J2):
    args = make_chain(L, J1, J2)
    om, osec, h, D = both(args, nod, (K, 0, 0))
    w = np.linalg.eigvalsh(osec.dense())
    NOE, NOK, NOM = 4, 6, 12
    r = h.trlan(NOE, NOK, NOM, maxitr=500, tol=1e-12, seed=11)
    np.testing.assert_allclose(r["ene"], w[:NOE], rtol=1e-10, atol=1e-10)
    assert r["resid"].max() < 1e-8
    # oracle TRLan from the same seeded start vector
    ene, _, _, conv = S.trlan(osec.hv, D, NOE, NOK, NOM, 500, 1e-12, S.start_vector(D, 11))
    np.testing.assert_allclose(r["ene"], ene[:NOE], rtol=1e-10, atol=1e-10)
    # FP32 storage + FP64 refinement reaches the same eigenvalues
    r32 = h.trlan(NOE, NOK, NOM, maxitr=500, tol=1e-12, precision=1, seed=11)
    np.testing.assert_allclose(r32["ene"], w[:NOE], rtol=1e-10, atol=1e-10)
    # complex(8) storage with double-float arithmetic on the FP32 pipe
    re = h.trlan(NOE, NOK, NOM, maxitr=500, tol=1e-12, precision=2, seed=11)
    np.testing.assert_allclose(re["ene"], w[:NOE], rtol=1e-10, atol=1e-10)
    assert re["resid"].max() < 1e-8
    # residual-based convergence
    rr = h.trlan(1, 4, 12, maxitr=500, tol=1e-10, conv_mode=1, seed=3)
    assert rr["resid"][0] <= 2e-10
    assert abs(rr["ene"][0] - w[0]) <= 1e-10 * max(1.0, abs(w[0]))
    h.close()


def test_start_vector_matches_oracle(qs3g):
    """The seeded start vector is generated identically on both sides."""
    args = make_chain(10, (1.0, 1.0), None)
    om, osec, h, D = both(args, 3, (0, 0, 0))
    st = S.start_vector(D, 1234)
    r1 = h.trlan(2, 3, 6, maxitr=200, tol=1e-13, seed=1234)
    r2 = h.trlan(2, 3, 6, maxitr=200, tol=1e-13, start=st)
    np.testing.assert_array_equal(r1["ene"], r2["ene"])
    h.close()


def test_lanczos(qs3g):
    args = make_chain(16, (1.0, 0.5), (0.3, 0.3))
    om, osec, h, D = both(args, 4, (0, 0, 0))
    w = np.linalg.eigvalsh(osec.dense())
    r = h.lanczos(maxitr=2000, minitr=20, itrint=5, tol=1e-14, seed=5)
    assert abs(r["ene"] - w[0]) <= 1e-10 * abs(w[0])
    psi = r["psi"]
    res = np.linalg.norm(osec.hv(psi) - r["ene"] * psi)
    assert res < 1e-6
    e2, p2, ite = S.lanczos(osec.hv, D, 2000, 20, 5, 1e-14, S.start_vector(D, 5))
    assert abs(r["ene"] - e2) <= 1e-10 * abs(e2)
    h.close()


def _dsf_case(spsmsz):
    # S^+ lowers N_down: start from N_down = 5 so the new sector (N_down = 4,
    # ~70 rows) is deep enough for 12 well-conditioned recursion levels
    L, nod = 14, (5 if spsmsz == 1 else 3)
    b, jxy, jz = inputs.chain_bonds(L, (1.0, 0.7), (0.2, 0.1))
    args = (L, L, 1, 1, b, jxy, jz)
    om, osec, h, D = both(args, nod, (0, 0, 0))
    w, V = np.linalg.eigh(osec.dense())
    psi = np.ascontiguousarray(V[:, 0])
    nod_new = {1: nod - 1, 2: nod + 1, 3: nod}[spsmsz]
    return L, nod, nod_new, om, osec, h, w, psi


def _oracle_new_sector(om, nod_new, q):
    rk = O.wavevector((0, 0, 0), om.Ls) + np.array([q, 0, 0])
    D2 = O.lib().ora_build_sector(om.h, nod_new, rk, None, None, 0, 0)
    ls = np.zeros(D2, np.int64)
    lr = np.zeros(D2)
    O.lib().ora_build_sector(om.h, nod_new, rk, ls.ctypes.data, lr.ctypes.data, D2, 0)
    return O.Sector(om, nod_new, (0, 0, 0), ls, lr, rk=rk)


@pytest.mark.parametrize("spsmsz", [1, 2, 3])
def test_sq_a_start_vectors(qs3g, spsmsz):
    """calcu_Sq_a: S^a(q)|GS> on the GPU (gather form) equals the oracle's scatter."""
    L, nod, nod_new, om, osec, h, w, psi = _dsf_case(spsmsz)
    Spos = inputs.chain_positions(L)
    for mq in (1, 4, 7, 10):
        q = 2 * np.pi * mq / L
        ns = _oracle_new_sector(om, nod_new, q)
        fo = O.sq_a(spsmsz, osec, ns, (q, 0, 0), Spos, psi)
        ls, fg = h.sq_a(psi, spsmsz, (q, 0, 0), Spos)
        np.testing.assert_array_equal(ls, ns.list_s)
        assert np.abs(fg - fo).max() <= 1e-13 * max(1.0, np.abs(fo).max())
    h.close()


@pytest.mark.parametrize("spsmsz", [1, 2, 3])
def test_dsf_small(qs3g, spsmsz):
    L, nod, nod_new, om, osec, h, w, psi = _dsf_case(spsmsz)
    Spos = inputs.chain_positions(L)
    mqs = (1, 4, 7, 10)
    qs = [2 * np.pi * m / L for m in mqs]
    itr = 12
    rfield = 0.1
    g = h.dsf(psi, w[0], spsmsz, [(q, 0, 0) for q in qs], Spos, itr, rfield)
    for iq, q in enumerate(qs):
        ns = _oracle_new_sector(om, nod_new, q)
        fn = O.sq_a(spsmsz, osec, ns, (q, 0, 0), Spos, psi)
        a, b2, n1, nl = S.dsf_recursion(ns.hv, fn, itr, rfield, L, nod_new)
        assert g["nlev"][iq] == nl
        np.testing.assert_allclose(g["norm1"][iq], n1, rtol=1e-12)
        np.testing.assert_allclose(g["E0"][iq], w[0] - rfield * (L / 2 - nod), rtol=1e-14)
        np.testing.assert_allclose(g["alpha"][iq, :nl], a, rtol=1e-8, atol=1e-10)
        np.testing.assert_allclose(g["beta2"][iq, :nl], b2, rtol=1e-8, atol=1e-10)
    h.close()


def test_cfrac(qs3g):
    from ed_gb300 import capi
    rng = np.random.default_rng(4)
    nq, N = 5, 40
    alpha = rng.uniform(-1, 3, (nq, N))
    beta2 = rng.uniform(0.1, 2, (nq, N))
    beta2[:, 0] = 0.0
    nlev = np.array([40, 30, 1, 2, 17], np.int32)
    norm1 = rng.uniform(0.5, 2, nq)
    E0 = rng.uniform(-5, -1, nq)
    om = np.linspace(0, 6, 2000)
    for compat in (True, False):
        S1 = capi.cfrac(alpha, beta2, nlev, norm1, E0, 0.05, om, compat)
        for q in range(nq):
            S0 = O.cfrac(alpha[q, :nlev[q]], beta2[q, :nlev[q]], norm1[q], E0[q], 0.05, om, compat)
            np.testing.assert_allclose(S1[q], S0, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("case", ["chain16", "chain14_k3", "square4x3"])
def test_correlations(qs3g, case):
    """get_cf_2_wave_vector / calcu_cf_trans_2 on the GPU equal the oracle for all NOS^2 pairs."""
    rng = np.random.default_rng(5)
    if case == "chain16":
        args, nod, K = make_chain(16, (1.0, 0.5), (0.3, 0.3)), 4, (0, 0, 0)
    elif case == "chain14_k3":
        args, nod, K = make_chain(14, (1.0, 1.0), None), 3, (3, 0, 0)
    else:
        b, jxy, jz = lattice_bonds(4, 3, 1, "square", rng)
        args, nod, K = (12, 4, 3, 1, b, jxy, jz), 3, (1, 0, 0)
    om, osec, h, D = both(args, nod, K)
    w, V = np.linalg.eigh(osec.dense())
    psi = np.ascontiguousarray(V[:, 0])
    zz0, pm0 = osec.corr(psi)
    zz1, pm1, lm1 = h.correlations(psi)
    np.testing.assert_allclose(zz1, zz0.T, rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(pm1, pm0.T, rtol=1e-12, atol=1e-13)
    NOS = args[0]
    np.testing.assert_allclose(lm1, 0.5 * (1 - 2 * nod / NOS), rtol=1e-12)
    # sum rule: sum_b <Sz_a Sz_b> = <Sz_a Sz_tot> = Sz_tot^2 / NOS for an Sz_tot eigenstate
    sz = NOS / 2 - nod
    np.testing.assert_allclose(zz1.sum(axis=1), sz * sz / NOS, rtol=1e-10)
    h.close()


def test_dsf_all_q_batched(qs3g):
    """Every q of a chain at once (one batched recursion): each q equals the
    oracle's own per-q recursion, and a sweep of one q equals the same q
    inside the full sweep bit for bit (results do not depend on the batch)."""
    # anisotropic couplings: with SU(2) symmetry S^-(q=0)|GS> is an eigenstate
    # and the recursion breaks down after one level (beta_2 = 0 up to rounding)
    L, nod = 24, 3
    b, jxy, jz = inputs.chain_bonds(L, (1.0, 0.6), (0.2, 0.1))
    om, osec, h, D = both((L, L, 1, 1, b, jxy, jz), nod, (0, 0, 0))
    w, V = np.linalg.eigh(osec.dense())
    psi = np.ascontiguousarray(V[:, 0])
    Spos = inputs.chain_positions(L)
    qs = [2 * np.pi * m / L for m in range(L)]
    itr = 40
    g = h.dsf(psi, w[0], 2, [(q, 0, 0) for q in qs], Spos, itr, 0.0)
    for m in (0, 1, 5, 12, 23):
        ns = _oracle_new_sector(om, nod + 1, qs[m])
        fn = O.sq_a(2, osec, ns, (qs[m], 0, 0), Spos, psi)
        a, b2, n1, nl = S.dsf_recursion(ns.hv, fn, itr, 0.0, L, nod + 1)
        assert g["nlev"][m] == nl
        np.testing.assert_allclose(g["norm1"][m], n1, rtol=1e-12)
        np.testing.assert_allclose(g["alpha"][m, :nl], a, rtol=1e-8, atol=1e-10)
        np.testing.assert_allclose(g["beta2"][m, :nl], b2, rtol=1e-8, atol=1e-10)
        one = h.dsf(psi, w[0], 2, [(qs[m], 0, 0)], Spos, itr, 0.0)
        np.testing.assert_array_equal(one["alpha"][0], g["alpha"][m])
        np.testing.assert_array_equal(one["beta2"][0], g["beta2"][m])
    h.close()


@pytest.mark.parametrize("LX,LY,LZ,nod,K,kind", [(4, 3, 1, 3, (1, 2, 0), "square"), (6, 6, 1, 3, (0, 0, 0), "square")])
def test_general_hv_schedules_identical(qs3g, LX, LY, LZ, nod, K, kind):
    """Warp-per-row and thread-per-row general H*v give bit-identical products;
    the autotuner settles on one of them after the first product."""
    rng = np.random.default_rng(2)
    b, jxy, jz = lattice_bonds(LX, LY, LZ, kind, rng)
    om, osec, h, D = both((LX * LY * LZ, LX, LY, LZ, b, jxy, jz), nod, K)
    x = rng.standard_normal(D) + 1j * rng.standard_normal(D)
    x32 = x.astype(np.complex64)
    out = {}
    for mode in (1, 2):
        h.hv_schedule(mode)
        out[mode] = (h.hv(x), h.hv32(x32))
        assert h.hv_schedule() == (mode, mode)
    np.testing.assert_array_equal(out[1][0], out[2][0])
    np.testing.assert_array_equal(out[1][1], out[2][1])
    y0 = osec.hv(x)
    assert np.abs(out[1][0] - y0).max() <= 1e-13 * np.abs(y0).max()
    h.hv_schedule(0)
    assert h.hv_schedule() == (0, 0)
    np.testing.assert_array_equal(h.hv(x), out[1][0])
    np.testing.assert_array_equal(h.hv32(x32), out[1][1])
    assert h.hv_schedule()[0] in (1, 2) and h.hv_schedule()[1] in (1, 2)
    h.close()


@pytest.mark.parametrize("L,nod,K,offsets", [(20, 4, 3, (1, 3, 4)), (18, 5, 0, (1, 2, 5)), (16, 3, 5, (2, 7)),
                                             (24, 2, 0, (1, 12)), (15, 6, 4, (1, 2, 3))])
def test_chain_long_range_bonds(qs3g, L, nod, K, offsets):
    """Chains whose bonds reach several sites: hops that pass over other down
    spins, land next to them or wrap round the ring take the general path, the
    rest the gap-lane path; both must give the oracle's connection table and
    H*v (complex(8), complex(4) and, at K = 0, real)."""
    rng = np.random.default_rng(L * 10 + nod)
    bonds = [(s, (s - 1 + o) % L + 1) for o in offsets for s in range(1, L + 1)]
    if L % 2 == 0 and L // 2 in offsets:  # the half-ring bond appears twice; keep one copy per pair
        seen, uniq = set(), []
        for a, b in bonds:
            key = (min(a, b), max(a, b))
            if key not in seen:
                seen.add(key)
                uniq.append((a, b))
        bonds = uniq
    bonds = np.array(bonds, np.int32)
    jxy = rng.uniform(0.5, 1.5, len(bonds))
    jz = rng.uniform(-1.0, 1.0, len(bonds))
    om, osec, h, D = both((L, L, 1, 1, bonds, jxy, jz), nod, (K, 0, 0))
    check_sector(osec, h, D)
    check_table(osec, h)
    check_hv(osec, h, seed=L)
    if K == 0:
        x = rng.standard_normal(D)
        np.testing.assert_array_equal(h.hv_real(x), h.hv(x.astype(np.complex128)).real)
    h.close()
