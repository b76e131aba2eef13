"""The benchmark workloads themselves under GPU-vs-oracle parity.

* The H*v benchmark sector: XXZ chain L=1000, nearest-neighbour (Jxy, Jz) =
  (1, 0.5), next-nearest (0.3, 0.3), N_down=4, k=0 (D = 41,417,250, 10-bit
  site packing, 1.66e8-entry anchored directory).  list_s is compared with
  the oracle's enumeration bit for bit and list_r to 1e-15; a sample of rows
  is re-checked with checkstate_SQ itself; on 10,000 rows spread over the
  sector H*v (complex(8), real, complex(4)) is compared with the oracle's
  ham_to_vec_wave_vector and on 3,000 rows the connection table bit for bit.
* Config 1: Heisenberg chain L=36, N_down=6, k=0 (D = 54,132), thick-restart
  Lanczos for the lowest 4 eigenpairs with the reference's convergence test
  at 1e-12, against the oracle's TRLan from the same seeded start vector,
  and <S^z_1 S^z_j>, <S^+_1 S^-_j> for every j against the oracle.

Tolerances as in test_gpu_parity.py: bit-exact integer tables, H*v 1e-13 of
max|y| (complex(4): 2e-6), eigenvalues 1e-10 relative, correlations 1e-12.
On the 2000-bond benchmark chain the H*v tolerance adds, per row, the
rounding bound of the reference's own diagonal (a running sum over all 2000
bonds, NOxxz * 2^-53 * sum|Jz|/4 * |x_i|), and 200 rows are summed exactly to
show that the GPU's row sums are the closer ones.
"""
import numpy as np
import pytest

from ed_gb300 import inputs
from oracle import oracle as O
from oracle import solvers as S

pytestmark = pytest.mark.gpu

L_BENCH, NOD_BENCH = 1000, 4


@pytest.fixture(scope="module")
def bench_sector(qs3g):
    from ed_gb300 import capi
    b, jxy, jz = inputs.chain_bonds(L_BENCH, (1.0, 0.5), (0.3, 0.3))
    h = capi.Handle(L_BENCH, L_BENCH, 1, 1, b, jxy, jz)
    D = h.build_sector(NOD_BENCH, (0, 0, 0))
    om = O.Model(L_BENCH, L_BENCH, 1, 1, b, jxy, jz, kmax=NOD_BENCH + 2)
    ls, lr = h.get_sector()
    yield h, D, om, ls, lr
    h.close()


def _blocks(D, nblk, size):
    starts = np.linspace(0, D - size, nblk).astype(np.int64)
    return [(int(s), int(s) + size) for s in starts]


def test_bench_sector_lists(bench_sector):
    h, D, om, ls, lr = bench_sector
    assert D == 41417250
    ls0, lr0 = O.chain_sector_lists(L_BENCH, NOD_BENCH, 0)
    np.testing.assert_array_equal(ls, ls0)
    np.testing.assert_allclose(lr, lr0, rtol=1e-15, atol=0)
    # checkstate_SQ (state_lists.f90:66-112) on sampled rows and on sampled ranks that are not rows
    rng = np.random.default_rng(7)
    rk = O.wavevector((0, 0, 0), om.Ls)
    for i in rng.integers(0, D, 300):
        np.testing.assert_allclose(om.checkstate(ls[i], NOD_BENCH, rk), lr[i] ** 2, rtol=1e-14)
    total = om.binom(L_BENCH, NOD_BENCH)
    cand = rng.integers(1, total + 1, 3000)
    pos = np.minimum(np.searchsorted(ls, cand), D - 1)
    absent = cand[ls[pos] != cand]
    assert len(absent) > 2000
    for s in absent[:300]:
        assert om.checkstate(int(s), NOD_BENCH, rk) <= 1e-15


def diag_sum_bound(jz, x):
    """Rounding bound of the reference's diagonal: ham2vec_v3.f90:56-67 adds
    +-Jz_b/4 * v1(i) for every one of the NOxxz bonds in sequence, so its result
    carries up to NOxxz * 2^-53 * sum_b |Jz_b|/4 * |v1(i)| of accumulated
    rounding (about 1e-13 of max|y| on the 2000-bond benchmark chain; the GPU
    adds a precomputed diagonal once)."""
    return len(jz) * 2.0 ** -53 * np.abs(0.25 * np.asarray(jz)).sum() * np.abs(x)


def exact_rows(osec, x, r0, r1):
    """y_i for rows [r0, r1) summed exactly (math.fsum of the rounded terms) from
    the oracle's connection table: diagonal sum_b +-Jz_b/4 (antiparallel bonds
    are the table's bonds: at k = 0 every hop lands on a row), plus the hops
    Jxy_b/2 * list_r(col)/list_r(row) * x(col)."""
    import math
    m = osec.model
    sz = 0.25 * m.Jz
    row, col, ell, bond = osec.connection_table(rows=(r0, r1))
    out = np.zeros(r1 - r0, np.complex128)
    for i in range(r0, r1):
        sel = row == i
        b, c = bond[sel], col[sel]
        d = math.fsum(sz) - 2.0 * math.fsum(sz[b])
        coef = (0.5 * m.Jxy[b]) * osec.list_r[c] / osec.list_r[i]
        re = math.fsum([d * x[i].real] + list(coef * x[c].real))
        im = math.fsum([d * x[i].imag] + list(coef * x[c].imag))
        out[i - r0] = re + 1j * im
    return out


def test_bench_sector_hv_rows(bench_sector):
    h, D, om, ls, lr = bench_sector
    osec = O.Sector(om, NOD_BENCH, (0, 0, 0), ls, lr)
    rng = np.random.default_rng(11)
    x = rng.standard_normal(D) + 1j * rng.standard_normal(D)
    y = h.hv(x)
    yr = h.hv_real(x.real)
    x32 = x.astype(np.complex64)
    y32 = h.hv32(x32)
    x32d = x32.astype(np.complex128)
    for r0, r1 in _blocks(D, 8, 1250):
        y0 = osec.hv(x, rows=(r0, r1))[r0:r1]
        tol = 1e-13 * np.abs(y0).max() + diag_sum_bound(om.Jz, x[r0:r1])
        assert (np.abs(y[r0:r1] - y0) <= tol).all()
        y0r = osec.hv(x.real.astype(np.complex128), rows=(r0, r1))[r0:r1]
        assert np.abs(y0r.imag).max() == 0.0
        tolr = 1e-13 * np.abs(y0r).max() + diag_sum_bound(om.Jz, x.real[r0:r1])
        assert (np.abs(yr[r0:r1] - y0r.real) <= tolr).all()
        y0b = osec.hv(x32d, rows=(r0, r1))[r0:r1]
        assert np.abs(y32[r0:r1] - y0b).max() <= 2e-6 * np.abs(y0b).max()
    # against exactly summed rows both sides are close, the GPU closer (its
    # diagonal is one precomputed product, the reference's a 2000-term running sum)
    r0, r1 = D // 2, D // 2 + 200
    ye = exact_rows(osec, x, r0, r1)
    y0 = osec.hv(x, rows=(r0, r1))[r0:r1]
    err_gpu = np.abs(y[r0:r1] - ye).max() / np.abs(ye).max()
    err_ora = np.abs(y0 - ye).max() / np.abs(ye).max()
    assert err_gpu <= 1e-14 and err_gpu <= err_ora


def test_bench_sector_connection_rows(bench_sector):
    h, D, om, ls, lr = bench_sector
    osec = O.Sector(om, NOD_BENCH, (0, 0, 0), ls, lr)
    nnz = 0
    for r0, r1 in _blocks(D, 3, 1000):
        ro, co, eo, bo = osec.connection_table(rows=(r0, r1))
        rg, cg, eg, bg = h.connection_table(rows=(r0, r1))
        np.testing.assert_array_equal(rg, ro + 1)
        np.testing.assert_array_equal(cg, co + 1)
        np.testing.assert_array_equal(eg, eo)
        np.testing.assert_array_equal(bg, bo + 1)
        nnz += len(ro)
    assert nnz > 30000


def test_config1_trlan_and_correlations(qs3g):
    from ed_gb300 import capi
    L, nod = 36, 6
    b, jxy, jz = inputs.chain_bonds(L, (1.0, 1.0))
    om = O.Model(L, L, 1, 1, b, jxy, jz, kmax=nod + 2)
    osec = om.build_sector(nod, (0, 0, 0))
    h = capi.Handle(L, L, 1, 1, b, jxy, jz)
    D = h.build_sector(nod, (0, 0, 0))
    assert D == osec.D == 54132
    ls, lr = h.get_sector()
    np.testing.assert_array_equal(ls, osec.list_s)
    np.testing.assert_allclose(lr, osec.list_r, rtol=1e-15, atol=0)
    r0, c0, e0, b0 = osec.connection_table()
    r1, c1, e1, b1 = h.connection_table()
    np.testing.assert_array_equal(r1, r0 + 1)
    np.testing.assert_array_equal(c1, c0 + 1)
    np.testing.assert_array_equal(e1, e0)
    np.testing.assert_array_equal(b1, b0 + 1)
    rng = np.random.default_rng(36)
    x = rng.standard_normal(D) + 1j * rng.standard_normal(D)
    y0 = osec.hv(x)
    assert np.abs(h.hv(x) - y0).max() <= 1e-13 * np.abs(y0).max()
    # TRLan, lowest 4, the reference's stagnation test at 1e-12 (eigen_solver.f90:150-159)
    NOE, NOK, NOM, seed = 4, 8, 24, 2024
    r = h.trlan(NOE, NOK, NOM, maxitr=5000, tol=1e-12, conv_mode=0, seed=seed)
    Hs = osec.sparse()
    assert np.abs(Hs @ x - y0).max() <= 1e-13 * np.abs(y0).max()
    ene, _, _, conv = S.trlan(lambda v: Hs @ v, D, NOE, NOK, NOM, 5000, 1e-12, S.start_vector(D, seed))
    assert conv
    np.testing.assert_allclose(r["ene"], ene[:NOE], rtol=1e-10, atol=0)
    assert r["resid"].max() < 1e-5
    # the list_cf_ss of the configuration: pairs (1, j), j = 1..36
    psi = r["psi"][0]
    zz1, pm1, lm1 = h.correlations(psi)
    pairs = np.array([(1, j) for j in range(1, L + 1)], np.int32)
    zz0, pm0 = osec.corr(psi, ss=np.stack([pairs[:, 1], pairs[:, 0]], axis=1))
    a, bb = pairs[:, 0] - 1, pairs[:, 1] - 1
    np.testing.assert_allclose(zz1.T[a, bb], zz0[a, bb], rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(pm1.T[a, bb], pm0[a, bb], rtol=1e-12, atol=1e-13)
    # <Sz_1 Sz_1> = 1/4 and sum_j <Sz_1 Sz_j> = Sz_tot^2 / L
    np.testing.assert_allclose(zz1[0, 0], 0.25, rtol=1e-13)
    np.testing.assert_allclose(zz1[0].sum(), (L / 2 - nod) ** 2 / L, rtol=1e-10)
    h.close()
