"""qs3g_trlan_batch: many independent problems solved concurrently give the
same eigenpairs as one-at-a-time qs3g_trlan and as dense diagonalisation."""
import numpy as np
import pytest

from oracle import oracle as O
from ed_gb300 import inputs

pytestmark = pytest.mark.gpu


def test_trlan_batch_matches_single_and_dense(qs3g):
    from ed_gb300 import capi, sweep
    probs = sweep.random_chains(seed=4, n=10, L_range=(14, 20), nods=(3, 4))
    recs, _, _ = sweep.solve(probs, NOE=2, NOK=4, NOM=12, tol=1e-10, precision=1, nthreads=4)
    for p, r in zip(probs, recs):
        assert r["status"] == 0, r
        b, jxy, jz = inputs.chain_bonds(p["L"], (1.0, p["delta"]), (p["j2"], p["j2"]))
        om = O.Model(p["L"], p["L"], 1, 1, b, jxy, jz, kmax=p["nod"] + 2)
        w = np.linalg.eigvalsh(om.build_sector(p["nod"], (p["K"], 0, 0)).dense())
        assert abs(r["ene"][0] - w[0]) <= 1e-9 * max(1.0, abs(w[0]))
        assert max(r["resid"]) <= 1e-10
        h = capi.Handle(p["L"], p["L"], 1, 1, b, jxy, jz)
        h.build_sector(p["nod"], (p["K"], 0, 0))
        one = h.trlan(2, 4, 12, maxitr=20000, tol=1e-10, precision=1, conv_mode=1, seed=1)
        np.testing.assert_allclose(r["ene"], one["ene"], rtol=0, atol=1e-10)
        h.close()


@pytest.mark.parametrize("precision", [1, 2])
def test_trlan_lockstep_matches_dense(qs3g, precision):
    """All problems in one launch sequence: each problem's two lowest levels
    equal dense diagonalisation, with FP64 residuals <= 1e-10."""
    from ed_gb300 import sweep
    probs = sweep.random_chains(seed=6, n=12, L_range=(14, 22), nods=(3, 4))
    recs, _, _ = sweep.solve(probs, NOE=2, NOK=4, NOM=12, tol=1e-10, precision=precision, lockstep=True)
    for p, r in zip(probs, recs):
        assert r["status"] == 0, r
        b, jxy, jz = inputs.chain_bonds(p["L"], (1.0, p["delta"]), (p["j2"], p["j2"]))
        om = O.Model(p["L"], p["L"], 1, 1, b, jxy, jz, kmax=p["nod"] + 2)
        w = np.linalg.eigvalsh(om.build_sector(p["nod"], (p["K"], 0, 0)).dense())
        assert abs(r["ene"][0] - w[0]) <= 1e-9 * max(1.0, abs(w[0])), (r["ene"], w[:3])
        assert max(r["resid"]) <= 1e-10


def test_trlan_lockstep_wide_basis_matches_dense(qs3g):
    """NOM = 90: the device Ritz solves keep their NOM x NOM matrices in
    global scratch instead of shared memory; same answers as dense."""
    from ed_gb300 import sweep
    probs = sweep.random_chains(seed=8, n=5, L_range=(24, 28), nods=(4,))
    recs, _, _ = sweep.solve(probs, NOE=2, NOK=40, NOM=90, tol=1e-10, precision=1, lockstep=True)
    for p, r in zip(probs, recs):
        assert r["status"] == 0, r
        b, jxy, jz = inputs.chain_bonds(p["L"], (1.0, p["delta"]), (p["j2"], p["j2"]))
        om = O.Model(p["L"], p["L"], 1, 1, b, jxy, jz, kmax=p["nod"] + 2)
        w = np.linalg.eigvalsh(om.build_sector(p["nod"], (p["K"], 0, 0)).dense())
        assert abs(r["ene"][0] - w[0]) <= 1e-9 * max(1.0, abs(w[0])), (r["ene"], w[:3])
        assert abs(r["ene"][1] - w[1]) <= 1e-9 * max(1.0, abs(w[1])), (r["ene"], w[:3])
        assert max(r["resid"]) <= 1e-10
