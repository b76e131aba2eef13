"""The learned start vector on the GPU (qs3g_mlp_*): forward pass, loss and
gradient against the float64 oracle (oracle/mlp_oracle.py), then training on
small-L ground states and the gain of the predicted start vector.

Tolerances: the GPU accumulates in float32 (tensor-core BF16 products) and
the oracle in float64, with the same BF16 roundings of inputs, parameters,
activations and back-propagated signals.  A value within an FP32 rounding of
a BF16 tie can round to different neighbours on the two sides (one BF16 unit,
2^-8 relative), so the loss agrees to 1e-4 relative and the gradient to
2e-3 in relative 2-norm, per layer; a wrong fragment layout or a missing term
would show as O(1).
"""
import numpy as np
import pytest

from oracle import mlp_oracle as M
from oracle import oracle as O
from ed_gb300 import inputs

pytestmark = pytest.mark.gpu


def _chain(L, delta, j2):
    b, jxy, jz = inputs.chain_bonds(L, (1.0, delta), (j2, j2))
    return b, jxy, jz


def _gs_case(L, nod, delta, j2):
    from ed_gb300 import capi
    b, jxy, jz = _chain(L, delta, j2)
    om = O.Model(L, L, 1, 1, b, jxy, jz, kmax=nod + 2)
    osec = om.build_sector(nod, (0, 0, 0))
    w, V = np.linalg.eigh(osec.dense())
    psi = np.ascontiguousarray(V[:, 0])
    h = capi.Handle(L, L, 1, 1, b, jxy, jz)
    h.build_sector(nod, (0, 0, 0))
    confs = np.array([om.list_fly(int(t), nod) for t in osec.list_s])
    return om, osec, h, psi, confs, w[0]


def test_mlp_loss_and_gradient_match_oracle(qs3g):
    from ed_gb300 import capi
    nod = 4
    cases = [(16, 0.5, 0.1), (20, 1.3, 0.4)]
    net = capi.Mlp(seed=3)
    p = M.init_params(np.random.default_rng(7))
    net.set_params(p)
    np.testing.assert_array_equal(net.params(), p.astype(np.float32).astype(np.float64))
    Xs, ts = [], []
    for L, delta, j2 in cases:
        om, osec, h, psi, confs, _ = _gs_case(L, nod, delta, j2)
        q0 = capi.band_minimum(1.0, j2)
        net.add_sample(h, psi, delta, j2, q0)
        Xs.append(M.features(confs, L, delta, j2, q0))
        ts.append(M.targets(psi, osec.list_r, confs, L, nod, q0))
        h.close()
    X, t = np.concatenate(Xs), np.concatenate(ts)
    loss0, g0 = M.loss_grad(p, X, t, nod)
    loss1, g1 = net.loss_grad()
    assert abs(loss1 - loss0) <= 1e-4 * loss0
    assert np.linalg.norm(g1 - g0) <= 2e-3 * np.linalg.norm(g0)
    # per-layer check so that no block of the gradient hides behind another's norm
    for a, b in [(M.OFF_W1, M.OFF_B1), (M.OFF_W2, M.OFF_B2), (M.OFF_W3, M.OFF_B3), (M.OFF_W4, M.OFF_B4 + 1)]:
        assert np.linalg.norm(g1[a:b] - g0[a:b]) <= 2e-3 * np.linalg.norm(g0[a:b]) + 1e-12
    net.close()


def test_mlp_training_gains_over_random_start(qs3g):
    """Trained on small chains, the network's start vector for an unseen
    (L, Delta, J2) overlaps the ground state far better than a random vector
    and TRLan needs fewer H*v products from it."""
    from ed_gb300 import capi
    nod = 4
    net = capi.Mlp(seed=5)
    rng = np.random.default_rng(2)
    for L in (16, 18, 20, 22, 24, 26, 28):
        for _ in range(3):
            delta, j2 = float(rng.uniform(0, 2)), float(rng.uniform(0, 0.5))
            b, jxy, jz = _chain(L, delta, j2)
            h = capi.Handle(L, L, 1, 1, b, jxy, jz)
            h.build_sector(nod, (0, 0, 0))
            r = h.trlan(1, 6, 20, maxitr=3000, tol=1e-12, seed=1)
            net.add_sample(h, r["psi"][0], delta, j2, capi.band_minimum(1.0, j2))
            h.close()
    l0, _ = net.loss_grad()
    for _ in range(4):
        net.train(150, 2048, 2e-3, seed=11)
        net.align()
    l1, _ = net.loss_grad()
    assert l1 < 0.2 * l0
    # held-out problem
    L, delta, j2 = 30, 0.7, 0.25
    b, jxy, jz = _chain(L, delta, j2)
    h = capi.Handle(L, L, 1, 1, b, jxy, jz)
    D = h.build_sector(nod, (0, 0, 0))
    exact = h.trlan(1, 6, 20, maxitr=3000, tol=1e-12, seed=1)
    gs = exact["psi"][0]
    v = net.predict(h, delta, j2, capi.band_minimum(1.0, j2))
    ov = abs(np.vdot(gs, v)) / np.linalg.norm(v)
    vr = S_random(D)
    ovr = abs(np.vdot(gs, vr)) / np.linalg.norm(vr)
    assert ov > 0.5 and ov > 5 * ovr, (ov, ovr)
    r_learn = h.trlan(1, 6, 20, maxitr=3000, tol=1e-10, conv_mode=1, start=v)
    r_rand = h.trlan(1, 6, 20, maxitr=3000, tol=1e-10, conv_mode=1, seed=9)
    assert abs(r_learn["ene"][0] - exact["ene"][0]) < 1e-9
    assert r_learn["iters"] <= r_rand["iters"]
    h.close()
    net.close()


def S_random(D):
    from oracle import solvers as S
    return S.start_vector(D, 9)
