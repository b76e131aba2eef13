"""CPU tests of the network oracle (oracle/mlp_oracle.py): its backward pass
against central finite differences, BF16 rounding, and the invariance of the
output under translations of a configuration."""
import numpy as np

from oracle import mlp_oracle as M


def _confs(L, nod, n, rng):
    out = []
    while len(out) < n:
        c = np.sort(rng.choice(np.arange(1, L + 1), nod, replace=False))
        out.append(c)
    return np.array(out)


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.0e-5, 65504.0], np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0                     # tie -> even (mantissa 0)
    assert r[2] == 1.0078125               # above the tie -> up
    assert abs(r[3] + 3.0e-5) < 2e-7
    u = r.astype(np.float32).view(np.uint32)
    assert np.all(u & 0xFFFF == 0)


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    L, nod = 24, 4
    confs = _confs(L, nod, 40, rng)
    X = M.features(confs, L, 0.7, 0.25, np.pi)
    t = rng.standard_normal(len(confs))
    p = M.init_params(rng)
    loss, g = M.loss_grad(p, X, t, nod, round_params=False, round_acts=False)
    idx = np.concatenate([rng.choice(np.arange(M.OFF_B1), 6, replace=False),
                          rng.choice(np.arange(M.OFF_W2, M.OFF_B2), 6, replace=False),
                          rng.choice(np.arange(M.OFF_W3, M.OFF_B3), 6, replace=False),
                          np.arange(M.OFF_B3, M.OFF_B3 + 3), np.arange(M.OFF_W4, M.OFF_W4 + 3), [M.OFF_B4]])
    eps = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += eps
        pm[k] -= eps
        lp, _ = M.loss_grad(pp, X, t, nod, round_params=False, round_acts=False)
        lm, _ = M.loss_grad(pm, X, t, nod, round_params=False, round_acts=False)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g[k])


def test_output_is_translation_invariant():
    rng = np.random.default_rng(1)
    L, nod = 30, 4
    p = M.init_params(rng)
    c = np.array([[2, 7, 8, 19]])
    shifted = np.sort((c - 1 + 11) % L + 1, axis=1)
    f0, _ = M.forward(p, M.features(c, L, 1.0, 0.2, np.pi), nod)
    f1, _ = M.forward(p, M.features(shifted, L, 1.0, 0.2, np.pi), nod)
    assert abs(f0[0] - f1[0]) < 1e-12


def test_rounded_gradient_is_close_to_the_exact_one():
    """The BF16 roundings of the activations and signals move the gradient by
    about the BF16 unit (2^-8) relative, not more."""
    rng = np.random.default_rng(2)
    L, nod = 24, 4
    confs = _confs(L, nod, 60, rng)
    X = M.features(confs, L, 0.7, 0.25, np.pi)
    t = rng.standard_normal(len(confs))
    p = M.init_params(rng)
    _, g0 = M.loss_grad(p, X, t, nod, round_acts=False)
    _, g1 = M.loss_grad(p, X, t, nod, round_acts=True)
    assert np.linalg.norm(g1 - g0) <= 2e-2 * np.linalg.norm(g0)
