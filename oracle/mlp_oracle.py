"""TEST INFRASTRUCTURE ONLY: a float64 numpy restatement of the learned
start-vector network (ed_gb300/csrc/mlp.cu), used to check the GPU's forward
pass, loss and gradients.  Only tests/ may import it.

It follows the same definitions: inputs and parameters rounded to BF16
(round to nearest even), hidden activations tanh rounded to BF16 (the GPU
keeps them as BF16 tensor-core operands), back-propagated signals
dz = dL/d(pre-activation) rounded to BF16 before they enter a matrix
product, output = mean over the NOD
cyclic rotations of the gap sequence, loss = mean over representatives of
(f - t)^2, targets t = Re(psi * phase) * list_r / L * sqrt(C(L, NOD)) with the
phase that makes the largest-modulus amplitude real and the sign that makes
sum_r t_r cos(q0 (g_0 + g_2 + ...)) >= 0.  Arithmetic is float64 here and
float32 on the GPU, so agreement is to float32 rounding, not bit-exact.
"""
from math import comb

import numpy as np

IN, HID = 16, 128
OFF_W1 = 0
OFF_B1 = OFF_W1 + IN * HID
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + HID * HID
OFF_W4 = OFF_B3 + HID
OFF_B4 = OFF_W4 + HID
NPARAMS = OFF_B4 + 1


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    u = np.ascontiguousarray(np.asarray(x, np.float32)).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p, round_params=True):
    p = bf16(np.asarray(p, np.float64).astype(np.float32)) if round_params else np.asarray(p, np.float64)
    W1 = p[OFF_W1:OFF_B1].reshape(IN, HID)
    b1 = p[OFF_B1:OFF_W2]
    W2 = p[OFF_W2:OFF_B2].reshape(HID, HID)
    b2 = p[OFF_B2:OFF_W3]
    W3 = p[OFF_W3:OFF_B3].reshape(HID, HID)
    b3 = p[OFF_B3:OFF_W4]
    w4 = p[OFF_W4:OFF_B4]
    b4 = p[OFF_B4]
    return W1, b1, W2, b2, W3, b3, w4, b4


def gaps(confs, L):
    """confs: (n, NOD) sorted 1-based sites -> (n, NOD) cyclic gaps."""
    c = np.asarray(confs, np.int64)
    g = np.empty_like(c)
    g[:, :-1] = c[:, 1:] - c[:, :-1]
    g[:, -1] = c[:, 0] + L - c[:, -1]
    return g


def features(confs, L, delta, j2, q0):
    """(n * NOD, 16) inputs: rotation s of rep r at row r * NOD + s."""
    g = gaps(confs, L)
    n, nod = g.shape
    h_all = np.arange(L + 1)
    cos_t = bf16(np.cos(q0 * h_all).astype(np.float32))
    sin_t = bf16(np.sin(q0 * h_all).astype(np.float32))
    invL = np.float32(1.0) / np.float32(L)
    X = np.zeros((n, nod, IN))
    for s in range(nod):
        h = np.roll(g, -s, axis=1)
        X[:, s, :nod] = bf16(h.astype(np.float32) * invL)
        X[:, s, nod:2 * nod] = cos_t[h]
        X[:, s, 2 * nod:3 * nod] = sin_t[h]
        X[:, s, 3 * nod] = bf16(np.float32(delta))
        X[:, s, 3 * nod + 1] = bf16(np.float32(j2))
    return X.reshape(n * nod, IN)


def forward(p, X, nod, round_params=True, round_acts=True):
    """round_acts=False: exact float64 activations (the smooth function whose
    gradient the finite-difference test checks); True: BF16 as on the GPU."""
    rd = bf16 if round_acts else (lambda v: v)
    W1, b1, W2, b2, W3, b3, w4, b4 = unpack(p, round_params)
    h1 = rd(np.tanh(X @ W1 + b1))
    h2 = rd(np.tanh(h1 @ W2 + b2))
    h3 = rd(np.tanh(h2 @ W3 + b3))
    out = h3 @ w4 + b4
    f = out.reshape(-1, nod).mean(axis=1)
    return f, (h1, h2, h3)


def targets(psi, list_r, confs, L, nod, q0):
    psi = np.asarray(psi, np.complex128)
    a = psi.real ** 2 + psi.imag ** 2
    i = int(np.argmax(a))
    ab = np.sqrt(a[i])
    ph = np.conj(psi[i]) / ab
    re = psi.real * ph.real - psi.imag * ph.imag
    g = gaps(confs, L)
    ge = g[:, 0::2].sum(axis=1)
    if np.sum(re * np.cos(q0 * ge)) < 0:
        re = -re
    scale = np.sqrt(float(comb(L, nod))) / L
    return (re * np.asarray(list_r) * scale).astype(np.float32).astype(np.float64)


def loss_grad(p, X, t, nod, round_params=True, round_acts=True):
    """Mean squared error over representatives and its gradient (NPARAMS).
    With round_acts the activations and the back-propagated signals are
    rounded to BF16 where the GPU rounds them (the gradient of the rounded
    forward pass taken through the roundings)."""
    rd = bf16 if round_acts else (lambda v: v)
    W1, b1, W2, b2, W3, b3, w4, b4 = unpack(p, round_params)
    f, (h1, h2, h3) = forward(p, X, nod, round_params, round_acts)
    B = len(t)
    e = f - t
    loss = float(np.sum(e * e) / B)
    dout = np.repeat(2.0 * e / B / nod, nod)
    g = np.zeros(NPARAMS)
    g[OFF_W4:OFF_B4] = h3.T @ dout
    g[OFF_B4] = dout.sum()
    dz3 = rd(np.outer(dout, w4) * (1 - h3 * h3))
    g[OFF_W3:OFF_B3] = (h2.T @ dz3).reshape(-1)
    g[OFF_B3:OFF_W4] = dz3.sum(axis=0)
    dz2 = rd((dz3 @ W3.T) * (1 - h2 * h2))
    g[OFF_W2:OFF_B2] = (h1.T @ dz2).reshape(-1)
    g[OFF_B2:OFF_W3] = dz2.sum(axis=0)
    dz1 = rd((dz2 @ W2.T) * (1 - h1 * h1))
    g[OFF_W1:OFF_B1] = (X.T @ dz1).reshape(-1)
    g[OFF_B1:OFF_W2] = dz1.sum(axis=0)
    return loss, g


def init_params(rng):
    p = np.zeros(NPARAMS)
    a1, a2, a4 = np.sqrt(6 / (IN + HID)), np.sqrt(6 / (2 * HID)), np.sqrt(6 / (HID + 1))
    p[OFF_W1:OFF_B1] = rng.uniform(-a1, a1, IN * HID)
    p[OFF_W2:OFF_B2] = rng.uniform(-a2, a2, HID * HID)
    p[OFF_W3:OFF_B3] = rng.uniform(-a2, a2, HID * HID)
    p[OFF_W4:OFF_B4] = rng.uniform(-a4, a4, HID)
    p[OFF_B1:OFF_W2] = rng.uniform(-0.1, 0.1, HID)
    p[OFF_B2:OFF_W3] = rng.uniform(-0.1, 0.1, HID)
    p[OFF_B3:OFF_W4] = rng.uniform(-0.1, 0.1, HID)
    p[OFF_B4] = 0.05
    return p
