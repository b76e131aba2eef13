"""Learned start vector for thick-restart Lanczos on XXZ chains.

The reference starts TRLan from a random vector (source/eigen_solver.f90:92-96).
Here a small network (ed_gb300/csrc/mlp.cu, the qs3g_mlp_* entry points)
predicts the k = 0 ground-state amplitude of every chain representative
from the gaps between its down spins, conditioned on (Delta, J2, q0).  The
pipeline, all on the GPU through the library:

1. ``training_problems``: a seeded grid of chains (L, Delta, J2);
2. ``generate``: their k = 0 ground states from qs3g_trlan, added as samples;
3. ``train``: Adam rounds on the BF16/FP32 kernels, with a global-sign
   alignment of every sample between rounds;
4. ``start_vector``: the prediction for a (larger, unseen) chain, passed to
   qs3g_trlan with start_mode = 1.  The random start stays the fallback: the
   converged residual, not the network, decides the result's accuracy.

Chains follow the bond convention of the configs: nearest-neighbour
(Jxy, Jz) = (1, Delta), next-nearest (J2, J2), periodic.
"""
from __future__ import annotations

import time

import numpy as np

from . import capi, inputs


def chain_handle(L: int, delta: float, j2: float) -> capi.Handle:
    b, jxy, jz = inputs.chain_bonds(L, (1.0, delta), (j2, j2) if j2 != 0.0 else None)
    return capi.Handle(L, L, 1, 1, b, jxy, jz)


def cond(delta: float, j2: float) -> tuple[float, float, float]:
    """(Delta, J2, q0) with q0 the magnon band minimum of cos q + J2 cos 2q."""
    return float(delta), float(j2), capi.band_minimum(1.0, j2)


def training_problems(seed: int = 1, Ls=(48, 64, 80, 96, 112, 128), per_L: int = 4,
                      delta_range=(0.0, 2.0), j2_range=(0.0, 0.5)):
    """Seeded (L, Delta, J2) grid: per_L draws of (Delta, J2) for every L."""
    rng = np.random.default_rng(seed)
    out = []
    for L in Ls:
        for _ in range(per_L):
            out.append((int(L), float(rng.uniform(*delta_range)), float(rng.uniform(*j2_range))))
    return out


def generate(net: capi.Mlp, problems, nod: int = 4, NOK: int = 8, NOM: int = 24, tol: float = 1e-10,
             precision: int = 2, seed: int = 1, log=None):
    """Solve every problem's k = 0 ground state with qs3g_trlan and add it to
    the network's training set.  Returns one record per problem."""
    recs = []
    for (L, delta, j2) in problems:
        h = chain_handle(L, delta, j2)
        D = h.build_sector(nod, (0, 0, 0))
        t0 = time.perf_counter()
        r = h.trlan(1, NOK, NOM, maxitr=20000, tol=tol, precision=precision, conv_mode=1, seed=seed)
        dt = time.perf_counter() - t0
        net.add_sample(h, r["psi"][0], *cond(delta, j2))
        rec = dict(L=L, delta=delta, j2=j2, D=D, E0=float(r["ene"][0]), hv=r["iters"], t=dt,
                   resid=float(r["resid"][0]))
        recs.append(rec)
        if log:
            log(rec)
        h.close()
    return recs


def train(net: capi.Mlp, rounds: int = 6, steps: int = 200, batch: int = 4096, lr: float = 2e-3,
          lr_decay: float = 0.7, seed: int = 1, log=None):
    """Adam rounds with a sign alignment of every sample between rounds.
    Returns the full-set loss after each round."""
    hist = [net.loss_grad()[0]]
    for k in range(rounds):
        net.train(steps, batch, lr * (lr_decay ** k), seed=seed + k)
        flips = net.align()
        hist.append(net.loss_grad()[0])
        if log:
            log(dict(round=k, loss=hist[-1], flipped=flips))
    return hist


def start_vector(net: capi.Mlp, h: capi.Handle, delta: float, j2: float) -> np.ndarray:
    """Predicted start vector for the handle's k = 0 chain sector (unnormalised)."""
    return net.predict(h, *cond(delta, j2))
