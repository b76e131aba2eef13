"""Many independent chain problems solved at once (qs3g_trlan_batch).

``random_chains`` draws problems the way the batched-solve workload is
specified: L uniform in {48..128}, N_down uniform in {3, 4, 5}, K uniform
over the L momenta, Delta = Jz/Jxy uniform in [0, 2], J2 uniform in [0, 0.5]
(both components), periodic.  ``solve`` builds every sector and runs the
lowest NOE eigenpairs of all problems concurrently.
"""
from __future__ import annotations

import time

import numpy as np

from . import capi, learned


def random_chains(seed: int = 1, n: int = 256, L_range=(48, 128), nods=(3, 4, 5), delta_range=(0.0, 2.0),
                  j2_range=(0.0, 0.5)):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        L = int(rng.integers(L_range[0], L_range[1] + 1))
        out.append(dict(L=L, nod=int(rng.choice(nods)), K=int(rng.integers(0, L)),
                        delta=float(rng.uniform(*delta_range)), j2=float(rng.uniform(*j2_range))))
    return out


def solve(problems, NOE=2, NOK=8, NOM=24, tol=1e-10, precision=1, maxitr=20000, nthreads=8, seed=1,
          lockstep=False, hv_cache=False):
    """Build every sector, then solve all problems with qs3g_trlan_batch
    (concurrent streams) or, with lockstep=True, qs3g_trlan_lockstep (one
    launch sequence for all problems).  hv_cache: cache each sector's
    connection table first (qs3g_hv_cache; skipped where it does not fit).
    Returns (records, build seconds, solve seconds)."""
    t0 = time.perf_counter()
    hs = []
    for p in problems:
        h = learned.chain_handle(p["L"], p["delta"], p["j2"])
        h.build_sector(p["nod"], (p["K"], 0, 0))
        if hv_cache:
            try:
                h.hv_cache(True)
            except capi.QS3GError as e:
                if e.code != capi.ENOMEM:
                    raise
        hs.append(h)
    t_build = time.perf_counter() - t0
    t0 = time.perf_counter()
    if lockstep:
        ene, iters, resid, status = capi.trlan_lockstep(hs, NOE, NOK, NOM, maxitr=maxitr, tol=tol,
                                                        precision=precision, conv_mode=1, seed=seed)
    else:
        ene, iters, resid, status = capi.trlan_batch(hs, NOE, NOK, NOM, maxitr=maxitr, tol=tol, precision=precision,
                                                     conv_mode=1, seed=seed, nthreads=nthreads)
    t_solve = time.perf_counter() - t0
    recs = []
    for p, h, e, it, r, st in zip(problems, hs, ene, iters, resid, status):
        recs.append(dict(p, D=h.D, ene=[float(x) for x in e], hv=int(it), resid=[float(x) for x in r],
                         status=int(st)))
        h.close()
    return recs, t_build, t_solve
