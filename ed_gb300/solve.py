"""Ground state of an XXZ chain sector from the command line (one JSON line).

    python -m ed_gb300.solve --L 400 --nod 4 --delta 0.5 --j2 0.3 --precision 1

Chain: nearest-neighbour (Jxy, Jz) = (1, delta), next-nearest (j2, j2),
periodic, sector (nod, k).  The solver is qs3g_trlan with a residual stop
(conv_mode 1: ||H psi - E psi|| <= tol, recomputed in FP64 at the end);
precision 0 = FP64 throughout, 1 = complex(4) storage + refinement,
2 = complex(8) storage with double-float arithmetic; --real adds QS3G_REAL
(real Krylov vectors; k = 0 only, where H is real symmetric).  --learned
trains the start-vector network first (ed_gb300.learned) and starts from its
prediction (k = 0, nod <= 4).

    python -m ed_gb300.solve --L 1000 --precision 1 --real --learned
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import capi, learned


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--L", type=int, default=400)
    ap.add_argument("--nod", type=int, default=4)
    ap.add_argument("--k", type=int, default=0)
    ap.add_argument("--delta", type=float, default=0.5)
    ap.add_argument("--j2", type=float, default=0.3)
    ap.add_argument("--precision", type=int, default=0, choices=[0, 1, 2])
    ap.add_argument("--nok", type=int, default=16)
    ap.add_argument("--nom", type=int, default=48)
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--maxitr", type=int, default=40000, help="cap on thick-restart cycles per phase")
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--learned", action="store_true")
    ap.add_argument("--real", action="store_true", help="real Krylov vectors (k = 0)")
    a = ap.parse_args(argv)
    h = learned.chain_handle(a.L, a.delta, a.j2)
    t0 = time.perf_counter()
    D = h.build_sector(a.nod, (a.k, 0, 0))
    out = dict(L=a.L, nod=a.nod, k=a.k, delta=a.delta, j2=a.j2, D=D, precision=a.precision, real=a.real,
               build_s=time.perf_counter() - t0)
    start = None
    if a.learned:
        t0 = time.perf_counter()
        net = capi.Mlp(seed=1)
        learned.generate(net, learned.training_problems(seed=1))
        learned.train(net, rounds=10, steps=300)
        start = learned.start_vector(net, h, a.delta, a.j2)
        out["learned_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    r = h.trlan(1, a.nok, a.nom, maxitr=a.maxitr, tol=a.tol, precision=a.precision, conv_mode=1, seed=a.seed,
                start=start, want_psi=start is not None, allow_unconverged=True, real=a.real)
    out.update(solve_s=time.perf_counter() - t0, hv=r["iters"], E0=float(r["ene"][0]), resid=float(r["resid"][0]),
               converged=bool(r["converged"]))
    if start is not None:
        out["start_overlap"] = float(abs(np.vdot(r["psi"][0], start)) / np.linalg.norm(start))
    print(json.dumps(out), flush=True)
    h.close()
    return 0  # "converged" in the JSON line tells whether the residual target was met


if __name__ == "__main__":
    raise SystemExit(main())
