"""Generate the golden fixtures in this directory.

The fixtures pin the CPU oracle to known answers that do not depend on it:
spectra from the independent dense exact diagonalisation (oracle/dense_ed.py,
bit-string basis + projection with translation characters), free-fermion XX
chain spectra, and single-magnon energies.  The reference QS3 ships no golden
outputs and cannot be compiled in this image (no Fortran compiler), so these
physics-derived values are the pin.

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import dense_ed as E  # noqa: E402

CASES = [
    # name, NOS, LX, LY, LZ, NOD, bonds spec
    ("chain10_nod3_heis", 10, 10, 1, 1, 3, ("chain", (1.0, 1.0), None)),
    ("chain12_nod4_xxz_j2", 12, 12, 1, 1, 4, ("chain", (1.0, 0.5), (0.3, 0.3))),
    ("chain12_nod6_heis", 12, 12, 1, 1, 6, ("chain", (1.0, 1.0), None)),
    ("chain11_nod2_fm", 11, 11, 1, 1, 2, ("chain", (-1.0, -1.0), None)),
    ("square4x3_nod3", 12, 4, 3, 1, 3, ("square", (1.0, 0.7), None)),
]


def bonds_for(spec, LX, LY):
    kind, a, b = spec
    if kind == "chain":
        return E.chain_bonds(LX, a, b)
    return E.square_bonds(LX, LY, a)


def main():
    out = {"cases": []}
    for name, NOS, LX, LY, LZ, nod, spec in CASES:
        bonds, jxy, jz = bonds_for(spec, LX, LY)
        sectors = {}
        for kz in range(LZ):
            for ky in range(LY):
                for kx in range(LX):
                    w = E.sector_spectrum(NOS, nod, (LX, LY, LZ), bonds, jxy, jz, (kx, ky, kz), +1)
                    sectors[f"{kx},{ky},{kz}"] = [float(v) for v in w]
        out["cases"].append({
            "name": name, "NOS": NOS, "LX": LX, "LY": LY, "LZ": LZ, "NOD": nod,
            "bonds": bonds.tolist(), "Jxy": jxy.tolist(), "Jz": jz.tolist(),
            "u1_spectrum": [float(v) for v in E.u1_spectrum(NOS, nod, bonds, jxy, jz)],
            "sectors": sectors,
        })
    # XX chain (Jz = 0): Jordan-Wigner free fermions
    L, N = 12, 3
    xx = {}
    for K in range(L):
        xx[str(K)] = E.xx_chain_sector_energies(L, N, 1.0, K)[1].tolist()
    out["xx_chain"] = {"L": L, "N": N, "Jxy": 1.0, "sector_energies": xx}
    # single magnon on a Heisenberg-XXZ chain: E(k) = L Jz/4 - Jz + Jxy cos k
    L, jxy1, jz1 = 16, 1.0, 0.6
    out["magnon"] = {"L": L, "Jxy": jxy1, "Jz": jz1,
                     "energies": [L * jz1 / 4 - jz1 + jxy1 * np.cos(2 * np.pi * k / L) for k in range(L)]}
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=0)
    print("wrote", os.path.join(HERE, "golden.json"))


if __name__ == "__main__":
    main()
