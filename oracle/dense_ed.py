"""Independent dense exact diagonalisation in numpy -- TEST INFRASTRUCTURE ONLY.

A second oracle that shares no code and no algorithm with ``qs3_oracle.cpp``:
it works in the full S^z_tot sector with bit-string configurations, builds the
XXZ Hamiltonian
    H = sum_b [ Jxy_b (Sx_i Sx_j + Sy_i Sy_j) + Jz_b Sz_i Sz_j ]
as a dense matrix, and obtains the momentum sectors by projecting with the
characters of the lattice translation group.  It pins the representative-basis
restatement (state_lists.f90 / ham2vec_v3.f90) through spectra, and the
free-fermion and magnon formulas below pin both.  Small lattices only
(C(NOS, NOD) up to a few thousand).
"""
from __future__ import annotations

import itertools

import numpy as np


def site_xyz(s, LX, LY):
    s0 = s - 1
    return s0 % LX, (s0 // LX) % LY, s0 // (LX * LY)


def translate_site(s, t, Ls):
    LX, LY, LZ = Ls
    x, y, z = site_xyz(s, LX, LY)
    x, y, z = (x + t[0]) % LX, (y + t[1]) % LY, (z + t[2]) % LZ
    return 1 + x + LX * (y + LY * z)


def u1_basis(NOS, NOD):
    confs = [tuple(c) for c in itertools.combinations(range(1, NOS + 1), NOD)]
    index = {c: i for i, c in enumerate(confs)}
    return confs, index


def u1_hamiltonian(NOS, NOD, bonds, Jxy, Jz):
    confs, index = u1_basis(NOS, NOD)
    D = len(confs)
    H = np.zeros((D, D))
    for a, c in enumerate(confs):
        down = set(c)
        for (i, j), jxy, jz in zip(bonds, Jxy, Jz):
            di, dj = i in down, j in down
            if di == dj:
                H[a, a] += jz / 4.0
            else:
                H[a, a] -= jz / 4.0
                nd = set(down)
                if di:
                    nd.remove(i); nd.add(j)
                else:
                    nd.remove(j); nd.add(i)
                H[index[tuple(sorted(nd))], a] += jxy / 2.0
    return H, confs, index


def translation_group(Ls):
    LX, LY, LZ = Ls
    return [(x, y, z) for z in range(LZ) for y in range(LY) for x in range(LX)]


def momentum_projector(confs, index, Ls, K, sign=+1):
    """P_K = (1/|G|) sum_t exp(sign*i k.t) T_t on the U(1) basis."""
    LX, LY, LZ = Ls
    k = 2 * np.pi * np.array([K[0] / LX, K[1] / LY, K[2] / LZ])
    D = len(confs)
    P = np.zeros((D, D), dtype=np.complex128)
    G = translation_group(Ls)
    for t in G:
        ph = np.exp(sign * 1j * np.dot(k, t))
        for a, c in enumerate(confs):
            tc = tuple(sorted(translate_site(s, t, Ls) for s in c))
            P[index[tc], a] += ph
    return P / len(G)


def sector_spectrum(NOS, NOD, Ls, bonds, Jxy, Jz, K, sign=+1):
    H, confs, index = u1_hamiltonian(NOS, NOD, bonds, Jxy, Jz)
    P = momentum_projector(confs, index, Ls, K, sign)
    w, V = np.linalg.eigh(P)
    Q = V[:, w > 0.5]
    if Q.shape[1] == 0:
        return np.zeros(0)
    return np.linalg.eigvalsh(Q.conj().T @ H @ Q)


def u1_spectrum(NOS, NOD, bonds, Jxy, Jz):
    H, _, _ = u1_hamiltonian(NOS, NOD, bonds, Jxy, Jz)
    return np.linalg.eigvalsh(H)


def xx_chain_sector_energies(L, N, Jxy, K):
    """XX chain (Jz = 0) by Jordan-Wigner: N fermions with eps(q) = Jxy cos q.

    Periodic spins give fermion momenta q = 2 pi (m + phi)/L with phi = 0 for N
    odd and 1/2 for N even.  Returns all N-fermion energies with total momentum
    congruent to +2 pi K / L or -2 pi K / L (the two orientations), as the
    sorted union of both sets per orientation.
    """
    phi = 0.0 if N % 2 == 1 else 0.5
    ms = np.arange(L)
    out = {+1: [], -1: []}
    for occ in itertools.combinations(ms, N):
        mt = sum(m + phi for m in occ)
        e = sum(Jxy * np.cos(2 * np.pi * (m + phi) / L) for m in occ)
        for sg in (+1, -1):
            if abs(((mt - sg * K) % L + L) % L) < 1e-9 or abs(((mt - sg * K) % L) - L) < 1e-9:
                out[sg].append(e)
    return {sg: np.sort(np.array(v)) for sg, v in out.items()}


def chain_bonds(L, J1=(1.0, 1.0), J2=None):
    """Periodic chain: (s, s+1) with (Jxy, Jz) = J1, plus (s, s+2) with J2 if given."""
    bonds, jxy, jz = [], [], []
    for s in range(1, L + 1):
        bonds.append((s, s % L + 1)); jxy.append(J1[0]); jz.append(J1[1])
    if J2 is not None:
        for s in range(1, L + 1):
            bonds.append((s, (s + 1) % L + 1)); jxy.append(J2[0]); jz.append(J2[1])
    return np.array(bonds, dtype=np.int32), np.array(jxy), np.array(jz)


def square_bonds(LX, LY, J=(1.0, 1.0)):
    bonds = []
    for y in range(LY):
        for x in range(LX):
            s = 1 + x + LX * y
            bonds.append((s, 1 + (x + 1) % LX + LX * y))
            bonds.append((s, 1 + x + LX * ((y + 1) % LY)))
    n = len(bonds)
    return np.array(bonds, dtype=np.int32), np.full(n, J[0]), np.full(n, J[1])
