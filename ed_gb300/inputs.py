"""QS3 input formats: the input.dat namelists and the list_* files.

Reads what read_ip (input_param.f90:58-117), allocate_expe_mem
(get_expectation_values.f90:11-38) and the solver namelists
(eigen_solver.f90:8,16; lanczos.f90:7,25) read from stdin and from disk,
so that an existing QS3 input directory drives this library unchanged.
Also writes chain bond lists in the list_xxz_term format (``i j Jxy Jz``).
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field

import numpy as np

_GROUP = re.compile(r"&(\w+)(.*?)(?:&end|/)", re.S | re.I)
_ITEM = re.compile(r"(\w+)\s*=\s*('(?:[^']*)'|\"(?:[^\"]*)\"|[^,\n]+)")


def _value(tok: str):
    t = tok.strip().rstrip(",").strip()
    if t[:1] in "'\"":
        return t[1:-1]
    tl = t.lower()
    if tl in (".true.", "t"):
        return True
    if tl in (".false.", "f"):
        return False
    try:
        return int(t)
    except ValueError:
        return float(tl.replace("d", "e"))


def _groups(text: str):
    """Yield (name, body) of every namelist group; a group ends at an unquoted
    '/' or at '&end' (quoted strings such as paths may contain '/')."""
    i, n = 0, len(text)
    while True:
        a = text.find("&", i)
        if a < 0:
            return
        m = re.match(r"&(\w+)", text[a:])
        if not m or m.group(1).lower() == "end":
            i = a + 1
            continue
        j = a + m.end()
        quote = None
        k = j
        while k < n:
            ch = text[k]
            if quote:
                if ch == quote:
                    quote = None
            elif ch in "'\"":
                quote = ch
            elif ch == "/" or (ch == "&" and text[k:k + 4].lower() == "&end"):
                break
            k += 1
        yield m.group(1), text[j:k]
        i = k + 1


def parse_namelists(text: str) -> dict:
    """Fortran namelist groups -> {group: {NAME: value}} (names upper-cased)."""
    out = {}
    for name, body in _groups(text):
        items = {}
        for it in _ITEM.finditer(body):
            items[it.group(1).upper()] = _value(it.group(2))
        out[name.lower()] = items
    return out


def read_fortran_reals(line: str):
    return [float(t.lower().replace("d", "e")) for t in line.split()]


def read_bonds(path: str, noxxz: int):
    """list_xxz_term: NOxxz lines 'i j Jxy Jz' (input_param.f90:91-103)."""
    bonds = np.zeros((noxxz, 2), np.int32)
    jxy = np.zeros(noxxz)
    jz = np.zeros(noxxz)
    with open(path) as f:
        lines = [ln for ln in f if ln.strip()]
    if len(lines) < noxxz:
        raise ValueError(f"{path}: {len(lines)} bonds, NOxxz = {noxxz}")
    for b in range(noxxz):
        v = read_fortran_reals(lines[b])
        bonds[b] = (int(v[0]), int(v[1]))
        jxy[b], jz[b] = v[2], v[3]
    return bonds, jxy, jz


def read_positions(path: str, nos: int):
    """list_site_position: NOS lines 'x y z' (get_expectation_values.f90:30-35)."""
    with open(path) as f:
        rows = [read_fortran_reals(ln) for ln in f if ln.strip()]
    return np.array(rows[:nos], dtype=np.float64)


def read_pairs(path: str, nocf: int):
    """list_cf_ss: NOCF lines 'a b' (get_expectation_values.f90:23-28)."""
    with open(path) as f:
        rows = [ln.split() for ln in f if ln.strip()]
    return np.array([(int(a), int(b)) for a, b in rows[:nocf]], dtype=np.int32)


def write_bonds(path: str, bonds, jxy, jz):
    with open(path, "w") as f:
        for (i, j), a, b in zip(bonds, jxy, jz):
            f.write(f"{int(i):5d}{int(j):5d}{a:23.15E}{b:23.15E}\n")


def chain_bonds(L: int, J1=(1.0, 1.0), J2=None):
    """Periodic chain: bonds (s, s+1) with (Jxy, Jz) = J1 and (s, s+2) with J2."""
    bonds, jxy, jz = [], [], []
    for s in range(1, L + 1):
        bonds.append((s, s % L + 1)); jxy.append(J1[0]); jz.append(J1[1])
    if J2 is not None:
        for s in range(1, L + 1):
            bonds.append((s, (s + 1) % L + 1)); jxy.append(J2[0]); jz.append(J2[1])
    return np.array(bonds, np.int32), np.array(jxy), np.array(jz)


def chain_positions(L: int):
    return np.stack([np.arange(L, dtype=np.float64), np.zeros(L), np.zeros(L)], axis=1)


@dataclass
class QS3Input:
    params: dict
    static: dict
    dynamic: dict
    lancz: dict = field(default_factory=dict)
    trlan: dict = field(default_factory=dict)

    @property
    def Ls(self):
        p = self.params
        return int(p.get("LX", p["NOS"])), int(p.get("LY", 1)), int(p.get("LZ", 1))

    @property
    def K(self):
        p = self.params
        return int(p.get("KX", 0)), int(p.get("KY", 0)), int(p.get("KZ", 0))


def read_input(text: str) -> QS3Input:
    g = parse_namelists(text)
    if "input_parameters" not in g:
        raise ValueError("input.dat: missing &input_parameters")
    return QS3Input(g["input_parameters"], g.get("input_static", {}), g.get("input_dynamic", {}),
                    g.get("input_lancz", {}), g.get("input_trlan", {}))
