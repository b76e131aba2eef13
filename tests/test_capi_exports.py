"""CPU tests of the boundary: libqs3g.so loads and exports every entry point
that include/qs3g.h declares (no compute call: no GPU here)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    text = open(os.path.join(ROOT, "include", "qs3g.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|const char\*)\s+(qs3g_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    names = declared()
    for must in ("qs3g_create", "qs3g_build_sector", "qs3g_hv", "qs3g_trlan", "qs3g_dsf", "qs3g_cfrac",
                 "qs3g_connection_table", "qs3g_destroy"):
        assert must in names


def test_library_loads_and_exports_all_declared_symbols():
    from ed_gb300 import build as b
    lib = b.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT\s+(qs3g_\w+)", out))
    missing = [n for n in declared() if n not in exported]
    assert not missing, missing
    L = ctypes.CDLL(lib)
    for n in declared():
        assert getattr(L, n) is not None


def test_library_is_sm103a_only():
    from ed_gb300 import build as b
    assert any("compute_103a" in a for a in b.ARCH) and any("sm_103a" in a for a in b.ARCH)


def test_binding_covers_the_header():
    from ed_gb300 import capi
    assert sorted(capi.EXPORTS) == declared()


def test_binding_constants_match_the_header():
    """Status codes, vector locations and the QS3G_REAL flag have the header's values."""
    from ed_gb300 import capi
    text = open(os.path.join(ROOT, "include", "qs3g.h")).read()
    consts = {k: int(v) for k, v in re.findall(r"\b(QS3G_[A-Z_0-9]+)\s*=\s*(\d+)", text)}
    assert consts["QS3G_REAL"] == capi.REAL
    assert consts["QS3G_HOST"] == capi.HOST and consts["QS3G_DEVICE"] == capi.DEVICE
    for name in ("OK", "EINVAL", "ESTATE", "ERANGE", "ENOTSUP", "EBREAKDOWN", "ENOTCONV"):
        assert consts["QS3G_" + name] == getattr(capi, name), name
