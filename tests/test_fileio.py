"""CPU tests of the result-file formats (host-only entry points of libqs3g.so).

wf<i>.bin is a Fortran unformatted sequential record (4-byte markers);
energy.dat is (2ES24.15); alpha_beta_values_*.d is (3I6, 8e23.15).  The
expected strings follow the Fortran edit-descriptor rules: ESw.d prints one
nonzero digit before the point, Ew.d prints 0.d1...dd, and the exponent field
is E+dd up to |exp| = 99 and +ddd (no letter) up to 999.
"""
import struct

import numpy as np
import pytest

from ed_gb300 import capi
from oracle import oracle as O


def test_wf_record_layout_and_roundtrip(tmp_path):
    rng = np.random.default_rng(0)
    psi = rng.standard_normal(37) + 1j * rng.standard_normal(37)
    p = tmp_path / "wf0.bin"
    capi.write_wf(p, psi)
    raw = p.read_bytes()
    n = 16 * psi.size
    assert len(raw) == n + 8
    assert struct.unpack("<i", raw[:4])[0] == n
    assert struct.unpack("<i", raw[-4:])[0] == n
    assert raw[4:-4] == psi.astype("<c16").tobytes()
    np.testing.assert_array_equal(capi.read_wf(p, psi.size), psi)
    # read(10) psi(1:dim) takes a prefix of a longer record
    np.testing.assert_array_equal(capi.read_wf(p, 10), psi[:10])
    with pytest.raises(capi.QS3GError):
        capi.read_wf(p, psi.size + 1)


def test_wf_reads_subrecords(tmp_path):
    """A record split into subrecords (negated leading markers while more
    follow, negated trailing markers after the first) reads as one record."""
    rng = np.random.default_rng(1)
    psi = rng.standard_normal(20) + 1j * rng.standard_normal(20)
    data = psi.astype("<c16").tobytes()
    cuts = [0, 100, 230, len(data)]  # subrecord boundaries need not align with values
    out = b""
    for j in range(3):
        seg = data[cuts[j]:cuts[j + 1]]
        lead = -len(seg) if j < 2 else len(seg)
        trail = -len(seg) if j > 0 else len(seg)
        out += struct.pack("<i", lead) + seg + struct.pack("<i", trail)
    p = tmp_path / "wf1.bin"
    p.write_bytes(out)
    np.testing.assert_array_equal(capi.read_wf(p, psi.size), psi)


def test_wf_empty_and_bad_markers(tmp_path):
    p = tmp_path / "wf2.bin"
    capi.write_wf(p, np.zeros(0, np.complex128))
    assert p.read_bytes() == struct.pack("<ii", 0, 0)
    p.write_bytes(struct.pack("<i", 16) + bytes(16) + struct.pack("<i", 32))
    with pytest.raises(capi.QS3GError, match="markers"):
        capi.read_wf(p, 1)


@pytest.mark.parametrize("x,w,d,kind,expect", [
    (1.0, 24, 15, "ES", "   1.000000000000000E+00"),
    (-0.4375, 24, 15, "ES", "  -4.375000000000000E-01"),
    (12.0, 24, 15, "ES", "   1.200000000000000E+01"),
    (0.0, 24, 15, "ES", "   0.000000000000000E+00"),
    (1.0e300, 23, 15, "E", "  0.100000000000000+301"),
    (0.0, 23, 15, "E", "  0.000000000000000E+00"),
    (12345.678, 23, 15, "E", "  0.123456780000000E+05"),
    (-1.0e-100, 23, 15, "E", " -0.100000000000000E-99"),
    (-1.0e-101, 23, 15, "E", " -0.100000000000000-100"),
    (-2.5, 23, 15, "E", " -0.250000000000000E+01"),
    (0.9999999999999999, 23, 15, "E", "  0.100000000000000E+01"),
    (1.0e300, 10, 3, "E", " 0.100+301"),
    (-1.0e300, 9, 3, "E", "-.100+301"),
])
def test_fortran_edit_descriptors(x, w, d, kind, expect):
    assert capi.format_real(x, w, d, kind) == expect


def test_energy_dat(tmp_path):
    ene = np.array([-5.123456789012345, -4.5, 0.125])
    p = tmp_path / "energy.dat"
    capi.write_energy(p, ene)
    lines = p.read_text().splitlines()
    assert lines[0] == "   1.000000000000000E+00  -5.123456789012345E+00"
    assert lines[1] == "   2.000000000000000E+00  -4.500000000000000E+00"
    assert lines[2] == "   3.000000000000000E+00   1.250000000000000E-01"
    np.testing.assert_allclose(capi.read_energy(p, 3), ene, rtol=1e-15)
    with pytest.raises(capi.QS3GError):
        capi.read_energy(p, 4)


def test_alpha_beta_file_and_dsflan_read(tmp_path):
    alpha = np.array([1.25, -0.5, 2.0, 1.0e300])
    beta2 = np.array([0.0, 0.75, 1.5, 0.0])
    p = tmp_path / "alpha_beta_values_E0-tmp.d"
    capi.write_alpha_beta(p, alpha[:2], beta2[:2], 0.875, -3.25, 1.0, append=False)
    capi.write_alpha_beta(p, alpha, beta2, 0.875, -3.25, 1.0, append=True)
    lines = p.read_text().splitlines()
    assert len(lines) == 6
    assert lines[0] == ("     1     1     1  0.125000000000000E+01  0.000000000000000E+00"
                        "  0.875000000000000E+00 -0.325000000000000E+01  0.100000000000000E+01")
    assert lines[5].startswith("     1     4     1  0.100000000000000+301")
    a, b2, n1, e0, sz = capi.read_alpha_beta(p)
    assert len(a) == 6
    np.testing.assert_array_equal(a[2:], alpha)
    np.testing.assert_array_equal(b2[2:], beta2)
    assert (n1, e0, sz) == (0.875, -3.25, 1.0)
    with pytest.raises(capi.QS3GError):
        capi.read_alpha_beta(p, cap=3)


def test_alpha_beta_roundtrip_feeds_cfrac(tmp_path):
    """Values written at 15 digits and read back give the same spectrum to 1e-12."""
    rng = np.random.default_rng(2)
    n = 30
    alpha = rng.uniform(-1, 3, n)
    beta2 = rng.uniform(0.1, 2, n)
    beta2[0] = 0.0
    p = tmp_path / "ab.d"
    capi.write_alpha_beta(p, alpha, beta2, 0.7, -2.0, 0.0, append=False)
    a, b2, n1, e0, _ = capi.read_alpha_beta(p)
    om = np.linspace(0, 5, 500)
    s0 = O.cfrac(alpha, beta2, 0.7, -2.0, 0.04, om)
    s1 = O.cfrac(a, b2, n1, e0, 0.04, om)
    np.testing.assert_allclose(s1, s0, rtol=1e-11, atol=1e-14)
