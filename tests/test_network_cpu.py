"""Network-parameter stage on the CPU: the oracle's convertParam restatement
pinned against closed-form results; the C-ABI Touchstone, CITIfile and Xyce
writers (host code, no GPU) against the oracle's text; the nodal matrices of
computeYBusFromParam bit-exact; the SPEF writer's elements against the
oracle's choices."""
import re

import numpy as np
import pytest

from oracle import network as onet

Z0 = 50.0


def test_oracle_one_port_reflection():
    # a load R on a Z0 line reflects (R - Z0) / (R + Z0)
    for r in (10.0, 50.0, 200.0):
        s = onet.convert_param("Z", "S", np.array([[[r + 0j]]]), [Z0])
        assert abs(s[0, 0, 0] - (r - Z0) / (r + Z0)) < 1e-15


def test_oracle_series_and_shunt_two_ports():
    # series impedance Zs between the ports: Y = y[[1, -1], [-1, 1]]
    zser = 30.0 + 40.0j
    y = 1.0 / zser
    s = onet.convert_param("Y", "S", np.array([[[y, -y], [-y, y]]]), [Z0, Z0])[0]
    np.testing.assert_allclose(s[0, 0], zser / (zser + 2 * Z0), rtol=1e-14)
    np.testing.assert_allclose(s[1, 0], 2 * Z0 / (zser + 2 * Z0), rtol=1e-14)
    # shunt impedance Zp to ground: Z = Zp[[1, 1], [1, 1]]
    zp = 25.0 - 10.0j
    s = onet.convert_param("Z", "S", np.array([[[zp, zp], [zp, zp]]]), [Z0, Z0])[0]
    np.testing.assert_allclose(s[0, 0], -Z0 / (2 * zp + Z0), rtol=1e-14)
    np.testing.assert_allclose(s[1, 0], 2 * zp / (2 * zp + Z0), rtol=1e-14)


def test_oracle_matched_and_unequal_references():
    zs = np.array([50.0, 75.0, 20.0])
    s = onet.convert_param("Z", "S", np.diag(zs).astype(complex)[None], zs)
    assert np.abs(s).max() < 1e-15
    # power waves with real references: S = F (Z - R)(Z + R)^-1 F^-1, F = diag(1 / (2 sqrt(R)))
    rng = np.random.default_rng(3)
    z = rng.standard_normal((3, 3)) + 1j * rng.standard_normal((3, 3)) + np.diag(zs)
    f = np.diag(1.0 / (2 * np.sqrt(zs)))
    r = np.diag(zs)
    want = f @ (z - r) @ np.linalg.inv(z + r) @ np.linalg.inv(f)
    np.testing.assert_allclose(onet.convert_param("Z", "S", z[None], zs)[0], want, rtol=1e-12, atol=1e-14)


def test_oracle_round_trips():
    rng = np.random.default_rng(7)
    zs = rng.uniform(20, 80, 4)
    z = rng.standard_normal((5, 4, 4)) + 1j * rng.standard_normal((5, 4, 4)) + 60 * np.eye(4)
    for a, b in (("Z", "Y"), ("Z", "S"), ("Y", "S"), ("S", "Z"), ("S", "Y")):
        start = onet.convert_param("Z", a, z, zs)
        back = onet.convert_param(b, a, onet.convert_param(a, b, start, zs), zs)
        np.testing.assert_allclose(back, start, rtol=1e-11, atol=1e-13)


def _lib_or_skip():
    from gds2para_gb300 import _lib, build
    try:
        build.build()
    except Exception as e:  # pragma: no cover - nvcc missing
        pytest.skip(f"library not buildable here: {e}")
    return _lib.load()


STAMP_TS = re.compile(r"^! Date/Time .*$", re.M)
STAMP_CITI = re.compile(r"^CONSTANT TIME .*$", re.M)


@pytest.mark.parametrize("nports,nfreq", [(1, 3), (2, 4), (3, 2), (5, 3), (12, 2)])
def test_writers_match_oracle_text(tmp_path, nports, nfreq):
    from gds2para_gb300 import api
    _lib_or_skip()
    rng = np.random.default_rng(nports * 100 + nfreq)
    zs = rng.choice([50.0, 75.0, 25.5], nports)
    freqs = np.geomspace(1e6, 3.2e10, nfreq)
    p = (rng.standard_normal((nfreq, nports, nports)) + 1j * rng.standard_normal((nfreq, nports, nports)))
    p *= 10.0 ** rng.integers(-12, 4, p.shape)
    p[0, 0, 0] = -0.0 + 0j
    para = api.Parasitics(zs)
    para.saveNetworkParam("Z", freqs, p.ravel())
    ts, ct = tmp_path / "a.sNp", tmp_path / "a.citi"
    assert api.dumpTouchstone(ts, para, "strip_Design")
    assert api.dumpCITI(ct, para, "strip_Design")
    got_ts, got_ct = ts.read_text(), ct.read_text()
    assert STAMP_TS.search(got_ts) and STAMP_CITI.search(got_ct)
    want_ts = onet.touchstone_text("Z", freqs, zs, p, "strip_Design", "T")
    want_ct = onet.citi_text("Z", freqs, p, "strip_Design", "T")
    assert STAMP_TS.sub("! Date/Time T", got_ts) == want_ts
    assert STAMP_CITI.sub("CONSTANT TIME T", got_ct) == want_ct


def test_writer_reports_unopenable_path(tmp_path):
    from gds2para_gb300 import api
    _lib_or_skip()
    para = api.Parasitics([50.0])
    para.saveNetworkParam("Z", [1e9], np.array([1 + 1j]))
    assert api.dumpTouchstone(tmp_path / "missing_dir" / "x.s1p", para) is False
    assert api.dumpCITI(tmp_path / "missing_dir" / "x.citi", para) is False


def test_writer_rejects_bad_arguments():
    L = _lib_or_skip()
    assert L.g2p_write_touchstone(b"/dev/null", b"Z", 0, 1, None, None, None, b"") == 1
    assert L.g2p_write_citi(None, b"Z", 1, 1, None, None, b"") == 1


def _nodal_case(n, seed, sym=True):
    rng = np.random.default_rng(seed)
    # a capacitive Z at 1 GHz: Im Z < 0 on and near the diagonal
    z = rng.uniform(0.1, 5.0, (n, n)) - 1j * rng.uniform(50.0, 500.0, (n, n))
    if sym:
        z = (z + z.T) / 2
    return z


@pytest.mark.parametrize("n,sym", [(1, True), (2, True), (4, False), (9, True)])
def test_ybus_and_xyce_match_oracle(tmp_path, n, sym):
    from gds2para_gb300 import api
    _lib_or_skip()
    z = _nodal_case(n, 40 + n, sym)
    f0 = 1.3e9
    para = api.Parasitics(np.full(n, 50.0), [f"net_{i}" for i in range(n)])
    para.saveNetworkParam("Z", [f0], z.ravel())
    g_ref, c_ref = onet.ybus_from_param("Z", z, f0)
    assert np.array_equal(para.matG, g_ref) and np.array_equal(para.matC, c_ref)     # same IEEE operations
    path = tmp_path / "x.cir"
    for thresh in (api.WRITE_THRESH, 0.05):
        assert api.dumpXyce(path, para, "dsgn", thresh)
        got = re.sub(r"^\* Date: .*$", "* Date: T", path.read_text(), flags=re.M)
        want = onet.xyce_text(str(path), "dsgn", para.port_names, f0, g_ref, c_ref, thresh, "T")
        assert got == want


def test_xyce_writes_inductors_for_negative_capacitance(tmp_path):
    from gds2para_gb300 import api
    _lib_or_skip()
    z = np.array([[1.0 + 80.0j, 0.5 - 200.0j], [0.5 - 200.0j, 2.0 - 90.0j]])
    para = api.Parasitics([50.0, 50.0])
    para.saveNetworkParam("Z", [1e9], z.ravel())
    assert api.dumpXyce(tmp_path / "x.cir", para, "d")
    text = (tmp_path / "x.cir").read_text()
    assert re.search(r"^L1 port1 0 ", text, re.M) and text.rstrip().endswith(".ends")
    want = onet.xyce_text(str(tmp_path / "x.cir"), "d", para.port_names, 1e9, para.matG, para.matC,
                          api.WRITE_THRESH, "T")
    assert re.sub(r"^\* Date: .*$", "* Date: T", text, flags=re.M) == want


def _parse_spef(text):
    sec, caps, ress, hdr = None, [], [], {}
    node = lambda t: int(t[1:])
    for line in text.splitlines():
        if line.startswith("*CAP"):
            sec = caps
            continue
        if line.startswith("*RES"):
            sec = ress
            continue
        if line.startswith("*END"):
            sec = None
            continue
        if line.startswith("*D_NET"):
            hdr["lcap"] = float(line.split()[2])
        if sec is not None and line.strip():
            t = line.split()
            a = node(t[1])
            b, v = (node(t[2]), float(t[3])) if len(t) == 4 else (0, float(t[2]))
            sec.append((a, b, v))
    return caps, ress, hdr


def test_spef_elements_match_oracle(tmp_path):
    from gds2para_gb300 import api
    _lib_or_skip()
    z = _nodal_case(5, 77, sym=False)
    para = api.Parasitics(np.full(5, 50.0), [f"p{i}" for i in range(5)], "IOBBI")
    para.saveNetworkParam("Z", [2e9], z.ravel())
    assert api.dumpSPEF(tmp_path / "x.spef", para, "dsgn")
    text = (tmp_path / "x.spef").read_text()
    assert text.startswith('*SPEF "IEEE 1481-1998"\n*DESIGN "dsgn"\n')
    assert "*1 p0\n" in text and "*P p1 O\n" in text and "*P p0 I\n" in text
    caps, ress, hdr = _parse_spef(text)
    want_c, want_r, ct = onet.spef_elements(para.matG, para.matC, api.WRITE_THRESH)
    assert [(a, b) for a, b, _ in caps] == [(a, b) for a, b, _ in want_c]
    assert [(a, b) for a, b, _ in ress] == [(a, b) for a, b, _ in want_r]
    np.testing.assert_allclose([v for *_, v in caps], [v for *_, v in want_c], rtol=1e-5)
    np.testing.assert_allclose([v for *_, v in ress], [v for *_, v in want_r], rtol=1e-5)
    assert abs(hdr["lcap"] - ct) <= 1e-5 * abs(ct)


def test_nodal_writers_reject_s_parameters_and_bad_arguments(tmp_path):
    from gds2para_gb300 import api
    L = _lib_or_skip()
    para = api.Parasitics([50.0])
    para.saveNetworkParam("S", [1e9], np.array([0.2 + 0.1j]))
    assert para.matG is None
    with pytest.raises(ValueError):
        api.dumpXyce(tmp_path / "x.cir", para, "d")
    assert L.g2p_write_xyce(b"/dev/null", b"d", 1, None, 1e9, None, None, 1e-5) == 1
