"""g2p_convert_param on the GPU against the oracle's convertParam
(src/solnoutclass.hpp:1456-1610), on random matrices and on a real
extraction's Z, plus its error paths.

Tolerance: the GPU inverts by Gauss-Jordan with partial pivoting, the oracle
by LAPACK's LU, so results agree to rounding scaled by the matrices'
condition numbers: relative 1e-10 of each matrix's largest entry for the
well-conditioned random cases, 1e-8 for the extraction's Z."""
import numpy as np
import pytest

from oracle import network as onet

pytestmark = pytest.mark.gpu

KINDS = ("Z", "Y", "S")


def _gpu_convert(frm, to, p, zs):
    from gds2para_gb300 import _lib
    nf, n, _ = p.shape
    buf = np.ascontiguousarray(p, np.complex128).view(np.float64).ravel().copy()
    out = np.zeros_like(buf)
    zs = np.ascontiguousarray(zs, np.float64)
    _lib.check(_lib.load().g2p_convert_param(frm.encode(), to.encode(), n, nf, zs.ctypes.data, buf.ctypes.data,
                                             out.ctypes.data))
    return out.view(np.complex128).reshape(nf, n, n)


def _close(got, want, rtol):
    scale = np.abs(want).max(axis=(1, 2), keepdims=True)
    assert np.all(np.abs(got - want) <= rtol * scale), float((np.abs(got - want) / scale).max())


@pytest.mark.parametrize("nports,nfreq", [(1, 5), (2, 40), (3, 7), (8, 33), (17, 4), (32, 64), (33, 2), (64, 3)])
def test_convert_matches_oracle(nports, nfreq):
    rng = np.random.default_rng(nports * 1000 + nfreq)
    zs = rng.uniform(20.0, 80.0, nports)
    z = rng.standard_normal((nfreq, nports, nports)) + 1j * rng.standard_normal((nfreq, nports, nports))
    z += 4.0 * np.sqrt(nports) * np.eye(nports)
    start = {k: onet.convert_param("Z", k, z, zs) for k in KINDS}
    for a in KINDS:
        for b in KINDS:
            got = _gpu_convert(a, b, start[a], zs)
            _close(got, onet.convert_param(a, b, start[a], zs), 1e-10)


def test_convert_extraction_z_and_write(tmp_path):
    from gds2para_gb300 import api, layout as lay
    d = lay.build(lay.multistrip(nx=24, ny=20, nz=8, n_strips=3, freq_start=1e8, freq_end=1e10, nfreq=4))
    with api.FdtdMesh(d) as m:
        api.generateStiff(m)
        z, _ = api.paraGenerator(m, api.default_params())
    zs = np.full(d.num_ports, 50.0)
    freqs = d.freqs()
    para = api.Parasitics(zs)
    para.saveNetworkParam("Z", freqs, z.ravel())
    para.convertParam("S")
    want = onet.convert_param("Z", "S", z, zs)
    _close(para.getParamMatrix(), want, 1e-8)
    assert para.getParamType() == "S"
    assert api.dumpCITI(tmp_path / "x.citi", para, "strip")
    text = (tmp_path / "x.citi").read_text()
    assert text.startswith("CITIFILE A.01.01\n") and text.count("\nBEGIN\n") == d.num_ports ** 2


def test_convert_device_pointers_and_in_place():
    import torch
    rng = np.random.default_rng(11)
    n, nf = 5, 9
    zs = rng.uniform(30, 60, n)
    z = rng.standard_normal((nf, n, n)) + 1j * rng.standard_normal((nf, n, n)) + 6 * np.eye(n)
    from gds2para_gb300 import _lib
    L = _lib.load()
    dz = torch.from_numpy(z.view(np.float64).ravel().copy()).cuda()
    dzs = torch.from_numpy(zs).cuda()
    _lib.check(L.g2p_convert_param(b"Z", b"S", n, nf, dzs.data_ptr(), dz.data_ptr(), dz.data_ptr()))
    got = dz.cpu().numpy().view(np.complex128).reshape(nf, n, n)
    _close(got, onet.convert_param("Z", "S", z, zs), 1e-10)


def test_convert_errors():
    from gds2para_gb300 import _lib
    L = _lib.load()
    one = np.array([1.0, 0.0])
    zs = np.array([50.0])
    out = np.zeros(2)
    assert L.g2p_convert_param(b"Z", b"S", 65, 1, None, None, None) == 1
    assert L.g2p_convert_param(b"Q", b"S", 1, 1, zs.ctypes.data, one.ctypes.data, out.ctypes.data) == 1
    assert L.g2p_convert_param(b"Z", b"S", 1, 1, None, one.ctypes.data, out.ctypes.data) == 1
    bad = np.array([-5.0])
    assert L.g2p_convert_param(b"Z", b"S", 1, 1, bad.ctypes.data, one.ctypes.data, out.ctypes.data) == 1
    sing = np.zeros(8)                         # 2 x 2 zero matrix: Z -> Y has no inverse
    out4 = np.zeros(8)
    assert L.g2p_convert_param(b"Z", b"Y", 2, 1, None, sing.ctypes.data, out4.ctypes.data) == 1
    assert b"singular" in L.g2p_last_error()
    # the library stays usable after the errors
    assert L.g2p_convert_param(b"Z", b"Y", 1, 1, None, one.ctypes.data, out.ctypes.data) == 0
    assert out[0] == 1.0 and out[1] == 0.0


def test_ybus_from_y_parameters_inverts_on_the_gpu():
    from gds2para_gb300 import api
    rng = np.random.default_rng(5)
    n = 6
    y = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) + 5 * np.eye(n)
    para = api.Parasitics(np.full(n, 50.0))
    para.saveNetworkParam("Y", [1e9], y.ravel())
    # G = Re Y^-1 and C = -1 / (Im Y^-1 * 2 pi f0): compare Y^-1 entrywise,
    # relative to its largest entry (the inverse is Gauss-Jordan vs LAPACK LU)
    inv = np.linalg.inv(y)
    scale = np.abs(inv).max()
    w = 2.0 * np.pi * 1e9
    assert np.abs(para.matG - inv.real).max() <= 1e-12 * scale
    assert np.abs(-1 / (para.matC * w) - inv.imag).max() <= 1e-12 * scale


# ---- convertParam on the GPU against the reference's own convertParam
# (src/solnoutclass.hpp compiled with an Eigen stand-in whose inverse is
# Gauss-Jordan with partial pivoting: equal to rounding, not bit for bit)

def _network_ref():
    import json
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "network_ref.npz"))
    return z, json.loads(bytes(z["_meta"]).decode())


@pytest.mark.parametrize("name", ["one_port", "two_port", "three_port", "five_port_small", "eight_port"])
def test_gpu_convert_param_matches_reference_convert_param(name, g2p):
    Z, meta = _network_ref()
    M = meta["network"][name]
    pre = name + "_"
    base = {"Z": Z[pre + "z"], "Y": Z[pre + "Z_to_Y"], "S": Z[pre + "Z_to_S"]}
    for a in "ZYS":
        for b in "ZYS":
            if a == b:
                continue
            para = g2p.Parasitics(Z[pre + "zs"], M["names"], M["dirs"])
            para.saveNetworkParam(a, Z[pre + "freqs"], base[a].reshape(-1))
            para.convertParam(b)
            want = Z[pre + f"{a}_to_{b}"]
            err = np.abs(para.matParam - want).max() / np.abs(want).max()
            assert err < 1e-12, (a, b, err)


def test_gpu_terminate_port_kron_reduction(g2p):
    rng = np.random.default_rng(5)
    n, freqs = 4, np.array([1e8, 2e8, 5e8])
    z = rng.normal(size=(3, n, n)) + 1j * rng.normal(size=(3, n, n)) + 10 * np.eye(n)
    zl = 50.0 + 10.0j
    for k in range(n):
        para = g2p.Parasitics([50.0] * n, [f"p{i}" for i in range(n)], "IOBI")
        para.saveNetworkParam("Z", freqs, z.reshape(-1))
        para.terminatePortZ(k, [zl])
        keep = [i for i in range(n) if i != k]
        for f in range(3):
            load = complex(zl.real, zl.imag * freqs[f] / freqs[0])
            want = z[f][np.ix_(keep, keep)] - np.outer(z[f][keep, k], z[f][k, keep]) / (z[f][k, k] + load)
            np.testing.assert_allclose(para.matParam[f], want, rtol=1e-13, atol=1e-13)
        assert para.getNPort() == n - 1 and para.port_names == [f"p{i}" for i in keep]


def test_gpu_terminate_port_t_network_input_impedance(g2p):
    za, zb, zc, zl = 10 + 2j, 20 - 5j, 30 + 1j, 50.0 + 0j
    z = np.array([[[za + zc, zc], [zc, zb + zc]]])
    para = g2p.Parasitics([50.0, 50.0])
    para.saveNetworkParam("Z", [1e9], z.reshape(-1))
    para.terminatePortZ(1, [zl])
    assert abs(para.matParam[0, 0, 0] - (za + zc * (zb + zl) / (zc + zb + zl))) < 1e-12


def test_gpu_y_from_circuit(g2p):
    rng = np.random.default_rng(6)
    g, c = rng.normal(size=(3, 3)), rng.normal(size=(3, 3)) * 1e-12
    freqs = np.array([1e8, 1e9])
    para = g2p.Parasitics([50.0] * 3)
    para.freqs = freqs
    para.matG, para.matC = g, c
    para.computeYParamFromCircuit()
    assert para.param == "Y"
    for f in range(2):
        np.testing.assert_allclose(para.matParam[f], g + 2j * np.pi * freqs[f] * c, rtol=1e-15, atol=0)
