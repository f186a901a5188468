"""The output stage and the .sim_input reader against the reference's own
code (tests/golden/network_ref.npz, made by
tests/golden/make_network_golden.py from src/solnoutclass.hpp compiled with
stand-ins for Eigen and Parser-SPEF), no GPU needed:

* computeYBusFromParam's G and C bit for bit;
* dumpTouchstone, dumpCITI and dumpXyce byte for byte, apart from the date
  and file-name lines (the reference formats an uninitialised time_t);
* toSPEF's element choices (name map, ports and directions, the net's
  connections, capacitances and resistances) from the library's SPEF file,
  whose rendering is the library's own (Parser-SPEF is absent);
* readSimInput + convertToFDTDMesh field for field, bit for bit.

The conversions themselves (convertParam, on the GPU) are checked in
tests/test_gpu_network.py against the same fixture."""
import json
import os
import re

import numpy as np
import pytest

from gds2para_gb300 import api

HERE = os.path.dirname(os.path.abspath(__file__))
EXAMPLES_DIR = os.path.join(os.environ.get("G2P_REFERENCE_ROOT", os.path.join(os.path.dirname(os.path.dirname(HERE)),
                                                                              "reference")), "examples")


def _fixture():
    z = np.load(os.path.join(HERE, "golden", "network_ref.npz"))
    return z, json.loads(bytes(z["_meta"]).decode())


Z, META = _fixture()
CASES = list(META["network"])


def _para(name, matrix=None, kind="Z"):
    M = META["network"][name]
    pre = name + "_"
    para = api.Parasitics(Z[pre + "zs"], M["names"], M["dirs"])
    para.saveNetworkParam(kind, Z[pre + "freqs"], (Z[pre + "z"] if matrix is None else matrix).reshape(-1))
    return para


def _text(name, fn):
    return bytes(Z[name + "_file_" + fn.replace(".", "_")]).decode()


VOLATILE = re.compile(r"^(! Date/Time|\* Date:|\* File:|CONSTANT TIME )")


def _same_but_dates(ref, got):
    a, b = ref.splitlines(), got.splitlines()
    assert len(a) == len(b), f"{len(a)} lines against {len(b)}"
    for x, y in zip(a, b):
        if x != y:
            assert VOLATILE.match(x) and VOLATILE.match(y), f"\n ref: {x!r}\n got: {y!r}"


@pytest.mark.parametrize("name", CASES)
def test_nodal_matrices_bit_exact(name):
    para = _para(name)
    np.testing.assert_array_equal(para.matG, Z[name + "_G"])
    np.testing.assert_array_equal(para.matC, Z[name + "_C"])


@pytest.mark.parametrize("name", CASES)
def test_touchstone_citi_xyce_match_reference_text(name, tmp_path):
    M = META["network"][name]
    para = _para(name)
    assert api.dumpTouchstone(tmp_path / "z.ts", para, M["design"])
    _same_but_dates(_text(name, "z.ts"), (tmp_path / "z.ts").read_text())
    assert api.dumpXyce(tmp_path / "z.cir", para, M["design"])
    _same_but_dates(_text(name, "z.cir"), (tmp_path / "z.cir").read_text())
    # the S data as the reference's convertParam left it
    s = _para(name, Z[name + "_Z_to_S"], "S")
    assert api.dumpCITI(tmp_path / "s.citi", s, M["design"])
    _same_but_dates(_text(name, "s.citi"), (tmp_path / "s.citi").read_text())
    assert api.dumpTouchstone(tmp_path / "s.ts", s, M["design"])
    _same_but_dates(_text(name, "s.ts"), (tmp_path / "s.ts").read_text())


def _ref_spef(text):
    out = {"names": {}, "ports": [], "conn": [], "cap": [], "res": []}
    for line in text.splitlines():
        t = line.split()
        if t[0] == "name":
            out["names"][t[1]] = t[2]
        elif t[0] == "port":
            out["ports"].append((t[1], "IOB"[int(t[2])]))
        elif t[0] == "net":
            out["lcap"] = float(t[2])
        elif t[0] == "conn":
            out["conn"].append((t[1], "IOB"[int(t[3])]))
        elif t[0] in ("cap", "res"):
            out[t[0]].append((t[1], None if t[2] == "-" else t[2], float(t[3])))
    return out


def _lib_spef(text):
    out = {"names": {}, "ports": [], "conn": [], "cap": [], "res": []}
    sec = None
    for line in text.splitlines():
        t = line.split()
        if not t:
            continue
        if t[0].startswith("*") and not t[0][1:].isdigit():
            sec = t[0]
            if sec == "*D_NET":
                out["lcap"] = float(t[2])
            if sec == "*P":
                out["conn"].append((t[1], t[2]))
            continue
        if sec == "*NAME_MAP":
            out["names"][t[0][1:]] = t[1]
        elif sec == "*PORTS":
            out["ports"].append((t[0], t[1]))
        elif sec in ("*CAP", "*RES"):
            key = "cap" if sec == "*CAP" else "res"
            out[key].append((t[1], t[2] if len(t) == 4 else None, float(t[-1])))
    return out


@pytest.mark.parametrize("name", CASES)
def test_spef_elements_match_reference_choices(name, tmp_path):
    M = META["network"][name]
    para = _para(name)
    assert api.dumpSPEF(tmp_path / "z.spef", para, M["design"])
    ref = _ref_spef(_text(name, "z.spef"))
    got = _lib_spef((tmp_path / "z.spef").read_text())
    assert got["names"] == ref["names"]
    dmap = {"I": "I", "O": "O", "B": "B"}
    assert [(p, dmap[d]) for p, d in got["ports"]] == ref["ports"]
    assert got["conn"] == ref["conn"]
    assert abs(got["lcap"] - ref["lcap"]) <= 1e-5 * abs(ref["lcap"])
    for key in ("cap", "res"):
        assert [(a, b) for a, b, _ in got[key]] == [(a, b) for a, b, _ in ref[key]], key
        for (_, _, x), (_, _, y) in zip(got[key], ref[key]):
            assert abs(x - y) <= 1e-5 * abs(y), (key, x, y)          # SPEF prints 6 significant digits


def _ref_simin(text):
    out = {"layers": [], "gds": [], "sides": [], "side_port": [], "dirs": []}
    for line in text.splitlines():
        t = line.split()
        if t[0] == "lim":
            out["lim"] = [float(v) for v in t[1:]]
        elif t[0] == "units":
            out["units"] = [float(v) for v in t[1:]]
        elif t[0] == "freq":
            out["freq"] = [int(v) for v in t[1:]]
        elif t[0] == "layer":
            out["layers"].append([float(v) for v in t[1:5]])
            out["gds"].append(int(t[5]))
        elif t[0] == "side":
            out["side_port"].append(int(t[1]))
            out["sides"].append([float(v) for v in t[2:8]])
            out["dirs"].append(int(t[8]))
    return out


def _check_simin(lib, ref):
    R = _ref_simin(ref)
    np.testing.assert_array_equal(lib["lim"], R["lim"])
    assert [lib["length_unit"], lib["freq_unit"], lib["freq_start"], lib["freq_end"]] == R["units"]
    assert [lib["nfreq"], lib["freq_scale"]] == R["freq"]
    np.testing.assert_array_equal(lib["layers"], np.array(R["layers"]).reshape(-1, 4))
    assert list(lib["layer_gdsii"]) == R["gds"]
    np.testing.assert_array_equal(lib["side_coords"], np.array(R["sides"]).reshape(-1, 6))
    assert list(lib["side_dir"]) == R["dirs"]
    port_of_side = np.searchsorted(lib["port_side_ptr"], np.arange(len(R["side_port"])), side="right") - 1
    assert list(port_of_side) == R["side_port"]


@pytest.mark.parametrize("name", [k for k in META["simin"] if not k.startswith("example_")])
def test_sim_input_reader_matches_reference_reader(name, tmp_path):
    S = META["simin"][name]
    p = tmp_path / "t.sim_input"
    p.write_text(S["text"])
    _check_simin(api.readSimInput(p), S["ref"])


@pytest.mark.skipif(not os.path.isdir(EXAMPLES_DIR), reason="the reference's example files are not here")
def test_sim_input_reader_matches_reference_reader_on_examples():
    names = [k for k in META["simin"] if k.startswith("example_")]
    assert names
    for k in names:
        S = META["simin"][k]
        _check_simin(api.readSimInput(os.path.join(EXAMPLES_DIR, S["file"])), S["ref"])
