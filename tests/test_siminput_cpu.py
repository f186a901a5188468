"""The .sim_input reader (g2p_sim_input_read, host code) and the host half
of the GDSII flow, no GPU needed.

The reference's reader (SolverDataBase::readSimInput) cannot be compiled
here (it needs Eigen), so the library's reader is checked against an
independent parse written below from the file format's rules, on synthetic
files covering each form, and on the reference's own example files when the
reference checkout is present.  The grid that the library builds from the
fixtures' polygons and settings must equal the reference meshAndMark's
(tests/golden/example_marks.npz)."""
import json
import os
import re

import numpy as np
import pytest

from gds2para_gb300 import api, _lib

HERE = os.path.dirname(os.path.abspath(__file__))
EXAMPLES_DIR = os.path.join(os.environ.get("G2P_REFERENCE_ROOT", os.path.join(os.path.dirname(os.path.dirname(HERE)),
                                                                              "reference")), "examples")


def independent_parse(text):
    """The format's rules, restated without the library: sections, '#'
    comment lines, "key = value", stack names -> GDSII numbers, port lines
    by their count of spaces, sides grouped by name (unnamed: "port1")."""
    lines = text.split("\n")
    complete = lines[:-1]                # a last line without newline is not read
    out = {"ports": {}}
    i = 0

    def nxt(j):
        j += 1
        while j < len(complete) and complete[j].startswith("#"):
            j += 1
        return j

    num = lambda s: float(re.match(r"\s*([-+]?[\d.]+(?:[eE][-+]?\d+)?)", s).group(1))
    while i < len(complete):
        line = complete[i]
        if line.startswith("TOTAL SIZE"):
            i = nxt(i)
            lim = [float(v) for v in complete[i].split("#")[0].split()[:6]]
            i = nxt(i)
            lu = num(complete[i].split("lengthUnit = ")[1])
            out["lim"] = [v * lu for v in lim]
            out["lu"] = lu
        elif line.startswith("FREQUENCY"):
            vals = []
            for key in ("freqUnit = ", "freqStart = ", "freqEnd = ", "nfreq = ", "freqScale = "):
                i = nxt(i)
                vals.append(num(complete[i].split(key)[1]))
            out["freq"] = vals
        elif line.startswith("DIELECTRIC STACK"):
            i = nxt(i)
            n = int(num(re.split(r"num(?:Stack|Layer) = ", complete[i])[1]))
            i = nxt(i)
            layers = []
            for _ in range(n):
                t = complete[i]
                name = t.split(" ")[0]
                digits = name[name.index("M") + 1:] if "M" in name else name
                g = int(digits) if digits.isdigit() else -1
                if "z = " in t:
                    z = num(t.split("z = ")[1]) * out["lu"]
                else:
                    z = layers[-1][0] + layers[-1][1] if layers else 0.0
                h = num(t.split("h = ")[1]) * out["lu"]
                e = num(t.split("e = ")[1])
                s = num(t.split("sigma = ")[1]) if "sigma = " in t else 0.0
                layers.append((z, h, e, s, g))
                i = nxt(i)
            out["layers"] = layers
            i -= 1
        elif line.startswith("PORT") and not out["ports"]:
            i = nxt(nxt(i))
            while i < len(complete) and len(complete[i]) >= 3:
                t = complete[i].split(" #")[0]
                tok = complete[i].split("#")[0].split()
                nsp = t.count(" ")
                u = out["lu"]
                if nsp == 4:
                    lay = [L for L in out["layers"] if L[4] == int(tok[4])][0]
                    c, name = [float(tok[0]) * u, float(tok[1]) * u, lay[0], float(tok[2]) * u, float(tok[3]) * u,
                               lay[0] + lay[1]], "port1"
                elif nsp == 6:
                    c, name = [float(v) * u for v in tok[:6]], "port1"
                else:
                    c, name = [float(v) * u for v in tok[1:7]], tok[0]
                out["ports"].setdefault(name, []).append(c)
                i = nxt(i)
            i -= 1
        i = nxt(i) if i + 1 < len(complete) and complete[i + 1].startswith("#") else i + 1
    return out


SYNTH = """TOTAL SIZE
0 300 -5 100 -0.3 +2.9
lengthUnit = 1.e-6

FREQUENCY
freqUnit = 1.0e+9
# a comment inside the section
freqStart = 1
freqEnd = 20
nfreq = 1
freqScale = 0

DIELECTRIC STACK
numLayer = 6
0         z = -0.3 h = 0.3 e = 4.1 sigma = 58000000 # ground
Sub z = 0.0 h = 0.000 e = 4.1 sigma = 5.e+7
ILDM1     z = +0.120 h = 0.285 e = 4.1 TanD = 0 sigma = 58000000
ILD1      h = 0.615 e = 3.9 TanD = 0
M2 z = 1.020 h = 0.120 e = 8.0 sigma = 5.8e7
7 z = 1.5 h = 1.4 e = 0.5

PORT
numPort = 3
near +155 +0.000 +0.12 +155 +0.000 0.00 +1 # first side
far +155 +100 +0.12 +155 +100 0.00 +1
near +155 +0.000 +0.405 +155 +0.000 +1.020 +1
10 20 0.12 10 20 0 -1
30 40 50 60 2
"""


def _read(tmp_path, text):
    p = tmp_path / "t.sim_input"
    p.write_text(text)
    return api.readSimInput(p)


def test_sim_input_forms_against_independent_parse(tmp_path):
    r = _read(tmp_path, SYNTH)
    ref = independent_parse(SYNTH)
    np.testing.assert_array_equal(r["lim"], ref["lim"])
    assert r["length_unit"] == ref["lu"]
    fu, fs, fe, nf, sc = ref["freq"]
    assert (r["freq_unit"], r["freq_start"], r["nfreq"], r["freq_scale"]) == (fu, fs, nf, sc)
    assert r["freq_end"] == fs                 # one point: the list holds freqStart only
    valid = [L for L in ref["layers"] if L[1] > 0 and L[2] >= 1 and L[3] >= 0]
    np.testing.assert_array_equal(r["layers"], [[L[0], L[0] + L[1], L[2], L[3]] for L in valid])
    np.testing.assert_array_equal(r["layer_gdsii"], [L[4] for L in valid])
    assert list(r["layer_gdsii"]) == [0, 1, -1, 2]
    # "ILD1" has no z: it continues from the layer below
    assert r["layers"][2][0] == ref["layers"][2][0] + ref["layers"][2][1]
    names = list(ref["ports"])
    assert names == ["near", "far", "port1"]
    sides = [c for nm in names for c in ref["ports"][nm]]
    np.testing.assert_array_equal(r["side_coords"], sides)
    np.testing.assert_array_equal(r["port_side_ptr"], [0, 2, 3, 5])
    want_dir = [1 if (c[0] > c[3] or c[1] > c[4] or c[2] > c[5]) else -1 for c in sides]
    np.testing.assert_array_equal(r["side_dir"], want_dir)
    # the 4-space form takes its z range from the layer with that GDSII number
    assert r["side_coords"][4][2] == ref["layers"][4][0]


def test_sim_input_last_line_without_newline_is_not_read(tmp_path):
    text = SYNTH.rstrip("\n")
    r = _read(tmp_path, text)
    assert len(r["side_coords"]) == 4            # the last port line is dropped, as the reference drops it


def test_sim_input_errors(tmp_path):
    with pytest.raises(_lib.G2PError):
        api.readSimInput(tmp_path / "missing.sim_input")
    with pytest.raises(_lib.G2PError):          # board outline file in place of the limits
        _read(tmp_path, "TOTAL SIZE\nboard.pcb 0.0 1.0\nlengthUnit = 1\n\n")
    with pytest.raises(_lib.G2PError):
        _read(tmp_path, "FREQUENCY\nfreqUnit = 1\nfreqStart = 1\nfreqEnd = 2\nnfreq = 0\nfreqScale = 1\n\n")


def _fixture():
    z = np.load(os.path.join(HERE, "golden", "example_marks.npz"))
    return z, json.loads(bytes(z["_meta"]).decode())


def test_example_grids_from_fixture_match_reference_mesher():
    z, meta = _fixture()
    for name in meta["examples"]:
        A = {k[len(name) + 1:]: z[k] for k in z.files if k.startswith(name + "_")}
        polys = (A["poly_layer"], A["poly_vptr"], A["poly_x"], A["poly_y"])
        grid = api.meshGrid(A["sim_lim"], polys, A["sim_side_coords"], A["sim_layers"])
        for got, key in zip(grid, ("xn", "yn", "zn", "stack_epsn", "stack_sign")):
            np.testing.assert_array_equal(got, A["ref_" + key], err_msg=f"{name} {key}")


@pytest.mark.skipif(not os.path.isdir(EXAMPLES_DIR), reason="the reference's example designs are not here")
def test_reader_on_the_reference_examples():
    z, meta = _fixture()
    for fn in sorted(os.listdir(EXAMPLES_DIR)):
        if not fn.endswith(".sim_input"):
            continue
        path = os.path.join(EXAMPLES_DIR, fn)
        try:
            r = api.readSimInput(path)
        except _lib.G2PError as e:
            assert "outline" in str(e)
            continue
        ref = independent_parse(open(path).read())
        np.testing.assert_array_equal(r["lim"], ref["lim"], err_msg=fn)
        sides = [c for nm in ref["ports"] for c in ref["ports"][nm]]
        np.testing.assert_array_equal(r["side_coords"], np.array(sides).reshape(-1, 6), err_msg=fn)
        name = fn[:-len(".sim_input")]
        if name in meta["examples"]:
            np.testing.assert_array_equal(r["side_coords"], z[name + "_sim_side_coords"])
            np.testing.assert_array_equal(r["layers"], z[name + "_sim_layers"])
            gds = os.path.join(EXAMPLES_DIR, name + ".gds")
            for got, key in zip(api.readGDSII(gds), ("layer", "vptr", "x", "y")):
                np.testing.assert_array_equal(got, z[f"{name}_poly_{key}"])
