"""meshAndMark's conductor marking and numbering and portSet on the GPU
(g2p_mesh_mark) against what the reference's own src/mesh.cpp produced for
the golden layouts, and against the host generator at the c2 bench size."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, check_golden_array, load_golden

pytestmark = pytest.mark.gpu

KEYS = ("mark_node", "mark_edge", "mark_port", "cdt_return", "side_edges", "side_area", "side_dir")


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_gpu_marking_and_ports_match_reference(name, g2p):
    from gds2para_gb300 import layout as lay
    arrays, meta = load_golden(name)
    out = g2p.meshAndMark(getattr(lay, meta["generator"])(**meta["kwargs"]))
    assert out["num_cdt"] == meta["numCdt"]
    for key in KEYS:
        check_golden_array(arrays, meta, key, out[key])


@pytest.mark.parametrize("config", ["c2", "c3"])
def test_gpu_marking_matches_host_generator_at_full_size(config, g2p):
    from gds2para_gb300 import layout as lay
    L = lay.config(config)
    d = lay.build(L)
    out = g2p.meshAndMark(L)
    assert out["num_cdt"] == d.num_cdt
    for key in KEYS:
        np.testing.assert_array_equal(out[key], getattr(d, key))
    np.testing.assert_array_equal(out["side_edge_ptr"], d.side_edge_ptr)


def test_gpu_marking_rejects_a_box_outside_the_grid(g2p):
    from gds2para_gb300 import layout as lay, _lib
    L = lay.microstrip(nx=13, ny=9, nz=6)
    L.boxes.append(lay.Box(0, 20, 0, 1, 0, 1))
    with pytest.raises(_lib.G2PError):
        g2p.meshAndMark(L)


# ---- the reference's example designs: GDSII polygons and .sim_input
# settings through the library's grid, polygon marking (findInsideCond),
# conductor numbering, findPortNode and portSet, against the reference's own
# meshAndMark + portSet (tests/golden/example_marks.npz, made by
# tests/golden/make_example_golden.py)

def _example(name):
    import json
    import os
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "example_marks.npz"))
    meta = json.loads(bytes(z["_meta"]).decode())
    return {k[len(name) + 1:]: z[k] for k in z.files if k.startswith(name + "_")}, meta


def _digest(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


EXAMPLES = ["singleStrip_100", "singleStrip_Detailed", "inv", "nand2", "xor", "SDFFRS_X2"]


def _marks(g2p, A):
    polys = (A["poly_layer"], A["poly_vptr"], A["poly_x"], A["poly_y"])
    grid = g2p.meshGrid(A["sim_lim"], polys, A["sim_side_coords"], A["sim_layers"])
    pz = g2p.polygonZ(polys, A["sim_layers"], A["sim_layer_gdsii"])
    mk = g2p.meshAndMarkPolygons(grid, polys, pz, A["sim_port_side_ptr"], A["sim_side_coords"], A["sim_side_dir"])
    return grid, mk


@pytest.mark.parametrize("name", EXAMPLES)
def test_gpu_polygon_marking_matches_reference_mesher(name, g2p):
    A, meta = _example(name)
    M = meta["cases"][name]
    grid, mk = _marks(g2p, A)
    for got, key in zip(grid, ("xn", "yn", "zn", "stack_epsn", "stack_sign")):
        np.testing.assert_array_equal(got, A["ref_" + key])
    assert mk["num_cdt"] == M["num_cdt"]
    assert _digest(mk["mark_node"]) == M["hashes"]["mark_node"], f"mark_node: sum {mk['mark_node'].sum()} vs {M['sums']['mark_node']}"
    assert _digest(mk["mark_edge"]) == M["hashes"]["mark_edge"], f"mark_edge: sum {mk['mark_edge'].sum()} vs {M['sums']['mark_edge']}"
    np.testing.assert_array_equal(mk["mark_port"], A["ref_mark_port"])
    for key in ("side_edge_ptr", "side_edges", "side_area", "side_dir"):
        np.testing.assert_array_equal(mk[key], A["ref_" + key], err_msg=key)
    np.testing.assert_array_equal(mk["side_coords"].reshape(-1), A["ref_side_coords"])


@pytest.mark.parametrize("name", ["singleStrip_100", "inv"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_example_design_end_to_end(name, precision, g2p):
    """From the design's polygons and settings to Z: the index maps equal
    the reference's mapEdge and bden, and Z the C restatement's (pinned to the
    reference's paraGenerator) on the reference's own mesh."""
    from gds2para_gb300.layout import MeshDesc
    A, meta = _example(name)
    M = meta["cases"][name]
    grid, mk = _marks(g2p, A)
    np.testing.assert_array_equal(mk["cdt_return"], A["cdt_return"])
    sptr = np.asarray(A["sim_port_side_ptr"], np.int32)
    d = MeshDesc(nx=len(grid[0]), ny=len(grid[1]), nz=len(grid[2]), xn=grid[0], yn=grid[1], zn=grid[2],
                 stack_epsn=grid[3], stack_sign=grid[4], mark_node=mk["mark_node"], mark_edge=mk["mark_edge"],
                 mark_node_raw=None, mark_edge_raw=None, num_cdt=mk["num_cdt"], mark_port=mk["mark_port"],
                 cdt_return=mk["cdt_return"], num_ports=len(sptr) - 1, port_side_ptr=sptr,
                 side_edge_ptr=mk["side_edge_ptr"], side_edges=mk["side_edges"], side_area=mk["side_area"],
                 side_dir=mk["side_dir"], side_coords=mk["side_coords"], freq_start=M["freq_start"],
                 freq_end=M["freq_end"], freq_unit=M["freq_unit"], nfreq=M["nfreq"], freq_scale=M["freq_scale"])
    with g2p.FdtdMesh(d) as m:
        me, bden = m.index_maps()
        assert bden == M["bden"]
        assert _digest(me) == M["hashes"]["map_edge"]
        g2p.generateStiff(m)
        rt = 1e-10 if precision == "fp64" else 1e-8
        Z, st = g2p.paraGenerator(m, g2p.default_params(precision=precision, rtol=rt))
    Zr = A["Z"]
    assert np.abs(Z - Zr).max() / np.abs(Zr).max() < (1e-7 if precision == "fp64" else 1e-6)
