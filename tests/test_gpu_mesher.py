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
