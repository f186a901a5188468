"""GDSII ingest on the CPU: the library's reader and flattener
(g2p_gdsii_read, host code) against the conductor polygons that the
reference's own AsciiDataBase + saveToMesh produce for synthetic GDSII files
(tests/golden/gdsii_cases.npz, made by tests/golden/make_gds_golden.py with
oracle/_ref/ref_gds).  Bit-exact: same polygons, order, layers and vertices."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gdsii_cases.npz")


def _api_or_skip():
    from gds2para_gb300 import api, build
    try:
        build.build()
    except Exception as e:  # pragma: no cover - nvcc missing
        pytest.skip(f"library not buildable here: {e}")
    return api


@pytest.mark.parametrize("case", ["flat", "hier", "hier_ignore"])
def test_gdsii_polygons_match_reference(tmp_path, case):
    api = _api_or_skip()
    g = np.load(GOLDEN)
    path = tmp_path / f"{case}.gds"
    path.write_bytes(g[f"{case}_gds"].tobytes())
    layer, vptr, x, y = api.readGDSII(path, g[f"{case}_ignore"])
    np.testing.assert_array_equal(layer, g[f"{case}_layer"])
    np.testing.assert_array_equal(vptr, g[f"{case}_vptr"])
    np.testing.assert_array_equal(x, g[f"{case}_x"])
    np.testing.assert_array_equal(y, g[f"{case}_y"])


def test_gdsii_fixture_covers_the_branches():
    g = np.load(GOLDEN)
    # paths give one rectangle per segment, boxes of BOXTYPE 1 are dropped,
    # the ignored layers leave, the array reference of one column is empty
    assert len(g["flat_layer"]) == 12 and set(g["flat_layer"]) == {1, 2, 4, 5, 3}
    assert len(g["hier_layer"]) == 44 and len(g["hier_ignore_layer"]) == 23
    assert not set(g["hier_ignore_layer"]) & {11, 13}


def test_gdsii_rejects_missing_and_malformed_files(tmp_path):
    api = _api_or_skip()
    from gds2para_gb300._lib import G2PError
    with pytest.raises(G2PError):
        api.readGDSII(tmp_path / "missing.gds")
    bad = tmp_path / "bad.gds"
    bad.write_bytes(b"\x00\x02\x00\x00not gdsii")
    with pytest.raises(G2PError):
        api.readGDSII(bad)


@pytest.mark.parametrize("case", ["flat", "hier"])
def test_mesh_grid_matches_reference_mesher(tmp_path, case):
    """Grid lines and per-layer constants (g2p_mesh_grid) against the
    reference's own meshAndMark on the same polygons, limits, layer stack
    and port sides (mesh.cpp:5-330): bit-exact."""
    api = _api_or_skip()
    g = np.load(GOLDEN)
    path = tmp_path / f"{case}.gds"
    path.write_bytes(g[f"{case}_gds"].tobytes())
    polys = api.readGDSII(path)
    got = api.meshGrid(g[f"{case}_grid_lim"], polys, g[f"{case}_grid_sides"], g[f"{case}_grid_stack"])
    for key, v in zip("XYZES", got):
        np.testing.assert_array_equal(v, g[f"{case}_grid_{key}"], err_msg=key)
    # lines ascend and the merge leaves none within disMin of the previous
    lim = g[f"{case}_grid_lim"]
    dmin = 1e-3 * min(lim[1] - lim[0], lim[3] - lim[2])
    assert np.diff(got[0]).min() > dmin and np.diff(got[1]).min() > dmin


def test_mesh_grid_rejects_a_stack_that_misses_the_grid(tmp_path):
    api = _api_or_skip()
    from gds2para_gb300._lib import G2PError
    g = np.load(GOLDEN)
    path = tmp_path / "flat.gds"
    path.write_bytes(g["flat_gds"].tobytes())
    polys = api.readGDSII(path)
    with pytest.raises(G2PError):
        # one layer covering only the lower half of the z range
        api.meshGrid(g["flat_grid_lim"], polys, [(0, 0, 5e-6, 0, 0, 6e-6)], [(0.0, 1e-6, 3.9, 0.0)])


def test_mesh_grid_rejects_empty_limits_and_runaway_fills(tmp_path):
    """Limits with no x or y extent (disMax = 0) and limits so small against
    the vertices' span that the disMax fill would need billions of lines are
    refused before any line is placed."""
    api = _api_or_skip()
    from gds2para_gb300._lib import G2PError
    g = np.load(GOLDEN)
    path = tmp_path / "flat.gds"
    path.write_bytes(g["flat_gds"].tobytes())
    polys = api.readGDSII(path)
    lim = np.array(g["flat_grid_lim"], np.float64)
    sides, stack = g["flat_grid_sides"], g["flat_grid_stack"]
    for bad in ((1, lim[0]), (1, lim[0] - 1e-6), (3, lim[2]), (2, float("nan"))):
        l2 = lim.copy()
        l2[bad[0]] = bad[1]
        with pytest.raises(G2PError):
            api.meshGrid(l2, polys, sides, stack)
    tiny = lim.copy()
    tiny[1] = tiny[0] + 1e-15          # disMax = 5e-18 m against micron spans
    with pytest.raises(G2PError, match="lines along"):
        api.meshGrid(tiny, polys, sides, stack)
