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
