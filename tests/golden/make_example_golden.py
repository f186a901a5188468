"""Makes tests/golden/example_marks.npz: the reference's own mesher on its
example designs, for the GDSII + .sim_input flow of the library.

For each design of EXAMPLES, from the reference checkout's examples folder:

* the conductor polygons of the reference's AsciiDataBase + saveToMesh
  (oracle/_ref/ref_gds; the library's readGDSII must give the same);
* the library's readSimInput of the design's .sim_input (the reference's
  reader needs Eigen, which is not here, so the reader itself is checked by
  tests/test_siminput_cpu.py against an independent parse);
* with those settings, the reference's meshAndMark and portSet
  (ref_gds --mark): grid lines and per-layer constants (whole), markNode,
  markEdge and mapEdge (SHA-256 digests), each conductor's markPort, the
  port sides' edges, areas, directions and coordinates after findPortNode,
  numCdt and bden;
* for Z_EXAMPLES, Z of the V0 path on that mesh from the C restatement
  (oracle/pipeline.c, pinned to the reference's own paraGenerator) at rtol
  1e-12; the return conductors that findBoundNodeEdge runs on are derived
  by meshAndMark's rule and checked through mapEdge.

usage: python tests/golden/make_example_golden.py [examples_dir]
    (default: $G2P_REFERENCE_ROOT/examples, else ../reference/examples)
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import make_gds_golden as mg  # noqa: E402

EXAMPLES = ["singleStrip_100", "singleStrip_Detailed", "inv", "nand2", "xor", "SDFFRS_X2"]
Z_EXAMPLES = ["singleStrip_100", "inv"]
DIGESTS = ("mark_node", "mark_edge", "map_edge")


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def cdt_return_of(mark_node, mark_port, ncdt, port_side_ptr, coords, xn, yn, zn):
    """The conductors meshAndMark hands to findBoundNodeEdge: each port's
    last-side return conductor, unless it was met before (mesh.cpp:941-953)."""
    ny, nns = len(yn), len(xn) * len(yn)
    idx = lambda c, v: max(int(np.searchsorted(c, v, side="right")) - 1, 0)
    node = lambda x, y, z: int(mark_node[idx(zn, z) * nns + idx(xn, x) * ny + idx(yn, y)])
    seen, ret = set(), np.zeros(ncdt, np.uint8)
    for p in range(len(port_side_ptr) - 1):
        c = coords[port_side_ptr[p + 1] - 1]
        c1, c2 = node(c[0], c[1], c[2]), node(c[3], c[4], c[5])
        seen.add(c1)
        if c2 not in seen:
            seen.add(c2)
            ret[c2 - 1] = 1
    return ret


def main():
    from gds2para_gb300 import api
    from gds2para_gb300.layout import MeshDesc
    folder = sys.argv[1] if len(sys.argv) > 1 else os.path.join(
        os.environ.get("G2P_REFERENCE_ROOT", os.path.join(os.path.dirname(ROOT), "reference")), "examples")
    subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh")], stdout=subprocess.DEVNULL)
    out, meta = {}, {"examples": EXAMPLES, "z_examples": Z_EXAMPLES, "cases": {}}
    for name in EXAMPLES:
        gds = os.path.join(folder, name + ".gds")
        polys = mg.parse_ref(subprocess.run([mg.REF_GDS, gds], check=True, capture_output=True, text=True,
                                            cwd=tempfile.gettempdir()).stdout)
        lib = api.readGDSII(gds)
        assert all(np.array_equal(a, b) for a, b in zip(polys, lib)), f"{name}: readGDSII differs"
        sim = api.readSimInput(os.path.join(folder, name + ".sim_input"))
        R = mg.run_ref_mark(gds, mg.mark_settings(sim))
        nx, ny, nz, ncdt, bden, st, st2 = (int(v) for v in R["meta"])
        assert st == 0 and st2 == 0, f"{name}: reference meshAndMark/portSet status {st}/{st2}"
        grid = api.meshGrid(sim["lim"], lib, sim["side_coords"], sim["layers"])
        assert all(np.array_equal(a, R[k]) for a, k in zip(grid, ("xn", "yn", "zn", "stack_epsn", "stack_sign"))), \
            f"{name}: library grid differs"
        pre = name + "_"
        for k, v in zip(("layer", "vptr", "x", "y"), polys):
            out[pre + "poly_" + k] = v
        for k in ("lim", "layers", "layer_gdsii", "port_side_ptr", "side_coords", "side_dir"):
            out[pre + "sim_" + k] = np.asarray(sim[k])
        for k in ("xn", "yn", "zn", "stack_epsn", "stack_sign", "mark_port", "side_edge_ptr", "side_edges",
                  "side_area", "side_dir", "side_coords"):
            out[pre + "ref_" + k] = R[k]
        case = {"nx": nx, "ny": ny, "nz": nz, "num_cdt": ncdt, "bden": bden, "freq_start": sim["freq_start"],
                "freq_end": sim["freq_end"], "freq_unit": sim["freq_unit"], "nfreq": sim["nfreq"],
                "freq_scale": sim["freq_scale"], "hashes": {k: digest(R[k]) for k in DIGESTS},
                "sums": {k: int(R[k].sum()) for k in DIGESTS}}
        if name in Z_EXAMPLES:
            from oracle.harness import COracle
            O = COracle()
            sptr = np.asarray(sim["port_side_ptr"], np.int32)
            coords = R["side_coords"].reshape(-1, 6)
            cr = cdt_return_of(R["mark_node"], R["mark_port"], ncdt, sptr, coords, R["xn"], R["yn"], R["zn"])
            d = MeshDesc(nx=nx, ny=ny, nz=nz, xn=R["xn"], yn=R["yn"], zn=R["zn"], stack_epsn=R["stack_epsn"],
                         stack_sign=R["stack_sign"], mark_node=R["mark_node"], mark_edge=R["mark_edge"],
                         mark_node_raw=None, mark_edge_raw=None, num_cdt=ncdt, mark_port=R["mark_port"],
                         cdt_return=cr, num_ports=len(sptr) - 1, port_side_ptr=sptr,
                         side_edge_ptr=R["side_edge_ptr"], side_edges=R["side_edges"], side_area=R["side_area"],
                         side_dir=R["side_dir"], side_coords=coords, freq_start=sim["freq_start"],
                         freq_end=sim["freq_end"], freq_unit=sim["freq_unit"], nfreq=sim["nfreq"],
                         freq_scale=sim["freq_scale"], name=name)
            me, _, _, bd = O.index_maps(d)
            assert bd == bden and np.array_equal(me, R["map_edge"]), f"{name}: derived return conductors disagree"
            z, zst = O.para_generator(d, O.default_opts(rtol=1e-12, maxit=4000, restart=60, reuse_setup=1))
            out[pre + "Z"] = z
            out[pre + "cdt_return"] = cr
            case["z_solves"] = int(zst.solves)
        meta["cases"][name] = case
        print(f"{name}: {nx} x {ny} x {nz}, {len(polys[0])} polygons, {ncdt} conductors, "
              f"{len(sim['port_side_ptr']) - 1} ports" + (", Z" if name in Z_EXAMPLES else ""), flush=True)
    out["_meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    path = os.path.join(HERE, "example_marks.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}: {os.path.getsize(path) / 1024:.1f} KiB")


if __name__ == "__main__":
    main()
