"""Makes tests/golden/network_ref.npz: the reference's own output stage and
.sim_input reader (src/solnoutclass.hpp, compiled unmodified by
oracle/build_ref.sh into oracle/_ref/ref_network against the project's
stand-ins for Eigen and Parser-SPEF, which are not in the image).

* NETWORK_CASES: seeded Z data (1-8 ports, 1-4 frequencies; some nearly
  reciprocal, some with entries below the writers' 1e-5 threshold) through
  Parasitics::saveNetworkParam('Z') (with computeYBusFromParam(0): G, C),
  convertParam between every pair of Z, Y and S, and the writers
  dumpTouchstone (Z and S), dumpCITI (S), dumpXyce and dumpSPEF (Z).  The
  SPEF file is the Parser-SPEF stand-in's listing of the Spef structure the
  reference's toSPEF fills (the stand-in has no SPEF renderer).
* SIM_INPUTS: synthetic .sim_input texts (written here) and, when the
  reference's examples folder is given, its example files: the fdtdMesh
  fields that readSimInput + convertToFDTDMesh leave (limits, frequency
  fields, valid stack layers with GDSII numbers, port sides and
  directions).  Only the reference's outputs are stored for the examples.

usage: python tests/golden/make_network_golden.py [examples_dir]
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref", "ref_network")

NETWORK_CASES = {
    # name: (ports, frequencies, seed, kind)
    "one_port": (1, 3, 11, "random"),
    "two_port": (2, 4, 12, "reciprocal"),
    "three_port": (3, 1, 13, "random"),
    "five_port_small": (5, 2, 14, "small"),
    "eight_port": (8, 3, 15, "reciprocal"),
}


def z_data(p, nf, seed, kind):
    r = np.random.default_rng(seed)
    z = np.empty((nf, p, p), np.complex128)
    for f in range(nf):
        a = r.normal(size=(p, p)) + 1j * r.normal(size=(p, p))
        if kind == "reciprocal":
            a = (a + a.T) / 2 + 1e-13 * r.normal(size=(p, p))      # nearly symmetric
        if kind == "small":
            a[r.random((p, p)) < 0.4] *= 1e-7                      # below the write threshold
        z[f] = 20 * np.eye(p) * (1 + 0.5j) + a
    return z


def sim_texts():
    base = open(os.path.join(ROOT, "tests", "test_siminput_cpu.py")).read()
    synth = base.split('SYNTH = """', 1)[1].split('"""', 1)[0]
    variants = {"synth": synth, "synth_no_last_newline": synth.rstrip("\n")}
    variants["two_points"] = synth.replace("nfreq = 1", "nfreq = 2").replace("freqScale = 0", "freqScale = 1")
    variants["log_sweep"] = synth.replace("nfreq = 1", "nfreq = 7")
    return variants


def run_sim(path):
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "o.txt")
        subprocess.run([REF, "simin", path, out], check=True, capture_output=True)
        return open(out).read()


def main():
    subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh")], stdout=subprocess.DEVNULL)
    arrays, meta = {}, {"network": {}, "simin": {}}
    for name, (p, nf, seed, kind) in NETWORK_CASES.items():
        z = z_data(p, nf, seed, kind)
        freqs = np.geomspace(1e8, 1e10, nf)
        zs = np.linspace(25.0, 100.0, p)
        names = [f"n{name[:3]}{i + 1}" for i in range(p)]
        dirs = "".join("IOB"[i % 3] for i in range(p))
        with tempfile.TemporaryDirectory() as d:
            inp = os.path.join(d, "in.txt")
            with open(inp, "w") as f:
                f.write(f"{p} {nf}\n" + " ".join(repr(float(v)) for v in freqs) + "\n")
                for i in range(p):
                    f.write(f"{names[i]} {dirs[i]} {float(zs[i])!r}\n")
                for v in z.reshape(-1):
                    f.write(f"{float(v.real)!r} {float(v.imag)!r}\n")
            out = os.path.join(d, "out")
            os.makedirs(out)
            subprocess.run([REF, "network", inp, out, "design_" + name], check=True, capture_output=True, cwd=d)
            pre = name + "_"
            arrays[pre + "z"] = z
            arrays[pre + "freqs"] = freqs
            arrays[pre + "zs"] = zs
            arrays[pre + "G"] = np.loadtxt(os.path.join(out, "G.txt")).reshape(p, p)
            arrays[pre + "C"] = np.loadtxt(os.path.join(out, "C.txt")).reshape(p, p)
            for a in "ZYS":
                for b in "ZYS":
                    if a != b:
                        v = np.loadtxt(os.path.join(out, f"{a}_to_{b}.txt")).reshape(-1, 2)
                        arrays[pre + f"{a}_to_{b}"] = (v[:, 0] + 1j * v[:, 1]).reshape(nf, p, p)
            for fn in ("z.ts", "z.cir", "z.spef", "s.citi", "s.ts"):
                arrays[pre + "file_" + fn.replace(".", "_")] = np.frombuffer(open(os.path.join(out, fn), "rb").read(),
                                                                             np.uint8)
        meta["network"][name] = {"ports": p, "nfreq": nf, "names": names, "dirs": dirs, "design": "design_" + name,
                                 "kind": kind}
        print(f"network {name}: {p} ports, {nf} frequencies")
    for name, text in sim_texts().items():
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "t.sim_input")
            with open(path, "w") as f:
                f.write(text)
            meta["simin"][name] = {"text": text, "ref": run_sim(path)}
    if len(sys.argv) > 1:
        folder = sys.argv[1]
        for fn in sorted(os.listdir(folder)):
            if fn.endswith(".sim_input"):
                meta["simin"]["example_" + fn[:-len(".sim_input")]] = {"file": fn,
                                                                        "ref": run_sim(os.path.join(folder, fn))}
    print(f"sim_input: {len(meta['simin'])} files")
    arrays["_meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    path = os.path.join(HERE, "network_ref.npz")
    np.savez_compressed(path, **arrays)
    print(f"wrote {path}: {os.path.getsize(path) / 1024:.1f} KiB")


if __name__ == "__main__":
    main()
