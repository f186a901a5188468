"""The full-wave (Vh) path of the C restatement against the reference's own
code: find_Vh(1000) and the per-port, per-frequency Vh correction, which the
reference compiles out (SKIP_VH), built in by oracle/ref_matrixcon_vh.cpp and
run by tests/golden/make_golden.py into tests/golden/strip_tiny_vh.npz.  The
dense LAPACK eigen and linear solves are the stand-ins of
oracle/lapacke_shim.cpp in both; everything else is each side's own code.
Bit-exact: the same Vh and the same Z."""
import hashlib

import numpy as np

from conftest import golden_layout


def _oracle_vh(coracle, d, k):
    job = coracle.job(d)
    job.enable_vh()
    o = coracle.default_opts(rtol=1e-13, maxit=4000, restart=60, reuse_setup=0)
    for s in range(3):
        job.stage(s, o, 1)
    vh = job.find_vh(k)
    z_vh, z_ref = job.vh_z(vh)
    v0 = job.z()
    job.close()
    return vh, z_vh, z_ref, v0


def test_oracle_full_wave_path_matches_reference(coracle):
    d, A, M = golden_layout("strip_tiny_vh")
    vh, z_vh, z_ref, z_v0 = _oracle_vh(coracle, d, 1000)
    assert vh.shape[1] == M["leng_Vh"]
    got = hashlib.sha256(np.ascontiguousarray(vh.T).astype(np.complex128).tobytes()).hexdigest()
    assert got == M["hashes"]["Vh"]
    np.testing.assert_array_equal(z_ref.reshape(-1), A["Z"])
    # after the first frequency the reference's entries are the Vh-corrected
    # Z alone; the first also carries the V0 Z it started from (a quirk of
    # its storage: Construct_Z_V0 and Construct_Z_V0_Vh share the slots)
    np.testing.assert_array_equal(z_ref[1:], z_vh[1:])
    assert np.abs(z_ref[0] - z_vh[0]).max() > 1e3 * np.abs(z_vh[0]).max()
    # the Vh correction moves the V0 answer by well under a percent here
    f = d.freqs()
    for i in range(d.nfreq):
        v0_i = z_v0[i].T if i else z_v0[i]
        assert np.abs(z_vh[i] - v0_i).max() / np.abs(v0_i).max() < 1e-2
