"""Full-size workloads, checked through size-independent properties (the
oracle does not run at these sizes):

* reciprocity: at the first frequency Z is symmetric (the reference's Z on
  the golden layouts is symmetric to 1e-14; here the solves stop at 1e-8);
* every solve reaches its tolerance;
* the mixed method agrees with the FP64 method within the 1e-6 Z bound;
* frequencies after the first carry the reference's f0/f rescale of Im Z,
  stored transposed (print_z_V0, src/fdtd.hpp:4249-4316)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(g2p, d, **kw):
    with g2p.FdtdMesh(d) as m:
        g2p.generateStiff(m)
        return g2p.paraGenerator(m, g2p.default_params(**kw))


def _reciprocal(z0, tol):
    err = np.abs(z0 - z0.T).max() / np.abs(z0).max()
    assert err < tol, err


def test_gpu_c2_mixed_matches_fp64_and_is_reciprocal(g2p):
    from gds2para_gb300 import layout as lay
    d = lay.build(lay.config("c2"))
    zm, sm = _run(g2p, d, precision="mixed", batch=1, rtol=1e-8)
    zf, sf = _run(g2p, d, precision="fp64", batch=1, rtol=1e-8)
    assert sm.max_rel_residual <= 1e-8 and sf.max_rel_residual <= 1e-8
    assert np.abs(zm - zf).max() / np.abs(zf).max() < 1e-6
    _reciprocal(zm[0], 1e-6)


def test_gpu_c5_large_layout(g2p):
    from gds2para_gb300 import layout as lay
    d = lay.build(lay.config("c5"))
    assert d.N_edge == 224034816
    z, st = _run(g2p, d, precision="mixed", batch=4, rtol=1e-8)
    assert st.max_rel_residual <= 1e-8
    assert st.rhs_block == 4 and st.solves == 3 * d.num_ports
    assert st.sizes.leng_S > 2 ** 31          # 64-bit row offsets in S
    _reciprocal(z[0], 1e-6)
    f = d.freqs()
    for i in range(1, d.nfreq):
        # Im Z(f) = Im Z(f0) * f0 / f, the real part unchanged; stored transposed
        np.testing.assert_allclose(z[i].T.imag, z[0].imag * f[0] / f[i], rtol=1e-12, atol=0)
        np.testing.assert_allclose(z[i].T.real, z[0].real, rtol=1e-12, atol=0)
