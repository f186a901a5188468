import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    meta = json.loads(bytes(z["_meta"]).decode())
    arrays = {k: z[k] for k in z.files if k != "_meta"}
    return arrays, meta


def golden_layout(name):
    from gds2para_gb300 import layout as lay
    arrays, meta = load_golden(name)
    d = lay.build(getattr(lay, meta["generator"])(**meta["kwargs"]))
    return d, arrays, meta


GOLDEN_CASES = ["strip_tiny", "strip_c1", "manhattan_small", "manhattan_sweep", "multistrip_small"]
# the bench configurations c2 and c3, pinned by digests of the reference's outputs
BENCH_CASES = ["manhattan_c2", "multistrip_c3"]


def check_golden_array(arrays, meta, key, value, exact=True, rtol=0.0):
    """Compares `value` with the fixture: whole array or SHA-256 + stats."""
    import hashlib
    value = np.ascontiguousarray(value)
    if key in arrays:
        ref = arrays[key]
        assert value.shape == ref.shape, f"{key}: shape {value.shape} vs {ref.shape}"
        if exact:
            np.testing.assert_array_equal(value, ref, err_msg=key)
        else:
            np.testing.assert_allclose(value, ref, rtol=rtol, atol=0, err_msg=key)
        return
    h = meta["hashes"][key]
    st = meta["stats"][key]
    assert value.size == st["size"], f"{key}: size {value.size} vs {st['size']}"
    if exact:
        got = hashlib.sha256(value.astype(np.dtype(st["dtype"])).tobytes()).hexdigest()
        assert got == h, f"{key}: digest differs"
    else:
        s = float(np.sum(value.astype(np.float64)))
        assert abs(s - st["sum"]) <= rtol * max(abs(st["sum"]), 1e-300) * 10 + 1e-300, f"{key}: sum {s} vs {st['sum']}"


@pytest.fixture(scope="session")
def coracle():
    from oracle.harness import COracle
    return COracle()


def have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def g2p():
    if not have_gpu():
        pytest.skip("no CUDA device")
    from gds2para_gb300 import api, _lib
    _lib.load()
    return api
