"""The extraction service (g2p_server_*): jobs of different grid sizes and
port counts run concurrently on one GPU, each on its own stream, and every
result is the same as the job run alone; admission follows the memory
budget.  The reference extracts one layout per process and has no
counterpart to compare with."""
import numpy as np
import pytest

from conftest import golden_layout

pytestmark = pytest.mark.gpu

CASES = ["manhattan_small", "multistrip_small", "manhattan_sweep", "strip_tiny"]


def _alone(g2p, d, p):
    with g2p.FdtdMesh(d) as m:
        g2p.generateStiff(m)
        Z, _ = g2p.paraGenerator(m, p)
    return Z


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_jobs_in_a_mix_match_each_job_alone(precision, g2p):
    p = g2p.default_params(precision=precision, batch=1, rtol=1e-10)
    layouts = [golden_layout(n)[0] for n in CASES]
    alone = [_alone(g2p, d, p) for d in layouts]
    # the whole path is deterministic: a second run is bit-identical
    np.testing.assert_array_equal(_alone(g2p, layouts[0], p), alone[0])
    with g2p.Server(mem_budget_bytes=64 << 30, max_active=4) as srv:
        jobs = [srv.submit(d, p) for d in layouts * 2]
        res = [srv.wait(j) for j in jobs]
    for i, (Z, st, t) in enumerate(res):
        np.testing.assert_array_equal(Z, alone[i % len(layouts)])
        assert st.solves == 3 * layouts[i % len(layouts)].num_ports
        assert t.total_ms >= t.run_ms > 0
    # the jobs did overlap on the device
    assert sum(t.ran_alone == 0 for _, _, t in res) >= 2


def test_budget_admits_one_job_at_a_time_when_nothing_else_fits(g2p):
    p = g2p.default_params(precision="mixed", batch=1, rtol=1e-10)
    layouts = [golden_layout(n)[0] for n in CASES[:3]]
    with g2p.Server(mem_budget_bytes=1, max_active=4) as srv:
        jobs = [srv.submit(d, p) for d in layouts]
        res = [srv.wait(j) for j in jobs]
    for Z, st, t in res:
        assert t.ran_alone == 1
        assert t.footprint_measured > 0 and t.footprint_estimate > 0
    # later jobs waited in the queue for the earlier ones
    assert res[2][2].queued_ms >= res[0][2].run_ms


def test_submit_rejects_a_bad_description(g2p):
    import ctypes as C
    from gds2para_gb300 import _lib
    L = _lib.load()
    h = C.c_void_p()
    _lib.check(L.g2p_server_create(1 << 30, 2, C.byref(h)))
    try:
        bad = _lib.MeshDescC()
        job = C.c_int64()
        assert L.g2p_server_submit(h, C.byref(bad), None, C.byref(job)) == 1
    finally:
        L.g2p_server_destroy(h)


def _model_estimate(g2p, d, p):
    """The service's footprint estimate of a job: the first job of a fresh
    server is estimated by the size model alone (no measured scale yet)."""
    with g2p.Server(mem_budget_bytes=1 << 40, max_active=1) as srv:
        _, _, t = srv.wait(srv.submit(d, p))
    return t.footprint_estimate


def test_a_job_that_fits_passes_one_that_does_not(g2p):
    """Admission is not head-of-line: with X running, Y does not fit the
    remaining budget but Z does, so Z starts first although Y was queued
    before it."""
    p = g2p.default_params(precision="fp64", batch=1, rtol=1e-12)
    X, Y, Z = (golden_layout(n)[0] for n in ("strip_c1", "manhattan_small", "strip_tiny"))
    ex, ey, ez = (_model_estimate(g2p, d, p) for d in (X, Y, Z))
    assert ey > ez
    budget = ex + (ey + ez) // 2          # X + Z fit, X + Y do not; each fits alone
    assert ex + ez <= budget < ex + ey and max(ex, ey, ez) <= budget
    with g2p.Server(mem_budget_bytes=budget, max_active=3) as srv:
        jobs = [srv.submit(d, p) for d in (X, Y, Z)]
        (_, _, tx), (_, _, ty), (_, _, tz) = [srv.wait(j) for j in jobs]
    assert tz.queued_ms < ty.queued_ms
    assert ty.queued_ms > 0
