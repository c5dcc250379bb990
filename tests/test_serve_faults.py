"""Failure handling of the serving loop, with every failure made on the host.

* a request whose plan can never fit under the HBM budget is rejected with a
  failed future, and the loop serves the next request;
* a device allocation that fails (the library's host-side hook
  pbi4g_debug_fail_alloc makes the next cudaMalloc of a plan report
  PBI4G_ERR_NOMEM without issuing it) fails that request's future with the
  library's error, and the same configuration is served on the next request;
* requests cancelled while queued are skipped, the others served;
* a producer thread that dies after submitting leaves the loop serving its
  requests and other producers' requests, and the server closes cleanly.

No GPU fault, trap or hang is involved: the loop runs small boxes on the GPU.
Results are checked against the same box run alone (tests/test_serve.py's
tolerance, 1e-6 relative on P0).
"""
import threading

import numpy as np
import pytest

from pbi4_gb300 import _lib, synthetic
from pbi4_gb300.estimator import Estimator, EstimatorConfig
from pbi4_gb300.serve import Request, Server

pytestmark = pytest.mark.gpu

SMALL = EstimatorConfig(grid=16, box=1000.0, nintp=3, interlacing=True, multipoles=False, do_bispectrum=False)


def _same_as_alone(res, req):
    alone = Estimator(req.cfg)
    pout, _ = alone.run_host(req.pos)
    alone.close()
    np.testing.assert_array_equal(res.pout[2], pout[2])
    ok = pout[1] != 0
    assert np.max(np.abs(res.pout[1][ok] / pout[1][ok] - 1)) < 1e-6


def test_plan_that_never_fits_is_rejected():
    srv = Server(hbm_budget_bytes=64 << 20, slots=2, max_npart=20000, batch=2)
    try:
        big = EstimatorConfig(grid=128, box=1000.0, nintp=4, interlacing=True, multipoles=True, kbin_bs=2.0,
                              kcenter_bs=2.0)
        f_big = srv.submit(Request(cfg=big, pos=synthetic.uniform_box(5000, seed=1), rid=0))
        req = Request(cfg=SMALL, pos=synthetic.uniform_box(8000, seed=2), rid=1)
        f_small = srv.submit(req)
        with pytest.raises(MemoryError):
            f_big.result(timeout=120)
        _same_as_alone(f_small.result(timeout=120), req)
        assert srv.rejected == 1
    finally:
        srv.close()


def test_allocation_failure_fails_one_request():
    lib = _lib.lib()
    srv = Server(hbm_budget_bytes=8 << 30, slots=1, max_npart=20000, batch=2)
    try:
        cfg = EstimatorConfig(grid=32, box=1000.0, nintp=2, interlacing=False, multipoles=False, do_bispectrum=False)
        r1 = Request(cfg=cfg, pos=synthetic.uniform_box(6000, seed=3), rid=1)
        r2 = Request(cfg=cfg, pos=synthetic.uniform_box(7000, seed=4), rid=2)
        assert lib.pbi4g_debug_fail_alloc(1) == 0  # the plan's first device buffer
        f1 = srv.submit(r1)
        with pytest.raises(_lib.Pbi4GpuError) as ei:
            f1.result(timeout=120)
        assert ei.value.code == 3 and "injected" in str(ei.value)   # PBI4G_ERR_NOMEM
        f2 = srv.submit(r2)
        _same_as_alone(f2.result(timeout=120), r2)
        assert srv.failed == 1
    finally:
        lib.pbi4g_debug_fail_alloc(0)
        srv.close()


def test_cancelled_requests_are_skipped():
    srv = Server(hbm_budget_bytes=8 << 30, slots=1, max_npart=20000, batch=4)
    try:
        reqs = [Request(cfg=SMALL, pos=synthetic.uniform_box(3000 + 500 * k, seed=10 + k), rid=k) for k in range(6)]
        with srv.lock:   # the loop cannot take requests while the test holds its lock
            futs = [srv.submit(r) for r in reqs]
            assert futs[1].cancel() and futs[4].cancel()
        for k, (r, f) in enumerate(zip(reqs, futs)):
            if k in (1, 4):
                assert f.cancelled()
            else:
                _same_as_alone(f.result(timeout=120), r)
        assert srv.cancelled == 2
        assert sorted(res.rid for res in srv.results) == [0, 2, 3, 5]
    finally:
        srv.close()


def test_producer_that_dies_leaves_the_loop_serving():
    srv = Server(hbm_budget_bytes=8 << 30, slots=2, max_npart=20000, batch=2)
    futs, reqs, errors = [], [], []

    def producer():
        for k in range(3):
            r = Request(cfg=SMALL, pos=synthetic.uniform_box(4000 + 1000 * k, seed=20 + k), rid=k)
            reqs.append(r)
            futs.append(srv.submit(r))
        raise RuntimeError("producer died")

    def hook(args):
        errors.append(args.exc_value)

    old = threading.excepthook
    threading.excepthook = hook
    try:
        t = threading.Thread(target=producer)
        t.start()
        t.join()
        assert len(errors) == 1 and "producer died" in str(errors[0])
        for r, f in zip(reqs, futs):
            _same_as_alone(f.result(timeout=120), r)
        late = Request(cfg=SMALL, pos=synthetic.uniform_box(5000, seed=30), rid=9)
        _same_as_alone(srv.submit(late).result(timeout=120), late)
    finally:
        threading.excepthook = old
        srv.close()
    assert not srv._thread.is_alive()
