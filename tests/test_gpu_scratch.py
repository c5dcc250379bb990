"""Shared assignment scratch (pbi4g_scratch_*, pbi4g_plan_use_scratch).

A plan that assigns through a shared scratch (with or without the graph
position slots), or moves between scratches, gives
its boxes the same density as with its own buffers, bit for bit: the records
are the same, only their addresses change.  P and B then agree within the
ordering of the floating-point atomics of the P bins and shell powers (1e-6);
mode and triangle counts are identical.  Captured graphs follow the binding.
Two plans of different configurations share one scratch in turn.  A scratch
too small for a plan is refused, and a scratch in use cannot be destroyed.
"""
import numpy as np
import pytest

from pbi4_gb300 import synthetic
from pbi4_gb300._lib import Pbi4GpuError
from pbi4_gb300.estimator import AssignScratch, Estimator, EstimatorConfig

pytestmark = pytest.mark.gpu

CFG_B = EstimatorConfig(grid=64, box=1000.0, nintp=4, interlacing=True, multipoles=True, kbin_bs=4.0, kcenter_bs=4.0,
                        precision="fp16split")
CFG_P = EstimatorConfig(grid=32, box=1000.0, nintp=2, interlacing=False, multipoles=False, do_bispectrum=False)


def _close(cfg, po, bo, p_ref, b_ref):
    modes = 4 if cfg.multipoles else 2  # the mode-count row of pout
    np.testing.assert_array_equal(po[modes], p_ref[modes])
    ok = p_ref[1] != 0
    assert np.max(np.abs(po[1][ok] / p_ref[1][ok] - 1)) < 1e-6
    if b_ref is not None:
        np.testing.assert_array_equal(bo[8], b_ref[8])  # triangle counts
        scale = np.maximum(np.abs(b_ref[6]), np.abs(b_ref[3] * b_ref[4]))
        assert np.max(np.abs(bo[6] - b_ref[6]) / scale) < 1e-6


def test_scratch_density_bit_identical():
    pos = synthetic.zeldovich_box(24, 1000.0, seed=3)
    est = Estimator(CFG_B)
    p0, b0 = est.run_host(pos)
    d0 = est.delta_half()
    sc = AssignScratch(128, pos.shape[1])
    est.use_scratch(sc)
    p1, b1 = est.run_host(pos)
    assert est.delta_half().tobytes() == d0.tobytes()
    _close(CFG_B, p1, b1, p0, b0)
    with pytest.raises(Pbi4GpuError):
        sc.close()  # still in use
    est.use_scratch(None)  # back to the plan's own buffers
    p2, b2 = est.run_host(pos)
    assert est.delta_half().tobytes() == d0.tobytes()
    _close(CFG_B, p2, b2, p0, b0)
    sc.close()
    est.close()


def test_scratch_follows_captured_graphs():
    import torch
    boxes = [synthetic.zeldovich_box(12 + 4 * k, 1000.0, seed=60 + k) for k in range(3)]
    cap = max(b.shape[1] for b in boxes)
    ref = []
    for b in boxes:
        alone = Estimator(CFG_B)
        ref.append(alone.run_host(b))
        alone.close()
    est = Estimator(CFG_B, stream=torch.cuda.Stream())
    est.graph_build(4, cap)
    # records only (positions stay in the plan's own slots), and records with four
    # position slots (the plan's own are freed)
    scratches = [AssignScratch(64, cap), AssignScratch(256, 4 * cap, boxes=4)]
    for sc in [None, scratches[0], scratches[1], None, scratches[1], scratches[0]]:
        est.use_scratch(sc)
        pouts = [np.empty((5, est.nbins_ps), order="F") for _ in boxes]
        bouts = [np.empty((est.brows, est.itot), order="F") for _ in boxes]
        est.graph_run_host(boxes, pouts, bouts)
        est.check()
        for k in range(len(boxes)):
            _close(CFG_B, pouts[k], bouts[k], *ref[k])
    est.close()
    for sc in scratches:
        sc.close()


def test_two_plans_share_one_scratch():
    pos_b = synthetic.zeldovich_box(20, 1000.0, seed=7)
    pos_p = synthetic.uniform_box(30000, seed=8)
    own_b, own_p = Estimator(CFG_B), Estimator(CFG_P)
    rb, rp = own_b.run_host(pos_b), own_p.run_host(pos_p)
    db, dp = own_b.delta_half(), own_p.delta_half()
    own_b.close()
    own_p.close()
    sc = AssignScratch(64, 30000)
    a, b = Estimator(CFG_B), Estimator(CFG_P)
    a.use_scratch(sc)
    b.use_scratch(sc)
    for _ in range(2):
        _close(CFG_B, *a.run_host(pos_b), *rb)
        assert a.delta_half().tobytes() == db.tobytes()
        _close(CFG_P, *b.run_host(pos_p), *rp)
        assert b.delta_half().tobytes() == dp.tobytes()
    a.close()
    b.close()
    sc.close()


def test_scratch_too_small_is_refused():
    sc = AssignScratch(32, 1000)
    est = Estimator(CFG_B)  # grid 64: more tiles than the scratch holds
    with pytest.raises(Pbi4GpuError):
        est.use_scratch(sc)
    small = Estimator(CFG_P)
    small.use_scratch(sc)
    with pytest.raises(Pbi4GpuError):  # 5000 particles above the scratch's 1000
        small.run_host(synthetic.uniform_box(5000, seed=9))
    small.use_scratch(None)
    small.run_host(synthetic.uniform_box(5000, seed=9))
    small.close()
    est.close()
    sc.close()
