"""Serving loop: each box's result is the same alone and in the mix.

Boxes of several configurations (grid sizes, assignment orders, interlacing,
P-only and P+B, FP32 and FP16-split) are submitted at once to a Server with
three CUDA-stream slots; every result is compared with the same box run alone
on a fresh plan through the direct path.  Same-configuration boxes on grids
that are multiples of 16 run as batches through captured CUDA graphs; the grid
of 48 runs box by box.  Tolerance: 1e-6 relative (the differences allowed are
the ordering of floating-point atomics in the P bins and shell powers, and the
fixed-point scale of the captured form, set by the server's particle capacity);
mode and triangle counts identical.  A second run squeezes the HBM budget so
plans are evicted and rebuilt, with the same check.
"""
import numpy as np
import pytest

from pbi4_gb300 import synthetic
from pbi4_gb300.estimator import Estimator, EstimatorConfig
from pbi4_gb300.serve import Request, Server

pytestmark = pytest.mark.gpu


def _requests():
    cfgs = [
        EstimatorConfig(grid=32, box=1000.0, nintp=4, interlacing=True, multipoles=True, kbin_bs=2.0, kcenter_bs=2.0),
        EstimatorConfig(grid=48, box=800.0, nintp=2, interlacing=False, multipoles=False, do_bispectrum=False),
        EstimatorConfig(grid=64, box=1000.0, nintp=3, interlacing=True, multipoles=False, kbin_bs=4.0,
                        kcenter_bs=4.0, precision="fp16split"),
    ]
    reqs = []
    rng = np.random.default_rng(5)
    for k in range(15):
        cfg = cfgs[k % 3]
        n = int(rng.integers(5000, 40000))
        pos = synthetic.uniform_box(n, seed=100 + k) if k % 2 else synthetic.zeldovich_box(20 + k, 1000.0, seed=k)
        reqs.append(Request(cfg=cfg, pos=pos, rid=k))
    return reqs


def _check(results, reqs):
    for r in reqs:
        res = results[r.rid]
        alone = Estimator(r.cfg)
        pout, bout = alone.run_host(r.pos)
        alone.close()
        np.testing.assert_array_equal(res.pout[4 if r.cfg.multipoles else 2], pout[4 if r.cfg.multipoles else 2])
        ok = pout[1] != 0
        assert np.max(np.abs(res.pout[1][ok] / pout[1][ok] - 1)) < 1e-6
        if bout is not None:
            np.testing.assert_array_equal(res.bout[8], bout[8])
            scale = np.maximum(np.abs(bout[6]), np.abs(bout[3] * bout[4]))
            assert np.max(np.abs(res.bout[6] - bout[6]) / scale) < 1e-6


@pytest.mark.parametrize("tight", [False, True])
def test_serving_mix_matches_alone(tight):
    from pbi4_gb300.estimator import footprint
    reqs = _requests()
    max_npart = 50000
    fp = sorted({footprint(r.cfg, max_npart) for r in reqs})
    # tight: room for the two largest plans only, so the loop must evict and rebuild
    budget = int(fp[-1] + fp[-2] + 1) if tight else int(40e9)
    srv = Server(hbm_budget_bytes=budget, slots=3, max_npart=max_npart)
    futs = [srv.submit(r) for r in reqs]
    results = {f.result(timeout=300).rid: f.result() for f in futs}
    stats = srv.stats()
    srv.close()
    assert stats["n"] == len(reqs) and stats["p99_ms"] >= stats["p50_ms"] > 0
    assert stats["batches"] < len(reqs)  # same-configuration boxes shared graph launches
    if tight:
        assert stats["evictions"] > 0
    _check(results, reqs)


def test_graph_batch_matches_direct():
    """One plan, four boxes of different sizes in one captured graph launch."""
    import torch
    cfg = EstimatorConfig(grid=64, box=1000.0, nintp=4, interlacing=True, multipoles=True, kbin_bs=4.0,
                          kcenter_bs=4.0, precision="fp16split")
    boxes = [synthetic.zeldovich_box(12 + 4 * k, 1000.0, seed=50 + k) for k in range(4)]
    st = torch.cuda.Stream()
    est = Estimator(cfg, stream=st)
    est.graph_build(4, max(b.shape[1] for b in boxes))
    for nb in (4, 3):  # a full and a partial batch (two captured graphs)
        pouts = [np.empty((5, est.nbins_ps), order="F") for _ in range(nb)]
        bouts = [np.empty((est.brows, est.itot), order="F") for _ in range(nb)]
        est.graph_run_host(boxes[:nb], pouts, bouts)
        est.check()
        for k in range(nb):
            ref = Estimator(cfg)
            p_ref, b_ref = ref.run_host(boxes[k])
            ref.close()
            np.testing.assert_array_equal(pouts[k][4], p_ref[4])
            ok = p_ref[1] != 0
            assert np.max(np.abs(pouts[k][1][ok] / p_ref[1][ok] - 1)) < 1e-6
            np.testing.assert_array_equal(bouts[k][8], b_ref[8])
            scale = np.maximum(np.abs(b_ref[6]), np.abs(b_ref[3] * b_ref[4]))
            assert np.max(np.abs(bouts[k][6] - b_ref[6]) / scale) < 1e-6
    est.close()


@pytest.mark.parametrize("precision", ["fp16split", "fp32"])
def test_two_plans_on_two_streams_match_one(precision):
    """Two plans of one configuration on two CUDA streams with their boxes in
    flight together (the two-in-flight form of the throughput figure) give the
    results each box gets alone on one plan: the k columns and counts identical,
    the rest within the ordering of the floating-point atomics (1e-6, P2 and P4
    relative to P0; the mean |k| of a P bin is summed with FP64 atomics once per
    plan, so two plans agree on it to the last bit only)."""
    import torch
    cfg = EstimatorConfig(grid=64, box=1000.0, nintp=4, interlacing=True, multipoles=True, kbin_bs=2.0,
                          kcenter_bs=2.0, nbins_bs=10, precision=precision)
    boxes = [synthetic.zeldovich_box(24, 1000.0, seed=40 + k) for k in range(4)]
    alone = Estimator(cfg)
    ref = [alone.run_host(b) for b in boxes]
    alone.close()
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    ests = [Estimator(cfg, stream=s) for s in streams]
    outs = [[e.alloc_outputs() for _ in range(2)] for e in ests]
    dpos = [torch.from_numpy(b).cuda() for b in boxes]
    torch.cuda.synchronize()
    for k in range(4):  # box k on plan k % 2, output slot k // 2; no host sync between the launches
        e = ests[k % 2]
        po, bo = outs[k % 2][k // 2]
        e.run_device(dpos[k].shape[1], dpos[k], po, bo)
    torch.cuda.synchronize()
    for e in ests:
        e.check()
    for k in range(4):
        po, bo = outs[k % 2][k // 2]
        p, b = po.cpu().numpy(), bo.cpu().numpy()
        pr, br = ref[k]
        np.testing.assert_array_equal(b[[0, 1, 2, 8]], br[[0, 1, 2, 8]])
        np.testing.assert_array_equal(p[4], pr[4])
        np.testing.assert_allclose(p[:2], pr[:2], rtol=1e-6, atol=0)
        # P2 and P4 against P0 of the bin (they are small differences of large terms)
        assert np.all(np.abs(p[2:4] - pr[2:4]) <= 1e-6 * np.abs(pr[1])), np.max(np.abs(p[2:4] - pr[2:4]) / np.abs(pr[1]))
        np.testing.assert_allclose(b, br, rtol=1e-6, atol=1e-9 * np.max(np.abs(br)))
