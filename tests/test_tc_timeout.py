"""A bounded wait of the tensor-core triangle sums that runs out is reported,
and the plan stays usable.

pbi4g_plan_debug_wait_limit sets, for one plan, how many polls a main-loop
barrier wait of the triangle-sum kernel makes before it gives up.  A limit of a
few polls makes the waits run out while the work is healthy (the barriers
complete a little later), so the launch takes its abort path: every role stops,
the copies and tensor-core work already in flight are waited for with the
normal limit, tensor memory is freed, and the error flag is set.  The host must
return PBI4G_ERR_TIMEOUT (5) from run_host and from pbi4g_plan_check, and the
next run with the normal limit must give the same results as before.  No GPU
fault, trap or endless wait is involved.
"""
import numpy as np
import pytest

from pbi4_gb300 import _lib, synthetic
from pbi4_gb300.estimator import Estimator, EstimatorConfig


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp16split", "tf32split", "bf16"])
def test_wait_that_runs_out_is_reported_and_plan_recovers(precision):
    lib = _lib.lib()
    cfg = EstimatorConfig(grid=64, box=1000.0, nintp=4, interlacing=True, multipoles=True, kbin_bs=2.0,
                          kcenter_bs=2.0, nbins_bs=10, precision=precision)
    pos = synthetic.zeldovich_box(24, 1000.0, seed=41)
    est = Estimator(cfg)
    try:
        p_ref, b_ref = est.run_host(pos)
        assert lib.pbi4g_plan_debug_wait_limit(est._h, 2) == 0
        with pytest.raises(_lib.Pbi4GpuError) as ei:
            est.run_host(pos)
        assert ei.value.code == 5, str(ei.value)
        assert "bounded wait" in str(ei.value)
        assert lib.pbi4g_plan_debug_wait_limit(est._h, 0) == 0
        p2, b2 = est.run_host(pos)
        est.check()
        np.testing.assert_array_equal(p2[4], p_ref[4])
        np.testing.assert_array_equal(b2[[0, 1, 2, 8]], b_ref[[0, 1, 2, 8]])
        ok = p_ref[4] > 0
        assert np.max(np.abs(p2[1][ok] / p_ref[1][ok] - 1)) < 1e-6
        scale = np.maximum(np.abs(b_ref[6]), np.abs(b_ref[3] * b_ref[4]))
        assert np.max(np.abs(b2[6] - b_ref[6]) / scale) < 1e-9
    finally:
        est.close()


def test_debug_wait_limit_rejects_bad_arguments():
    """Host-side argument check (no GPU needed)."""
    lib = _lib.lib()
    assert lib.pbi4g_plan_debug_wait_limit(None, 1) == 1
