"""Admission accounting of the serving loop, on the host (no device work).

With one assignment scratch per slot, a plan's footprint leaves out the record
buffers and the graph position slots the scratch holds (FP32-family plans on
grids up to the scratch's grid); larger grids and the FP64 form keep their own,
and a captured plan without a shared scratch adds its own position slots.
"""
from pbi4_gb300.estimator import EstimatorConfig, footprint, scratch_footprint
from pbi4_gb300.serve import Server, graph_capable


def _server(shared: bool, grid_max: int = 1024, npart: int = 10 ** 7, batch: int = 4):
    # the accounting only: no slots, streams or scratch allocations
    srv = object.__new__(Server)
    srv.shared_scratch, srv.scratch_grid_max, srv.max_npart, srv.batch = shared, grid_max, npart, batch
    return srv


def test_footprint_leaves_out_the_slot_scratch():
    cfg = EstimatorConfig(grid=256, box=1000.0, nintp=4, interlacing=True, multipoles=True, kbin_bs=3.0,
                          kcenter_bs=3.0, nbins_bs=21, precision="fp16split")
    n = 10 ** 7
    own = _server(False)._footprint(cfg)
    shared = _server(True)._footprint(cfg)
    assert graph_capable(cfg)
    assert own == footprint(cfg, n) + 4 * 3 * n * 8  # its own graph position slots
    assert shared == footprint(cfg, n) - scratch_footprint(256, n)  # records and slots in the slot's scratch
    assert own - shared == scratch_footprint(256, n, 4)


def test_grids_above_the_scratch_and_fp64_keep_their_own():
    n = 10 ** 6
    big = EstimatorConfig(grid=1024, box=1000.0, nintp=2, interlacing=False, multipoles=False, do_bispectrum=False)
    srv = _server(True, grid_max=512, npart=n)
    assert srv._footprint(big) == footprint(big, n) + 4 * 3 * n * 8
    f64 = EstimatorConfig(grid=64, box=1000.0, nintp=2, interlacing=False, multipoles=False, do_bispectrum=False,
                          precision="fp64")
    assert not graph_capable(f64)
    assert _server(True, npart=n)._footprint(f64) == footprint(f64, n)
