"""Batched form on the GPU: every instance of a batch advances exactly as the same
instance advanced alone (single-instance contexts are checked against the oracle)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batch_matches_single_instances(wb):
    cfgs, ics = wb.batch_workload(n=12, seed_base=77, nmin=16, nmax=70)
    # one cell per thread everywhere, so the batch kernel and the single grid's kernel run
    # the same instructions per cell (two-cells-per-thread kernels may contract FMAs
    # differently: test_batch_autotune_and_pinned_tiles_keep_results)
    for c in cfgs:
        c.tile_x, c.tile_y, c.cells_per_thread = 32, 8, 1
    with wb.Batch(cfgs) as b:
        b.init_perturbation(ics)
        b.step(9)        # eager phases + one graph replay of six steps
        b.step(7, 2e-4)  # fixed-dt arguments rebuilt
        b.sync()
        outs = [b.download(i) for i in range(len(cfgs))]
        total = b.dofs
    assert total == sum(4 * wb.num_modes(c.order, c.basis) * c.nx * c.ny for c in cfgs)
    for i, (c, ic) in enumerate(zip(cfgs, ics)):
        with wb.Solver(config=c) as s:
            s.init_perturbation(ic)
            s.step(9)
            s.step(7, 2e-4)
            ref = s.download()
        np.testing.assert_array_equal(outs[i], ref, err_msg="instance %d" % i)


def test_batch_mixed_physics_matches_single_instances(wb):
    """Instances of one degree and tile that differ in their physical constants, boundary
    conditions or limiter run in separate groups (each launch carries one set of constants);
    every instance still advances exactly as alone."""
    cfgs, ics = wb.batch_workload(n=8, seed_base=123, nmin=20, nmax=60)
    for c in cfgs:
        c.order = 1
        c.tile_x, c.tile_y, c.cells_per_thread = 32, 8, 1
    cfgs[1].gamma = 5.0 / 3.0
    cfgs[2].gy = 0.5
    cfgs[3].gx, cfgs[3].gy = 0.3, 0.8
    cfgs[4].bc_x = wb.BC_PERIODIC
    cfgs[5].limiter = wb.LIMITER_MINMOD
    cfgs[6].kpoly, cfgs[6].eq_kind = 0.7, wb.EQ_POLYTROPE
    with wb.Batch(cfgs) as b:
        b.init_perturbation(ics)
        b.step(8)
        b.sync()
        outs = [b.download(i) for i in range(len(cfgs))]
    for i, (c, ic) in enumerate(zip(cfgs, ics)):
        with wb.Solver(config=c) as s:
            s.init_perturbation(ic)
            s.step(8)
            ref = s.download()
        np.testing.assert_array_equal(outs[i], ref, err_msg="instance %d" % i)


def test_batch_sync_names_the_nonphysical_instance(wb):
    """wb_batch_sync reads every instance's device error word in one copy and reports the
    first instance whose cell means went non-physical."""
    cfgs, ics = wb.batch_workload(n=4, seed_base=31, nmin=24, nmax=40)
    ics[2].amp = -5.0  # the pressure bump drives the centre's pressure below zero
    with wb.Batch(cfgs) as b:
        b.init_perturbation(ics)
        b.step(2, 1e-4)
        with pytest.raises(wb.WbError) as ei:
            b.sync()
    assert ei.value.status == wb.WB_ERR_NONPHYSICAL
    assert "instance 2" in str(ei.value)


def test_batch_zero_perturbation_stays_zero(wb):
    cfgs, ics = wb.batch_workload(n=6, seed_base=5, nmin=16, nmax=40)
    for ic in ics:
        ic.amp = 0.0
    with wb.Batch(cfgs) as b:
        b.init_perturbation(ics)
        b.step(12)
        b.sync()
        for i in range(len(cfgs)):
            assert np.all(b.download(i) == 0.0)


def test_batch_rejects_mixed_precision(wb):
    cfgs, _ = wb.batch_workload(n=2, nmin=16, nmax=20)
    cfgs[1].precision = wb.PREC_FP64
    with pytest.raises(wb.WbError) as ei:
        wb.Batch(cfgs)
    assert ei.value.status == wb.WB_ERR_CONFIG


def test_batch_autotune_and_pinned_tiles_keep_results(wb):
    """wb_batch_autotune changes no state and only regroups the work list: instances on
    any tile shape (chosen or pinned by the config) still advance as alone."""
    cfgs, ics = wb.batch_workload(n=10, seed_base=91, nmin=24, nmax=200)
    cfgs[3].tile_x, cfgs[3].tile_y = 16, 16   # pinned
    cfgs[5].tile_x, cfgs[5].tile_y, cfgs[5].cells_per_thread = 32, 16, 2
    with wb.Batch(cfgs) as b:
        b.init_perturbation(ics)
        b.step(2)
        tiles = b.autotune(2)
        allowed = {(32, 8, 1), (16, 16, 1), (32, 16, 2), (32, 32, 4)}
        assert set(tiles.values()) <= allowed
        assert all(t != (32, 32, 4) for (k, _), t in tiles.items() if k > 0)
        b.step(8)
        b.autotune(1)
        b.step(3)
        b.sync()
        outs = [b.download(i) for i in range(len(cfgs))]
    for i, (c, ic) in enumerate(zip(cfgs, ics)):
        with wb.Solver(config=c) as s:
            s.init_perturbation(ic)
            s.step(13)
            ref = s.download()
        if c.order >= 1:
            # the autotuner or the pin may run these instances at two cells per thread,
            # which may round differently from the single grid's kernel (the compiler's FMA
            # contraction): FP32 rounding level; degree 0 stays bit for bit
            assert np.max(np.abs(outs[i] - ref)) <= 1e-5 * np.max(np.abs(ref)), i
        else:
            np.testing.assert_array_equal(outs[i], ref, err_msg="instance %d" % i)


def test_batch_rejects_unsupported_tile(wb):
    cfgs, _ = wb.batch_workload(n=2, nmin=16, nmax=20)
    cfgs[0].tile_x, cfgs[0].tile_y = 16, 8
    with pytest.raises(wb.WbError) as ei:
        wb.Batch(cfgs)
    assert ei.value.status == wb.WB_ERR_CONFIG
