"""Batched and FP32 paths on the GPU."""
import numpy as np
import pytest

import gdc
from helpers import interior, rel_l2, scheme

pytestmark = pytest.mark.gpu


def test_member_alone_equals_member_in_mix(native):
    """Continuous batching must not change results: a member advanced alone
    and inside a mixed batch (other grids, members joining and leaving) is
    bitwise identical."""
    p = scheme(gdc, 360, 181, 240.0)
    ic = gdc.ic_seeded(360, 181, seed=9)
    alone = gdc.Batch(p)
    a = alone.add(360, 181, 240.0, 12, *ic)
    alone.step(12)
    mix = gdc.Batch(p)
    o1 = mix.add(180, 91, 480.0, 5, *gdc.ic_seeded(180, 91, seed=1))
    mix.step(2)
    b = mix.add(360, 181, 240.0, 12, *ic)
    o2 = mix.add(720, 361, 120.0, 3, *gdc.ic_seeded(720, 361, seed=2))
    mix.step(20)
    mix.sync()
    assert mix.info(b)[0] == 12 and mix.info(b)[1]
    for x, y in zip(alone.get_state(a), mix.get_state(b)):
        assert np.array_equal(x, y)
    assert mix.info(o1)[0] == 5 and mix.info(o2)[0] == 3


@pytest.mark.parametrize("prec", [gdc.FP64, gdc.FP32])
def test_batch_member_matches_single_model(native, prec):
    N, M = 180, 91
    p = scheme(gdc, N, M, 480.0, precision=prec)
    ic = gdc.ic_seeded(N, M, seed=5)
    m = gdc.Model(p)
    m.set_state(*ic)
    m.run(7)
    b = gdc.Batch(p)
    i = b.add(N, M, 480.0, 7, *ic)
    b.step(7)
    for x, y in zip(m.get_state(), b.get_state(i)):
        assert np.array_equal(x, y)


def test_fp32_compensated_vs_fp64(native):
    """Zonal flow over three mountains on 720x361 (dt 120 s), one model day:
    FP32 with compensated time levels vs the FP64 path; gd relative L2
    <= 1e-5 (the stated bound).  The zonal flow makes the reference's
    filter rescale noise-driven on filtered rows, so both runs use the
    rescale guard."""
    N, M = 720, 361
    ic = gdc.ic_seeded(N, M, seed=1, lmax=0, gd0=5960 * gdc.G, gd_rms=0, psi_rms=0, u0=20.0, n_mountains=3)
    out = {}
    for prec in (gdc.FP64, gdc.FP32):
        p = scheme(gdc, N, M, 120.0, precision=prec, cutoff=(4,) * 10)
        p.filter_rescale_rtol = 1e-5
        m = gdc.Model(p)
        m.set_state(*ic)
        m.run(720)
        out[prec] = m.get_state()
    e = [rel_l2(a, b) for a, b in zip(out[gdc.FP32], out[gdc.FP64])]
    assert e[2] <= 1e-5, e


@pytest.mark.parametrize("tile", [(8, 32), (8, 64), (4, 128), (16, 64), (4, 32)])
def test_every_tile_shape_matches_oracle_on_ragged_grid(native, tile):
    """720 columns leave a ragged last column block under every tile shape
    (16, 16 and 80 columns), whose halo columns wrap to 0 and 1; 4x32 tiles
    have fewer points than the block has threads."""
    from oracle.oracle import OracleModel
    N, M = 720, 361
    p = scheme(gdc, N, M, 120.0, subcycles=2, cutoff=(4,) * 5)
    ic = gdc.ic_seeded(N, M, seed=5)
    b = gdc.Batch(p)
    b.set_tile(*tile)
    mid = b.add(N, M, 120.0, 1, *ic)
    b.step(1)
    b.sync()
    got = b.get_state(mid)
    b.close()
    o = OracleModel.from_params(p)
    o.set_state(*ic)
    o.step(1)
    ref = o.get_state()
    for name, a in zip(("u", "v", "gd"), got):
        assert np.array_equal(interior(a), interior(ref[name])), (tile, name)


@pytest.mark.parametrize("tile", [(8, 32), (8, 64), (4, 128), (16, 64)])
def test_every_fp32_tile_shape_near_oracle_on_ragged_grid(native, tile):
    """The FP32 kernels (column pairs where the tile allows) under every tile
    shape: one step within 1e-5 (relative L2) of the FP64 oracle, on the
    serving scheme of this grid (8 subcycles, 10 filtered rows: the gravity
    waves of the first unfiltered row are within their CFL limit)."""
    from oracle.oracle import OracleModel
    N, M = 720, 361
    p = scheme(gdc, N, M, 120.0, subcycles=8, cutoff=(4,) * 10, precision=gdc.FP32)
    p.filter_rescale_rtol = 1e-5
    ic = gdc.ic_seeded(N, M, seed=5)
    b = gdc.Batch(p)
    b.set_tile(*tile)
    mid = b.add(N, M, 120.0, 1, *ic)
    b.step(1)
    b.sync()
    got = b.get_state(mid)
    b.close()
    o = OracleModel.from_params(p)
    o.set_state(*ic)
    o.step(1)
    ref = o.get_state()
    for name, a in zip(("u", "v", "gd"), got):
        assert rel_l2(a, ref[name]) < 1e-5, (tile, name, rel_l2(a, ref[name]))


@pytest.mark.parametrize("shape", [(8, 30), (16, 30), (32, 30), (64, 30)])
@pytest.mark.parametrize("N,M", [(720, 361), (200, 101)])
def test_warp_strips_match_oracle(native, shape, N, M):
    """Warp strips evaluate the same point formulas as the tiles: FP64 stays
    bitwise equal to the oracle, including a grid whose width is not a
    multiple of the 30-column strip (200 = 6 x 30 + 20) and bands cut short
    by the filtered rows."""
    from oracle.oracle import OracleModel
    dt = 120.0 if N == 720 else 480.0
    p = scheme(gdc, N, M, dt, subcycles=2, cutoff=(4,) * 5)
    ic = gdc.ic_seeded(N, M, seed=6)
    b = gdc.Batch(p)
    b.set_tile(*shape)
    mid = b.add(N, M, dt, 2, *ic)
    b.step(2)
    b.sync()
    got = b.get_state(mid)
    diag = b.diag(mid)
    b.close()
    o = OracleModel.from_params(p)
    o.set_state(*ic)
    o.step(2)
    ref = o.get_state()
    for name, a in zip(("u", "v", "gd"), got):
        assert np.array_equal(interior(a), interior(ref[name])), (shape, name)
    assert diag == o.diag()


@pytest.mark.parametrize("split,adv", [(gdc.SPLIT_ISP, 0), (gdc.SPLIT_CSP2, 1), (gdc.SPLIT_NONE, 0)])
def test_warp_strips_other_schemes_match_oracle(native, split, adv):
    from oracle.oracle import OracleModel
    N, M = 200, 101
    dt = 90.0 if split == gdc.SPLIT_NONE else 480.0
    p = scheme(gdc, N, M, dt, split=split, adv=adv, subcycles=3, cutoff=(4,) * 5, lat_beta=0.5, lon_beta=0.25)
    ic = gdc.ic_seeded(N, M, seed=7)
    b = gdc.Batch(p)
    b.set_tile(16, 30)
    mid = b.add(N, M, dt, 2, *ic)
    b.step(2)
    b.sync()
    got = b.get_state(mid)
    b.close()
    o = OracleModel.from_params(p)
    o.set_state(*ic)
    o.step(2)
    ref = o.get_state()
    for name, a in zip(("u", "v", "gd"), got):
        assert np.array_equal(interior(a), interior(ref[name])), (split, adv, name)


@pytest.mark.parametrize("split", [0, 1])
def test_every_schedule_matches_oracle(native, split):
    """Whole-row or per-field row tasks, the final update launched or formed
    by the next predict_correct's first stage, row tasks on one block or
    split over the two blocks of a cluster: the FP64 path stays bitwise the
    oracle's (csp2 with 6 subcycles: seven fused updates per step)."""
    from oracle.oracle import OracleModel
    N, M = 360, 181
    p = scheme(gdc, N, M, 240.0)
    ic = gdc.ic_seeded(N, M, seed=6)
    o = OracleModel.from_params(p)
    o.set_state(*ic)
    o.step(3)
    ref = o.get_state()
    for fuse, pair in ((0, 0), (1, 0), (0, 1)):
        b = gdc.Batch(p)
        b.set_schedule(split, fuse, pair)
        mid = b.add(N, M, 240.0, 3, *ic)
        b.step(3)
        b.sync()
        assert b.schedule()["fuse_final"] == fuse and b.schedule()["pair_rows"] == pair
        for name, a in zip(("u", "v", "gd"), b.get_state(mid)):
            assert np.array_equal(interior(a), interior(ref[name])), (split, fuse, pair, name)
        b.close()


def test_paired_rows_in_a_mixed_batch(native):
    """Row tasks split over block pairs in a mixed-grid FP64 batch (members
    of different widths -- 180 columns split at 88, not at the middle --
    whole-row and per-field tasks, pole rows) are bitwise the unpaired
    batch's.  (The single-member FP64 model pairs its rows by default, and
    its debug tendency -- a launch without clusters, where part 0 does a
    paired task whole -- is checked against the oracle by the tendency
    parity tests.)  FP32 batches never pair."""
    grids = [(360, 181, 240.0), (180, 91, 480.0), (144, 73, 600.0)]
    p = scheme(gdc, 360, 181, 240.0)
    for split in (0, 1):
        out = []
        for pair in (0, 1):
            b = gdc.Batch(p)
            b.set_schedule(split, 0, pair)
            ids = [b.add(N, M, dt, 4, *gdc.ic_seeded(N, M, seed=k)) for k, (N, M, dt) in enumerate(grids)]
            b.step(4)
            assert b.schedule()["pair_rows"] == pair
            out.append([b.get_state(i) for i in ids])
            b.close()
        for s0, s1 in zip(*out):
            for x, y in zip(s0, s1):
                assert np.array_equal(x, y), split
    b = gdc.Batch(scheme(gdc, 360, 181, 240.0, precision=gdc.FP32))
    b.set_schedule(1, 0, 1)
    b.add(180, 91, 480.0, 2, *gdc.ic_seeded(180, 91, seed=0))
    b.step(2)
    assert b.schedule()["pair_rows"] == 0
    b.close()


def test_fp32_fused_schedule_matches_launched(native):
    """FP32 under the fused schedule: the update's arithmetic is
    final_kernel's, so the state is bitwise the launched schedule's."""
    N, M = 180, 91
    p = scheme(gdc, N, M, 480.0, precision=gdc.FP32)
    ic = gdc.ic_seeded(N, M, seed=3)
    out = []
    for fuse in (0, 1):
        b = gdc.Batch(p)
        b.set_schedule(-1, fuse)
        mid = b.add(N, M, 480.0, 10, *ic)
        b.step(10)
        out.append(b.get_state(mid))
        b.close()
    for x, y in zip(*out):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("prec", [gdc.FP64, gdc.FP32])
def test_autotune_advances_no_forecast(native, prec):
    """Autotuning times every schedule on the live members and restores
    them: the state right after is the state before, and the run continues
    exactly as in an untuned twin batch (bitwise in FP64 under any chosen
    schedule; in FP32 the twin uses the same schedule)."""
    p = scheme(gdc, 360, 181, 240.0, precision=prec)
    ics = [gdc.ic_seeded(360, 181, seed=1), gdc.ic_seeded(180, 91, seed=2)]
    grids = [(360, 181, 240.0), (180, 91, 480.0)]
    a, b = gdc.Batch(p), gdc.Batch(p)
    ia = [a.add(N, M, dt, 9, *ic) for (N, M, dt), ic in zip(grids, ics)]
    ib = [b.add(N, M, dt, 9, *ic) for (N, M, dt), ic in zip(grids, ics)]
    a.step(2)
    b.step(2)
    before = [a.get_state(i) for i in ia]
    diag_before = [a.diag(i) for i in ia]
    r, c, ms = a.autotune()
    assert ms > 0 and (r, c) == a.schedule()["tile"]
    for i, s0, d0 in zip(ia, before, diag_before):
        for x, y in zip(s0, a.get_state(i)):
            assert np.array_equal(x, y)
        assert a.diag(i) == d0 and a.info(i)[0] == 2
    sch = a.schedule()
    if prec == gdc.FP32:
        b.set_tile(*sch["tile"])
        b.set_schedule(sch["split_rows"], sch["fuse_final"], sch["pair_rows"])
    a.step(7)
    b.step(7)
    for i, j in zip(ia, ib):
        assert a.info(i)[:2] == (9, 1)
        for x, y in zip(a.get_state(i), b.get_state(j)):
            assert np.array_equal(x, y)
