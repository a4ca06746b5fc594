"""CUDA path vs the CPU oracle, through the C ABI (FP64 plain path).

The FP64 kernels and the host tables are compiled without FMA contraction,
so every point-wise expression rounds exactly as the oracle's, and every
sum (filter s1/s2 and projections, pole caps, beta, diagnostics) is the
correctly rounded sum on both sides.  The plain path is therefore expected
to be bitwise identical to the oracle; the stated bound (relative L2
<= 1e-12 after 360 steps of the seeded 360x181 state, mass drift equal
within 1e-13) is asserted as well.
"""
import numpy as np
import pytest

import gdc
from helpers import interior, rel_l2, rel_linf, scheme
from oracle.oracle import OracleModel

pytestmark = pytest.mark.gpu


def pair(p, ic):
    m = gdc.Model(p)
    m.set_state(*ic)
    o = OracleModel.from_params(p)
    o.set_state(*ic)
    return m, o


@pytest.mark.parametrize("adv", [gdc.ADV_CENTER_DIFF, gdc.ADV_UPWIND, gdc.ADV_WENO])
@pytest.mark.parametrize("pass_", [0, 1, 2])
def test_tendency_parity(native, pass_, adv):
    N, M = 360, 181
    p = scheme(gdc, N, M, 240.0, adv=adv, lat_beta=0.5, lon_beta=0.25)
    ic = gdc.ic_seeded(N, M, seed=11)
    m, o = pair(p, ic)
    g = m.tendency(pass_)
    r = o.tendency(pass_)
    for name, a, b in zip(("du", "dv", "dgd"), g, r):
        if pass_ == 2 and name == "dgd":
            assert np.all(interior(a) == 0)
        assert np.array_equal(interior(a), interior(b)), (name, rel_l2(a, b))


@pytest.mark.parametrize("split,adv", [(gdc.SPLIT_NONE, 0), (gdc.SPLIT_CSP2, 0), (gdc.SPLIT_ISP, 0),
                                       (gdc.SPLIT_CSP2, 1), (gdc.SPLIT_NONE, gdc.ADV_WENO)])
def test_step_parity(native, split, adv):
    N, M = 180, 91
    # Without splitting the gravity-wave step must satisfy the CFL limit of
    # the first unfiltered row (~110 s at 2 degrees): dt 90 s.
    dt = 90.0 if split == gdc.SPLIT_NONE else 480.0
    p = scheme(gdc, N, M, dt, split=split, cutoff=(3, 3, 3), adv=adv, lat_beta=0.5, lon_beta=0.25)
    ic = gdc.ic_seeded(N, M, seed=2)
    m, o = pair(p, ic)
    for n in (1, 9):
        m.run(n)
        o.step(n)
        s = o.get_state()
        u, v, gd = m.get_state()
        for a, b in ((gd, s["gd"]), (u, s["u"]), (v, s["v"])):
            assert rel_l2(a, b) <= 1e-12
            assert np.array_equal(interior(a), interior(b))
    assert m.diag() == o.diag()


def test_diffusion_parity(native):
    """Rossby-Haurwitz wave with diffusion (cutoff 4 as the reference's RH
    namelist; with cutoff 3 the kept cos(4 lon) mode is orthogonal to the
    wave-4 weights and the reference's s2 vanishes)."""
    N, M = 180, 91
    p = scheme(gdc, N, M, 480.0, diffusion=True, diffusion_coef=1.0e5, cutoff=(4, 4, 4))
    ic = gdc.ic_rossby_haurwitz(N, M)
    m, o = pair(p, ic)
    m.run(10)
    o.step(10)
    s = o.get_state()
    u, v, gd = m.get_state()
    for a, b in ((gd, s["gd"]), (u, s["u"]), (v, s["v"])):
        assert rel_l2(a, b) <= 1e-12
        assert np.array_equal(interior(a), interior(b))


@pytest.mark.slow
def test_seeded_360x181_one_day(native):
    """The seeded state on 360x181, dt=240 s, 360 steps, filter on, no topography."""
    N, M = 360, 181
    p = scheme(gdc, N, M, 240.0)
    ic = gdc.ic_seeded(N, M, seed=0)
    m, o = pair(p, ic)
    m0, _, _ = m.diag()
    o0, _, _ = o.diag()
    m.run(360)
    assert o.step(360) == 0
    s = o.get_state()
    u, v, gd = m.get_state()
    errs = {k: rel_l2(a, s[k]) for k, a in (("gd", gd), ("u", u), ("v", v))}
    assert all(e <= 1e-12 for e in errs.values()), errs
    for k, a in (("gd", gd), ("u", u), ("v", v)):
        assert np.array_equal(interior(a), interior(s[k])), k
    m1, _, _ = m.diag()
    o1, _, _ = o.diag()
    drift_g, drift_o = (m1 - m0) / m0, (o1 - o0) / o0
    assert abs(drift_g - drift_o) <= 1e-13, (drift_g, drift_o)


def test_graph_replay_matches_direct_launches(native):
    """A model step replayed from the CUDA graph is bitwise the launch-by-launch step."""
    N, M = 180, 91
    p = scheme(gdc, N, M, 480.0)
    ic = gdc.ic_seeded(N, M, seed=4)
    a = gdc.Batch(p)
    b = gdc.Batch(p)
    ia = a.add(N, M, 480.0, 6, *ic)
    ib = b.add(N, M, 480.0, 6, *ic)
    a.step(6)
    b.profile(6)
    for x, y in zip(a.get_state(ia), b.get_state(ib)):
        assert np.array_equal(x, y)


def test_rescale_guard_parity(native):
    """Zonal flow over mountains: gd+ghs is constant along each row, so the
    reference's s1 on filtered rows is rounding noise.  With the guard
    (filter_rescale_rtol) both paths skip that noise rescale and agree."""
    N, M = 360, 181
    p = scheme(gdc, N, M, 240.0, cutoff=(8,) * 10)
    p.filter_rescale_rtol = 1e-9
    ic = gdc.ic_seeded(N, M, seed=1, lmax=0, gd0=5960 * gdc.G, gd_rms=0, psi_rms=0, u0=20.0, n_mountains=3)
    m, o = pair(p, ic)
    m.run(5)
    o.step(5)
    s = o.get_state()
    u, v, gd = m.get_state()
    assert rel_l2(gd, s["gd"]) <= 1e-12 and rel_l2(u, s["u"]) <= 1e-11
    assert rel_l2(v, s["v"]) <= 1e-9  # v starts at 0: relative to a small field


def test_nan_member_is_evicted(native):
    N, M = 180, 91
    p = scheme(gdc, N, M, 480.0)
    good = gdc.ic_seeded(N, M, seed=1)
    bad = [x.copy() for x in good]
    bad[2][40, 40] = np.nan  # NaN in gd: the host-side fault
    b = gdc.Batch(p)
    ig = b.add(N, M, 480.0, 4, *good)
    ib = b.add(N, M, 480.0, 4, *bad)
    b.step(2)
    b.sync()
    _, fin_b, nan_b = b.info(ib)
    assert fin_b and nan_b >= 0
    b.step(2)
    b.sync()
    s, fin_g, nan_g = b.info(ig)
    assert s == 4 and fin_g and nan_g == -1
    m = gdc.Model(p)
    m.set_state(*bad)
    m.step(1)
    with pytest.raises(gdc.GdcError) as e:
        m.sync()
    assert e.value.code == gdc.E_NAN


def test_device_ic_run_parity_shallow_water_wave(native):
    """The shallow-water Rossby wave generated in device memory and stepped
    in a batch is bitwise the oracle's run from the host-built state."""
    N, M = 144, 73
    p = scheme(gdc, N, M, 300.0, subcycles=4, cutoff=(3, 3, 3))
    b = gdc.Batch(p)
    mid = b.add_ic(N, M, 300.0, 12, gdc.ic_spec(gdc.IC_SHALLOW_WATER_WAVES))
    o = OracleModel.from_params(p)
    o.set_state(*gdc.ic_shallow_water_waves(N, M))
    b.step(12)
    b.sync()
    o.step(12)
    s = o.get_state()
    for a, r in zip(b.get_state(mid), (s["u"], s["v"], s["gd"])):
        assert np.array_equal(interior(a), interior(r))
    assert b.diag(mid) == o.diag()
    b.close()


@pytest.mark.parametrize("split", [gdc.SPLIT_CSP2, gdc.SPLIT_ISP])
def test_weno_split_blows_up_at_the_oracles_step(native, split):
    """The reference's WENO (zero split fluxes on the pole rows, no lat
    halos) is unstable under csp2 and isp splitting: the oracle's total
    energy turns NaN within a few steps on this state, and the CUDA path
    stops at the same step."""
    N, M = 180, 91
    p = scheme(gdc, N, M, 480.0, split=split, cutoff=(3, 3, 3), adv=gdc.ADV_WENO)
    ic = gdc.ic_seeded(N, M, seed=2)
    m, o = pair(p, ic)
    bad = next(k for k in range(1, 13) if o.step(1) != 0)
    with pytest.raises(gdc.GdcError, match=f"NaN at step {bad}"):
        m.run(12)
    m.close()


def test_weno_batch_mixed_grids_parity_and_fp32(native):
    """uv_adv_scheme weno in a batch of two grids (no splitting, dt 90 s:
    stable for these 12 steps): each FP64 member is bitwise the oracle's run
    (diffusion on, so the given-u/v path is exercised after each diffusion
    step); FP32 members stay within 1e-5 (gd relative L2) of FP64; other tile
    shapes are refused."""
    runs = {}
    grids = [(180, 91, 90.0), (200, 101, 90.0)]
    for prec in (gdc.FP64, gdc.FP32):
        p = scheme(gdc, 180, 91, 90.0, split=gdc.SPLIT_NONE, adv=gdc.ADV_WENO, cutoff=(3, 3, 3, 3), diffusion=True,
                   precision=prec)
        b = gdc.Batch(p)
        with pytest.raises(gdc.GdcError):
            b.set_tile(16, 64)
        ids = [b.add(N, M, dt, 12, *gdc.ic_seeded(N, M, seed=N)) for N, M, dt in grids]
        b.step(12)
        b.sync()
        runs[prec] = [b.get_state(i) for i in ids]
        b.close()
    for (N, M, dt), st in zip(grids, runs[gdc.FP64]):
        o = OracleModel.from_params(scheme(gdc, N, M, dt, split=gdc.SPLIT_NONE, adv=gdc.ADV_WENO, cutoff=(3, 3, 3, 3),
                                           diffusion=True))
        o.set_state(*gdc.ic_seeded(N, M, seed=N))
        o.step(12)
        s = o.get_state()
        for a, r in zip(st, (s["u"], s["v"], s["gd"])):
            assert np.array_equal(interior(a), interior(r))
    for a, b in zip(runs[gdc.FP32], runs[gdc.FP64]):
        assert rel_l2(a[2], b[2]) <= 1e-5


def test_iap_and_derived_state_read_back_bitwise(native):
    """gdc_get_iap / gdc_get_state after steps: iap u, iap v, iap gd = sqrt(gd)
    and the recovered u, v equal the oracle's state arrays bit for bit."""
    N, M = 180, 91
    p = scheme(gdc, N, M, 480.0, cutoff=(3, 3, 3))
    m, o = pair(p, gdc.ic_seeded(N, M, seed=8))
    m.run(3)
    o.step(3)
    s = o.get_state()
    iu, iv, ig = m.get_iap()
    u, v, gd = m.get_state()
    for a, name in ((iu, "iu"), (iv, "iv"), (ig, "ig"), (u, "u"), (v, "v"), (gd, "gd")):
        assert np.array_equal(interior(a), interior(s[name])), name
    m.close()


def test_large_filter_cutoffs_match_oracle(native):
    """Cutoffs up to num_lon/2 - 1 (the reference's factor rows hold 2 (c+1)
    <= num_lon entries): every mode kept (c = 71 at 144 columns, with the
    Nyquist coefficient), 61 and 35 kept pairs, and the usual 4 -- the
    tendencies of every pass and 5 steps (rows split over block pairs by
    default) are bitwise the oracle's; c = 72 is refused."""
    N, M = 144, 73
    cut = (71, 60, 35, 10, 4)
    p = scheme(gdc, N, M, 600.0, cutoff=cut)
    ic = gdc.ic_seeded(N, M, seed=4)
    for pass_ in (0, 1, 2):
        m, o = pair(p, ic)
        for name, a, b in zip(("du", "dv", "dgd"), m.tendency(pass_), o.tendency(pass_)):
            assert np.array_equal(interior(a), interior(b)), (pass_, name, rel_l2(a, b))
        m.close()
    m, o = pair(p, ic)
    m.run(5)
    o.step(5)
    s = o.get_state()
    for a, name in zip(m.get_state(), ("u", "v", "gd")):
        assert np.array_equal(interior(a), interior(s[name])), name
    assert m.diag() == o.diag()
    m.close()
    b = gdc.Batch(p)
    with pytest.raises(gdc.GdcError):
        b.add(N, M, 600.0, 1, *ic, cutoff=[72] + [4] * 4)
    b.close()


@pytest.mark.parametrize("grid", [(16, 11), (20, 9)])
def test_tiny_grids_match_oracle(native, grid):
    """Grids smaller than one tile (16 or 20 columns: one partial tile per
    row band, the wrap seam inside it) with two filtered rows per pole:
    10 csp2 steps bitwise the oracle's."""
    N, M = grid
    p = scheme(gdc, N, M, 1800.0, cutoff=(2, 1))
    ic = gdc.ic_seeded(N, M, seed=9, lmax=2)
    m, o = pair(p, ic)
    m.run(10)
    o.step(10)
    s = o.get_state()
    for a, name in zip(m.get_state(), ("u", "v", "gd")):
        assert np.array_equal(interior(a), interior(s[name])), (name, rel_l2(a, s[name]))
    assert m.diag() == o.diag()
    m.close()
