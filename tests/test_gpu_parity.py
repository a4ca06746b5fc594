"""CUDA path vs the CPU oracle, through the C ABI (FP64 plain path).

The FP64 kernels are compiled without FMA contraction, so every point-wise
expression rounds exactly as the oracle's; the two differ only in the order
of their sums (filter s1/s2 and projections, pole caps, beta, diagnostics).

Tolerances (FP64): operator level (one space_operators call) relative L2
<= 1e-13 for du and dv, <= 1e-11 for dgd (on filtered rows s1 = sum of
dgd*(gd+ghs) inherits the near-cancellation of the row's mass flux, so the
rescale factor s1/s2 carries ~1e-12 of summation-order noise); one model
step <= 1e-12; config 0 (360x181, dt 240 s, csp2 with 6 subcycles, filter
4,4,4,4,4) after 360 steps: relative L2 of gd, u, v <= 1e-12, and the
total-mass drift equal to the oracle's within 1e-13.
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


@pytest.mark.parametrize("adv", [0, 1])
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
            continue
        tol = 1e-11 if name == "dgd" else 1e-13
        assert rel_l2(a, b) <= tol, (name, rel_l2(a, b))
        assert rel_linf(a, b) <= 100 * tol, (name, rel_linf(a, b))


@pytest.mark.parametrize("split", [gdc.SPLIT_NONE, gdc.SPLIT_CSP2, gdc.SPLIT_ISP])
def test_step_parity(native, split):
    N, M = 180, 91
    p = scheme(gdc, N, M, 480.0, split=split, cutoff=(3, 3, 3))
    ic = gdc.ic_seeded(N, M, seed=2)
    m, o = pair(p, ic)
    m.run(1)
    o.step(1)
    s = o.get_state()
    u, v, gd = m.get_state()
    for a, b in ((gd, s["gd"]), (u, s["u"]), (v, s["v"])):
        assert rel_l2(a, b) <= 1e-12
    m.run(9)
    o.step(9)
    s = o.get_state()
    u, v, gd = m.get_state()
    for a, b in ((gd, s["gd"]), (u, s["u"]), (v, s["v"])):
        assert rel_l2(a, b) <= 1e-12
    mg, eg, bg = m.diag()
    mo, eo, bo = o.diag()
    assert abs(mg - mo) / mo < 1e-13 and abs(eg - eo) / eo < 1e-12
    assert abs(bg - bo) < 1e-9


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


@pytest.mark.slow
def test_config0_360_steps(native):
    """Config 0: 360x181, dt=240 s, 360 steps, filter on, no topography."""
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
