"""Initial conditions generated in device memory (gdc_batch_add_ic) against
the host generators (gdc_ic_*): the reference's barotropic test cases
(src/test_cases/barotropic/*_test_mod.F90: Rossby-Haurwitz wave, steady
geostrophic flow, mountain zonal flow, shallow-water wave) and the seeded
harmonic state, with and without white noise.

The separable states (the reference's four) are products of host factor
tables or exact operations on the mesh: bitwise equal, and so are runs
started from them.  The seeded state and the noise evaluate sin, cos, exp,
log per point and sum the RMS normalisation in another order, so they
agree to a few units in the last place: gd within 1e-13 of its maximum, u
within 1e-12 (the seeded u is a difference of a streamfunction ~1e7), v
within 1e-10 (v = dpsi/dlon / (a cos lat): on the rows next to the poles
1/cos amplifies psi's last bits).  Runs started from them stay as close as
runs started from the host state and from the host state with gd perturbed
by one unit in the last place: the filter's s1/s2 rescale makes the step
itself amplify last-bit differences on some rows.
"""
import numpy as np
import pytest

import gdc
from helpers import interior, rel_l2, rel_linf, scheme

pytestmark = pytest.mark.gpu


def stable_scheme(N, M, precision):
    """A CFL-stable scheme for the grid, with the filter's rescale guard on:
    without it the reference's s1/s2 rescale of rows whose filtered
    tendency is rounding noise (zonal flows) amplifies last-bit differences
    of the initial state."""
    dt, cutoff = (240.0, (8,) * 10) if N >= 360 else (480.0, (4, 4, 4, 4))
    p = scheme(gdc, N, M, dt, cutoff=cutoff, precision=precision)
    p.filter_rescale_rtol = 1e-9
    return p, dt


def ulp_perturbed(ic):
    u, v, gd, ghs = (a.copy() for a in ic)
    gd[2:-2, 2:-2] *= 1 + 2.0 ** -52
    return u, v, gd, ghs


def host_ic(kind, N, M, spec):
    if kind == gdc.IC_ROSSBY_HAURWITZ:
        ic = gdc.ic_rossby_haurwitz(N, M)
    elif kind == gdc.IC_STEADY_GEOSTROPHIC:
        ic = gdc.ic_steady_geostrophic(N, M)
    elif kind == gdc.IC_MOUNTAIN_ZONAL_FLOW:
        ic = gdc.ic_mountain_zonal_flow(N, M)
    elif kind == gdc.IC_SHALLOW_WATER_WAVES:
        ic = gdc.ic_shallow_water_waves(N, M)
    else:
        ic = gdc.ic_seeded(N, M, seed=spec.seed, lmax=spec.lmax, gd0=spec.gd0, gd_rms=spec.gd_rms,
                           psi_rms=spec.psi_rms, u0=spec.u0, n_mountains=spec.n_mountains,
                           mountain_height=spec.mountain_height, mountain_radius_deg=spec.mountain_radius_deg)
    if spec.noise_sigma > 0:
        gdc.ic_add_noise(ic[2], N, M, spec.noise_seed, spec.noise_sigma)
    return ic


CASES = [
    (gdc.IC_ROSSBY_HAURWITZ, {}),
    (gdc.IC_STEADY_GEOSTROPHIC, {}),
    (gdc.IC_MOUNTAIN_ZONAL_FLOW, {}),
    (gdc.IC_SEEDED, {"seed": 11}),
    (gdc.IC_SEEDED, {"seed": 5, "n_mountains": 3, "u0": 15.0, "lmax": 9}),
    (gdc.IC_SEEDED, {"seed": 2, "noise_seed": 77, "noise_sigma": 3.0}),
    (gdc.IC_ROSSBY_HAURWITZ, {"noise_seed": 4, "noise_sigma": 10.0}),
    (gdc.IC_SHALLOW_WATER_WAVES, {}),
]
# Built from host factor tables or exact operations only: bitwise equal.
SEPARABLE = (gdc.IC_ROSSBY_HAURWITZ, gdc.IC_STEADY_GEOSTROPHIC, gdc.IC_MOUNTAIN_ZONAL_FLOW,
             gdc.IC_SHALLOW_WATER_WAVES)


@pytest.mark.parametrize("N,M", [(360, 181), (200, 101)])
@pytest.mark.parametrize("kind,kw", CASES)
def test_device_ic_matches_host_fp64(native, N, M, kind, kw):
    spec = gdc.ic_spec(kind, **kw)
    ic = host_ic(kind, N, M, spec)
    p, dt = stable_scheme(N, M, gdc.FP64)
    b = gdc.Batch(p)
    ih = b.add(N, M, dt, 6, *ic)
    idv = b.add_ic(N, M, dt, 6, spec)
    ip = b.add(N, M, dt, 6, *ulp_perturbed(ic))
    hu, hv, hg = b.get_state(ih)
    du, dv, dg = b.get_state(idv)
    d0 = [rel_l2(x, y) for x, y in ((du, hu), (dv, hv), (dg, hg))]
    assert rel_linf(dg, hg) < 1e-13
    assert rel_linf(du, hu) < 1e-12 and rel_linf(dv, hv) < 1e-10
    exact = kind in SEPARABLE and spec.noise_sigma == 0
    if exact:
        for x, y in ((du, hu), (dv, hv), (dg, hg)):
            assert np.array_equal(interior(x), interior(y))
    assert np.all(interior(du)[[0, -1]] == 0)  # pole-row u
    # ghs through the history's gh = gd + ghs
    gh_h, gh_d = b.history(ih)["gh"], b.history(idv)["gh"]
    assert np.max(np.abs(interior(gh_d - dg) - interior(gh_h - hg))) <= 1e-12 * np.max(np.abs(interior(hg)))
    mh, eh, _ = b.diag(ih)
    md, ed, _ = b.diag(idv)
    assert abs(md - mh) <= 1e-13 * abs(mh) and abs(ed - eh) <= 1e-12 * abs(eh)
    b.step(6)
    b.sync()
    assert b.info(idv)[:2] == (6, True)
    # no more amplification than a last-bit perturbation, or than the
    # initial difference itself
    for x, y, z in zip(b.get_state(idv), b.get_state(ih), b.get_state(ip)):
        assert rel_l2(x, y) <= max(1e-13, 20 * rel_l2(z, y), 20 * max(d0))
        assert rel_l2(x, y) < 1e-9
        if exact:
            assert np.array_equal(x, y)
    b.close()


@pytest.mark.parametrize("kind,kw", [CASES[0], CASES[2], CASES[4]])
def test_device_ic_matches_host_fp32(native, kind, kw):
    N, M = 360, 181
    spec = gdc.ic_spec(kind, **kw)
    ic = host_ic(kind, N, M, spec)
    p, dt = stable_scheme(N, M, gdc.FP32)
    b = gdc.Batch(p)
    ih = b.add(N, M, dt, 6, *ic)
    idv = b.add_ic(N, M, dt, 6, spec)
    for x, y in zip(b.get_state(idv), b.get_state(ih)):
        assert rel_linf(x, y) < 1e-6
    b.step(6)
    b.sync()
    for x, y in zip(b.get_state(idv), b.get_state(ih)):
        assert rel_l2(x, y) < 1e-5
    b.close()


def test_device_ic_large_grid_seeded(native):
    """The 0.25-degree grid (1440 x 721) with mountains and noise."""
    N, M = 1440, 721
    spec = gdc.ic_spec(gdc.IC_SEEDED, seed=9, n_mountains=4, u0=10.0, noise_seed=1, noise_sigma=2.0)
    ic = host_ic(gdc.IC_SEEDED, N, M, spec)
    b = gdc.Batch(scheme(gdc, N, M, 60.0, subcycles=8, precision=gdc.FP64))
    ih = b.add(N, M, 60.0, 1, *ic)
    idv = b.add_ic(N, M, 60.0, 1, spec)
    hu, hv, hg = b.get_state(ih)
    du, dv, dg = b.get_state(idv)
    assert rel_linf(dg, hg) < 1e-13
    assert rel_linf(du, hu) < 1e-12 and rel_linf(dv, hv) < 1e-10
    b.close()


def test_device_ic_rejects_bad_specs(native):
    N, M = 180, 91
    b = gdc.Batch(scheme(gdc, N, M, 480.0, precision=gdc.FP64))
    for spec in (gdc.ic_spec(7), gdc.ic_spec(gdc.IC_SEEDED, lmax=65), gdc.ic_spec(gdc.IC_SEEDED, n_mountains=-1),
                 gdc.ic_spec(gdc.IC_ROSSBY_HAURWITZ, noise_sigma=-1.0)):
        with pytest.raises(gdc.GdcError):
            b.add_ic(N, M, 480.0, 2, spec)
    with pytest.raises(gdc.GdcError):
        b.add_ic(90, M, 480.0, 2, gdc.ic_spec(gdc.IC_SEEDED))  # num_lon not a multiple of 4
    assert b.active() == 0
    mid = b.add_ic(N, M, 480.0, 2, gdc.ic_spec(gdc.IC_SEEDED))
    assert b.active() == 1 and b.info(mid)[:2] == (0, False)
    b.close()
