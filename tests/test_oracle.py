"""Oracle self-checks (CPU): the restatement against known answers.

The reference ships no golden vectors and cannot be built here, so the
oracle is pinned by identities the reference's own code implies:
FFTPACK 5.1's coefficient packing (checked against numpy's FFT), the
filter's row sets and kept modes, exact mass conservation with the filter
off, and the antisymmetry identities of check_antisymmetry
(src/dycore_mod.F90:794-851).
"""
import numpy as np
import pytest

from helpers import interior
from oracle.oracle import OracleModel


def test_correctly_rounded_sum():
    """The oracle's sums are correctly rounded (compared with math.fsum)."""
    import math
    from oracle.oracle import fsum
    rng = np.random.default_rng(0)
    for trial in range(200):
        n = int(rng.integers(1, 3000))
        x = rng.standard_normal(n) * np.exp(rng.uniform(-40, 40, n))
        if trial % 3 == 0:  # heavy cancellation
            x = np.concatenate([x, -x[: n // 2] * (1 + 1e-15)])
        assert fsum(x) == math.fsum(x)
    assert fsum([1e16, 1.0, -1e16]) == 1.0
    assert fsum([]) == 0.0


def fftpack_projection(x, c):
    """FFTPACK rfft1f -> keep packed indices 1..2(c+1) -> rfft1b, via numpy."""
    N = len(x)
    X = np.fft.rfft(x)
    Y = np.zeros_like(X)
    Y[: c + 1] = X[: c + 1]
    Y[c + 1] = X[c + 1].real
    return np.fft.irfft(Y, n=N)


@pytest.mark.parametrize("N,c", [(360, 4), (180, 3), (720, 8), (96, 1)])
def test_filter_matches_fftpack_packing(N, c):
    M = 31
    o = OracleModel(N, M, 100.0, cutoff=[c])
    rng = np.random.default_rng(N + c)
    x = np.zeros(N + 4)
    x[2:-2] = rng.standard_normal(N)
    y = o.filter_row(0, 2, x)  # full row Fortran 2 is flagged by cutoff entry 1
    ref = fftpack_projection(x[2:-2], c)
    assert np.max(np.abs(y[2:-2] - ref)) < 1e-13 * np.max(np.abs(x))
    # halos untouched
    assert np.all(y[:2] == 0) and np.all(y[-2:] == 0)


def test_filter_kept_modes():
    N, c = 360, 4
    o = OracleModel(N, 31, 100.0, cutoff=[c])
    lam = 2 * np.pi * np.arange(N) / N
    def run(f):
        x = np.zeros(N + 4)
        x[2:-2] = f
        return o.filter_row(0, 2, x)[2:-2]
    for k in range(0, c + 1):
        assert np.allclose(run(np.cos(k * lam)), np.cos(k * lam), atol=1e-13)
        assert np.allclose(run(np.sin(k * lam)), np.sin(k * lam), atol=1e-13)
    # the cosine of wavenumber c+1 passes, its sine does not (quirk of the
    # factor indices 1..2(c+1), src/filter_mod.F90:79-84)
    assert np.allclose(run(np.cos((c + 1) * lam)), np.cos((c + 1) * lam), atol=1e-13)
    assert np.allclose(run(np.sin((c + 1) * lam)), 0, atol=1e-13)
    for k in (c + 2, c + 7, N // 2 - 1):
        assert np.allclose(run(np.cos(k * lam)), 0, atol=1e-13)
        assert np.allclose(run(np.sin(k * lam)), 0, atol=1e-13)


def test_filter_row_sets():
    """South filters half rows 1..n, north only n-1 half rows (the flag
    index of src/filter_mod.F90:56 is one past the factor index of :95)."""
    N, M, n = 360, 181, 5
    o = OracleModel(N, M, 240.0, cutoff=[4] * n)
    ff, fh, cf, ch = o.filter_flags()
    assert [j for j in range(M) if ff[j]] == list(range(1, n + 1)) + list(range(M - 1 - n, M - 1))
    assert [j for j in range(M - 1) if fh[j]] == list(range(0, n)) + list(range(M - n, M - 1))
    assert all(cf[j] == 4 for j in range(M) if ff[j])
    assert all(ch[j] == 4 for j in range(M - 1) if fh[j])
    # a half row whose factor row is unset keeps nothing
    o2 = OracleModel(N, M, 240.0, cutoff=[4, 0, 3])
    ff, fh, cf, ch = o2.filter_flags()
    assert fh[M - 3] == 1 and ch[M - 3] == -1  # flagged by entry 3, factors of entry 2 (zero)


def _seeded(N, M, seed=0):
    import gdc
    return gdc.ic_seeded(N, M, seed=seed)


@pytest.mark.parametrize("split", [0, 2, 3])
def test_mass_conserved_without_filter(split):
    """With the filter and diffusion off the flux-form mass divergence and
    its pole caps telescope: total mass is conserved to round-off."""
    N, M = 72, 37
    u, v, gd, ghs = _seeded(N, M, seed=3)
    o = OracleModel(N, M, 600.0, subcycles=4, split_scheme=split, use_zonal_tend_filter=0, cutoff=[])
    o.set_state(u, v, gd, ghs)
    m0, _, _ = o.diag()
    assert o.step(12) == 0
    m1, _, _ = o.diag()
    assert abs(m1 - m0) / m0 < 1e-13


def test_antisymmetry_identities():
    """check_antisymmetry's four sums vanish to round-off relative to the
    magnitudes of the terms they combine (filter off)."""
    N, M = 72, 37
    u, v, gd, ghs = _seeded(N, M, seed=5)
    o = OracleModel(N, M, 600.0, use_zonal_tend_filter=0, cutoff=[])
    o.set_state(u, v, gd, ghs)
    du, dv, dgd = o.tendency(0)
    s = o.antisymmetry()
    scale = np.sqrt(np.sum(interior(du) ** 2) + np.sum(interior(dv) ** 2)) * 1e4 * N * M
    assert np.all(np.abs(s) < 1e-10 * scale), s


def test_energy_conserving_without_filter():
    """The quadratic-conservation beta keeps total energy nearly constant
    (the design goal of the IAP scheme); with qcon off it drifts more."""
    N, M = 72, 37
    u, v, gd, ghs = _seeded(N, M, seed=7)
    def drift(qcon):
        o = OracleModel(N, M, 300.0, subcycles=4, split_scheme=0, qcon_modified=qcon, use_zonal_tend_filter=0,
                        cutoff=[])
        o.set_state(u, v, gd, ghs)
        _, e0, _ = o.diag()
        o.step(20)
        _, e1, b = o.diag()
        return abs(e1 - e0) / e0, b
    d_on, b_on = drift(1)
    d_off, b_off = drift(0)
    assert d_on < 1e-10
    assert b_off == 1.0 and b_on != 1.0


def test_steady_geostrophic_stays_steady():
    import gdc
    N, M = 72, 37
    u, v, gd, ghs = gdc.ic_steady_geostrophic(N, M)
    o = OracleModel(N, M, 600.0, subcycles=4, split_scheme=2, cutoff=[3, 3])
    o.set_state(u, v, gd, ghs)
    o.step(24)
    s = o.get_state()
    err = np.sqrt(np.mean((interior(s["gd"]) - interior(gd)) ** 2)) / np.mean(interior(gd))
    assert err < 1e-3, err  # truncation error of a 5-degree grid after 4 hours


def test_history_fields_known_answers():
    """A-grid wind, gh, div and vor of the oracle (src/history_mod.F90:101-108,
    src/diag_mod.F90:49-68) on the seeded state: its u, v come from a
    streamfunction differenced at C-grid corners, so the discrete divergence
    vanishes; the vorticity is that streamfunction's discrete Laplacian-like
    field (nonzero); u is 0 on the pole rows; gh = gd + ghs exactly."""
    N, M = 72, 37
    u, v, gd, ghs = _seeded(N, M, seed=4)
    o = OracleModel(N, M, 600.0, subcycles=4, split_scheme=2, cutoff=[4])
    o.set_state(u, v, gd, ghs)
    h = o.history()
    a, dlon = 6.37122e6, 2 * np.pi / N
    scale = np.abs(u).max() / (a * dlon)
    assert np.abs(h["div"]).max() < 1e-12 * scale
    assert np.abs(interior(h["vor"])).max() > 1e-3 * scale
    assert np.array_equal(interior(h["gh"]), interior(gd) + interior(ghs))
    assert np.all(h["u_a"][2] == 0) and np.all(h["u_a"][M + 1] == 0)
    # A-grid averages: interior columns and the periodic wrap
    assert np.array_equal(h["u_a"][5, 3:N + 2], 0.5 * (u[5, 3:N + 2] + u[5, 2:N + 1]))
    assert h["u_a"][5, 2] == 0.5 * (u[5, 2] + u[5, N + 1])
    assert np.array_equal(h["v_a"][2, 2:N + 2], 0.5 * v[2, 2:N + 2])          # south pole row
    assert np.array_equal(h["v_a"][M + 1, 2:N + 2], 0.5 * v[M, 2:N + 2])      # north pole row


def _weno2(fp1, fp2, fp3, fn2, fn3, fn4):
    """weno_2nd_order_pass (src/weno_mod.F90:249-298) restated with numpy."""
    eps = 1.0e-6

    def part(fs1, fs2, b1, b2):  # stencil fluxes, smoothness indicators
        w1 = (1.0 / 3.0) / (eps + b1) ** 2
        w2 = (2.0 / 3.0) / (eps + b2) ** 2
        sw = w1 + w2
        return (w1 / sw) * fs1 + (w2 / sw) * fs2

    f = part(-0.5 * fp1 + 1.5 * fp2, 0.5 * fp2 + 0.5 * fp3, (fp2 - fp1) ** 2, (fp3 - fp2) ** 2)
    return f + part(-0.5 * fn4 + 1.5 * fn3, 0.5 * fn3 + 0.5 * fn2, (fn3 - fn4) ** 2, (fn2 - fn3) ** 2)


def weno_terms(s, N, M):
    """-(u_adv_lon + u_adv_lat), -(v_adv_lon + v_adv_lat) of src/weno_mod.F90
    (weno_order 2) restated with numpy on 0-based interior arrays: zero
    split fluxes off the interior rows, u_adv_lon over half_dlon."""
    Mh, A = M - 1, 6.37122e6
    dlon, dlat = 2 * np.pi / N, np.pi / Mh
    full_lat = -0.5 * np.pi + np.arange(M) * dlat
    full_lat[-1] = 0.5 * np.pi
    half_lat = full_lat[:-1] + 0.5 * dlat
    hdlon = (A * dlon * np.cos(half_lat))[:, None]
    fdlat = (A * dlat * np.cos(full_lat))[:, None]
    hdlat = (A * dlat * np.cos(half_lat))[:, None]
    u, v, iu, iv = (interior(s[k]) for k in ("u", "v", "iu", "iv"))
    sh = lambda a, k: np.roll(a, -k, axis=1)  # a[:, i + k]
    w = lambda f, g, k: _weno2(sh(f, k - 1), sh(f, k), sh(f, k + 1), sh(g, k), sh(g, k + 1), sh(g, k + 2))
    # zonal, u points
    fp, fn = 0.5 * (u + 20.0) * iu, 0.5 * (u - 20.0) * iu
    fu = w(fp, fn, 0)
    ual = (fu - sh(fu, -1) - (sh(u, 1) - sh(u, -1)) * iu * 0.25)[:Mh] / hdlon
    # zonal, v points
    um = sh(u, -1)
    ub = 0.25 * (um[:-1] + um[1:] + u[:-1] + u[1:])
    fpv, fnv = 0.5 * (ub + 20.0) * iv, 0.5 * (ub - 20.0) * iv
    fv = w(fpv, fnv, 0)
    val = (fv - sh(fv, -1) - (u[:-1] + u[1:] - um[:-1] - um[1:]) * iv * 0.25) / hdlon
    # meridional, u points: split fluxes on rows 1..M-2, zero elsewhere
    pad = lambda a: np.vstack([np.zeros((2, N)), a, np.zeros((2, N))])  # row r -> r + 2
    vb = np.zeros((M, N))
    vs = sh(v, 1)
    vb[1:M - 1] = 0.25 * (v[:-1] + v[1:] + vs[:-1] + vs[1:])
    mp, mn = 0.5 * (vb + 20.0) * iu, 0.5 * (vb - 20.0) * iu
    mp[[0, M - 1]] = 0.0
    mn[[0, M - 1]] = 0.0
    P, Q = pad(mp), pad(mn)
    g = np.zeros((M + 4, N))
    for r in range(1, M - 1):
        g[r + 2] = _weno2(P[r + 1], P[r + 2], P[r + 3], Q[r + 2], Q[r + 3], Q[r + 4])
    vm = sh(v, -1)
    uat = np.zeros((M, N))
    for j in range(1, M - 1):
        uat[j] = (g[j + 2] - g[j + 1] - (vm[j] + v[j] - vm[j - 1] - v[j - 1]) * iu[j] * 0.25) / fdlat[j]
    # meridional, v points
    pv, nv = pad(0.5 * (v + 20.0) * iv), pad(0.5 * (v - 20.0) * iv)
    gv = np.zeros((Mh + 4, N))
    for r in range(Mh):
        gv[r + 2] = _weno2(pv[r + 1], pv[r + 2], pv[r + 3], nv[r + 2], nv[r + 3], nv[r + 4])
    V = pad(v)
    vat = np.zeros((Mh, N))
    for j in range(Mh):
        vat[j] = (gv[j + 2] - gv[j + 1] - (V[j + 3] - V[j + 1]) * iv[j] * 0.25) / hdlat[j]
    du = np.zeros((M, N))
    du[1:M - 1] = -ual[1:M - 1] - uat[1:M - 1]
    return du, -val - vat


@pytest.mark.parametrize("seed", [6, 9])
def test_weno_tendency_matches_restatement(seed):
    """The oracle's WENO advection (slow pass, filter off) against a numpy
    restatement of src/weno_mod.F90 with the reference's index choices."""
    N, M = 72, 37
    u, v, gd, ghs = _seeded(N, M, seed=seed)
    o = OracleModel(N, M, 600.0, subcycles=4, split_scheme=2, uv_adv_scheme=2, use_zonal_tend_filter=0,
                    cutoff=[])
    o.set_state(u, v, gd, ghs)
    du, dv, dgd = o.tendency(2)
    ru, rv = weno_terms(o.get_state(), N, M)
    assert np.max(np.abs(interior(du) - ru)) <= 1e-12 * np.max(np.abs(ru))
    assert np.max(np.abs(interior(dv) - rv)) <= 1e-12 * np.max(np.abs(rv))
    assert np.all(interior(dgd) == 0)


def test_weno_uniform_zonal_flow_known_answers():
    """u = u0 cos(lat), v = 0 (steady geostrophic state): iap v is zero, so
    every v-point split flux and term vanishes exactly; every u-point input
    is constant along a row, so the zonal terms vanish (f_u(i) = f_u(i-1)
    exactly) and du is the same in every column of a row; the meridional
    term is nonzero (iap u varies with latitude)."""
    import gdc
    N, M = 72, 37
    u, v, gd, ghs = gdc.ic_steady_geostrophic(N, M)
    o = OracleModel(N, M, 600.0, subcycles=4, split_scheme=2, uv_adv_scheme=2, use_zonal_tend_filter=0,
                    cutoff=[])
    o.set_state(u, v, gd, ghs)
    du, dv, _ = o.tendency(2)
    assert np.all(interior(dv) == 0)
    d = interior(du)
    assert np.all(d == d[:, :1])
    assert np.abs(d[1:M - 1]).min() > 0
    ru, _ = weno_terms(o.get_state(), N, M)
    assert np.max(np.abs(d - ru)) <= 1e-12 * np.max(np.abs(ru))


def test_diffusion_known_answers():
    """ordinary_diffusion (src/diffusion_mod.F90:74-217, order 2): its
    Laplacian is in flux form with zonal-sum pole caps, so with the tendency
    filter off the total mass stays exact; it dissipates energy that the
    qcon scheme otherwise conserves; and a resting uniform layer stays
    exactly at rest and uniform."""
    N, M = 72, 37
    ic = _seeded(N, M, seed=3)

    def run(diff):
        o = OracleModel(N, M, 600.0, subcycles=4, split_scheme=2, use_zonal_tend_filter=0, cutoff=[],
                        use_diffusion=int(diff), diffusion_coef=1.0e5)
        o.set_state(*ic)
        m0, e0, _ = o.diag()
        assert o.step(12) == 0
        m1, e1, _ = o.diag()
        return (m1 - m0) / m0, (e1 - e0) / e0

    dm, de = run(True)
    _, de0 = run(False)
    assert abs(dm) < 1e-14
    assert de < -1e-7 and abs(de0) < 1e-9
    import gdc
    u, v, gd, ghs = gdc.ic_seeded(N, M, seed=0, lmax=0, gd_rms=0, psi_rms=0)
    o = OracleModel(N, M, 600.0, subcycles=4, split_scheme=2, cutoff=[3, 3], use_diffusion=1,
                    diffusion_coef=1.0e5)
    o.set_state(u, v, gd, ghs)
    assert o.step(5) == 0
    s = o.get_state()
    assert np.all(interior(s["u"]) == 0) and np.all(interior(s["v"]) == 0)
    assert np.array_equal(interior(s["gd"]), interior(gd))


def test_upwind_with_zero_beta_is_centred():
    """The upwind advection (src/dycore_mod.F90:393-415, :450-469) with
    uv_adv_upwind_lon/lat_beta = 0 is the centred scheme rewritten:
    u2 (ic + ip) - u1 (ic + im) - (u2 - u1) ic = u2 ip - u1 im.  Equal to
    round-off; with beta > 0 it differs (the upwind dissipation)."""
    N, M = 72, 37
    ic = _seeded(N, M, seed=12)

    def slow(adv, beta):
        o = OracleModel(N, M, 600.0, split_scheme=2, uv_adv_scheme=adv, upwind_lon_beta=beta, upwind_lat_beta=beta,
                        use_zonal_tend_filter=0, cutoff=[])
        o.set_state(*ic)
        du, dv, _ = o.tendency(2)
        return interior(du), interior(dv)

    cu, cv = slow(0, 0.0)
    uu, uv = slow(1, 0.0)
    assert np.max(np.abs(uu - cu)) <= 1e-12 * np.max(np.abs(cu))
    assert np.max(np.abs(uv - cv)) <= 1e-12 * np.max(np.abs(cv))
    bu, _ = slow(1, 0.5)
    assert np.max(np.abs(bu - cu)) > 1e-3 * np.max(np.abs(cu))
