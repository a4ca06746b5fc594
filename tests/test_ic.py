"""Host initial conditions (CPU): the shallow-water Rossby wave of Shamir and
Paldor (src/test_cases/barotropic/shallow_water_waves_test_mod.F90) and the
Rossby-Haurwitz wave (rossby_haurwitz_wave_test_mod.F90:33-85) against
numpy restatements of the reference's formulas, the phase speeds against
the cubic they solve, and the oracle's propagation of the wave against the
analytic phase speed.
"""
import numpy as np
import pytest

import gdc
from helpers import interior
from oracle.oracle import OracleModel

G, A, OMEGA, H0 = 9.80616, 6371220.0, 7.29212e-5, 5.0e3
N_MODE, K = 5, 10


def mesh(N, M):
    dlat = np.pi / (M - 1)
    full_lat = -0.5 * np.pi + np.arange(M) * dlat
    full_lat[-1] = 0.5 * np.pi
    half_lat = full_lat[:-1] + 0.5 * dlat
    full_lon = np.arange(N) * (2 * np.pi / N)
    half_lon = full_lon + 0.5 * (2 * np.pi / N)
    return full_lat, half_lat, full_lon, half_lon


@pytest.mark.parametrize("flag", [0, 1, -1])
def test_sw_phase_speeds_are_cubic_roots(flag):
    """getPhaseSpeed's Cardano roots solve k^2 C^3 - En C - 2 g H0 omega / a^2 = 0."""
    sigma = 0.5 + np.sqrt(0.25 + K * K)
    En = G * H0 / A ** 2 * (N_MODE + sigma) ** 2
    d = 2 * G * H0 * OMEGA / A ** 2
    roots = np.sort(np.roots([K * K, 0.0, -En, -d]).real)
    c = gdc.sw_waves_phase_speed(flag)
    scale = max(abs(K * K * c ** 3), abs(En * c), d)
    assert abs(K * K * c ** 3 - En * c - d) < 1e-12 * scale
    want = {0: -np.min(np.abs(roots)), 1: roots[-1], -1: roots[0]}[flag]
    assert abs(c - want) < 1e-10 * abs(want)


def sw_amplitudes(lat, C):
    """getPsi + getAmplitudes (Rossby wave) restated with numpy."""
    sigma = 0.5 + np.sqrt(0.25 + K * K)
    a3 = sigma * (sigma + 1) * (sigma + 2)
    a4, a5 = a3 * (sigma + 3), a3 * (sigma + 3) * (sigma + 4)
    s, c, t = np.sin(lat), np.cos(lat), np.tan(lat)
    C5 = (4 * a5 * s ** 4 - 20 * a4 * s ** 2 + 15 * a3) * s / 15
    C5p = (4 * a5 * s ** 4 - 12 * a4 * s ** 2 + 3 * a3) * c / 3
    psi = 1e-8 * c ** sigma * C5
    dpsi = 1e-8 * c ** sigma * (-sigma * t * C5 + C5p)
    o2 = 2 * OMEGA
    Kp = (G * H0 + A ** 2 * C ** 2 * c ** 2) / (C * c)
    Km = (G * H0 - A ** 2 * C ** 2 * c ** 2) / (C * c)
    vt = (o2 * np.abs(Km) / c ** 2) ** 0.5 * psi
    ht = (o2 * np.abs(Km) * A ** 2 * H0 ** 2) ** 0.5 / Km * (dpsi + t * (0.5 * Kp / Km - o2 / C) * psi)
    ut = (o2 * s / C) * vt + (G / A / c / C) * ht
    return ut, K * vt, ht


@pytest.mark.parametrize("N,M", [(144, 73), (360, 181)])
def test_sw_fields_match_formulas(N, M):
    u, v, gd, ghs = gdc.ic_shallow_water_waves(N, M)
    full_lat, _, full_lon, half_lon = mesh(N, M)
    C = gdc.sw_waves_phase_speed(0)
    ut, vt, ht = sw_amplitudes(full_lat, C)
    eu = np.outer(ut, np.cos(K * half_lon))
    eu[[0, -1]] = 0.0  # pole rows (below 1e-100 in the reference) are zero
    # v's half row j takes the amplitude of full row j (getFields' indexing)
    ev = np.outer(vt[:M - 1], np.cos(K * full_lon - 0.5 * np.pi))
    eh = np.outer(ht, np.cos(K * full_lon))
    assert np.max(np.abs(interior(u) - eu)) <= 1e-12 * np.max(np.abs(eu))
    assert np.max(np.abs(interior(v) - ev)) <= 1e-12 * np.max(np.abs(ev))
    assert np.max(np.abs(interior(gd) - (G * eh + 5e4))) <= 1e-12 * G * np.max(np.abs(eh))
    assert np.all(ghs == 0)
    assert np.all(np.abs(np.outer(ut, np.ones(N))[[0, -1]]) < 1e-100)
    # periodic halos
    assert np.array_equal(u[:, :2], u[:, N:N + 2]) and np.array_equal(u[:, N + 2:], u[:, 2:4])


def test_rh_tables_match_direct_formula():
    N, M = 180, 91
    u, v, gd, _ = gdc.ic_rossby_haurwitz(N, M)
    full_lat, half_lat, full_lon, half_lon = mesh(N, M)
    R, omg, a, Om = 4.0, 7.848e-6, 6.37122e6, 2 * np.pi / 86400
    cl, sl = np.cos(full_lat), np.sin(full_lat)
    cl[[0, -1]] = 0.0
    sl[0], sl[-1] = -1.0, 1.0
    lon_h, lon_f = half_lon[None, :], full_lon[None, :]
    c_, s_ = cl[:, None], sl[:, None]
    eu = a * omg * (c_ + R * c_ ** (R - 1) * s_ ** 2 * np.cos(R * lon_h) - c_ ** (R + 1) * np.cos(R * lon_h))
    ch, sh = np.cos(half_lat)[:, None], np.sin(half_lat)[:, None]
    ev = -a * omg * R * ch ** (R - 1) * sh * np.sin(R * lon_f)
    A_ = 0.5 * omg * (2 * Om + omg) * c_ ** 2 + 0.25 * omg ** 2 * (
        (R + 1) * c_ ** (2 * R + 2) + (2 * R * R - R - 2) * c_ ** (2 * R) - 2 * R * R * c_ ** (2 * R - 2))
    B_ = 2 * (Om + omg) * omg * c_ ** R * (R * R + 2 * R + 2 - (R + 1) ** 2 * c_ ** 2) / (R + 1) / (R + 2)
    C_ = 0.25 * omg ** 2 * c_ ** (2 * R) * ((R + 1) * c_ ** 2 - R - 2)
    eg = 8.0e3 * G + a * a * (A_ + B_ * np.cos(R * lon_f) + C_ * np.cos(2 * R * lon_f))
    assert np.max(np.abs(interior(u) - eu)) <= 1e-13 * np.max(np.abs(eu))
    assert np.max(np.abs(interior(v) - ev)) <= 1e-13 * np.max(np.abs(ev))
    assert np.max(np.abs(interior(gd) - eg)) <= 1e-14 * np.max(np.abs(eg))


def test_oracle_propagates_sw_wave_at_its_phase_speed():
    """The wave is a linear solution travelling at C: after 12 hours the
    oracle's k = 10 mode of gd has moved by k C t to within 10 % (2.5 degree
    grid) and stayed in that mode; its amplitude stays within 25 % (the
    discrete state is not exactly balanced: gravity waves of a few hours'
    period ride on it)."""
    N, M, dt = 144, 73, 300.0
    u, v, gd, ghs = gdc.ic_shallow_water_waves(N, M)
    C = gdc.sw_waves_phase_speed(0)
    o = OracleModel(N, M, dt, subcycles=4, split_scheme=2, cutoff=[3, 3, 3])
    o.set_state(u, v, gd, ghs)
    nsteps = 144
    assert o.step(nsteps) == 0
    h0 = interior(gd) - 5e4
    h1 = interior(o.get_state()["gd"]) - 5e4
    f0, f1 = np.fft.rfft(h0, axis=1), np.fft.rfft(h1, axis=1)
    shift = np.angle(np.sum(f1[:, K] * np.conj(f0[:, K])))
    want = -K * C * nsteps * dt
    assert abs(shift - want) < 0.1 * abs(want)
    assert abs(np.linalg.norm(f1[:, K]) / np.linalg.norm(f0[:, K]) - 1) < 0.25
    f1[:, K] = 0
    assert np.linalg.norm(np.fft.irfft(f1, n=N, axis=1)) < 0.05 * np.linalg.norm(h1)


def test_oracle_seeded_state_is_the_library_state(native):
    """The oracle's copy of the seeded-state definition (used where the
    product library must not be loaded: the benchmark's reference arm) is
    bitwise the library's, noise included."""
    from oracle import oracle as O
    cases = [(360, 181, {}), (180, 91, dict(seed=3)),
             (72, 37, dict(seed=5, lmax=12, n_mountains=3, u0=20.0)),
             (144, 73, dict(lmax=0, gd_rms=0.0, psi_rms=0.0, u0=20.0, n_mountains=3, gd0=5960 * gdc.G))]
    for N, M, kw in cases:
        a, b = gdc.ic_seeded(N, M, **kw), O.ic_seeded(N, M, **kw)
        for x, y in zip(a, b):
            assert np.array_equal(x, y), (N, M)
        g1 = gdc.ic_add_noise(a[2].copy(), N, M, seed=1001, sigma=gdc.G)
        g2 = O.ic_add_noise(b[2].copy(), N, M, 1001, gdc.G)
        assert np.array_equal(g1, g2)


def test_reference_arm_worker_runs_without_the_product_library():
    """bench.py's reference arm: a worker process builds its members from
    the oracle alone, advances them, and reports that libgdc.so is not
    mapped in it."""
    import multiprocessing as mp
    import bench
    ctx = mp.get_context("spawn")
    a, b = ctx.Pipe()
    task = dict(N=72, M=37, dt=1200.0, nsteps=3, cutoff=[3, 3], seed=1000)
    pr = ctx.Process(target=bench._ref_worker, args=(b, [str(bench.ROOT)], [task]))
    pr.start()
    tag, mapped = a.recv()
    assert tag == "ready" and mapped is False
    a.send(5)  # more steps than the member's length: it stops at 3
    done, nan = a.recv()
    assert done == 72 * 37 * 3 and nan == 0
    a.send(None)
    pr.join(timeout=60)
    assert pr.exitcode == 0
