"""Host-side pieces (no GPU): the C ABI's exports, the namelist reader, the
run length, the initial-condition hooks and the byte accounting."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

import gdc
from helpers import interior

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = Path(__file__).resolve().parent / "golden"


def test_library_exports_every_declared_symbol(native):
    decl = set(re.findall(r"\b(gdc_\w+)\s*\(", (ROOT / "include" / "gdc.h").read_text()))
    assert len(decl) > 30
    for name in sorted(decl):
        assert hasattr(native, name), name


def test_namelist_matches_reference_keys(native):
    p, tc, cn = gdc.read_namelist(GOLDEN / "namelist.mountain")
    assert (tc, cn) == ("mountain_zonal_flow", "mz.180x90.dt720")
    assert (p.num_lon, p.num_lat, p.time_step_size, p.subcycles) == (180, 90, 720.0, 8)
    assert p.split_scheme == gdc.SPLIT_CSP2 and p.uv_adv_scheme == gdc.ADV_UPWIND
    assert p.uv_adv_upwind_lat_beta == 0.1 and p.uv_adv_upwind_lon_beta == 0.0
    assert p.qcon_modified == 1 and p.use_zonal_tend_filter == 1
    assert list(p.zonal_tend_filter_cutoff_wavenumber)[:4] == [4, 4, 4, 0]
    assert p.run_days == 50 and gdc.steps_for_run(p) == 50 * 86400 // 720


def test_namelist_rejects_unknown_key(native):
    """gfortran rejects keys absent from /dycore_params/ (e.g. `days`)."""
    with pytest.raises(gdc.GdcError) as e:
        gdc.read_namelist(GOLDEN / "namelist.bad_key")
    assert "days" in str(e.value)


def test_defaults_follow_params_mod(native):
    p = gdc.default_params()
    assert p.subcycles == 4 and p.diffusion_order == 2 and p.uv_adv_upwind_lat_beta == 0.5
    assert p.use_zonal_tend_filter == 1 and p.uv_adv_scheme == gdc.ADV_CENTER_DIFF
    # the calling thread's current CUDA device (0 without one)
    import torch
    expect = torch.cuda.current_device() if torch.cuda.is_available() else 0
    assert p.device == expect


def test_seeded_state_is_nondivergent(native):
    """u, v from the streamfunction differenced at C-grid corners: the
    reference's discrete divergence (src/diag_mod.F90:49-58) vanishes."""
    N, M = 72, 37
    u, v, gd, ghs = gdc.ic_seeded(N, M, seed=4)
    G = gdc.G
    assert abs(np.sqrt(np.mean((interior(gd) - 8000 * G) ** 2)) - 100 * G) < 1e-6 * G
    assert np.all(u[2, :] == 0) and np.all(u[M + 1, :] == 0)  # pole rows
    dlon, dlat, a = 2 * np.pi / N, np.pi / (M - 1), 6.37122e6
    lat = -0.5 * np.pi + np.arange(M) * dlat
    hc = np.cos(lat[:-1] + 0.5 * dlat)
    div = []
    for j in range(1, M - 1):
        fc = np.cos(lat[j])
        ui = u[j + 2, 2:N + 2]
        um = u[j + 2, 1:N + 1]
        vp = v[j + 2, 2:N + 2] * hc[j]
        vm = v[j + 1, 2:N + 2] * hc[j - 1]
        div.append((ui - um) / (a * dlon * fc) + (vp - vm) / (a * dlat * fc))
    scale = np.abs(u).max() / (a * dlon)
    assert np.abs(np.array(div)).max() < 1e-12 * scale


def test_reference_ic_hooks(native):
    N, M = 72, 37
    u, v, gd, ghs = gdc.ic_rossby_haurwitz(N, M)
    assert np.all(u[2, :] == 0) and np.all(u[M + 1, :] == 0)
    assert abs(interior(gd).mean() - 8000 * gdc.G) < 0.2 * 8000 * gdc.G
    u, v, gd, ghs = gdc.ic_mountain_zonal_flow(N, M)
    assert interior(ghs).max() == pytest.approx(2000 * gdc.G, rel=0.05)
    assert np.all(np.abs(interior(v)) == 0)
    # periodic longitude halo as parallel_fill_halo leaves it
    assert np.array_equal(gd[:, 0], gd[:, N]) and np.array_equal(gd[:, N + 3], gd[:, 3])


def test_algorithmic_bytes(native):
    p = gdc.default_params(split_scheme=gdc.SPLIT_CSP2, subcycles=6, precision=gdc.FP32)
    # 8 predict_correct calls of 39 words (+6 compensation words in FP32)
    # and the diagnostics' read of the new level (7 words FP32, 4 FP64)
    assert gdc.algorithmic_bytes_per_gpt_step(p) == (45 * 8 + 7) * 4
    p.precision = gdc.FP64
    assert gdc.algorithmic_bytes_per_gpt_step(p) == (39 * 8 + 4) * 8
    assert gdc.member_bytes(p, 360, 181) > 20 * 360 * 181 * 8


def test_driver_prints_usage_without_arguments(native):
    """The dycore_test program (src/dycore_test.F90:15-18): no namelist
    argument is a usage error, exit status 1, before any device work."""
    import subprocess
    build = __import__("build")
    out = subprocess.run([str(build.OUT / "dycore_test")], capture_output=True, text=True, timeout=60)
    assert out.returncode == 1 and "Usage" in out.stdout
