"""Shared helpers for the parity tests: configurations and error norms."""
from __future__ import annotations

import numpy as np

G = 9.80616


def interior(a: np.ndarray) -> np.ndarray:
    return a[2:-2, 2:-2]


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    """Relative L2 norm of a - b over the interior (b is the reference)."""
    x, y = interior(a), interior(b)
    den = np.sqrt(np.sum(y * y))
    num = np.sqrt(np.sum((x - y) ** 2))
    return float(num / den) if den > 0 else float(num)


def rel_linf(a: np.ndarray, b: np.ndarray) -> float:
    x, y = interior(a), interior(b)
    den = np.max(np.abs(y))
    return float(np.max(np.abs(x - y)) / den) if den > 0 else float(np.max(np.abs(x - y)))


def scheme(gdc, N, M, dt, split=2, subcycles=6, cutoff=(4, 4, 4, 4, 4), adv=0, diffusion=False,
           diffusion_coef=1.0e5, precision=0, filt=True, qcon=True, lat_beta=0.5, lon_beta=0.0):
    return gdc.default_params(num_lon=N, num_lat=M, time_step_size=dt, subcycles=subcycles, split_scheme=split,
                              qcon_modified=int(qcon), uv_adv_scheme=adv, use_zonal_tend_filter=int(filt),
                              zonal_tend_filter_cutoff_wavenumber=list(cutoff), use_diffusion=int(diffusion),
                              diffusion_coef=diffusion_coef, precision=precision,
                              uv_adv_upwind_lat_beta=lat_beta, uv_adv_upwind_lon_beta=lon_beta)
