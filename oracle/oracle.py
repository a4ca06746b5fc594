"""ctypes wrapper of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use
this module, to check the CUDA path; the product never imports it.  Arrays use the
reference's padded layout, numpy shape (rows + 4, num_lon + 4).
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import build as _build

_libs = {}
_P = ctypes.POINTER(ctypes.c_double)


def lib(kind: str = "exact") -> ctypes.CDLL:
    """One build of the oracle: "exact" (correctly rounded sums,
    the filter as a projection -- the CUDA path's arithmetic), "ref" (the
    reference's order: plain running sums in its loop order; FFTPACK's
    transforms with fft=True) or "fast" (the reference-order arithmetic at
    -Ofast: the timed CPU baseline, never used to check)."""
    if kind is True:
        kind = "fast"
    elif kind is False:
        kind = "exact"
    if kind not in _libs:
        _build.build()
        L = ctypes.CDLL(str(_build.LIBS[kind][0]))
        vp, dp, i = ctypes.c_void_p, _P, ctypes.c_int
        ip = ctypes.POINTER(ctypes.c_int)
        L.gdo_create.restype = vp
        L.gdo_create.argtypes = [i, i, ctypes.c_double, i, i, i, i, ctypes.c_double, ctypes.c_double, i, ip, i,
                                 ctypes.c_double, i]
        L.gdo_destroy.argtypes = [vp]
        L.gdo_set_rescale_rtol.argtypes = [vp, ctypes.c_double]
        L.gdo_set_fft.argtypes = [vp, i]
        L.gdo_set_fft.restype = i
        L.gdo_rescale_record.argtypes = [vp, dp, ip, ip]
        ull, d = ctypes.c_ulonglong, ctypes.c_double
        L.gdo_ic_seeded.argtypes = [i, i, ull, i, d, d, d, d, i, d, d, dp, dp, dp, dp]
        L.gdo_ic_seeded.restype = i
        L.gdo_ic_add_noise.argtypes = [i, i, ull, d, dp]
        L.gdo_ic_add_noise.restype = i
        L.gdo_rfft_row.argtypes = [i, i, dp]
        L.gdo_rfft_row.restype = i
        L.gdo_fsum.argtypes = [dp, i]
        L.gdo_fsum.restype = ctypes.c_double
        L.gdo_set_state.argtypes = [vp, dp, dp, dp, dp]
        L.gdo_run_init.argtypes = [vp]
        L.gdo_step.argtypes = [vp, i]
        L.gdo_step.restype = i
        L.gdo_get_state.argtypes = [vp, dp, dp, dp, dp, dp, dp]
        L.gdo_diag.argtypes = [vp, dp, dp, dp]
        L.gdo_tendency.argtypes = [vp, i, dp, dp, dp]
        L.gdo_antisymmetry.argtypes = [vp, dp]
        L.gdo_history.argtypes = [vp, dp, dp, dp, dp, dp]
        L.gdo_filter_row.argtypes = [vp, i, i, dp]
        L.gdo_filter_flags.argtypes = [vp, ip, ip, ip, ip]
        _libs[kind] = L
    return _libs[kind]


def rfft(x, backward: bool = False) -> np.ndarray:
    """FFTPACK 5.1's rfft1f (or rfft1b) of one row, as the oracle restates it."""
    a = np.ascontiguousarray(x, dtype=np.float64).copy()
    if lib("ref").gdo_rfft_row(len(a), int(backward), _ptr(a)) != 0:
        raise ValueError(f"length {len(a)} has a prime factor above 5")
    return a


def _ptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_P)


def fsum(x) -> float:
    """The oracle's correctly rounded summation."""
    a = np.ascontiguousarray(x, dtype=np.float64)
    return lib().gdo_fsum(_ptr(a), len(a))


G = 9.80616


def ic_seeded(N, M, seed=0, lmax=6, gd0=8000 * G, gd_rms=100 * G, psi_rms=1.0e7, u0=0.0, n_mountains=0,
              mountain_height=2000.0, mountain_radius_deg=20.0):
    """The benchmark's seeded state (padded layout), built by the oracle
    without the product library; bitwise the library's gdc_ic_seeded."""
    u, v, gd, ghs = _pad(M, N), _pad(M - 1, N), _pad(M, N), _pad(M, N)
    rc = lib("exact").gdo_ic_seeded(N, M, seed, lmax, gd0, gd_rms, psi_rms, u0, n_mountains, mountain_height,
                                    mountain_radius_deg, _ptr(u), _ptr(v), _ptr(gd), _ptr(ghs))
    if rc:
        raise ValueError("gdo_ic_seeded: invalid arguments")
    return u, v, gd, ghs


def ic_add_noise(gd, N, M, seed, sigma):
    """N(0, sigma) noise on gd's interior, in place (gdc_ic_add_noise's draws)."""
    if lib("exact").gdo_ic_add_noise(N, M, seed, sigma, _ptr(gd)):
        raise ValueError("gdo_ic_add_noise: invalid arguments")
    return gd


def _pad(rows, N):
    return np.zeros((rows + 4, N + 4))


class OracleModel:
    """The reference's dycore_init/run on the CPU, FP64, one thread."""

    def __init__(self, num_lon, num_lat, time_step_size, subcycles=4, split_scheme=0, qcon_modified=1,
                 uv_adv_scheme=0, upwind_lon_beta=0.0, upwind_lat_beta=0.5, use_zonal_tend_filter=1,
                 cutoff=(), use_diffusion=0, diffusion_coef=0.0, diffusion_order=2, rescale_rtol=0.0,
                 fast=False, kind=None, fft=None):
        """kind: "exact" (default), "ref" or "fast" (see lib()); fft: run the
        filter through FFTPACK's transforms (default: on for "ref" and
        "fast", off for "exact")."""
        self.N, self.M = num_lon, num_lat
        kind = kind or ("fast" if fast else "exact")
        self.kind = kind
        self._L = lib(kind)
        c = (ctypes.c_int * 20)(*([0] * 20))
        for k, x in enumerate(cutoff):
            c[k] = int(x)
        self.h = self._L.gdo_create(num_lon, num_lat, time_step_size, subcycles, split_scheme, qcon_modified,
                                  uv_adv_scheme, upwind_lon_beta, upwind_lat_beta, use_zonal_tend_filter, c,
                                  use_diffusion, diffusion_coef, diffusion_order)
        if rescale_rtol:
            self._L.gdo_set_rescale_rtol(self.h, rescale_rtol)
        if fft is None:
            fft = kind != "exact"
        if fft and self._L.gdo_set_fft(self.h, 1) != 0:
            raise ValueError(f"num_lon {num_lon} has a prime factor above 5: no FFTPACK restatement for it")
        self.fft = bool(fft)

    @classmethod
    def from_params(cls, p, kind=None, fft=None):
        """Build from a gdc.Params (any object with the same attribute names)."""
        return cls(p.num_lon, p.num_lat, p.time_step_size, p.subcycles, p.split_scheme, p.qcon_modified,
                   p.uv_adv_scheme, p.uv_adv_upwind_lon_beta, p.uv_adv_upwind_lat_beta, p.use_zonal_tend_filter,
                   list(p.zonal_tend_filter_cutoff_wavenumber), p.use_diffusion, p.diffusion_coef,
                   p.diffusion_order, getattr(p, "filter_rescale_rtol", 0.0), kind=kind, fft=fft)

    def set_state(self, u, v, gd, ghs):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (u, v, gd, ghs)]
        self._L.gdo_set_state(self.h, *map(_ptr, arrs))
        self._L.gdo_run_init(self.h)

    def step(self, n=1):
        return self._L.gdo_step(self.h, n)

    def get_state(self):
        N, M = self.N, self.M
        u, v, gd = _pad(M, N), _pad(M - 1, N), _pad(M, N)
        iu, iv, ig = _pad(M, N), _pad(M - 1, N), _pad(M, N)
        self._L.gdo_get_state(self.h, _ptr(u), _ptr(v), _ptr(gd), _ptr(iu), _ptr(iv), _ptr(ig))
        return dict(u=u, v=v, gd=gd, iu=iu, iv=iv, ig=ig)

    def history(self):
        """A-grid u, v, gh, div, vor of state(old) (padded layout)."""
        N, M = self.N, self.M
        ua, va, gh, dv = _pad(M, N), _pad(M, N), _pad(M, N), _pad(M, N)
        vo = _pad(M - 1, N)
        self._L.gdo_history(self.h, _ptr(ua), _ptr(va), _ptr(gh), _ptr(dv), _ptr(vo))
        return dict(u_a=ua, v_a=va, gh=gh, div=dv, vor=vo)

    def diag(self):
        m, e, b = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._L.gdo_diag(self.h, ctypes.byref(m), ctypes.byref(e), ctypes.byref(b))
        return m.value, e.value, b.value

    def tendency(self, pass_=0):
        N, M = self.N, self.M
        du, dv, dgd = _pad(M, N), _pad(M - 1, N), _pad(M, N)
        self._L.gdo_tendency(self.h, pass_, _ptr(du), _ptr(dv), _ptr(dgd))
        return du, dv, dgd

    def rescale_record(self):
        """Worst conditioning of the filter rescale since the last call:
        [(sum|t w| / |s1|, field, row), (same for s2)], field 0 du, 1 dv, 2 dgd."""
        c = (ctypes.c_double * 2)()
        f, r = (ctypes.c_int * 2)(), (ctypes.c_int * 2)()
        self._L.gdo_rescale_record(self.h, c, f, r)
        return [(c[k], ("du", "dv", "dgd")[f[k]], r[k]) for k in range(2)]

    def antisymmetry(self):
        out = np.zeros(4)
        self._L.gdo_antisymmetry(self.h, _ptr(out))
        return out

    def filter_row(self, half, lat_idx, x):
        x = np.ascontiguousarray(x, dtype=np.float64).copy()
        self._L.gdo_filter_row(self.h, int(half), int(lat_idx), _ptr(x))
        return x

    def filter_flags(self):
        M = self.M
        ff, fh = (ctypes.c_int * M)(), (ctypes.c_int * (M - 1))()
        cf, ch = (ctypes.c_int * M)(), (ctypes.c_int * (M - 1))()
        self._L.gdo_filter_flags(self.h, ff, fh, cf, ch)
        return list(ff), list(fh), list(cf), list(ch)

    def close(self):
        if self.h:
            self._L.gdo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
