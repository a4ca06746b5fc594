"""Python host side of the GB300-native gamil-dycore barotropic step.

A thin ctypes mirror of the C ABI in ``include/gdc.h``: the reference's
``dycore_init / dycore_run / dycore_final`` entry points become
``Model(params)``, ``Model.set_state`` + ``Model.run`` and ``Model.close``;
the batched ensemble / serving engine is ``Batch``.  Fields use the
reference's padded layout: numpy arrays of shape ``(rows + 4, num_lon + 4)``
(lon fastest, halo 2), full rows ``rows = num_lat`` for u and gd,
``num_lat - 1`` for v.

The CUDA library is required: importing works without it, but every call
that needs it raises ``RuntimeError`` when ``_build/libgdc.so`` is missing.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent.parent
LIB_PATH = PKG / "_build" / "libgdc.so"

OK, E_CONFIG, E_CUDA, E_OOM, E_NAN, E_TIMEOUT, E_STATE = range(7)
SPLIT_NONE, SPLIT_CSP1, SPLIT_CSP2, SPLIT_ISP = range(4)
ADV_CENTER_DIFF, ADV_UPWIND, ADV_WENO = range(3)
FP64, FP32 = 0, 1
ALL_PASS, FAST_PASS, SLOW_PASS = 0, 1, 2
G = 9.80616  # src/params_mod.F90:11


class GdcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"gdc error {code}: {msg}")
        self.code = code


class Params(ctypes.Structure):
    """Mirror of ``gdc_params`` (namelist /dycore_params/ + precision)."""

    _fields_ = [
        ("num_lon", ctypes.c_int),
        ("num_lat", ctypes.c_int),
        ("time_step_size", ctypes.c_double),
        ("subcycles", ctypes.c_int),
        ("split_scheme", ctypes.c_int),
        ("qcon_modified", ctypes.c_int),
        ("uv_adv_scheme", ctypes.c_int),
        ("uv_adv_upwind_lon_beta", ctypes.c_double),
        ("uv_adv_upwind_lat_beta", ctypes.c_double),
        ("use_zonal_tend_filter", ctypes.c_int),
        ("zonal_tend_filter_cutoff_wavenumber", ctypes.c_int * 20),
        ("use_diffusion", ctypes.c_int),
        ("diffusion_coef", ctypes.c_double),
        ("diffusion_order", ctypes.c_int),
        ("run_days", ctypes.c_int),
        ("run_hours", ctypes.c_int),
        ("run_minutes", ctypes.c_int),
        ("run_seconds", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("device", ctypes.c_int),
        ("filter_rescale_rtol", ctypes.c_double),
    ]


IC_ROSSBY_HAURWITZ, IC_STEADY_GEOSTROPHIC, IC_MOUNTAIN_ZONAL_FLOW, IC_SEEDED, IC_SHALLOW_WATER_WAVES = 0, 1, 2, 3, 4


class ICSpec(ctypes.Structure):
    """Mirror of ``gdc_ic_spec``: an initial condition generated on the device."""

    _fields_ = [
        ("kind", ctypes.c_int),
        ("lmax", ctypes.c_int),
        ("seed", ctypes.c_ulonglong),
        ("gd0", ctypes.c_double),
        ("gd_rms", ctypes.c_double),
        ("psi_rms", ctypes.c_double),
        ("u0", ctypes.c_double),
        ("n_mountains", ctypes.c_int),
        ("reserved", ctypes.c_int),
        ("mountain_height", ctypes.c_double),
        ("mountain_radius_deg", ctypes.c_double),
        ("noise_seed", ctypes.c_ulonglong),
        ("noise_sigma", ctypes.c_double),
    ]


_lib = None
_P = ctypes.POINTER(ctypes.c_double)


def lib() -> ctypes.CDLL:
    """Load libgdc.so (fails loudly when the native build is missing)."""
    global _lib
    if _lib is None:
        path = Path(os.environ.get("GDC_LIB", LIB_PATH))
        if not path.exists():
            raise RuntimeError(
                f"native library {path} not found: run gamil-dycore_gb300/build.py "
                "(there is no CPU fallback)")
        L = ctypes.CDLL(str(path))
        vp, ip, dp, i64p = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), _P, ctypes.POINTER(ctypes.c_longlong)
        sig = {
            "gdc_params_default": (None, [ctypes.POINTER(Params)]),
            "gdc_params_read_namelist": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(Params), ctypes.c_char_p,
                                                        ctypes.c_int, ctypes.c_char_p, ctypes.c_int,
                                                        ctypes.c_char_p, ctypes.c_int]),
            "gdc_steps_for_run": (ctypes.c_int, [ctypes.POINTER(Params)]),
            "gdc_create": (ctypes.c_int, [ctypes.POINTER(Params), ctypes.POINTER(vp)]),
            "gdc_destroy": (None, [vp]),
            "gdc_last_error": (ctypes.c_char_p, [vp]),
            "gdc_set_state": (ctypes.c_int, [vp, dp, dp, dp, dp, ctypes.c_int]),
            "gdc_step": (ctypes.c_int, [vp, ctypes.c_int]),
            "gdc_sync": (ctypes.c_int, [vp]),
            "gdc_run": (ctypes.c_int, [vp, ctypes.c_int]),
            "gdc_get_state": (ctypes.c_int, [vp, dp, dp, dp, ctypes.c_int]),
            "gdc_get_iap": (ctypes.c_int, [vp, dp, dp, dp, ctypes.c_int]),
            "gdc_diag": (ctypes.c_int, [vp, dp, dp, dp]),
            "gdc_steps_done": (ctypes.c_int, [vp, i64p]),
            "gdc_debug_tendency": (ctypes.c_int, [vp, ctypes.c_int, dp, dp, dp, ctypes.c_int]),
            "gdc_set_stream": (ctypes.c_int, [vp, vp]),
            "gdc_ic_rossby_haurwitz": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, dp, dp, dp, dp, ctypes.c_int]),
            "gdc_ic_steady_geostrophic": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, dp, dp, dp, dp, ctypes.c_int]),
            "gdc_ic_mountain_zonal_flow": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, dp, dp, dp, dp, ctypes.c_int]),
            "gdc_ic_seeded": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong, ctypes.c_int,
                                             ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                             ctypes.c_int, ctypes.c_double, ctypes.c_double, dp, dp, dp, dp,
                                             ctypes.c_int]),
            "gdc_ic_shallow_water_waves": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, dp, dp, dp, dp,
                                                          ctypes.c_int]),
            "gdc_sw_waves_phase_speed": (ctypes.c_double, [ctypes.c_int]),
            "gdc_ic_add_noise": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong, ctypes.c_double,
                                                dp, ctypes.c_int]),
            "gdc_batch_create": (ctypes.c_int, [ctypes.POINTER(Params), ctypes.POINTER(vp)]),
            "gdc_batch_destroy": (None, [vp]),
            "gdc_batch_last_error": (ctypes.c_char_p, [vp]),
            "gdc_batch_set_stream": (ctypes.c_int, [vp, vp]),
            "gdc_member_bytes": (ctypes.c_size_t, [ctypes.POINTER(Params), ctypes.c_int, ctypes.c_int]),
            "gdc_device_mem_info": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_size_t),
                                                   ctypes.POINTER(ctypes.c_size_t)]),
            "gdc_batch_add": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_longlong,
                                             ip, dp, dp, dp, dp, ctypes.c_int, ctypes.c_size_t, ip]),
            "gdc_ic_spec_default": (None, [ctypes.POINTER(ICSpec), ctypes.c_int]),
            "gdc_batch_add_ic": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_longlong,
                                                ip, ctypes.POINTER(ICSpec), ctypes.c_size_t, ip]),
            "gdc_batch_remove": (ctypes.c_int, [vp, ctypes.c_int]),
            "gdc_batch_step": (ctypes.c_int, [vp, ctypes.c_int]),
            "gdc_batch_sync": (ctypes.c_int, [vp]),
            "gdc_batch_member_info": (ctypes.c_int, [vp, ctypes.c_int, i64p, ip, i64p]),
            "gdc_batch_get_state": (ctypes.c_int, [vp, ctypes.c_int, dp, dp, dp, ctypes.c_int]),
            "gdc_batch_diag": (ctypes.c_int, [vp, ctypes.c_int, dp, dp, dp]),
            "gdc_batch_active": (ctypes.c_int, [vp, ip]),
            "gdc_batch_set_tile": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int]),
            "gdc_batch_set_schedule": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
            "gdc_batch_get_schedule": (ctypes.c_int, [vp, ip, ip, ip, ip, ip]),
            "gdc_batch_checkpoint": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_char_p]),
            "gdc_batch_restore": (ctypes.c_int, [vp, ctypes.c_char_p, ctypes.c_size_t, ip]),
            "gdc_write_restart": (ctypes.c_int, [vp, ctypes.c_char_p]),
            "gdc_history": (ctypes.c_int, [vp, dp, dp, dp, dp, dp, ctypes.c_int]),
            "gdc_batch_history": (ctypes.c_int, [vp, ctypes.c_int, dp, dp, dp, dp, dp, ctypes.c_int]),
            "gdc_read_restart": (ctypes.c_int, [vp, ctypes.c_char_p]),
            "gdc_batch_autotune": (ctypes.c_int, [vp, ip, ip, dp]),
            "gdc_batch_profile": (ctypes.c_int, [vp, ctypes.c_int, dp, i64p]),
            "gdc_algorithmic_bytes_per_gpt_step": (ctypes.c_double, [ctypes.POINTER(Params)]),
            "gdc_fp64_fma_rate": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
            "gdc_tendency_noalloc": (ctypes.c_int, [ctypes.POINTER(Params), ctypes.c_int, vp, vp, vp, vp, vp, vp,
                                                    vp, vp, vp, vp]),
            "gdc_noalloc_last_error": (ctypes.c_char_p, []),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_P)


def ic_spec(kind: int, **kw) -> ICSpec:
    """gdc_ic_spec_default(kind) with fields overridden by keyword."""
    spec = ICSpec()
    lib().gdc_ic_spec_default(ctypes.byref(spec), kind)
    for k, v in kw.items():
        if not hasattr(spec, k):
            raise AttributeError(f"gdc_ic_spec has no field {k}")
        setattr(spec, k, v)
    return spec


def _cutoff_array(cutoff):
    if cutoff is None:
        return None
    cut = (ctypes.c_int * 20)(*([0] * 20))
    for q, c in enumerate(cutoff):
        cut[q] = int(c)
    return cut


def padded(rows: int, num_lon: int) -> np.ndarray:
    """Zero field in the reference's padded layout."""
    return np.zeros((rows + 4, num_lon + 4), dtype=np.float64)


def default_params(**kw) -> Params:
    p = Params()
    lib().gdc_params_default(ctypes.byref(p))
    for k, v in kw.items():
        if k == "zonal_tend_filter_cutoff_wavenumber":
            arr = (ctypes.c_int * 20)(*([0] * 20))
            for q, c in enumerate(v):
                arr[q] = int(c)
            p.zonal_tend_filter_cutoff_wavenumber = arr
        else:
            setattr(p, k, v)
    return p


def read_namelist(path: str) -> tuple[Params, str, str]:
    p = Params()
    tc = ctypes.create_string_buffer(256)
    cn = ctypes.create_string_buffer(256)
    err = ctypes.create_string_buffer(512)
    rc = lib().gdc_params_read_namelist(str(path).encode(), ctypes.byref(p), tc, 256, cn, 256, err, 512)
    if rc:
        raise GdcError(rc, err.value.decode())
    return p, tc.value.decode(), cn.value.decode()


def steps_for_run(p: Params) -> int:
    return lib().gdc_steps_for_run(ctypes.byref(p))


def algorithmic_bytes_per_gpt_step(p: Params) -> float:
    return lib().gdc_algorithmic_bytes_per_gpt_step(ctypes.byref(p))


def fp64_fma_rate(device: int = 0) -> float:
    """The device's FP64 fused multiply-add rate, 1e9 FMA/s (the FP64 path's roof)."""
    r = ctypes.c_double()
    rc = lib().gdc_fp64_fma_rate(device, ctypes.byref(r))
    if rc:
        raise GdcError(rc, "gdc_fp64_fma_rate failed")
    return r.value


def member_bytes(p: Params, num_lon: int, num_lat: int) -> int:
    return lib().gdc_member_bytes(ctypes.byref(p), num_lon, num_lat)


def device_mem_info(device: int = 0) -> tuple[int, int]:
    f, t = ctypes.c_size_t(), ctypes.c_size_t()
    rc = lib().gdc_device_mem_info(device, ctypes.byref(f), ctypes.byref(t))
    if rc:
        raise GdcError(rc, "cudaMemGetInfo failed")
    return f.value, t.value


# ------------------------------------------------------------ initial conditions

def _ic(fn, N: int, M: int):
    u, v, gd, ghs = padded(M, N), padded(M - 1, N), padded(M, N), padded(M, N)
    rc = fn(N, M, _ptr(u), _ptr(v), _ptr(gd), _ptr(ghs), N + 4)
    if rc:
        raise GdcError(rc, "initial condition failed")
    return u, v, gd, ghs


def ic_rossby_haurwitz(N: int, M: int):
    return _ic(lib().gdc_ic_rossby_haurwitz, N, M)


def ic_steady_geostrophic(N: int, M: int):
    return _ic(lib().gdc_ic_steady_geostrophic, N, M)


def ic_mountain_zonal_flow(N: int, M: int):
    return _ic(lib().gdc_ic_mountain_zonal_flow, N, M)


def ic_seeded(N: int, M: int, seed: int = 0, lmax: int = 6, gd0: float = 8000 * G, gd_rms: float = 100 * G,
              psi_rms: float = 1.0e7, u0: float = 0.0, n_mountains: int = 0, mountain_height: float = 2000.0,
              mountain_radius_deg: float = 20.0):
    """Seeded harmonics / mountains initial state (padded layout)."""
    u, v, gd, ghs = padded(M, N), padded(M - 1, N), padded(M, N), padded(M, N)
    rc = lib().gdc_ic_seeded(N, M, seed, lmax, gd0, gd_rms, psi_rms, u0, n_mountains, mountain_height,
                             mountain_radius_deg, _ptr(u), _ptr(v), _ptr(gd), _ptr(ghs), N + 4)
    if rc:
        raise GdcError(rc, "gdc_ic_seeded failed")
    return u, v, gd, ghs


def ic_shallow_water_waves(N: int, M: int):
    """Shamir-Paldor shallow-water Rossby wave (padded layout)."""
    u, v, gd, ghs = padded(M, N), padded(M - 1, N), padded(M, N), padded(M, N)
    rc = lib().gdc_ic_shallow_water_waves(N, M, _ptr(u), _ptr(v), _ptr(gd), _ptr(ghs), N + 4)
    if rc:
        raise GdcError(rc, "gdc_ic_shallow_water_waves failed")
    return u, v, gd, ghs


def sw_waves_phase_speed(wave_flag: int = 0) -> float:
    """Phase speed (rad/s) of the shallow-water wave: 0 Rossby, 1 EIG, -1 WIG."""
    return lib().gdc_sw_waves_phase_speed(wave_flag)


def ic_add_noise(gd: np.ndarray, N: int, M: int, seed: int, sigma: float) -> np.ndarray:
    rc = lib().gdc_ic_add_noise(N, M, seed, sigma, _ptr(gd), N + 4)
    if rc:
        raise GdcError(rc, "gdc_ic_add_noise failed")
    return gd


# ------------------------------------------------------------------- model

class Model:
    """One model: dycore_init (constructor), the initial-condition hook +
    dycore_run prologue (set_state), the run loop (step / run), and
    dycore_final (close)."""

    def __init__(self, params: Params):
        self.p = params
        self.N, self.M = params.num_lon, params.num_lat
        h = ctypes.c_void_p()
        rc = lib().gdc_create(ctypes.byref(params), ctypes.byref(h))
        if rc:
            raise GdcError(rc, "gdc_create failed")
        self.h = h

    def _check(self, rc: int):
        if rc:
            raise GdcError(rc, lib().gdc_last_error(self.h).decode())

    def set_state(self, u, v, gd, ghs):
        ld = self.N + 4
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (u, v, gd, ghs)]
        self._check(lib().gdc_set_state(self.h, *map(_ptr, arrs), ld))

    def step(self, n: int = 1):
        self._check(lib().gdc_step(self.h, n))

    def sync(self):
        self._check(lib().gdc_sync(self.h))

    def run(self, n: int):
        self._check(lib().gdc_run(self.h, n))

    def get_state(self):
        u, v, gd = padded(self.M, self.N), padded(self.M - 1, self.N), padded(self.M, self.N)
        self._check(lib().gdc_get_state(self.h, _ptr(u), _ptr(v), _ptr(gd), self.N + 4))
        return u, v, gd

    def get_iap(self):
        iu, iv, ig = padded(self.M, self.N), padded(self.M - 1, self.N), padded(self.M, self.N)
        self._check(lib().gdc_get_iap(self.h, _ptr(iu), _ptr(iv), _ptr(ig), self.N + 4))
        return iu, iv, ig

    def diag(self):
        m, e, b = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._check(lib().gdc_diag(self.h, ctypes.byref(m), ctypes.byref(e), ctypes.byref(b)))
        return m.value, e.value, b.value

    def steps_done(self) -> int:
        s = ctypes.c_longlong()
        self._check(lib().gdc_steps_done(self.h, ctypes.byref(s)))
        return s.value

    def tendency(self, pass_: int = ALL_PASS):
        du, dv, dgd = padded(self.M, self.N), padded(self.M - 1, self.N), padded(self.M, self.N)
        self._check(lib().gdc_debug_tendency(self.h, pass_, _ptr(du), _ptr(dv), _ptr(dgd), self.N + 4))
        return du, dv, dgd

    def history(self):
        """A-grid u, v, gh = gd + ghs, divergence and vorticity of state(old)."""
        N, M = self.N, self.M
        out = [padded(M, N) for _ in range(4)] + [padded(M - 1, N)]
        self._check(lib().gdc_history(self.h, *map(_ptr, out), N + 4))
        return dict(zip(("u_a", "v_a", "gh", "div", "vor"), out))

    def write_restart(self, path: str):
        self._check(lib().gdc_write_restart(self.h, str(path).encode()))

    def read_restart(self, path: str):
        self._check(lib().gdc_read_restart(self.h, str(path).encode()))

    def set_stream(self, cuda_stream: int | None):
        self._check(lib().gdc_set_stream(self.h, ctypes.c_void_p(cuda_stream) if cuda_stream else None))

    def close(self):
        if getattr(self, "h", None):
            lib().gdc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tendency_noalloc(params: Params, pass_: int, gd: int, iap_u: int, iap_v: int, ghs: int, du: int, dv: int,
                     dgd: int, given_u: int | None = None, given_v: int | None = None, stream: int | None = None):
    """space_operators into caller-owned device buffers (interior layout,
    FP64), without any device allocation by the library.  Arguments are
    device addresses (e.g. torch tensors' data_ptr())."""
    vp = ctypes.c_void_p
    rc = lib().gdc_tendency_noalloc(ctypes.byref(params), pass_, vp(gd), vp(iap_u), vp(iap_v), vp(ghs),
                                    vp(given_u) if given_u else None, vp(given_v) if given_v else None,
                                    vp(du), vp(dv), vp(dgd), vp(stream) if stream else None)
    if rc:
        raise GdcError(rc, lib().gdc_noalloc_last_error().decode())


class Batch:
    """Batched ensemble / serving engine (gdc_batch_*)."""

    def __init__(self, scheme: Params):
        self.p = scheme
        b = ctypes.c_void_p()
        rc = lib().gdc_batch_create(ctypes.byref(scheme), ctypes.byref(b))
        if rc:
            raise GdcError(rc, "gdc_batch_create failed")
        self.b = b
        self.grids: dict[int, tuple[int, int]] = {}

    def _check(self, rc: int):
        if rc:
            raise GdcError(rc, lib().gdc_batch_last_error(self.b).decode())

    def add(self, N: int, M: int, dt: float, nsteps: int, u, v, gd, ghs, reserve_bytes: int = 0,
            cutoff=None) -> int:
        """Admit a member; `cutoff` overrides the scheme's filter cutoffs."""
        mid = ctypes.c_int()
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (u, v, gd, ghs)]
        rc = lib().gdc_batch_add(self.b, N, M, dt, nsteps, _cutoff_array(cutoff), *map(_ptr, arrs), N + 4,
                                 reserve_bytes, ctypes.byref(mid))
        self._check(rc)
        self.grids[mid.value] = (N, M)
        return mid.value

    def add_ic(self, N: int, M: int, dt: float, nsteps: int, spec: ICSpec, reserve_bytes: int = 0,
               cutoff=None) -> int:
        """Admit a member whose initial condition (`spec`, see ``ic_spec``)
        is generated in device memory."""
        mid = ctypes.c_int()
        rc = lib().gdc_batch_add_ic(self.b, N, M, dt, nsteps, _cutoff_array(cutoff), ctypes.byref(spec),
                                    reserve_bytes, ctypes.byref(mid))
        self._check(rc)
        self.grids[mid.value] = (N, M)
        return mid.value

    def remove(self, mid: int):
        self._check(lib().gdc_batch_remove(self.b, mid))
        self.grids.pop(mid, None)

    def step(self, n: int = 1):
        self._check(lib().gdc_batch_step(self.b, n))

    def sync(self):
        self._check(lib().gdc_batch_sync(self.b))

    def info(self, mid: int):
        s, f, n = ctypes.c_longlong(), ctypes.c_int(), ctypes.c_longlong()
        self._check(lib().gdc_batch_member_info(self.b, mid, ctypes.byref(s), ctypes.byref(f), ctypes.byref(n)))
        return s.value, bool(f.value), n.value

    def get_state(self, mid: int):
        N, M = self.grids[mid]
        u, v, gd = padded(M, N), padded(M - 1, N), padded(M, N)
        self._check(lib().gdc_batch_get_state(self.b, mid, _ptr(u), _ptr(v), _ptr(gd), N + 4))
        return u, v, gd

    def diag(self, mid: int):
        m, e, b = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._check(lib().gdc_batch_diag(self.b, mid, ctypes.byref(m), ctypes.byref(e), ctypes.byref(b)))
        return m.value, e.value, b.value

    def active(self) -> int:
        n = ctypes.c_int()
        self._check(lib().gdc_batch_active(self.b, ctypes.byref(n)))
        return n.value

    def history(self, mid: int):
        """A-grid u, v, gh = gd + ghs, divergence and vorticity of a member."""
        N, M = self.grids[mid]
        out = [padded(M, N) for _ in range(4)] + [padded(M - 1, N)]
        self._check(lib().gdc_batch_history(self.b, mid, *map(_ptr, out), N + 4))
        return dict(zip(("u_a", "v_a", "gh", "div", "vor"), out))

    def checkpoint(self, mid: int, path: str):
        self._check(lib().gdc_batch_checkpoint(self.b, mid, str(path).encode()))

    def restore(self, path: str, reserve_bytes: int = 0) -> int:
        """Admit a checkpoint as a new member; returns its id."""
        mid = ctypes.c_int()
        self._check(lib().gdc_batch_restore(self.b, str(path).encode(), reserve_bytes, ctypes.byref(mid)))
        with open(path, "rb") as f:
            hdr = f.read(24)
        N, M = int.from_bytes(hdr[16:20], "little"), int.from_bytes(hdr[20:24], "little")
        self.grids[mid.value] = (N, M)
        return mid.value

    def set_tile(self, rows: int, cols: int):
        self._check(lib().gdc_batch_set_tile(self.b, rows, cols))

    def set_schedule(self, split_rows: int = -1, fuse_final: int = 0, pair_rows: int = -1):
        """Launch schedule: whole-row tasks split by field (-1 auto, 0, 1),
        the final update fused into the next stage (1) or launched (0), and
        whole-row tasks split over the two blocks of a cluster (-1 auto, 0,
        1)."""
        self._check(lib().gdc_batch_set_schedule(self.b, split_rows, fuse_final, pair_rows))

    def autotune(self):
        """Time every launch schedule on the current members and keep the
        fastest; the members' states are restored.  Returns (tile rows, tile
        columns, ms per model step)."""
        r, c, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        self._check(lib().gdc_batch_autotune(self.b, ctypes.byref(r), ctypes.byref(c), ctypes.byref(ms)))
        return r.value, c.value, ms.value

    def schedule(self) -> dict:
        """The launch schedule in use: tile shape, row-task split, fusion."""
        v = [ctypes.c_int() for _ in range(5)]
        self._check(lib().gdc_batch_get_schedule(self.b, *[ctypes.byref(x) for x in v]))
        return {"tile": (v[0].value, v[1].value), "split_rows": v[2].value, "fuse_final": v[3].value,
                "pair_rows": v[4].value}

    def profile(self, nsteps: int):
        ms = (ctypes.c_double * 5)()
        n = (ctypes.c_longlong * 5)()
        self._check(lib().gdc_batch_profile(self.b, nsteps, ms, n))
        return list(ms), list(n)

    def set_stream(self, cuda_stream: int | None):
        self._check(lib().gdc_batch_set_stream(self.b, ctypes.c_void_p(cuda_stream) if cuda_stream else None))

    def close(self):
        if getattr(self, "b", None):
            lib().gdc_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
