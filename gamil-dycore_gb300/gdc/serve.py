"""Forecast serving with continuous batching on one GPU.

Requests (a grid, a forecast length and an arrival time) are admitted as
they arrive and as free device memory allows (``gdc_batch_add`` refuses a
member that would leave less than ``reserve_bytes`` free) into the batch of
their grid's subcycle count -- one ``gdc.Batch`` per count, each on its own
CUDA stream, so that every member runs the fast subcycles its grid needs
and the batches' steps overlap on the device; their state stays resident
and every tick advances all resident members together in the batched
steps.  A member that reaches its length is read back (optionally),
removed, and its memory serves the next request.  Time to completion is
measured from arrival.

The reference has no serving path: this loop is built on the batch engine's
C ABI (``gdc_batch_add / _step / _sync / _member_info / _remove``), and the
engine's per-member arithmetic does not depend on the other members, so a
request's result is the same alone and in the mix.
"""
from __future__ import annotations

import collections
import dataclasses
import math
import time

import numpy as np

from . import (E_OOM, FP32, G, IC_SEEDED, SPLIT_CSP2, Batch, GdcError, ICSpec, default_params, ic_add_noise,
               ic_seeded, ic_spec)

# grid (degrees of resolution) -> num_lon, num_lat, time step (240 s per
# degree), steps per model day, filter cutoffs of the near-pole rows
GRIDS = {
    180: (180, 91, 480.0, 180, [4] * 3),
    360: (360, 181, 240.0, 360, [4] * 5),
    720: (720, 361, 120.0, 720, [4] * 10),
    1440: (1440, 721, 60.0, 1440, [4] * 20),
}


@dataclasses.dataclass
class Request:
    rid: int
    grid: int            # key of GRIDS
    nsteps: int
    arrival: float       # seconds after the start of the stream
    admitted: float = math.nan
    finished: float = math.nan
    member: int = -1
    nan_step: int = -1
    result: tuple | None = None

    @property
    def points(self) -> int:
        N, M = GRIDS[self.grid][:2]
        return N * M

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def poisson_stream(n: int = 2000, rate: float = 20.0, seed: int = 0, grids=(180, 360, 720, 1440),
                   min_hours: float = 6.0, max_days: float = 5.0) -> list[Request]:
    """The request stream: Poisson arrivals at `rate` per second, grid drawn
    uniformly from `grids`, forecast length uniform in [min_hours, max_days]."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    g = rng.choice(np.asarray(grids), size=n)
    length_s = rng.uniform(min_hours * 3600.0, max_days * 86400.0, size=n)
    out = []
    for k in range(n):
        dt = GRIDS[int(g[k])][2]
        out.append(Request(rid=k, grid=int(g[k]), nsteps=max(1, int(round(length_s[k] / dt))), arrival=float(t[k])))
    return out


# fast subcycles per grid for forecasts of up to 5 days: 6 (the benchmark's
# scheme) at 180x91 and 360x181 (stable for 5 days); at 720x361 and
# 1440x721 the fast step dt/6 exceeds the fast-wave CFL limit at the first
# unfiltered row (gravity-wave Courant number ~1.2 at 5 degrees from the
# pole; the seeded 1440x721 state goes NaN after about 1.3 model days).  8
# keep 720x361 stable; at 1440x721 8 still left one noisy FP32 member of
# 200 going NaN (Courant number ~0.83 at the first unfiltered row, 5.25
# degrees from the pole), and 10 (the reference's rh_test setting) bring it
# to ~0.66.
SUBCYCLES = {180: 6, 360: 6, 720: 8, 1440: 10}


# The filter's s1/s2 rescale (src/dycore_mod.F90:212-219) divides by a sum
# that can cancel to 1e-5..1e-6 of its terms on polar rows; FP32 tendencies
# determine such a sum only to ~1e-7 of the terms, so the FP32 rescale factor
# there is noise.  One 720x361 request of the 2000-request stream went NaN
# at step 1263 in FP32 (alone as in the batch) while the FP64 path ran it to
# its end; with the rescale skipped where s1 or s2 is below 1e-5 of the sum
# of its terms' magnitudes (gdc_params::filter_rescale_rtol) the FP32 run
# completes, as far from the FP64 run as the guard itself moves FP64.  FP32
# serving uses that guard; FP64 keeps the reference's unguarded rescale.
FP32_RESCALE_RTOL = 1e-5


def serving_scheme(precision: int = FP32, subcycles: int = 6):
    """csp2 with `subcycles` fast subcycles (the batch of one subcycle class);
    FP32 with the rescale guard (FP32_RESCALE_RTOL)."""
    return default_params(num_lon=360, num_lat=181, time_step_size=240.0, subcycles=subcycles,
                          split_scheme=SPLIT_CSP2, qcon_modified=1, use_zonal_tend_filter=1,
                          zonal_tend_filter_cutoff_wavenumber=[4] * 5, precision=precision,
                          filter_rescale_rtol=FP32_RESCALE_RTOL if precision == FP32 else 0.0)


class InitialStates:
    """Seeded initial states: the degree 1..6 harmonic state of each grid
    plus N(0, 1 m) noise on gd seeded per request.  With `device` (the
    default) the state is generated in device memory at admission
    (``gdc_batch_add_ic``); otherwise the host builds it (the base state
    once per grid) and uploads it."""

    def __init__(self, seed: int = 0, noise_m: float = 1.0, device: bool = True):
        self.seed = seed
        self.noise = noise_m * G
        self.device = device
        self.base = {}

    def __call__(self, req: Request):
        if self.device:
            return ic_spec(IC_SEEDED, seed=self.seed, noise_seed=1000 + req.rid, noise_sigma=self.noise)
        N, M = GRIDS[req.grid][:2]
        if req.grid not in self.base:
            self.base[req.grid] = ic_seeded(N, M, seed=self.seed)
        u, v, gd, ghs = self.base[req.grid]
        gd = ic_add_noise(gd.copy(), N, M, seed=1000 + req.rid, sigma=self.noise)
        return u, v, gd, ghs


class Server:
    """The request loop.  `batch_factory(subcycles)` builds the engine of one
    subcycle class (a ``gdc.Batch`` by default); `steps_per_tick` model
    steps are taken between admission and completion checks.  Each batch is
    autotuned (``gdc_batch_autotune``: its launch schedule, without
    advancing any member) once it first holds `tune_at` members, and again
    every `retune_ticks` ticks (0: never again)."""

    def __init__(self, precision: int = FP32, steps_per_tick: int = 4, reserve_bytes: int = 2 << 30,
                 max_members: int = 1000, batch_factory=None, initial_states=None, clock=time.perf_counter,
                 sleep=time.sleep, cuda_stream: int | None = None, tune_at: int = 4, retune_ticks: int = 0):
        self.precision = precision
        self.steps_per_tick = steps_per_tick
        self.reserve = reserve_bytes
        self.max_members = max_members
        self.clock = clock
        self.sleep = sleep
        self.ics = initial_states or InitialStates()
        self.factory = batch_factory or (lambda m: Batch(serving_scheme(precision, m)))
        self.cuda_stream = cuda_stream
        self.tune_at = tune_at
        self.retune_ticks = retune_ticks
        self.batches: dict[int, object] = {}
        self.tuned: dict[int, int] = {}  # subcycles -> tick of the last tuning
        self.ticks = 0
        self.max_resident = 0

    def batch(self, subcycles: int):
        if subcycles not in self.batches:
            b = self.factory(subcycles)
            if self.cuda_stream is not None:
                b.set_stream(self.cuda_stream)
            self.batches[subcycles] = b
        return self.batches[subcycles]

    def close(self):
        for b in self.batches.values():
            b.close()
        self.batches = {}

    def _maybe_tune(self, resident: dict[int, int]):
        for m, n in resident.items():
            last = self.tuned.get(m)
            due = (last is None and n >= self.tune_at) or (
                last is not None and self.retune_ticks and self.ticks - last >= self.retune_ticks)
            if due and hasattr(self.batches[m], "autotune"):
                self.batches[m].autotune()
                self.tuned[m] = self.ticks

    def run(self, requests: list[Request], keep_results: bool = False, max_wall: float | None = None) -> dict:
        """Serve `requests` (sorted by arrival).  With `max_wall`, arrivals
        after that many seconds are not admitted and the loop ends once the
        admitted requests complete."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        waiting = collections.deque()
        running: dict[tuple[int, int], Request] = {}  # (subcycles, member) -> request
        done: list[Request] = []
        nxt = 0
        t0 = self.clock()
        while True:
            now = self.clock() - t0
            cutoff = now if max_wall is None else min(now, max_wall)
            while nxt < len(reqs) and reqs[nxt].arrival <= cutoff:
                waiting.append(reqs[nxt])
                nxt += 1
            # admission: first come first served, while memory and slots last
            while waiting and len(running) < self.max_members:
                r = waiting[0]
                N, M, dt, _, cut = GRIDS[r.grid]
                m = SUBCYCLES[r.grid]
                b = self.batch(m)
                ic = self.ics(r)
                try:
                    if isinstance(ic, ICSpec):
                        mid = b.add_ic(N, M, dt, r.nsteps, ic, reserve_bytes=self.reserve, cutoff=cut)
                    else:
                        mid = b.add(N, M, dt, r.nsteps, *ic, reserve_bytes=self.reserve, cutoff=cut)
                except GdcError as e:
                    if e.code == E_OOM and running:
                        break  # wait for completions to free memory
                    raise
                r.member = mid
                r.admitted = self.clock() - t0
                running[(m, mid)] = r
                waiting.popleft()
            self.max_resident = max(self.max_resident, len(running))
            arrivals_left = nxt < len(reqs) and (max_wall is None or reqs[nxt].arrival <= max_wall)
            if not running:
                if not arrivals_left and not waiting:
                    break
                if arrivals_left:
                    self.sleep(max(0.0, reqs[nxt].arrival - (self.clock() - t0)))
                continue
            resident = collections.Counter(m for m, _ in running)
            self._maybe_tune(resident)
            live = [self.batches[m] for m in resident]
            for b in live:  # enqueue every class's steps, then wait for all
                b.step(self.steps_per_tick)
            for b in live:
                b.sync()
            self.ticks += 1
            now = self.clock() - t0
            for (m, mid), r in list(running.items()):
                b = self.batches[m]
                steps, fin, nan = b.info(mid)
                if fin or nan >= 0:
                    r.finished = now
                    r.nan_step = nan
                    if keep_results:
                        r.result = b.get_state(mid)
                    b.remove(mid)
                    del running[(m, mid)]
                    done.append(r)
        return summarize(done, len(reqs))


def summarize(done: list[Request], offered: int) -> dict:
    if not done:
        return {"completed": 0, "offered": offered}
    lat = np.array([r.latency for r in done])
    wait = np.array([r.admitted - r.arrival for r in done])
    # a member stopped by a NaN did only the steps before it
    work = sum(r.points * (r.nan_step if r.nan_step >= 0 else r.nsteps) for r in done)
    span = max(r.finished for r in done) - min(r.arrival for r in done)
    return {
        "completed": len(done),
        "offered": offered,
        "p50_s": float(np.percentile(lat, 50)),
        "p99_s": float(np.percentile(lat, 99)),
        "mean_s": float(lat.mean()),
        "p50_admission_wait_s": float(np.percentile(wait, 50)),
        "gpt_steps": float(work),
        "span_s": float(span),
        "gpt_steps_per_s": float(work / span) if span > 0 else float("nan"),
        "nan_members": int(sum(1 for r in done if r.nan_step >= 0)),
        "nan_members_by_grid": {str(g): int(sum(1 for r in done if r.nan_step >= 0 and r.grid == g))
                                for g in sorted({r.grid for r in done})},
        "nan_requests": [{"rid": r.rid, "grid": r.grid, "nsteps": r.nsteps, "nan_step": r.nan_step}
                         for r in done if r.nan_step >= 0],
    }
