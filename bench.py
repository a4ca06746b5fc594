#!/usr/bin/env python
"""Benchmark of the GB300-native barotropic time step (one JSON line).

Default workload (the metric's headline configuration): a 64-member FP32
ensemble in one batch -- 16 x 180x91 (dt 480 s), 32 x 360x181 (dt 240 s),
16 x 720x361 (dt 120 s), one model day each -- from the seeded harmonic
state (gd0 = 8000 m g, degree 1..6, 100 m / 1e7 m^2 s^-1 RMS) plus
N(0, 1 m) g white noise per member.  Scheme: predict_correct, csp2 with 6
subcycles, qcon_modified, center_diff, zonal filter cutoff 4 on the rows
within ~5 degrees of each pole.  A "step" is one model step of every active
member; --steps 720 (default) is the whole job.  `value` is grid-point
steps per second over the timed steps with the inputs resident in HBM; the
plain FP64 path (360x181, 360 steps) is timed beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload batch|plain|serve|large-run] [--requests N]

--impl reference times the reference's arithmetic on the host cores: the
oracle's reference-order restatement (the Fortran reference cannot be built
here) advancing the same 64 members for the same --steps and --warmup, one
process per core, without loading the product library.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for _p in (ROOT, ROOT / "gamil-dycore_gb300"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

G = 9.80616
# grid -> (num_lon, num_lat, dt, steps per model day, filter cutoffs)
GRIDS = {
    180: (180, 91, 480.0, 180, [4] * 3),
    360: (360, 181, 240.0, 360, [4] * 5),
    720: (720, 361, 120.0, 720, [4] * 10),
    1440: (1440, 721, 60.0, 1440, [4] * 20),
}
ENSEMBLE = [(180, 16), (360, 32), (720, 16)]
ENSEMBLE_CONFIG = {"workload": "ensemble: 16x180x91@480s + 32x360x181@240s + 16x720x361@120s, one model day each, "
                               "csp2 m=6, filter on",
                   "scheme": "predict_correct+csp2(6)+qcon",
                   "l2_cache": "inputs larger than L2 (working set ~0.8 GB vs 129 MB L2)"}


def peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        return {}


def scheme(gdc, precision, subcycles=6):
    return gdc.default_params(num_lon=360, num_lat=181, time_step_size=240.0, subcycles=subcycles,
                              split_scheme=gdc.SPLIT_CSP2, qcon_modified=1, uv_adv_scheme=gdc.ADV_CENTER_DIFF,
                              use_zonal_tend_filter=1, zonal_tend_filter_cutoff_wavenumber=[4] * 5,
                              precision=precision)


def ensemble_ics(gdc):
    """Per-member initial states of the 64-member ensemble (host arrays)."""
    base = {g: gdc.ic_seeded(GRIDS[g][0], GRIDS[g][1], seed=0) for g, _ in ENSEMBLE}
    members = []
    k = 0
    for g, count in ENSEMBLE:
        N, M, dt, nsteps, cut = GRIDS[g]
        for _ in range(count):
            u, v, gd, ghs = base[g]
            gd = gdc.ic_add_noise(gd.copy(), N, M, seed=1000 + k, sigma=1.0 * G)
            members.append(dict(N=N, M=M, dt=dt, nsteps=nsteps, cutoff=cut, ic=(u, v, gd, ghs)))
            k += 1
    return members


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 9:
                    rows.append(f)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        load = [s for s in sm if s > 0.5 * (max(mx) if mx else 2070)] or sm
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup(n_gpus):
    if n_gpus <= 1 or "RANK" not in os.environ:
        return 0, 1, None
    import torch
    import torch.distributed as dist
    rank, world = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", rank)))
    dist.init_process_group("nccl")
    return rank, world, dist


def reduce_max(dist, x: float, device: str = "cuda") -> float:
    """Max over ranks (replicas): the job is done when the slowest replica is."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(dist, points_per_rank: float, ms: float, device: str = "cuda") -> tuple[float, float]:
    """Whole-job throughput of N independent replicas: all ranks' grid points
    over the slowest rank's time.  Returns (value, max ms)."""
    world = dist.get_world_size() if dist is not None else 1
    ms_all = reduce_max(dist, ms, device)
    return world * points_per_rank / (ms_all / 1e3), ms_all


def barrier(dist):
    if dist is not None:
        dist.barrier()


# ------------------------------------------------------------------ ours

def time_batch(gdc, torch, members, steps, warmup, precision, ts):
    """Warm up, then time `steps` model steps of the whole ensemble with CUDA
    events on the stream the kernels are launched on."""
    b = gdc.Batch(scheme(gdc, precision))
    b.set_stream(ts.cuda_stream)
    ids = []
    for m in members:
        ids.append(b.add(m["N"], m["M"], m["dt"], warmup + m["nsteps"], *m["ic"], cutoff=m["cutoff"]))
    b.step(warmup)
    b.sync()
    # the launch schedule picked by the batch's autotuner (restores the members)
    b.autotune()
    sched = b.schedule()
    gpt = sum(m["N"] * m["M"] * min(steps, m["nsteps"]) for m in members)
    launches_per_step = step_launches(fused=bool(sched["fuse_final"]))
    active_steps = sum(min(steps, m["nsteps"]) for m in members)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(ts)
    b.step(steps)
    e1.record(ts)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    b.sync()
    nan = [b.info(i)[2] for i in ids]
    b.close()
    return ms, gpt, launches_per_step * max(min(steps, m["nsteps"]) for m in members), active_steps, nan, sched


SUBCYCLES = 6


def step_launches(subcycles=SUBCYCLES, fused=True):
    """Kernel launches of one csp2 model step: per predict_correct 3 stage
    launches and beta, the final update of the step's last predict_correct
    (the others are formed by the next one's first stage when fused), then
    diag + diag_finalize."""
    pcs = subcycles + 2
    return 4 * pcs + (1 if fused else pcs) + 2


def stage_words_per_launch(subcycles=SUBCYCLES, fused=True):
    """Algorithmic prognostic words per grid point of a stage launch, mean
    over a step: predict 1 reads the level and ghs, writes S1 (7); with the
    previous final update fused it also reads that update's base level and
    T_new and writes the level instead of reading it (13); predict 2 reads
    S1, the base level and ghs, writes T_old and S2 (13); correct reads S2,
    ghs and T_old, writes T_new (10).  FP32 compensation words are not
    counted."""
    pcs = subcycles + 2
    s1 = 7 + (pcs - 1) * (13 if fused else 7)
    return (s1 + 13 * pcs + 10 * pcs) / (3 * pcs)


def apply_schedule(b, sched):
    if sched:
        b.set_tile(*sched["tile"])
        b.set_schedule(sched["split_rows"], sched["fuse_final"], sched["pair_rows"])


def e2e_batch(gdc, torch, members, steps, precision, sched=None):
    """The same job through the C ABI from host buffers: admit (H2D), step,
    read every member's state back (D2H), all inside the timed region; the
    schedule the autotuner picked for the ensemble is set, not re-tuned."""
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b = gdc.Batch(scheme(gdc, precision))
    apply_schedule(b, sched)
    ids = [b.add(m["N"], m["M"], m["dt"], min(steps, m["nsteps"]), *m["ic"], cutoff=m["cutoff"]) for m in members]
    b.step(steps)
    b.sync()
    outs = [b.get_state(i) for i in ids]
    t1 = time.perf_counter()
    b.close()
    h2d = sum(sum(a.nbytes for a in m["ic"]) for m in members)
    d2h = sum(sum(a.nbytes for a in o) for o in outs)
    gpt = sum(m["N"] * m["M"] * min(steps, m["nsteps"]) for m in members)
    return (t1 - t0) * 1e3, gpt, h2d, d2h


def profile_kernels(gdc, members, precision, nsteps=2, sched=None):
    """Per-kernel-kind device time, launch by launch with CUDA events."""
    b = gdc.Batch(scheme(gdc, precision))
    apply_schedule(b, sched)
    for m in members:
        b.add(m["N"], m["M"], m["dt"], nsteps + 1, *m["ic"], cutoff=m["cutoff"])
    b.step(1)  # module load, attributes
    b.sync()
    ms, n = b.profile(nsteps)
    b.close()
    return ms, n


def plain_fp64(gdc, torch, ts, steps=360):
    """The seeded 360x181 state (dt 240 s) through the plain FP64 path: one
    member, 360 steps."""
    N, M, dt, _, cut = GRIDS[360]
    ic = gdc.ic_seeded(N, M, seed=0)
    p = gdc.default_params(num_lon=N, num_lat=M, time_step_size=dt, subcycles=6, split_scheme=gdc.SPLIT_CSP2,
                           qcon_modified=1, zonal_tend_filter_cutoff_wavenumber=cut, precision=gdc.FP64)
    out = {}
    for prec in (gdc.FP64, gdc.FP32):
        p.precision = prec
        m = gdc.Model(p)
        m.set_stream(ts.cuda_stream)
        m.set_state(*ic)
        m.run(3)
        m.set_state(*ic)
        m.run(1)
        m.set_state(*ic)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(ts)
        m.step(steps)
        e1.record(ts)
        torch.cuda.synchronize()
        m.sync()
        out[prec] = (e0.elapsed_time(e1), m.get_state())
        m.close()
    import numpy as np
    def rl2(a, b):
        x, y = a[2:-2, 2:-2], b[2:-2, 2:-2]
        return float(np.sqrt(np.sum((x - y) ** 2) / np.sum(y * y)))
    s64, s32 = out[gdc.FP64][1], out[gdc.FP32][1]
    return {"value": N * M * steps / (out[gdc.FP64][0] / 1e3), "ms": out[gdc.FP64][0],
            "fp32_value": N * M * steps / (out[gdc.FP32][0] / 1e3),
            "l2_fp32_vs_fp64": {"gd": rl2(s32[2], s64[2]), "u": rl2(s32[0], s64[0]), "v": rl2(s32[1], s64[1])},
            "fp64_fma_gfma_per_s": gdc.fp64_fma_rate(torch.cuda.current_device())}


def stage_traffic():
    """DRAM bytes per stage launch from the committed ncu capture of this
    workload (the .traffic.json beside its summary under profiles/)."""
    try:
        rec = json.loads((ROOT / "profiles" / "stage_kernel_f32_16x64_ensemble64.traffic.json").read_text())
        return rec["mean_dram_bytes_per_launch"]
    except Exception:
        return None


def beside_path(gdc, torch):
    """Timings of the rows beside the hot path (host-visible, CUDA-synchronised
    wall clock): admitting a 1440x721 FP32 member from host arrays vs
    generating its state on the device; checkpoint, restore and the history
    fields of that member; and the WENO advection option against the centred
    scheme on 64 x 180x91 FP32 members (no splitting, dt 90 s, 8 steps after
    2 warm-up steps: the range in which the reference's WENO stays stable)."""
    out = {}

    def timed(f):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = f()
        torch.cuda.synchronize()
        return r, (time.perf_counter() - t0) * 1e3

    try:
        N, M, dt, _, cut = GRIDS[1440]
        b = gdc.Batch(scheme(gdc, gdc.FP32, subcycles=8))
        spec = gdc.ic_spec(gdc.IC_SEEDED, seed=1, noise_seed=7, noise_sigma=gdc.G)

        def host_add():
            ic = gdc.ic_seeded(N, M, seed=1)
            gdc.ic_add_noise(ic[2], N, M, 7, gdc.G)
            return b.add(N, M, dt, 4, *ic, cutoff=cut)

        _, host_ms = timed(host_add)
        idv, dev_ms = timed(lambda: b.add_ic(N, M, dt, 4, spec, cutoff=cut))
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "member.rst")
            _, ck_ms = timed(lambda: b.checkpoint(idv, path))
            _, rs_ms = timed(lambda: b.restore(path))
        _, hist_ms = timed(lambda: b.history(idv))
        b.close()
        out["admission_1440x721_ms"] = {"host_arrays": host_ms, "device_generated": dev_ms}
        out["checkpoint_1440x721_ms"] = ck_ms
        out["restore_1440x721_ms"] = rs_ms
        out["history_fields_1440x721_ms"] = hist_ms
        rates, nans = {}, {}
        ic = gdc.ic_seeded(180, 91, seed=2)
        for name, adv in (("center_diff", gdc.ADV_CENTER_DIFF), ("weno", gdc.ADV_WENO)):
            q = gdc.default_params(num_lon=180, num_lat=91, time_step_size=90.0, subcycles=6,
                                   split_scheme=gdc.SPLIT_NONE, qcon_modified=1, uv_adv_scheme=adv,
                                   use_zonal_tend_filter=1, zonal_tend_filter_cutoff_wavenumber=[3] * 3,
                                   precision=gdc.FP32)
            bb = gdc.Batch(q)
            ids = [bb.add(180, 91, 90.0, 10, *ic) for _ in range(64)]
            bb.step(2)
            bb.sync()
            _, ms = timed(lambda: (bb.step(8), bb.sync()))
            rates[name] = 64 * 180 * 91 * 8 / (ms / 1e3)
            nans[name] = sum(1 for i in ids if bb.info(i)[2] >= 0)
            bb.close()
        out["uv_adv_scheme_grid_pt_steps_per_s"] = rates
        out["uv_adv_scheme_nan_members"] = nans
    except Exception as e:  # a failure here must not cost the headline line
        out["error"] = repr(e)
    return out


def serve_sample(gdc, ts, n=40, rate=20.0, seed=0):
    """The serving loop on the first `n` requests of the Poisson stream
    (20 requests/s; grids 180x91..1440x721; 6 h to 5 days), FP32; one batch
    per subcycle class, each on its own stream."""
    from gdc import serve
    reqs = serve.poisson_stream(n=2000, rate=rate, seed=seed)[:n]
    srv = serve.Server(precision=gdc.FP32, steps_per_tick=4)
    st = srv.run(reqs)
    srv.close()
    st.update({"max_resident": srv.max_resident, "ticks": srv.ticks, "steps_per_tick": 4,
               "subcycles": dict((str(g), m) for g, m in serve.SUBCYCLES.items()),
               "sample": f"first {n} of 2000 requests of the Poisson stream (rate {rate}/s, seed {seed}); "
                         f"offered load exceeds one GPU's rate, so latency includes queueing"})
    return st


def serve_run(args):
    """The serving configuration: a Poisson stream of --requests requests at
    20 per second (grid uniform over 180x91..1440x721, length uniform in
    6 h..5 days, dt 240 s per degree), admitted by free device memory into
    continuously batched FP32 steps; p50/p99 time to completion and the
    aggregate grid-point steps per second."""
    import __graft_entry__
    __graft_entry__.build()
    import gdc
    from gdc import serve
    reqs = serve.poisson_stream(n=args.requests, rate=20.0, seed=0)
    srv = serve.Server(precision=gdc.FP32, steps_per_tick=4)
    t0 = time.perf_counter()
    st = srv.run(reqs)
    wall = time.perf_counter() - t0
    srv.close()
    st.update({"workload": "serve", "wall_s": wall, "max_resident": srv.max_resident, "ticks": srv.ticks,
               "steps_per_tick": 4, "subcycles": dict((str(g), m) for g, m in serve.SUBCYCLES.items()),
               "stream": f"{args.requests} requests, Poisson 20/s, seed 0", "dtype": "f32"})
    print(json.dumps(st), flush=True)


def _rl2(a, b):
    x, y = a[2:-2, 2:-2], b[2:-2, 2:-2]
    return float((((x - y) ** 2).sum() / (y * y).sum()) ** 0.5)


def large_run(args):
    """1440x721, dt 60 s, 8 subcycles: FP32 (compensated levels; FP64 pole
    caps and integrals) for args.days model days and the FP64 path (bitwise
    equal to the oracle) for args.fp64_days, with mass and total-energy
    drift per day; for each FP64 day the relative L2 of gd, u, v FP32 vs
    FP64, beside a perturbation-growth control: the FP64 run started from
    its state with gd perturbed by 1e-13 relative (seeded), vs the FP64
    run.  Initial state: degree 1..12 seeded harmonics plus 3 seeded 2000 m
    mountains."""
    import numpy as np
    import __graft_entry__
    __graft_entry__.build()
    import gdc
    N, M, dt, spd, cut = GRIDS[1440]
    ic = gdc.ic_seeded(N, M, seed=0, lmax=12, n_mountains=3, mountain_height=2000.0, mountain_radius_deg=20.0)
    gd_p = ic[2].copy()
    gd_p[2:-2, 2:-2] *= 1.0 + 1e-13 * np.random.default_rng(0).uniform(-1.0, 1.0, size=gd_p[2:-2, 2:-2].shape)
    ic_p = (ic[0], ic[1], gd_p, ic[3])
    out = {"workload": "large-run", "grid": f"{N}x{M}", "dt": dt, "subcycles": 8, "days": args.days,
           "fp64_days": args.fp64_days, "perturbation": "gd x (1 + 1e-13 U(-1,1)), seed 0"}
    states = {}
    for key, prec, days, start in (("fp32", gdc.FP32, args.days, ic), ("fp64", gdc.FP64, args.fp64_days, ic),
                                   ("fp64_perturbed", gdc.FP64, args.fp64_days, ic_p)):
        p = gdc.default_params(num_lon=N, num_lat=M, time_step_size=dt, subcycles=8, split_scheme=gdc.SPLIT_CSP2,
                               qcon_modified=1, zonal_tend_filter_cutoff_wavenumber=cut, precision=prec)
        b = gdc.Batch(p)
        mid = b.add(N, M, dt, days * spd, *start)
        m0, e0, _ = b.diag(mid)
        rows = []
        t = time.perf_counter()
        for d in range(1, days + 1):
            b.step(spd)
            b.sync()
            m, e, beta = b.diag(mid)
            rows.append({"day": d, "mass_drift": (m - m0) / m0, "energy_drift": (e - e0) / e0, "beta": beta,
                         "nan_step": b.info(mid)[2]})
            if d <= args.fp64_days:
                states[(key, d)] = b.get_state(mid)
        secs = time.perf_counter() - t
        b.close()
        out[key] = {"per_day": rows, "seconds": secs, "grid_pt_steps_per_s": N * M * days * spd / secs}
    out["l2_vs_fp64"] = []
    for d in range(1, min(args.days, args.fp64_days) + 1):
        ref = states[("fp64", d)]
        row = {"day": d}
        for key in ("fp32", "fp64_perturbed"):
            s_ = states[(key, d)]
            row[key] = {"gd": _rl2(s_[2], ref[2]), "u": _rl2(s_[0], ref[0]), "v": _rl2(s_[1], ref[1])}
        out["l2_vs_fp64"].append(row)
    print(json.dumps(out), flush=True)


def precision_config1(gdc, torch, ts, rtol=1e-5):
    """The precision configuration: 720x361, dt 120 s, 720 steps (one model
    day), a uniform zonal flow u = 20 cos(lat) m/s in geostrophic balance
    over 3 seeded 2000 m Gaussian mountains (20 degree e-folding radius),
    gd0 = 5960 m g; FP32 with compensated time levels against the FP64 path.
    The zonal flow makes the reference's filter rescale noise-driven on the
    filtered rows, so both runs use the rescale guard (rtol)."""
    N, M, dt = 720, 361, 120.0
    ic = gdc.ic_seeded(N, M, seed=1, lmax=0, gd0=5960 * G, gd_rms=0.0, psi_rms=0.0, u0=20.0, n_mountains=3,
                       mountain_height=2000.0, mountain_radius_deg=20.0)
    out, st = {}, {}
    for name, prec in (("fp64", gdc.FP64), ("fp32", gdc.FP32)):
        p = gdc.default_params(num_lon=N, num_lat=M, time_step_size=dt, subcycles=6, split_scheme=gdc.SPLIT_CSP2,
                               qcon_modified=1, zonal_tend_filter_cutoff_wavenumber=[4] * 10, precision=prec,
                               filter_rescale_rtol=rtol)
        m = gdc.Model(p)
        m.set_stream(ts.cuda_stream)
        m.set_state(*ic)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(ts)
        m.step(720)
        e1.record(ts)
        torch.cuda.synchronize()
        m.sync()
        out[name + "_grid_pt_steps_per_s"] = N * M * 720 / (e0.elapsed_time(e1) / 1e3)
        st[name] = m.get_state()
        m.close()
    u32, v32, g32 = st["fp32"]
    u64, v64, g64 = st["fp64"]
    out["l2_fp32_vs_fp64"] = {"gd": _rl2(g32, g64), "u": _rl2(u32, u64), "v": _rl2(v32, v64)}
    out["config"] = "720x361 dt 120 s, 720 steps, zonal flow over 3 mountains, csp2 6, cutoffs 4 x 10"
    out["filter_rescale_rtol"] = rtol
    return out


def plain_run(args):
    """The plain FP64 path alone: the seeded 360x181 state, dt 240 s, csp2
    with 6 subcycles, for --steps steps (default one model day) after
    --warmup steps, timed with CUDA events.  Short runs of this workload
    are the FP64 profiling case."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    import gdc
    ts = torch.cuda.Stream()
    N, M, dt, spd, cut = GRIDS[360]
    steps = args.steps if args.steps_given else spd
    ic = gdc.ic_seeded(N, M, seed=0)
    p = gdc.default_params(num_lon=N, num_lat=M, time_step_size=dt, subcycles=6, split_scheme=gdc.SPLIT_CSP2,
                           qcon_modified=1, zonal_tend_filter_cutoff_wavenumber=cut, precision=gdc.FP64)
    m = gdc.Model(p)
    m.set_stream(ts.cuda_stream)
    m.set_state(*ic)
    m.run(args.warmup)
    m.set_state(*ic)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(ts)
    m.step(steps)
    e1.record(ts)
    torch.cuda.synchronize()
    m.sync()
    ms = e0.elapsed_time(e1)
    m.close()
    print(json.dumps({"workload": "plain", "grid": f"{N}x{M}", "dtype": "f64", "steps": steps,
                      "value": N * M * steps / (ms / 1e3), "unit": "grid-pt-steps/s", "ms": ms}), flush=True)


def cpu_baseline_sample(seconds_target=12.0):
    """The oracle (port of the reference, 1 thread) on a 360x181 member."""
    import gdc
    from oracle.oracle import OracleModel
    N, M, dt, _, cut = GRIDS[360]
    ic = gdc.ic_seeded(N, M, seed=0)
    o = OracleModel(N, M, dt, subcycles=6, split_scheme=2, qcon_modified=1, cutoff=cut, kind="fast")
    o.set_state(*ic)
    t0 = time.perf_counter()
    o.step(2)
    per = (time.perf_counter() - t0) / 2
    n = max(2, int(seconds_target / per))
    t0 = time.perf_counter()
    o.step(n)
    t = time.perf_counter() - t0
    return {"value": N * M * n / t, "unit": "grid-pt-steps/s", "cores": 1, "kind": "port",
            "sample": f"oracle restatement of the reference (FP64, running sums in the reference's order, FFTPACK "
                      f"transforms, -Ofast as the reference's build, 1 thread): one 360x181 member, {n} csp2 steps"}


def run_ours(args, rank, world, dist):
    import torch
    import __graft_entry__
    __graft_entry__.build()
    import gdc
    torch.cuda.init()
    ts = torch.cuda.Stream()
    members = ensemble_ics(gdc)
    if args.profile_only:
        # Short run of the batched step for profilers (ncu launch lists).
        b = gdc.Batch(scheme(gdc, gdc.FP32))
        for m in members:
            b.add(m["N"], m["M"], m["dt"], args.warmup + args.steps, *m["ic"], cutoff=m["cutoff"])
        b.step(args.warmup + args.steps)
        b.sync()
        b.close()
        return
    pk = peaks()
    # Warm the FP32 kernels and the FP64 plain path before anything is timed.
    barrier(dist)
    with Clocks(int(os.environ.get("LOCAL_RANK", 0))) as clk:
        ms, gpt, launches, active_steps, nan, sched = time_batch(gdc, torch, members, args.steps, args.warmup,
                                                                 gdc.FP32, ts)
    clocks = clk.summary()
    value, ms_all = replica_value(dist, gpt, ms)
    plain = plain_fp64(gdc, torch, ts)
    precision = precision_config1(gdc, torch, ts)
    # one untimed job first (as the warm-up steps of the device-side figure:
    # first-use costs of the process -- page-locked staging, the host pool,
    # the allocator -- are not per-job costs), then the timed job
    e2e_batch(gdc, torch, members, min(args.steps, 2), gdc.FP32, sched)
    e2e_ms, e2e_gpt, h2d, d2h = e2e_batch(gdc, torch, members, args.steps, gdc.FP32, sched)
    e2e_ms = reduce_max(dist, e2e_ms)
    prof_ms, prof_n = profile_kernels(gdc, members, gdc.FP32, sched=sched)
    serving = serve_sample(gdc, ts) if rank == 0 else None
    if rank != 0:
        return
    beside = beside_path(gdc, torch)
    # Roofline of the dominant kernel (the stage kernel): algorithmic bytes
    # per launch = the mean prognostic words per grid point of a stage launch
    # (stage_words_per_launch) x 4 bytes x active points.
    cells = sum(m["N"] * m["M"] for m in members)
    stage_ms = prof_ms[0] / max(prof_n[0], 1)
    stage_words = stage_words_per_launch(fused=bool(sched["fuse_final"]))
    stage_bytes = stage_words * 4 * cells
    achieved = stage_bytes / (stage_ms / 1e3) / 1e9
    hbm = pk.get("hbm_gbs")
    peak_src = "measured" if hbm else "fallback"
    hbm = hbm or 6800.0
    algo_bytes = gdc.algorithmic_bytes_per_gpt_step(scheme(gdc, gdc.FP32))
    line = {
        "metric": "grid-pt-steps/s batched FP32 vs plain FP64 on GB300 @L2<=1e-5; p50/p99 latency",
        "value": value,
        "unit": "grid-pt-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_all / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded spherical-harmonic states + per-member N(0,1 m) noise)",
        "config": dict(ENSEMBLE_CONFIG, members=len(members), grid_pt_steps=gpt,
                       parallelism=f"replicas x{world}",
                       schedule=f"autotuned: tiles {sched['tile'][0]}x{sched['tile'][1]}, "
                                f"row tasks {('auto', 'whole', 'split')[sched['split_rows'] + 1]}, "
                                f"final update {'fused' if sched['fuse_final'] else 'launched'}"
                                f"{', row tasks split over block pairs' if sched['pair_rows'] else ''}"),
        "clocks": clocks,
        "e2e": {"value": world * e2e_gpt / (e2e_ms / 1e3), "unit": "grid-pt-steps/s",
                "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": stage_traffic(), "traffic_unit": "bytes per launch (ncu, mean of one predict_correct)",
                     "kernel": f"stage_kernel<float, pass, 0, {sched['tile'][0]}, {sched['tile'][1]}>",
                     "peak_source": peak_src,
                     "stage_ms_per_launch": stage_ms, "bytes_per_launch": stage_bytes,
                     "words_per_point_per_launch": stage_words,
                     "kernel_ms": {"stage": prof_ms[0], "final": prof_ms[1], "beta": prof_ms[4],
                                   "diag": prof_ms[2]},
                     "kernel_launches": {"stage": prof_n[0], "final": prof_n[1], "beta": prof_n[4],
                                         "diag": prof_n[2]},
                     "whole_step_frac": (gpt / (ms / 1e3)) * algo_bytes / 1e9 / hbm},
        "plain_fp64": {"value": plain["value"], "unit": "grid-pt-steps/s",
                       "config": "360x181 dt 240 s, 360 steps, FP64, one member",
                       "fp32_single_member_value": plain["fp32_value"],
                       "l2_fp32_vs_fp64_after_1_day": plain["l2_fp32_vs_fp64"],
                       "batched_fp32_over_plain_fp64": value / plain["value"],
                       # the plain path's roof is the FP64 unit, not HBM (the ncu
                       # summary of its stage kernel: FP64 pipe 62-66 % busy)
                       "fp64_roof": {"fma_rate_measured_gfma_per_s": plain["fp64_fma_gfma_per_s"],
                                     "kernel": "an FMA-chain kernel on every SM (gdc_fp64_fma_rate)"}},
        "precision_720x361": precision,
        "serving": serving,
        "beside_path": beside,
        "nan_members": sum(1 for x in nan if x >= 0),
        "cpu_baseline": cpu_baseline_sample(),
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------- reference
# The reference's CPU implementation of the path is the oracle's restatement
# (the Fortran reference cannot be built here): its reference-order build
# (running sums in the reference's loop order, FFTPACK's transforms in the
# filter) compiled with the reference's flags (-Ofast).  This process tree
# never loads the product library: the initial states come from the
# oracle's own copy of the seeded-state definition (bitwise the library's).

def _product_library_mapped() -> bool:
    """Whether this process has the product library (libgdc.so) mapped."""
    try:
        with open("/proc/self/maps") as f:
            return any("libgdc.so" in line for line in f)
    except OSError:
        return False


def _ref_worker(conn, paths, tasks):
    """One host process: builds its members' states and oracle models, then
    advances them by the step counts the parent sends."""
    for p in paths:
        if p not in sys.path:
            sys.path.insert(0, p)
    from oracle.oracle import OracleModel, ic_add_noise, ic_seeded
    base, models = {}, []
    for t in tasks:
        N, M = t["N"], t["M"]
        if (N, M) not in base:
            base[(N, M)] = ic_seeded(N, M, seed=0)
        u, v, gd, ghs = base[(N, M)]
        gd = ic_add_noise(gd.copy(), N, M, t["seed"], 1.0 * G)
        o = OracleModel(N, M, t["dt"], subcycles=6, split_scheme=2, qcon_modified=1, cutoff=t["cutoff"],
                        kind="fast")
        o.set_state(u, v, gd, ghs)
        models.append([o, t["nsteps"], N * M])
    conn.send(("ready", _product_library_mapped()))
    while True:
        n = conn.recv()
        if n is None:
            break
        done, nan = 0, 0
        for rec in models:
            k = min(n, rec[1])
            if k > 0:
                nan += rec[0].step(k)
                rec[1] -= k
                done += rec[2] * k
        conn.send((done, nan))
    conn.close()


def _plain_reference(seconds_target=10.0):
    """The plain FP64 configuration (seeded 360x181, dt 240 s, csp2 6) on one
    host core: the reference-order oracle at -Ofast, bounded sample."""
    from oracle.oracle import OracleModel, ic_seeded
    N, M, dt, _, cut = GRIDS[360]
    o = OracleModel(N, M, dt, subcycles=6, split_scheme=2, qcon_modified=1, cutoff=cut, kind="fast")
    o.set_state(*ic_seeded(N, M, seed=0))
    t0 = time.perf_counter()
    o.step(2)
    per = (time.perf_counter() - t0) / 2
    n = max(2, int(seconds_target / per))
    t0 = time.perf_counter()
    o.step(n)
    t = time.perf_counter() - t0
    return {"value": N * M * n / t, "unit": "grid-pt-steps/s", "cores": 1,
            "config": "360x181 dt 240 s, FP64, one member", "sample": f"{n} csp2 steps"}


def run_reference(args, rank, world, dist):
    if rank != 0:
        return
    import multiprocessing as mp
    from oracle import build as oracle_build
    oracle_build.build()
    cores = os.cpu_count() or 1
    tasks = []
    k = 0
    for g, count in ENSEMBLE:
        N, M, dt, nsteps, cut = GRIDS[g]
        for _ in range(count):
            tasks.append(dict(N=N, M=M, dt=dt, nsteps=args.warmup + nsteps, cutoff=cut, seed=1000 + k))
            k += 1
    # Members to processes, largest first onto the least loaded (the cost of
    # a member step is proportional to its grid points).
    nproc = min(cores, len(tasks))
    load, parts = [0] * nproc, [[] for _ in range(nproc)]
    for t in sorted(tasks, key=lambda t: -t["N"] * t["M"]):
        q = load.index(min(load))
        parts[q].append(t)
        load[q] += t["N"] * t["M"]
    ctx = mp.get_context("spawn")
    paths = [str(ROOT)]
    pipes, procs = [], []
    for part in parts:
        a, b = ctx.Pipe()
        pr = ctx.Process(target=_ref_worker, args=(b, paths, part))
        pr.start()
        pipes.append(a)
        procs.append(pr)
    mapped = _product_library_mapped()
    for a in pipes:
        tag, m = a.recv()
        assert tag == "ready"
        mapped = mapped or m

    def advance(n):
        for a in pipes:
            a.send(n)
        got = [a.recv() for a in pipes]
        return sum(d for d, _ in got), sum(x for _, x in got)

    advance(args.warmup)
    t0 = time.perf_counter()
    done, nan = advance(args.steps)
    t = time.perf_counter() - t0
    for a in pipes:
        a.send(None)
    for pr in procs:
        pr.join()
    value = done / t
    plain = _plain_reference()
    sample = (f"oracle restatement of the reference (FP64, running sums in the reference's order, FFTPACK "
              f"transforms, -Ofast as the reference's build), {nproc} processes over the 64-member ensemble, "
              f"{args.steps} timed steps after {args.warmup} warm-up steps, every member as on the GPU")
    print(json.dumps({
        "impl": "reference",
        "metric": "grid-pt-steps/s batched FP32 vs plain FP64 on GB300 @L2<=1e-5; p50/p99 latency",
        "value": value, "unit": "grid-pt-steps/s", "higher_is_better": True, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3 / max(args.steps, 1),
        "dtype": "f64", "data": "synthetic (seeded spherical-harmonic states + per-member N(0,1 m) noise)",
        "config": ENSEMBLE_CONFIG, "grid_pt_steps": done, "nan_members": nan,
        "product_library_loaded": mapped,
        "cpu_baseline": {"value": value, "unit": "grid-pt-steps/s", "cores": nproc, "kind": "port",
                         "sample": sample},
        "plain_fp64": plain,
        "e2e": {"value": value, "unit": "grid-pt-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=720)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--requests", type=int, default=2000, help="serve: requests of the stream")
    ap.add_argument("--workload", default="batch", choices=["batch", "plain", "serve", "large-run"],
                    help="plain: the FP64 path alone on the seeded 360x181 state; "
                         "large-run: 1440x721 FP32 for --days model days with per-day mass and energy drift, "
                         "beside the FP64 path for --fp64-days")
    ap.add_argument("--days", type=int, default=10)
    ap.add_argument("--fp64-days", type=int, default=2)
    ap.add_argument("--profile-only", action="store_true",
                    help="run warmup+steps of the ensemble batch and exit (for ncu)")
    args = ap.parse_args()
    args.steps_given = any(a == "--steps" or a.startswith("--steps=") for a in sys.argv[1:])
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    rank, world, dist = dist_setup(args.gpus) if args.impl == "ours" else (
        int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), None)
    if args.impl == "reference":
        run_reference(args, rank, world, dist)
    elif args.workload == "large-run":
        large_run(args)
    elif args.workload == "plain":
        plain_run(args)
    elif args.workload == "serve":
        serve_run(args)
    else:
        run_ours(args, rank, world, dist)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
