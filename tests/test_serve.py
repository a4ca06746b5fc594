"""Serving loop: the request stream and the scheduling logic, on the CPU
against a fake batch engine (no device calls)."""
import numpy as np
import pytest

import gdc
from gdc import serve


def test_poisson_stream_matches_the_configuration():
    reqs = serve.poisson_stream(n=2000, rate=20.0, seed=3)
    t = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(t) > 0)
    assert abs(np.mean(np.diff(t)) - 1 / 20.0) < 0.05 / 20.0 * 3
    grids = [r.grid for r in reqs]
    assert set(grids) == {180, 360, 720, 1440}
    for g in (180, 360, 720, 1440):
        assert abs(grids.count(g) / 2000 - 0.25) < 0.05
    for r in reqs:
        dt = serve.GRIDS[r.grid][2]
        length = r.nsteps * dt
        assert 6 * 3600 - dt <= length <= 5 * 86400 + dt
    # the time step is 240 s per degree of resolution
    assert [serve.GRIDS[g][2] for g in (180, 360, 720, 1440)] == [480.0, 240.0, 120.0, 60.0]
    again = serve.poisson_stream(n=2000, rate=20.0, seed=3)
    assert [(r.grid, r.nsteps, r.arrival) for r in again] == [(r.grid, r.nsteps, r.arrival) for r in reqs]


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, s):
        self.t += max(s, 0.0)


class FakeBatch:
    """Members advance one step per step(); each step costs `step_s` of
    fake time per resident member; admission fails past `capacity`."""

    def __init__(self, clock, capacity=3, step_s=0.01):
        self.clock, self.capacity, self.step_s = clock, capacity, step_s
        self.members = {}
        self.next_id = 0
        self.adds = []
        self.specs = []

    def add(self, N, M, dt, nsteps, u, v, gd, ghs, reserve_bytes=0, cutoff=None):
        if len(self.members) >= self.capacity:
            raise gdc.GdcError(gdc.E_OOM, "full")
        mid = self.next_id
        self.next_id += 1
        self.members[mid] = [0, nsteps]
        self.adds.append((mid, N, nsteps))
        return mid

    def add_ic(self, N, M, dt, nsteps, spec, reserve_bytes=0, cutoff=None):
        self.specs.append(spec)
        return self.add(N, M, dt, nsteps, None, None, None, None, reserve_bytes, cutoff)

    def step(self, n):
        for _ in range(n):
            self.clock.t += self.step_s * max(1, len(self.members))
            for m in self.members.values():
                if m[0] < m[1]:
                    m[0] += 1

    def sync(self):
        pass

    def info(self, mid):
        s, n = self.members[mid]
        return s, s >= n, -1

    def get_state(self, mid):
        return ("state", mid)

    def remove(self, mid):
        del self.members[mid]

    def set_stream(self, s):
        pass

    def close(self):
        pass


def fake_server(capacity=3, steps_per_tick=2):
    clock = FakeClock()
    fb = FakeBatch(clock, capacity=capacity)
    srv = serve.Server(steps_per_tick=steps_per_tick, batch_factory=lambda m: fb,
                       initial_states=lambda r: (0, 0, 0, 0), clock=clock, sleep=clock.sleep)
    return srv, fb, clock


def test_server_admits_by_memory_and_completes_everything():
    reqs = [serve.Request(rid=k, grid=180, nsteps=3 + k, arrival=0.001 * k) for k in range(8)]
    srv, fb, clock = fake_server(capacity=3)
    stats = srv.run(reqs, keep_results=True)
    assert stats["completed"] == 8 and stats["offered"] == 8
    assert srv.max_resident == 3  # admission stopped at the memory limit
    assert [a[0] for a in fb.adds] == list(range(8))  # first come, first served
    for r in reqs:
        assert r.arrival <= r.admitted <= r.finished
        assert r.result == ("state", r.member)
    lat = [r.latency for r in reqs]
    assert stats["p50_s"] == pytest.approx(np.percentile(lat, 50))
    assert stats["p99_s"] == pytest.approx(np.percentile(lat, 99))
    assert stats["gpt_steps"] == sum(r.points * r.nsteps for r in reqs)
    assert not fb.members  # every member removed


def test_server_idles_until_the_next_arrival_and_honours_max_wall():
    reqs = [serve.Request(rid=0, grid=360, nsteps=2, arrival=1.0),
            serve.Request(rid=1, grid=360, nsteps=2, arrival=5.0),
            serve.Request(rid=2, grid=360, nsteps=2, arrival=50.0)]
    srv, fb, clock = fake_server(capacity=4)
    stats = srv.run(reqs, max_wall=10.0)
    assert stats["completed"] == 2 and stats["offered"] == 3
    assert reqs[0].admitted >= 1.0 and reqs[1].admitted >= 5.0
    assert np.isnan(reqs[2].finished)


def test_server_raises_when_a_request_can_never_fit():
    srv, fb, clock = fake_server(capacity=0)
    with pytest.raises(gdc.GdcError):
        srv.run([serve.Request(rid=0, grid=180, nsteps=1, arrival=0.0)])


def test_device_initial_states_go_through_add_ic():
    """The default initial states are specs of the seeded state generated on
    the device (one noise seed per request); the server admits them with
    add_ic, and host-built states with add."""
    reqs = [serve.Request(rid=k, grid=360, nsteps=2, arrival=0.0) for k in range(3)]
    clock = FakeClock()
    fb = FakeBatch(clock, capacity=5)
    srv = serve.Server(steps_per_tick=2, batch_factory=lambda m: fb, clock=clock, sleep=clock.sleep)
    stats = srv.run(reqs)
    assert stats["completed"] == 3
    assert [sp.kind for sp in fb.specs] == [gdc.IC_SEEDED] * 3
    assert [sp.noise_seed for sp in fb.specs] == [1000, 1001, 1002]
    assert all(sp.noise_sigma == pytest.approx(gdc.G) for sp in fb.specs)


def test_each_grid_runs_in_the_batch_of_its_subcycle_count():
    """180x91 and 360x181 members share the 6-subcycle batch, 1440x721
    members run in the 10-subcycle one; both batches step every tick; each
    is tuned once it holds `tune_at` members."""
    clock = FakeClock()
    made = {}

    class Tunable(FakeBatch):
        tunes = 0

        def autotune(self):
            self.tunes += 1
            return 16, 64, 1.0

    def factory(m):
        made[m] = Tunable(clock, capacity=10)
        return made[m]

    reqs = [serve.Request(rid=k, grid=g, nsteps=4, arrival=0.0) for k, g in enumerate([180, 1440, 360, 1440, 180])]
    srv = serve.Server(steps_per_tick=2, batch_factory=factory, initial_states=lambda r: (0, 0, 0, 0),
                       clock=clock, sleep=clock.sleep, tune_at=2)
    stats = srv.run(reqs)
    assert stats["completed"] == 5 and set(made) == {6, 10}
    assert sorted(N for _, N, _ in made[6].adds) == [180, 180, 360] and len(made[10].adds) == 2
    assert made[6].tunes == 1 and made[10].tunes == 1
    assert serve.SUBCYCLES == {180: 6, 360: 6, 720: 8, 1440: 10}


def test_nan_member_is_reported_and_counted_to_its_stop():
    """A member whose mass or energy turns NaN is stopped and listed; its
    grid-point steps count only the steps it did."""
    clock = FakeClock()

    class NanAt2(FakeBatch):
        def info(self, mid):
            s, n = self.members[mid]
            if mid == 1 and s >= 2:
                return s, False, 2
            return s, s >= n, -1

    fb = NanAt2(clock, capacity=4)
    reqs = [serve.Request(rid=k, grid=180, nsteps=6, arrival=0.0) for k in range(3)]
    srv = serve.Server(steps_per_tick=2, batch_factory=lambda m: fb, initial_states=lambda r: (0, 0, 0, 0),
                       clock=clock, sleep=clock.sleep)
    st = srv.run(reqs)
    assert st["completed"] == 3 and st["nan_members"] == 1
    assert st["nan_requests"] == [{"rid": 1, "grid": 180, "nsteps": 6, "nan_step": 2}]
    assert st["gpt_steps"] == reqs[0].points * (6 + 2 + 6)


def test_fp32_serving_guards_the_rescale():
    """FP32 serving skips the ill-conditioned s1/s2 rescale (guard 1e-5);
    FP64 serving keeps the reference's rescale."""
    assert serve.serving_scheme(gdc.FP32, 8).filter_rescale_rtol == pytest.approx(1e-5)
    assert serve.serving_scheme(gdc.FP64, 8).filter_rescale_rtol == 0.0
