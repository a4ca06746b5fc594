"""Serving on the GPU: requests folded into the batched step as they arrive
give the same result as the same request advanced alone (bitwise: a
member's arithmetic does not depend on the other members)."""
import numpy as np
import pytest

import gdc
from gdc import serve

pytestmark = pytest.mark.gpu


def solo(req, ics):
    N, M, dt, _, cut = serve.GRIDS[req.grid]
    b = gdc.Batch(serve.serving_scheme(gdc.FP32, serve.SUBCYCLES[req.grid]))
    ic = ics(req)
    if isinstance(ic, gdc.ICSpec):
        mid = b.add_ic(N, M, dt, req.nsteps, ic, cutoff=cut)
    else:
        mid = b.add(N, M, dt, req.nsteps, *ic, cutoff=cut)
    b.step(req.nsteps)
    b.sync()
    out = b.get_state(mid)
    b.close()
    return out


@pytest.mark.parametrize("device_ic", [True, False])
def test_served_results_equal_solo_runs(native, device_ic):
    rng = np.random.default_rng(5)
    reqs = [serve.Request(rid=k, grid=int(rng.choice([180, 360])), nsteps=int(rng.integers(3, 25)),
                          arrival=0.001 * k) for k in range(10)]
    ics = serve.InitialStates(seed=0, device=device_ic)
    srv = serve.Server(steps_per_tick=3, initial_states=ics, tune_at=1 << 30)
    stats = srv.run(reqs, keep_results=True)
    srv.close()
    assert stats["completed"] == 10 and stats["nan_members"] == 0
    assert srv.max_resident >= 2  # requests overlapped on the device
    for r in reqs:
        ref = solo(r, ics)
        for a, b in zip(r.result, ref):
            assert np.array_equal(a, b), r
