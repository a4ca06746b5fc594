"""History output (A-grid wind, gh, divergence, vorticity) computed on the
device against the oracle: bitwise in FP64 for the initial condition (given
u, v) and after steps (u, v recovered from the IAP state), close in FP32."""
import numpy as np
import pytest

import gdc
from helpers import interior, scheme
from oracle.oracle import OracleModel

pytestmark = pytest.mark.gpu

FIELDS = ("u_a", "v_a", "gh", "div", "vor")


@pytest.mark.parametrize("steps", [0, 3])
def test_history_matches_oracle_fp64(native, steps):
    N, M = 360, 181
    p = scheme(gdc, N, M, 240.0, subcycles=2)
    ic = gdc.ic_seeded(N, M, seed=21, n_mountains=2)
    m = gdc.Model(p)
    m.set_state(*ic)
    m.run(steps)
    got = m.history()
    m.close()
    o = OracleModel.from_params(p)
    o.set_state(*ic)
    o.step(steps)
    ref = o.history()
    for f in FIELDS:
        assert np.array_equal(interior(got[f]), interior(ref[f])), f


def test_history_of_batch_member_fp32(native):
    # 6 fast subcycles: with 2 (fast step 120 s) the first unfiltered row at
    # 1 degree exceeds the fast-wave CFL limit and FP32 and FP64 part at once
    N, M = 360, 181
    p = scheme(gdc, N, M, 240.0, subcycles=6, precision=gdc.FP32)
    ic = gdc.ic_seeded(N, M, seed=22)
    b = gdc.Batch(p)
    mid = b.add(N, M, 240.0, 3, *ic)
    b.step(3)
    b.sync()
    got = b.history(mid)
    b.close()
    o = OracleModel.from_params(scheme(gdc, N, M, 240.0, subcycles=6))
    o.set_state(*ic)
    o.step(3)
    ref = o.history()
    for f in ("u_a", "v_a", "gh"):
        x, y = interior(got[f]), interior(ref[f])
        assert np.sqrt(np.sum((x - y) ** 2) / np.sum(y * y)) < 1e-5, f
    # div and vor difference nearby winds over the short polar dx: an FP32
    # state's 1e-7 relative error shows up there at ~0.5 % of their scale
    for f in ("div", "vor"):
        x, y = interior(got[f]), interior(ref[f])
        assert np.abs(x - y).max() < 1e-2 * np.abs(y).max(), f
