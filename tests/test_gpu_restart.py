"""Checkpoint / restart: a restored member continues bitwise as if never
interrupted (FP64 and FP32), from an initial condition (its given u, v) and
from the middle of a run, in another batch at another time-level parity; the
file also holds the reference's restart fields u, v, gd, ghs."""
import numpy as np
import pytest

import gdc
from helpers import scheme

pytestmark = pytest.mark.gpu

HEADER = 136  # bytes before the FP64 reference fields


@pytest.mark.parametrize("prec", [gdc.FP64, gdc.FP32])
@pytest.mark.parametrize("at", [0, 4])
def test_restored_member_continues_bitwise(native, tmp_path, prec, at):
    N, M, total = 360, 181, 10
    p = scheme(gdc, N, M, 240.0, subcycles=2, precision=prec)
    ic = gdc.ic_seeded(N, M, seed=12)
    a = gdc.Batch(p)
    ia = a.add(N, M, 240.0, total, *ic)
    a.step(at)
    a.sync()
    path = tmp_path / "member.rst"
    a.checkpoint(ia, path)
    a.step(total - at)
    a.sync()
    ref, dref = a.get_state(ia), a.diag(ia)
    a.close()

    b = gdc.Batch(p)
    b.add(180, 91, 480.0, 3, *gdc.ic_seeded(180, 91, seed=1))
    b.step(1)  # the restored member lands at the other time-level parity
    ib = b.restore(path)
    assert b.info(ib)[0] == at
    b.step(total - at)
    b.sync()
    assert b.info(ib)[:2] == (total, True)
    for x, y in zip(b.get_state(ib), ref):
        assert np.array_equal(x, y)
    assert b.diag(ib) == dref
    b.close()


def test_single_model_restart_and_reference_fields(native, tmp_path):
    N, M = 180, 91
    p = scheme(gdc, N, M, 480.0, subcycles=2)
    m = gdc.Model(p)
    m.set_state(*gdc.ic_seeded(N, M, seed=3))
    m.run(3)
    path = tmp_path / "run.rst"
    m.write_restart(path)
    u3, v3, gd3 = m.get_state()
    m.run(4)
    ref = m.get_state()
    m.close()

    raw = path.read_bytes()
    f = np.frombuffer(raw, dtype=np.float64, count=3 * N * M + N * (M - 1), offset=HEADER)
    fu = f[:N * M].reshape(M, N)
    fv = f[N * M:N * M + N * (M - 1)].reshape(M - 1, N)
    fg = f[N * M + N * (M - 1):2 * N * M + N * (M - 1)].reshape(M, N)
    assert np.array_equal(fu, u3[2:-2, 2:-2]) and np.array_equal(fv, v3[2:-2, 2:-2])
    assert np.array_equal(fg, gd3[2:-2, 2:-2])

    m2 = gdc.Model(p)
    m2.read_restart(path)
    assert m2.steps_done() == 3
    m2.run(4)
    for x, y in zip(m2.get_state(), ref):
        assert np.array_equal(x, y)
    m2.close()


def test_restore_rejects_other_precision_and_truncated_files(native, tmp_path):
    N, M = 180, 91
    a = gdc.Batch(scheme(gdc, N, M, 480.0, precision=gdc.FP64))
    ia = a.add(N, M, 480.0, 2, *gdc.ic_seeded(N, M, seed=4))
    path = tmp_path / "a.rst"
    a.checkpoint(ia, path)
    a.close()
    b = gdc.Batch(scheme(gdc, N, M, 480.0, precision=gdc.FP32))
    with pytest.raises(gdc.GdcError):
        b.restore(path)
    b.close()
    cut = tmp_path / "cut.rst"
    cut.write_bytes(path.read_bytes()[:-8])
    c = gdc.Batch(scheme(gdc, N, M, 480.0, precision=gdc.FP64))
    with pytest.raises(gdc.GdcError):
        c.restore(cut)
    assert c.active() == 0
    c.close()
