"""The oracle's reference-order arithmetic (no GPU).

The exact-sum oracle evaluates every reduction as a correctly rounded sum and
the polar filter as a projection onto the kept modes; the reference-order
build instead keeps the reference's running sums in its loop order and runs
the filter through FFTPACK 5.1's transforms (lib/fft/rfftf1.f, rfftb1.f and
their radix passes), restated in oracle/gdc_fftpack.c.  These tests pin that
restatement to the transform it computes and bound how far the two
arithmetics sit apart after one step.
"""
import numpy as np
import pytest

import gdc
from helpers import interior, rel_l2
from oracle.oracle import OracleModel, rfft

LENGTHS = [8, 12, 20, 30, 36, 144, 180, 200, 360, 720, 1440]


def packed(x):
    """FFTPACK 5.1's packing of rfft1f (lib/fft/rfftf1.f:87-109) from numpy:
    r(1) = a0, (r(2k), r(2k+1)) = (a_k, b_k) with x_n = a0 + sum_k a_k
    cos(2 pi k n/N) + b_k sin(2 pi k n/N) (+ r(N) (-1)^n for even N)."""
    n = len(x)
    X = np.fft.rfft(x)
    r = np.zeros(n)
    r[0] = X[0].real / n
    m = (n - 1) // 2
    r[1:2 * m + 1:2] = 2 * X[1:m + 1].real / n
    r[2:2 * m + 2:2] = -2 * X[1:m + 1].imag / n
    if n % 2 == 0:
        r[n - 1] = X[n // 2].real / n
    return r


@pytest.mark.parametrize("n", LENGTHS)
def test_forward_transform_is_fftpack_packing(n):
    x = np.random.default_rng(n).standard_normal(n)
    r = rfft(x)
    assert np.max(np.abs(r - packed(x))) <= 1e-15 * max(1.0, np.max(np.abs(x)))


@pytest.mark.parametrize("n", LENGTHS)
def test_backward_inverts_forward(n):
    x = np.random.default_rng(100 + n).standard_normal(n)
    y = rfft(rfft(x), backward=True)
    assert np.max(np.abs(y - x)) <= 1e-14


def test_general_radix_is_refused():
    with pytest.raises(ValueError):
        rfft(np.ones(14))  # 2 x 7: FFTPACK's general-radix pass


def test_single_mode_passes_through_the_kept_band():
    n, c = 360, 4
    lon = 2 * np.pi * np.arange(n) / n
    kept = np.cos(3 * lon) + 0.5 * np.sin(4 * lon) + 0.25 * np.cos(5 * lon)  # a_(c+1) is kept
    removed = np.sin(5 * lon) + np.cos(9 * lon)
    r = rfft(kept + removed)
    r[2 * (c + 1):] = 0.0  # filter_init's factor row: 1 for indices 1..2(c+1)
    y = rfft(r, backward=True)
    assert np.max(np.abs(y - kept)) <= 1e-14


def test_fftpack_filter_matches_projection_filter(native):
    """Both filters compute the same truncated transform; they differ only
    in rounding."""
    N, M = 360, 181
    p = dict(subcycles=6, split_scheme=2, cutoff=(4, 4, 4, 4, 4))
    a = OracleModel(N, M, 240.0, kind="exact", **p)
    b = OracleModel(N, M, 240.0, kind="ref", fft=True, **p)
    rng = np.random.default_rng(5)
    for half, j in ((0, 2), (0, 6), (1, 1), (1, 5), (0, M - 1), (1, M - 2)):
        x = np.zeros(N + 4)
        x[2:-2] = rng.standard_normal(N)
        ya, yb = a.filter_row(half, j, x), b.filter_row(half, j, x)
        assert np.max(np.abs(ya[2:-2] - yb[2:-2])) <= 1e-15, (half, j)


@pytest.mark.parametrize("kind,fft", [("ref", True), ("ref", False), ("exact", True)])
def test_reference_order_one_step_within_rounding(native, kind, fft):
    """One csp2 step of the seeded 360x181 state: the reference's order of
    summation and its transforms move the state by rounding only."""
    N, M = 360, 181
    ic = gdc.ic_seeded(N, M, seed=0)
    p = dict(subcycles=6, split_scheme=2, qcon_modified=1, cutoff=(4, 4, 4, 4, 4))
    a = OracleModel(N, M, 240.0, kind="exact", **p)
    b = OracleModel(N, M, 240.0, kind=kind, fft=fft, **p)
    for o in (a, b):
        o.set_state(*ic)
        o.step(1)
    sa, sb = a.get_state(), b.get_state()
    for f in ("gd", "u", "v", "iu", "iv"):
        assert rel_l2(sb[f], sa[f]) <= 1e-14, f
    ma, ea, ba = a.diag()
    mb, eb, bb = b.diag()
    # a plain running sum over the grid carries up to ~n eps of rounding
    assert abs(mb - ma) <= 1e-13 * abs(ma) and abs(eb - ea) <= 1e-13 * abs(ea) and abs(bb - ba) <= 1e-13


def test_rescale_record_names_the_worst_row(native):
    """The diagnostic the design notes quote: the conditioning of the
    filter's s1/s2 rescale, with the field and row where it was worst."""
    N, M = 180, 91
    o = OracleModel(N, M, 480.0, subcycles=6, split_scheme=2, cutoff=(4, 4, 4), kind="ref", fft=True)
    o.set_state(*gdc.ic_seeded(N, M, seed=0))
    o.step(2)
    (c1, f1, r1), (c2, f2, r2) = o.rescale_record()
    assert c1 >= 1.0 and c2 >= 1.0
    assert f1 in ("du", "dv", "dgd") and 1 <= r1 <= M
    assert o.rescale_record()[0][0] == 0.0  # the record resets
