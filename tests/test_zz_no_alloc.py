"""gdc_tendency_noalloc: the tendency for callers that cannot allocate.

Such callers (hosts whose allocator owns all device memory, processes under
a fixed device-memory budget) pass their own device buffers; the library
keeps its tables in a static device array.  The entry point must give the same
tendencies as the existing one (gdc_debug_tendency), call after call, and
must not change the device's free memory once set up.  Collected last so a
failure here does not stop the other tests.
"""
import ctypes

import numpy as np
import pytest

import gdc
from helpers import interior, rel_l2, scheme

pytestmark = pytest.mark.gpu


def test_noalloc_matches_existing_entry_point(native):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    free_before = None
    # Two calls in a row on different grids, passes and states: the shared
    # scratch is rewritten by each call.
    for call, (N, M, seed, pass_) in enumerate([(360, 181, 3, gdc.ALL_PASS), (180, 91, 8, gdc.FAST_PASS)]):
        p = scheme(gdc, N, M, 240.0 if N == 360 else 480.0, cutoff=(4, 4, 4))
        u, v, gd, ghs = gdc.ic_seeded(N, M, seed=seed)
        m = gdc.Model(p)
        m.set_state(u, v, gd, ghs)
        ref = m.tendency(pass_)
        iu, iv, _ = m.get_iap()
        m.close()
        # Caller-owned device buffers, interior layout (rows x N).
        t = {k: torch.from_numpy(np.ascontiguousarray(interior(a))).to(dev)
             for k, a in (("gd", gd), ("iu", iu), ("iv", iv), ("ghs", ghs), ("u", u), ("v", v))}
        out = {"du": torch.zeros((M, N), dtype=torch.float64, device=dev),
               "dv": torch.zeros((M - 1, N), dtype=torch.float64, device=dev),
               "dgd": torch.zeros((M, N), dtype=torch.float64, device=dev)}
        torch.cuda.synchronize()
        if call == 1:
            free_before = torch.cuda.mem_get_info()[0]
        gdc.tendency_noalloc(p, pass_, t["gd"].data_ptr(), t["iu"].data_ptr(), t["iv"].data_ptr(),
                             t["ghs"].data_ptr(), out["du"].data_ptr(), out["dv"].data_ptr(), out["dgd"].data_ptr(),
                             given_u=t["u"].data_ptr(), given_v=t["v"].data_ptr())
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before
        for name, r in zip(("du", "dv", "dgd"), ref):
            got = out[name].cpu().numpy()
            want = interior(r)
            # FP64 parity tolerance of the tendency tests (bitwise expected).
            assert rel_l2(np.pad(got, 2), np.pad(want, 2)) <= 1e-13, (call, name)
            assert np.array_equal(got, want), (call, name)


def test_noalloc_rejects_oversized_grid(native):
    p = scheme(gdc, 2880, 1441, 30.0)
    with pytest.raises(gdc.GdcError) as e:
        gdc.tendency_noalloc(p, 0, 1, 1, 1, 1, 1, 1, 1)
    assert e.value.code == gdc.E_CONFIG
