"""The allocation-free single-step assembly, tdbem_gh_driver_noalloc.

Callers that cannot allocate device memory (a host application that reserves
all of it at start-up, or a latency-critical loop that cannot take the device
synchronisation of cudaMalloc/cudaFree) pass their own device output buffers;
the kernels' scratch lives in a fixed array inside the library.  Two calls in a
row (two different steps, so the shared scratch array holds the first call's
contents when the second starts) must each match tdbem_gh_driver, which
allocates, within the parity tolerance of the other GPU tests.  This file is
collected last so that a first failure here leaves every other test run."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden, rel_max

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module")
def tdlib():
    import build as b
    b.build()
    from tdbem import lib
    lib.load()
    return lib


def test_noalloc_matches_allocating_entry_point_twice(tdlib):
    torch = pytest.importorskip("torch")
    z, m = load_golden("ref_spherical_cavity_1_40")
    lo, hi = 5, 120
    rows = 3 * (hi - lo + 1)
    L = tdlib.load()
    with tdlib.Context(m) as ctx:
        torch.cuda.set_device(0)
        outs = [torch.full((rows, ctx.D), float("nan"), dtype=torch.float64, device="cuda")
                for _ in range(4)]
        for step in (1, 3):  # C term on the first call only; scratch reused by the second
            ref = ctx.gh_driver(step, lo, hi)  # G_I, G_J, H_I, H_J from the allocating path
            rc = L.tdbem_gh_driver_noalloc(ctx.h, step, lo, hi,
                                           *[ctypes.c_void_p(o.data_ptr()) for o in outs], None)
            assert rc == 0, L.tdbem_last_error().decode()
            torch.cuda.synchronize()
            for got, want, name in zip(outs, ref, ["G_I", "G_J", "H_I", "H_J"]):
                g = got.cpu().numpy()
                assert np.isfinite(g).all(), name
                assert rel_max(g, want) <= TOL, f"step {step} {name}: {rel_max(g, want):.3e}"


def test_noalloc_rejects_bad_arguments(tdlib):
    z, m = load_golden("ref_bar1")
    L = tdlib.load()
    with tdlib.Context(m) as ctx:
        assert L.tdbem_gh_driver_noalloc(ctx.h, 1, 0, m.nnd, None, None, None, None, None) == -1
        assert L.tdbem_gh_driver_noalloc(ctx.h, 0, 0, 3, ctypes.c_void_p(8), ctypes.c_void_p(8),
                                         ctypes.c_void_p(8), ctypes.c_void_p(8), None) == -1
