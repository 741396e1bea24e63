"""The allocation-free single-step assembly, tdbem_gh_driver_noalloc.

Callers that cannot allocate device memory (a host application that reserves
all of it at start-up, or a latency-critical loop that cannot take the device
synchronisation of cudaMalloc/cudaFree) pass their own device output buffers;
the kernels' scratch lives in a fixed array inside the library.  Two calls in a
row (two different steps, so the shared scratch array holds the first call's
contents when the second starts) must each match tdbem_gh_driver, which
allocates, and the oracle (exact-zero mode), within the parity tolerance of the
other GPU tests; on the context's stream and on a stream of the caller; with the
full chunk sizes and with chunk limits lowered so that the node-chunked paths
(pair windows and the C term) run many chunks.  This file is collected last so
that a first failure here leaves every other test run."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden, rel_max

pytestmark = pytest.mark.gpu

TOL = 1e-10
NAMES = ["G_I", "G_J", "H_I", "H_J"]


@pytest.fixture(scope="module")
def tdlib():
    import build as b
    b.build()
    from tdbem import lib
    lib.load()
    return lib


def _run_twice(tdlib, torch, m, lo, hi, stream, oracle=None):
    """Steps 1 (C term) and 3 through the allocation-free call into the same
    device buffers, each checked against the allocating call (and the oracle)."""
    rows = 3 * (hi - lo + 1)
    L = tdlib.load()
    with tdlib.Context(m) as ctx:
        torch.cuda.set_device(0)
        outs = [torch.full((rows, ctx.D), float("nan"), dtype=torch.float64, device="cuda")
                for _ in range(4)]
        for step in (1, 3):
            ref = ctx.gh_driver(step, lo, hi)  # G_I, G_J, H_I, H_J from the allocating path
            torch.cuda.synchronize()
            handle = None if stream is None else ctypes.c_void_p(stream.cuda_stream)
            rc = L.tdbem_gh_driver_noalloc(ctx.h, step, lo, hi,
                                           *[ctypes.c_void_p(o.data_ptr()) for o in outs], handle)
            assert rc == 0, L.tdbem_last_error().decode()
            if stream is None:
                torch.cuda.synchronize()
            else:
                stream.synchronize()
            want_o = None if oracle is None else oracle.gh_driver(step * m.dt, m.dt, lo, hi)
            for b, (got, want, name) in enumerate(zip(outs, ref, NAMES)):
                g = got.cpu().numpy()
                assert np.isfinite(g).all(), name
                assert rel_max(g, want) <= TOL, f"step {step} {name}: {rel_max(g, want):.3e}"
                if want_o is not None:
                    e = rel_max(g, want_o[b])
                    assert e <= TOL, f"step {step} {name} vs oracle: {e:.3e}"


def test_noalloc_matches_allocating_entry_point_and_oracle_twice(tdlib, oracle_mod):
    torch = pytest.importorskip("torch")
    z, m = load_golden("ref_spherical_cavity_1_40")
    _run_twice(tdlib, torch, m, 5, 120, None, oracle_mod.Oracle(m, clean=True))


def test_noalloc_on_caller_stream_in_small_chunks(tdlib, monkeypatch):
    """A non-default stream of the caller, and per-launch limits of 64 pairs and 7
    collocation nodes: every colour runs one node per chunk and the C term 17 chunks
    (row offsets of later chunks inside the caller's row block)."""
    torch = pytest.importorskip("torch")
    monkeypatch.setenv("TDBEM_NOALLOC_CHUNK_PAIRS", "64")
    monkeypatch.setenv("TDBEM_NOALLOC_CHUNK_NODES", "7")
    z, m = load_golden("ref_spherical_cavity_1_40")
    torch.cuda.set_device(0)
    _run_twice(tdlib, torch, m, 5, 120, torch.cuda.Stream())


def test_noalloc_q8_bar(tdlib):
    """8-node elements (two threads per pair, singular sub-elements)."""
    torch = pytest.importorskip("torch")
    z, m = load_golden("ref_bar2")
    _run_twice(tdlib, torch, m, 3, 30, None)


def test_noalloc_rejects_bad_arguments(tdlib):
    z, m = load_golden("ref_bar1")
    L = tdlib.load()
    with tdlib.Context(m) as ctx:
        assert L.tdbem_gh_driver_noalloc(ctx.h, 1, 0, m.nnd, None, None, None, None, None) == -1
        assert L.tdbem_gh_driver_noalloc(ctx.h, 0, 0, 3, ctypes.c_void_p(8), ctypes.c_void_p(8),
                                         ctypes.c_void_p(8), ctypes.c_void_p(8), None) == -1
