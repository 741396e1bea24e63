"""Bounded pipeline waits of the tcgen05 convolution kernel (k_conv_tc).

Every mbarrier wait of the kernel's producer, MMA and epilogue roles gives up
after a limit (tdbem_set_pipeline_wait; 2 s by default).  Here the limit is
set to one nanosecond, so waits run out in every launch: the march must fail
with TDBEM_ERR_CUDA naming the wait, every CTA must have released its tensor
memory (the kernel counts CTAs holding TMEM: +1 after tcgen05.alloc, -1 after
tcgen05.dealloc), and with the default limit restored the same context must
march again to bitwise the histories it gave before.  No wait is left
unbounded and nothing faults: a run-out wait only makes the roles stop, drain
their copies and MMAs (with the 2 s drain limit) and return."""
import re

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tdlib():
    import build as b
    b.build()
    from tdbem import lib
    lib.load()
    return lib


def _check_timeout(err):
    assert err.code == -2  # TDBEM_ERR_CUDA
    msg = str(err)
    m = re.search(r"timed out \(code (\d)", msg)
    assert m and 1 <= int(m.group(1)) <= 4, msg
    h = re.search(r"still holding TMEM: (-?\d+)", msg)
    assert h and int(h.group(1)) == 0, msg


def test_march_wait_runs_out_and_context_recovers(tdlib):
    from tdbem import meshes
    m = meshes.cubed_sphere(8, numstep=80)
    with tdlib.Context(m) as ctx:
        ctx.set_alpha(0.25, 0.0)
        ctx.assemble(precision=tdlib.MIXED)
        u0, t0 = ctx.march()
        ctx.set_pipeline_wait(1e-9)
        with pytest.raises(tdlib.TdbemError) as e:
            ctx.march()
        _check_timeout(e.value)
        ctx.set_pipeline_wait(0)
        u1, t1 = ctx.march()
    assert np.array_equal(u0, u1) and np.array_equal(t0, t1)


def test_batch_wait_runs_out_and_context_recovers(tdlib):
    from tdbem import loads, meshes
    m = meshes.cubed_sphere(8, numstep=60)
    trac, amp = loads.gaussian_patch_cases(m, 4, seed=3)
    with tdlib.Context(m) as ctx:
        ctx.set_alpha(0.25, 0.0)
        ctx.assemble(precision=tdlib.MIXED)
        u0, t0 = ctx.march_batch(trac, amp)
        ctx.set_pipeline_wait(1e-9)
        with pytest.raises(tdlib.TdbemError) as e:
            ctx.march_batch(trac, amp)
        _check_timeout(e.value)
        ctx.set_pipeline_wait(0)
        u1, t1 = ctx.march_batch(trac, amp)
    assert np.array_equal(u0, u1) and np.array_equal(t0, t1)


def test_wait_limit_range(tdlib):
    from tdbem import meshes
    with tdlib.Context(meshes.cubed_sphere(4, numstep=10)) as ctx:
        for bad in (-1.0, 61.0, float("nan")):
            with pytest.raises(tdlib.TdbemError):
                ctx.set_pipeline_wait(bad)
