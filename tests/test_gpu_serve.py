"""Serving (tdbem_server_*): continuous batching of transient solves.

Each result must be the same alone and in the mix: the histories of a request
served among others equal, bitwise, those of the same solve run alone through
tdbem_march (the kernels are deterministic and contexts share no device data).
Admission keeps the resident footprint within the budget; a failing request
fails alone."""
import copy
import threading
import time

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


@pytest.fixture(scope="module")
def mix():
    from tdbem import meshes
    reqs = []
    for k, m in enumerate([meshes.bar(1, 1, 3, per_unit=3, numstep=120),
                           meshes.cubed_sphere(8, numstep=100),
                           meshes.halfspace_cavity(n_sphere=4, numstep=110),
                           meshes.bar(1, 1, 6, per_unit=2, numstep=150),
                           meshes.cubed_sphere(6, numstep=130)]):
        amp = None
        if k % 2:
            t = np.arange(m.numstep) * m.dt
            amp = np.exp(-0.5 * ((t - 15 * m.dt) / (5 * m.dt)) ** 2)
        reqs.append((m, amp))
    return reqs


def alone(lib, m, amp, precision):
    with lib.Context(m) as ctx:
        ctx.set_alpha(0.25, 0.0)
        if amp is not None:
            ctx.set_load_history(amp)
        ctx.assemble(precision=precision)
        return ctx.march()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_results_same_alone_and_in_mix(tdlib, mix, precision):
    prec = tdlib.MIXED if precision == "mixed" else tdlib.FP64
    ref = [alone(tdlib, m, a, prec) for m, a in mix]
    with tdlib.Server(0, 0, slots=4) as srv:
        ids = [srv.submit(m, amp=a, precision=prec) for m, a in mix]
        out = []
        for rid in ids:
            assert srv.wait(rid) == tdlib.REQ_DONE
            out.append(srv.result(rid))
    for (u, t), (us, ts, times) in zip(ref, out):
        assert np.array_equal(u, us) and np.array_equal(t, ts)
        assert times["latency_s"] >= times["run_s"] > 0 and times["queued_s"] >= 0


def test_admission_keeps_within_budget(tdlib, mix):
    """Budget of 1.2 x the largest footprint: never two large solves at once,
    small ones may share; everything completes; used <= budget throughout."""
    fps = [tdlib.footprint(m, tdlib.MIXED) for m, _ in mix]
    budget = int(1.2 * max(fps))
    seen = []
    with tdlib.Server(0, budget, slots=4) as srv:
        stop = threading.Event()

        def poll():
            while not stop.is_set():
                seen.append(srv.stats())
                time.sleep(0.002)

        th = threading.Thread(target=poll)
        th.start()
        ids = [srv.submit(m, amp=a) for m, a in mix + mix]
        for rid in ids:
            assert srv.wait(rid) == tdlib.REQ_DONE
            srv.result(rid)
        stop.set()
        th.join()
        st = srv.stats()
    assert st["completed"] == 2 * len(mix) and st["used_bytes"] == 0
    assert all(s["used_bytes"] <= budget for s in seen)
    assert max(s["active"] for s in seen) >= 1


def test_failing_request_fails_alone(tdlib, mix):
    m, a = mix[0]
    bad = copy.deepcopy(m)
    bad.fbc_dofs = np.array([10 ** 6], np.int32)  # out of range: tdbem_set_bc refuses it
    bad.fbc_vals = np.array([1.0])
    u_ref, _ = alone(tdlib, m, a, tdlib.MIXED)
    with tdlib.Server(0, 0, slots=2) as srv:
        r_bad = srv.submit(bad)
        r_ok = srv.submit(m, amp=a)
        assert srv.wait(r_bad) == tdlib.REQ_FAILED
        with pytest.raises(tdlib.TdbemError) as ei:
            srv.result(r_bad)
        assert ei.value.code == -1 and "out of range" in str(ei.value)
        assert srv.wait(r_ok) == tdlib.REQ_DONE
        u, _, _ = srv.result(r_ok)
    assert np.array_equal(u, u_ref)


def test_request_larger_than_budget_is_refused(tdlib, mix):
    m, _ = mix[1]
    with tdlib.Server(0, 1 << 20, slots=1) as srv:
        with pytest.raises(tdlib.TdbemError) as ei:
            srv.submit(m)
        assert ei.value.code == -3  # TDBEM_ERR_NOMEM


def test_poisson_stream_latencies(tdlib):
    from tdbem import serve
    reqs = serve.request_mix(6, rate_hz=20.0, seed=2, kinds=("bar", "sphere"),
                             sphere_range=(6, 8), steps_range=(100, 120))
    with tdlib.Server(0, 0, slots=3) as srv:
        res = serve.run_stream(srv, reqs)
    assert len(res["records"]) == 6
    assert 0 < res["p50_s"] <= res["p99_s"] <= res["wall_s"]
    assert res["dof_steps_per_s"] > 0
