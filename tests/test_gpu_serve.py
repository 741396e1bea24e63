"""Serving (tdbem_server_*): continuous batching of transient solves.

The server batches the time steps of its resident solves: every prepared solve
advances by a time block in one grouped launch, each at its own step, and solves
join and leave at block boundaries.  Each result must be the same alone and in
the mix: the histories of a request served among others equal, bitwise, those
of the same request served alone (the grouped kernels reduce each row in a fixed
order whatever else is resident).  They also match the solve run alone through
tdbem_march: FP64 at 1e-10 per step (max-norm relative, another summation
order), the mixed form at 1e-4 relative L2 (the server marches FP32 levels on
the CUDA cores, tdbem_march split-BF16 products on the tensor cores).
Admission keeps the resident footprint within the budget; a failing request
fails alone; with requests arriving while others march, grouped launches carry
several solves at once."""
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


def served(lib, reqs, prec, slots=4):
    with lib.Server(0, 0, slots=slots) as srv:
        ids = [srv.submit(m, amp=a, precision=prec) for m, a in reqs]
        out = []
        for rid in ids:
            assert srv.wait(rid) == lib.REQ_DONE
            out.append(srv.result(rid))
        stats = srv.march_stats()
    return out, stats


def rel_step_max(u, ur):
    return max((np.abs(u[s] - ur[s]).max() / np.abs(ur[s]).max()) if np.abs(ur[s]).max() else
               np.abs(u[s]).max() for s in range(ur.shape[0]))


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_results_same_alone_and_in_mix(tdlib, mix, precision):
    prec = tdlib.MIXED if precision == "mixed" else tdlib.FP64
    solo = [served(tdlib, [(m, a)], prec, slots=1)[0][0] for m, a in mix]
    out, stats = served(tdlib, mix, prec)
    assert stats["launches"] > 0 and stats["solve_steps"] > 0
    for (u1, t1, _), (us, ts, times), (m, a) in zip(solo, out, mix):
        assert np.array_equal(u1, us) and np.array_equal(t1, ts)
        assert times["latency_s"] >= times["run_s"] > 0 and times["queued_s"] >= 0
        u, t = alone(tdlib, m, a, prec)
        if prec == tdlib.FP64:
            assert rel_step_max(us, u) <= 1e-10 and rel_step_max(ts, t) <= 1e-10
        else:
            assert np.linalg.norm(us - u) / np.linalg.norm(u) <= 1e-4


def test_co_resident_steps_share_launches(tdlib):
    """Six solves of 300 steps submitted together: their marches overlap, so the
    grouped launches carry more than one resident solve on average and there are
    fewer launches than the solves' time blocks.  (How far above one the average
    goes depends on how the solves' assembly times line up, not on the engine.)"""
    from tdbem import meshes
    reqs = [(meshes.cubed_sphere(n, numstep=300), None) for n in (4, 5, 6, 6)]
    reqs += [(meshes.bar(1, 1, L, per_unit=2, numstep=300), None) for L in (3, 5)]
    out, stats = served(tdlib, reqs, tdlib.MIXED, slots=6)
    assert len(out) == 6
    blocks = sum(-(-(m.numstep - 1) // 12) for m, _ in reqs)
    print(f"launches {stats['launches']}, solve blocks {blocks}, "
          f"mean resident {stats['mean_resident']:.2f}")
    assert stats["mean_resident"] > 1.0
    assert stats["launches"] < blocks


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
    (u_solo, _, _), = served(tdlib, [(m, a)], tdlib.MIXED, slots=1)[0]
    assert np.array_equal(u, u_solo)
    assert np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref) <= 1e-4


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
