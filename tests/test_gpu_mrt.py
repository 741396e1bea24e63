"""Two-region solver (tdbem_mrt_*, SolverMRT) on the GPU against the oracle and
the reference's goldens.

Bar: 1e-10 relative per step against the oracle in its exact-zero mode, with
the displacement unknowns and the interface tractions compared apart (their
scales differ by the material stiffness), and the region displacement
histories likewise; against the reference's raw outputs, 1e-10 plus twice the
reference's round-off floor of that step (clean oracle vs reference), as for
one region.
"""
import numpy as np
import pytest

from conftest import load_mrt_golden, mrt_golden_cases, rel_max

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module")
def tdlib():
    import build as b
    b.build()
    from tdbem import lib
    lib.load()
    return lib


@pytest.fixture(scope="module")
def oracle_cache(oracle_mod):
    cache = {}

    def get(name, amp=None):
        key = (name, None if amp is None else tuple(amp))
        if key not in cache:
            z, m1, m2 = load_mrt_golden(name)
            mr = oracle_mod.MultiRegion(m1, m2, int(z["max_step"]), clean=True)
            GG, HH = mr.assemble_levels()
            X, u1, u2 = mr.march(GG, HH, amp=amp)
            cache[key] = (z, m1, m2, mr, X, u1, u2)
        return cache[key]

    return get


def check_steps(a, b, what, floor_ref=None):
    for s in range(b.shape[0]):
        if np.abs(b[s]).max() == 0:
            assert np.abs(a[s]).max() == 0, f"{what} step {s}"
            continue
        tol = TOL if floor_ref is None else TOL + 2 * rel_max(floor_ref[s], b[s])
        e = rel_max(a[s], b[s])
        assert e <= tol, f"{what} step {s}: {e:.3e} > {tol:.3e}"


def split(X, mr):
    """Displacement unknowns and interface tractions of the combined vector."""
    k = mr.NI1 + mr.NI2 + mr.NZ
    return X[:, :k], X[:, k:]


@pytest.mark.parametrize("name", mrt_golden_cases())
def test_mrt_matches_oracle_and_reference(name, tdlib, oracle_cache):
    z, m1, m2, mr, Xo, u1o, u2o = oracle_cache(name)
    with tdlib.MultiRegion(m1, m2, int(z["max_step"])) as g:
        assert (g.N, g.NG) == (mr.N, mr.NG)
        for r in (1, 2):
            u, t = g.columns(r)
            assert np.array_equal(u, mr.ucol[r - 1]) and np.array_equal(t, mr.tcol[r - 1])
        g.assemble()
        X, u1, t1, u2, t2 = g.march()
    xu, xt = split(X, mr)
    xuo, xto = split(Xo, mr)
    check_steps(xu, xuo, "x displacements")
    check_steps(xt, xto, "x interface tractions")
    check_steps(u1, u1o, "u1")
    check_steps(u2, u2o, "u2")
    # tractions of the regions: the interface traction (region 2 with the opposite
    # sign) and the interior loads
    ifc1, ifc2 = mr.tcol[0] >= 0, mr.tcol[1] >= 0
    np.testing.assert_array_equal(t1[:, ifc1], X[:, mr.tcol[0][ifc1]])
    np.testing.assert_array_equal(t2[:, ifc2], -X[:, mr.tcol[1][ifc2]])
    # against the reference's raw outputs (its ExtractField lags one step)
    ns = int(z["numstep"])
    xr_u, xr_t = split(z["x"], mr)
    check_steps(xu, xr_u, "x displacements vs reference", floor_ref=xuo)
    check_steps(xt, xr_t, "x tractions vs reference", floor_ref=xto)
    check_steps(u1[:ns], z["u1"][:ns], "u1 vs reference", floor_ref=u1o[:ns])
    check_steps(u2[:ns], z["u2"][:ns], "u2 vs reference", floor_ref=u2o[:ns])


def test_mrt_load_history(tdlib, oracle_cache):
    """A load history in place of the built-in pulse (Heaviside here)."""
    z, m1, m2 = load_mrt_golden("mrt_bar_2x2")
    amp = np.ones(m1.numstep + 1)
    _, _, _, mr, Xo, u1o, u2o = oracle_cache("mrt_bar_2x2", amp=list(amp))
    with tdlib.MultiRegion(m1, m2, int(z["max_step"])) as g:
        g.set_load_history(amp)
        g.assemble()
        X, u1, _, u2, _ = g.march()
    check_steps(u1, u1o, "u1")
    check_steps(u2, u2o, "u2")


def test_mrt_rerun_is_bitwise_and_refine_off_close(tdlib):
    z, m1, m2 = load_mrt_golden("mrt_layer_test0")
    with tdlib.MultiRegion(m1, m2, int(z["max_step"])) as g:
        g.assemble()
        a = g.march()
        b = g.march()
        g.set_refine(0)
        c = g.march()
    for p, q in zip(a, b):
        assert np.array_equal(p, q)
    check_steps(c[1], a[1], "u1 without refinement")


def test_mrt_errors(tdlib):
    z, m1, m2 = load_mrt_golden("mrt_bar_2x2")
    with tdlib.MultiRegion(m1, m2, 10) as g:
        with pytest.raises(tdlib.TdbemError) as e:
            g.march(5)
        assert e.value.code == -6  # levels not assembled
        g.assemble(5)
        with pytest.raises(tdlib.TdbemError) as e:
            g.march(8)  # levels for 5 steps, 8 needed
        assert e.value.code == -6
    bad = m2.interface.copy()
    bad[0] = bad[1]
    with pytest.raises(tdlib.TdbemError) as e:
        tdlib.MultiRegion(m1, m2, 10, iface2=bad)
    assert e.value.code == -1  # listed twice
    shifted = m2.interface.copy()
    shifted[0] = np.setdiff1d(np.arange(m2.nnd), m2.interface)[0]
    with pytest.raises(tdlib.TdbemError) as e:
        tdlib.MultiRegion(m1, m2, 10, iface2=shifted)
    assert e.value.code == -1 and "mismatch" in str(e.value)


def test_mrt_stepwise_equals_whole_run(tdlib):
    """Per-step placement (tdbem_update_gh_linear with tdbem_gh_driver blocks of each
    region, steps <= max_step) + tdbem_mrt_step gives the whole run's histories."""
    z, m1, m2 = load_mrt_golden("mrt_bar_2x2")
    L, ns = int(z["max_step"]), m1.numstep
    with tdlib.MultiRegion(m1, m2, L) as g:
        g.assemble()
        X, u1, _, u2, _ = g.march()
    with tdlib.MultiRegion(m1, m2, L) as g:
        g.begin(ns)
        xs = [np.zeros(g.N)]
        for n in range(1, ns + 1):
            if n <= L:
                for ctx in g.regions:
                    GI, GJ, HI, HJ = ctx.gh_driver(n)
                    ctx.update_gh_linear(n, GI, GJ, HI, HJ)
            xs.append(g.step(n)[0])
    Xs = np.array(xs)
    assert Xs.shape == X.shape
    mr_k = g.N - (g.N - g.NG) // 2  # displacement unknowns: NI1 + NI2 + NZ
    check_steps(Xs[:, :mr_k], X[:, :mr_k], "stepwise x displacements")
    check_steps(Xs[:, mr_k:], X[:, mr_k:], "stepwise x tractions")
