"""GPU (sm_103a) plain FP64 path against the oracle and the reference's goldens.

Parity bar: 1e-10 relative, measured per level as max|G_gpu - G_oracle| /
max|G_oracle| (likewise H), and per time step as max|u_gpu - u_oracle| /
max|u_oracle| (likewise t), against the oracle in its exact-zero mode: once
both wave fronts have passed a quadrature point at both evaluation times the
step response is identically zero, and the reference's arithmetic leaves only
round-off there (up to ~6e-8 of the level norm on some inputs).  Against the
reference's raw outputs the bar is 1e-10 plus twice that measured round-off
floor, level by level and step by step.
"""
import numpy as np
import pytest

from conftest import golden_cases, load_golden, rel_max

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

    def get(name):
        if name not in cache:
            z, m = load_golden(name)
            o = oracle_mod.Oracle(m, clean=True)
            G, H = o.assemble_levels()
            u, t = o.march(G, H, float(z["a1"]), float(z["a2"]))
            cache[name] = (z, m, G, H, u, t)
        return cache[name]

    return get


def floor(a_clean, a_ref):
    """The reference's round-off floor of one level / step: clean oracle vs reference."""
    return rel_max(a_clean, a_ref)


def check_steps(u, uo, what, clean=None):
    for s in range(uo.shape[0]):
        if np.abs(uo[s]).max() == 0:
            assert np.abs(u[s]).max() == 0, f"{what} step {s}"
            continue
        tol = TOL if clean is None else TOL + 2 * floor(clean[s], uo[s])
        e = rel_max(u[s], uo[s])
        assert e <= tol, f"{what} step {s}: {e:.3e} > {tol:.3e}"


@pytest.mark.parametrize("name", golden_cases())
def test_levels_match_oracle_and_reference(name, tdlib, oracle_cache):
    z, m, Go, Ho, uo, to = oracle_cache(name)
    with tdlib.Context(m) as ctx:
        assert ctx.M == Go.shape[0] - 1
        ctx.assemble()
        G, H = ctx.levels()
    for k in range(ctx.M + 1):
        assert rel_max(G[k], Go[k]) <= TOL, f"G level {k}: {rel_max(G[k], Go[k]):.3e}"
        assert rel_max(H[k], Ho[k]) <= TOL, f"H level {k}: {rel_max(H[k], Ho[k]):.3e}"
    w = np.random.default_rng(int(z["seed"])).standard_normal(ctx.D)
    for k in range(ctx.M + 1):  # against the reference's own outputs, above its round-off
        tg = TOL + 2 * floor(Go[k] @ w, z["G_w"][k])
        th = TOL + 2 * floor(w @ Ho[k], z["w_H"][k])
        assert rel_max(G[k] @ w, z["G_w"][k]) <= tg, f"G level {k} vs reference"
        assert rel_max(w @ H[k], z["w_H"][k]) <= th, f"H level {k} vs reference"


@pytest.mark.parametrize("name", golden_cases())
def test_histories_match_oracle_and_reference(name, tdlib, oracle_cache):
    z, m, Go, Ho, uo, to = oracle_cache(name)
    with tdlib.Context(m) as ctx:
        ctx.set_alpha(float(z["a1"]), float(z["a2"]))
        ctx.assemble()
        u, t = ctx.march()
    check_steps(u, uo, "u")
    check_steps(t, to, "t")
    d = z["dofs"]
    check_steps(u[:, d], z["u"], "u vs reference", clean=uo[:, d])
    check_steps(t[:, d], z["t"], "t vs reference", clean=to[:, d])


@pytest.mark.parametrize("step", [1, 2, 5])
def test_gh_driver_matches_oracle(step, tdlib, oracle_mod):
    z, m = load_golden("ref_spherical_cavity_1_40")
    o = oracle_mod.Oracle(m, clean=True)
    lo, hi = 17, 80
    ref = o.gh_driver(step * m.dt, m.dt, lo, hi)
    with tdlib.Context(m) as ctx:
        got = ctx.gh_driver(step, lo, hi)
    for a, b, nm in zip(got, ref, ["G_I", "G_J", "H_I", "H_J"]):
        assert rel_max(a, b) <= TOL, f"{nm}: {rel_max(a, b):.3e}"


@pytest.mark.parametrize("step", [1, 3])
def test_gh_driver_q8_matches_oracle(step, tdlib, oracle_mod):
    """8-node elements: serendipity shapes, corner and midside singular nodes
    (sub-element Duffy rules), the C term, on a row block of the reference's bar."""
    z, m = load_golden("ref_bar2")
    assert m.etype == 2
    o = oracle_mod.Oracle(m, clean=True)
    lo, hi = 5, 40
    ref = o.gh_driver(step * m.dt, m.dt, lo, hi)
    with tdlib.Context(m) as ctx:
        got = ctx.gh_driver(step, lo, hi)
    for a, b, nm in zip(got, ref, ["G_I", "G_J", "H_I", "H_J"]):
        assert rel_max(a, b) <= TOL, f"{nm}: {rel_max(a, b):.3e}"


def test_reruns_are_bitwise_identical(tdlib):
    z, m = load_golden("sphere_6x4x4")
    with tdlib.Context(m) as ctx:
        ctx.set_alpha(0.25, 0.0)
        ctx.assemble()
        G1, H1 = ctx.level(3, 0), ctx.level(3, 1)
        u1, t1 = ctx.march(40)
        ctx.assemble()
        u2, t2 = ctx.march(40)
        assert np.array_equal(G1, ctx.level(3, 0)) and np.array_equal(H1, ctx.level(3, 1))
        assert np.array_equal(u1, u2) and np.array_equal(t1, t2)


def test_sphere_against_closed_form(tdlib):
    """Second oracle: radial wall displacement of the spherical cavity under step
    pressure.  A 6x8x8 cubed sphere (beta = 0.6, alpha = (0.25, 0)) must stay stable and
    settle near the static value p a / (4 mu) = 0.25 (discretisation error of this mesh)."""
    from tdbem import meshes
    m = meshes.cubed_sphere(8, numstep=240)
    with tdlib.Context(m) as ctx:
        ctx.set_alpha(0.25, 0.0)
        ctx.assemble()
        u, _ = ctx.march()
    rh = m.coords / np.linalg.norm(m.coords, axis=1, keepdims=True)
    ur = (u.reshape(u.shape[0], -1, 3) * rh).sum(2).mean(1)[:-1]
    cf = meshes.sphere_cavity_closed_form(np.arange(len(ur)) * m.dt)
    late = slice(len(ur) // 2, None)
    assert np.abs(ur[late] - cf[late]).max() < 0.03
    assert np.abs(ur).max() < 0.5  # no blow-up


def test_errors_are_status_codes(tdlib):
    z, m = load_golden("ref_halfspace_plane_1e")
    with tdlib.Context(m) as ctx:
        with pytest.raises(tdlib.TdbemError) as e:
            ctx.march(5)
        assert e.value.code == -6  # TDBEM_ERR_STATE: no levels yet
        with pytest.raises(tdlib.TdbemError) as e:
            ctx.set_alpha(0.9, 0.5)
        assert e.value.code == -1
        with pytest.raises(tdlib.TdbemError):
            ctx.set_bc([ctx.D], [0.0], [], [])
        with pytest.raises(tdlib.TdbemError):
            ctx.level(0, 0)
