"""Mixed precision (FP32 far-field quadrature, FP32 levels, time-blocked FP32
convolution, FP32 inverse with FP64 refinement) against the plain FP64 GPU form.

Bar: relative L2 error of the displacement and traction histories <= 1e-4
(||u_mixed - u_fp64||_2 / ||u_fp64||_2 over all steps and dofs)."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

TOL_L2 = 1e-4


@pytest.fixture(scope="module")
def tdlib():
    import build as b
    b.build()
    from tdbem import lib
    lib.load()
    return lib


def rel_l2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def run(lib, m, precision, alpha=(0.25, 0.0), block=12, refine=1, numstep=None, engine=None,
        amp=None):
    with lib.Context(m) as ctx:
        ctx.set_alpha(*alpha)
        ctx.set_march_options(block, refine)
        if engine is not None:
            ctx.set_march_engine(engine)
        if amp is not None:
            ctx.set_load_history(amp)
        ctx.assemble(precision=precision)
        u, t = ctx.march(numstep)
        lev = (ctx.level(3, 0), ctx.level(3, 1), ctx.level(ctx.M, 1))
    return u, t, lev


@pytest.fixture(scope="module")
def sphere8(tdlib):
    from tdbem import meshes
    m = meshes.cubed_sphere(8, numstep=160)
    return m, run(tdlib, m, tdlib.FP64)


def test_mixed_levels_close_to_fp64(tdlib, sphere8):
    m, (u, t, lev) = sphere8
    _, _, lev32 = run(tdlib, m, tdlib.MIXED)
    for a, b in zip(lev32, lev):
        assert np.abs(a - b).max() <= 2e-5 * np.abs(b).max()


def test_mixed_every_level_close_to_fp64(tdlib):
    """Every level of the FP32 store against the FP64 levels (oracle-pinned), 2e-5 of
    the level's max-norm: the far pairs' settled levels (P front passed at every
    Gauss point, S front at none: one quasi-static block per pair scaled by
    (k - 1/2) dt) and the levels at both fronts (the tau form) alike."""
    from tdbem import meshes
    m = meshes.cubed_sphere(8, numstep=60)
    levels = {}
    for prec in (tdlib.FP64, tdlib.MIXED):
        with tdlib.Context(m) as ctx:
            ctx.assemble(precision=prec)
            M = ctx.M
            levels[prec] = [(ctx.level(k, 0), ctx.level(k, 1)) for k in range(2, M + 1)]
    assert M > 20
    worst = 0.0
    for k, (a, b) in enumerate(zip(levels[tdlib.MIXED], levels[tdlib.FP64]), start=2):
        for x, y, nm in zip(a, b, "GH"):
            if np.abs(y).max() == 0:
                assert np.abs(x).max() == 0, f"level {k} {nm}"
                continue
            e = np.abs(x - y).max() / np.abs(y).max()
            worst = max(worst, e)
            assert e <= 2e-5, f"level {k} {nm}: {e:.2e}"
    print(f"worst level error {worst:.2e} over levels 2..{M}")


def test_mixed_c_term_close_to_fp64(tdlib):
    """Levels 0 and 1 of the mixed form (the LHS of its solves) hold the C term,
    its regular elements in FP32: the diagonal blocks stay within 1e-6 of FP64."""
    from tdbem import meshes
    m = meshes.cubed_sphere(4, numstep=20)
    out = {}
    for prec in (tdlib.FP64, tdlib.MIXED):
        with tdlib.Context(m) as ctx:
            ctx.assemble(precision=prec)
            out[prec] = [ctx.level(k, 1) for k in (0, 1)]
    n = 3 * m.nnd
    blk = np.kron(np.eye(m.nnd), np.ones((3, 3))) > 0
    for a, b in zip(out[tdlib.MIXED], out[tdlib.FP64]):
        assert a.shape == (n, n)
        assert np.abs(a - b)[blk].max() <= 1e-6 * np.abs(b[blk]).max()


@pytest.mark.parametrize("block", [1, 8, 12, 16, 24, 32])
def test_mixed_histories_within_1e4(tdlib, sphere8, block):
    m, (u, t, _) = sphere8
    u32, t32, _ = run(tdlib, m, tdlib.MIXED, block=block)
    assert rel_l2(u32, u) <= TOL_L2
    assert rel_l2(t32, t) <= TOL_L2


def test_mixed_bar_with_prescribed_displacements(tdlib):
    """UBC columns swapped into the LHS, alpha_2 != 0, traction at the loaded end."""
    z, m = load_golden("bar_1x1x4_q2_alpha")
    u, t, _ = run(tdlib, m, tdlib.FP64, alpha=(0.25, 0.1))
    u32, t32, _ = run(tdlib, m, tdlib.MIXED, alpha=(0.25, 0.1))
    assert rel_l2(u32, u) <= TOL_L2 and rel_l2(t32, t) <= TOL_L2


def bar_with_prescribed_values(seed=3):
    """The alpha bar with nonzero prescribed displacements, and its last dof both
    displacement- and traction-prescribed (the state update keeps the prescribed
    traction in that dof's history)."""
    import copy
    _, m = load_golden("bar_1x1x4_q2_alpha")
    m = copy.copy(m)
    D = 3 * m.nnd
    rng = np.random.default_rng(seed)
    m.ubc_dofs = np.unique(np.append(m.ubc_dofs, D - 1)).astype(np.int32)
    m.ubc_vals = 1e-3 * rng.standard_normal(len(m.ubc_dofs))
    m.fbc_dofs = np.append(m.fbc_dofs, D - 1).astype(np.int32)
    m.fbc_vals = np.append(m.fbc_vals, 0.5 * np.abs(m.fbc_vals).max())
    return m


@pytest.mark.parametrize("engine", ["tcgen05", "fp32"])
def test_mixed_prescribed_values_and_load_history(tdlib, engine):
    """Known values in every history term: nonzero prescribed displacements, a
    prescribed traction on a displacement-prescribed last dof, and a ramped load
    history, in both march engines against the plain FP64 march."""
    m = bar_with_prescribed_values()
    amp = np.minimum(1.0, np.arange(m.numstep + 1) / 20.0)
    eng = tdlib.ENGINE_TCGEN05 if engine == "tcgen05" else tdlib.ENGINE_FP32
    u, t, _ = run(tdlib, m, tdlib.FP64, alpha=(0.25, 0.1), amp=amp)
    for block in (4, 16):
        u32, t32, _ = run(tdlib, m, tdlib.MIXED, alpha=(0.25, 0.1), amp=amp, engine=eng,
                          block=block)
        assert rel_l2(u32, u) <= TOL_L2 and rel_l2(t32, t) <= TOL_L2


def test_long_blocks_need_the_tcgen05_engine(tdlib):
    _, m = load_golden("bar_1x1x4_q2_alpha")
    with tdlib.Context(m) as ctx:
        ctx.set_march_options(32, 0)
        ctx.set_march_engine(tdlib.ENGINE_FP32)
        ctx.assemble(precision=tdlib.MIXED)
        with pytest.raises(tdlib.TdbemError) as e:
            ctx.march()
        assert e.value.code == -1 and "tcgen05" in str(e.value)
        with pytest.raises(tdlib.TdbemError):
            ctx.set_march_options(20, 0)


def test_load_history_of_exactly_numstep_values(tdlib):
    """A load history with one value per step (the shortest accepted) marches like the
    same history with an extra trailing value, in both engines."""
    m = bar_with_prescribed_values()
    amp = np.minimum(1.0, np.arange(m.numstep) / 20.0)
    for engine in (tdlib.ENGINE_TCGEN05, tdlib.ENGINE_FP32):
        u1, t1, _ = run(tdlib, m, tdlib.MIXED, alpha=(0.25, 0.1), amp=amp, engine=engine)
        u2, t2, _ = run(tdlib, m, tdlib.MIXED, alpha=(0.25, 0.1), engine=engine,
                        amp=np.append(amp, 7.0))
        assert np.array_equal(u1, u2) and np.array_equal(t1, t2)


def test_new_boundary_values_reach_the_merged_levels(tdlib):
    """tdbem_set_bc between two marches of one assembly: the second march uses the
    new values (the merged levels and their known part are rebuilt)."""
    _, m0 = load_golden("bar_1x1x4_q2_alpha")
    m1 = bar_with_prescribed_values()
    ref, _, _ = run(tdlib, m1, tdlib.MIXED, alpha=(0.25, 0.1))
    with tdlib.Context(m0) as ctx:
        ctx.set_alpha(0.25, 0.1)
        ctx.set_march_options(12, 1)
        ctx.assemble(precision=tdlib.MIXED)
        ctx.march()
        ctx.set_bc(m1.ubc_dofs, m1.ubc_vals, m1.fbc_dofs, m1.fbc_vals)
        u, _ = ctx.march()
    assert np.array_equal(u, ref)


@pytest.mark.parametrize("case", ["alpha_bar", "prescribed", "q8"])
def test_default_options_within_1e4(tdlib, case):
    """The library's default march options (tcgen05 engine, 16-step blocks, no
    refinement sweep) on the bars with prescribed displacements, known values in
    every history term, and 8-node elements."""
    if case == "q8":
        z, m = load_golden("ref_bar2_alpha")
        a = (float(z["a1"]), float(z["a2"]))
    else:
        m = bar_with_prescribed_values() if case == "prescribed" else \
            load_golden("bar_1x1x4_q2_alpha")[1]
        a = (0.25, 0.1)
    u, t, _ = run(tdlib, m, tdlib.FP64, alpha=a)
    with tdlib.Context(m) as ctx:
        ctx.set_alpha(*a)
        ctx.assemble(precision=tdlib.MIXED)
        u32, t32 = ctx.march()
    assert rel_l2(u32, u) <= TOL_L2 and rel_l2(t32, t) <= TOL_L2


def test_mixed_q8_bar(tdlib):
    """8-node elements in mixed precision: every pair through the FP64 quadrature
    into the FP32 store, FP32 convolution and FP32 inverse with refinement."""
    z, m = load_golden("ref_bar2_alpha")
    a = (float(z["a1"]), float(z["a2"]))
    u, t, _ = run(tdlib, m, tdlib.FP64, alpha=a)
    u32, t32, _ = run(tdlib, m, tdlib.MIXED, alpha=a)
    assert rel_l2(u32, u) <= TOL_L2
    assert rel_l2(t32, t) <= TOL_L2


def test_refinement_recovers_fp64_solve(tdlib, sphere8):
    """With FP32 convolution products the inverse's error dominates; refinement
    removes it (under split-BF16 products the convolution's ~1e-5 dominates)."""
    m, (u, t, _) = sphere8
    e0 = rel_l2(run(tdlib, m, tdlib.MIXED, refine=0, engine=tdlib.ENGINE_FP32)[0], u)
    e2 = rel_l2(run(tdlib, m, tdlib.MIXED, refine=2, engine=tdlib.ENGINE_FP32)[0], u)
    assert e2 <= e0 and e2 <= TOL_L2


@pytest.mark.parametrize("block", [8, 16])
def test_march_engines(tdlib, sphere8, block):
    """Old-history pass on the tensor cores (split-BF16, the default) and on the CUDA
    cores (FP32 products): both within the bar, the FP32 one near FP32 round-off."""
    m, (u, t, _) = sphere8
    u_tc, t_tc, _ = run(tdlib, m, tdlib.MIXED, block=block, engine=tdlib.ENGINE_TCGEN05)
    u_32, t_32, _ = run(tdlib, m, tdlib.MIXED, block=block, engine=tdlib.ENGINE_FP32)
    assert rel_l2(u_tc, u) <= TOL_L2 and rel_l2(t_tc, t) <= TOL_L2
    assert rel_l2(u_32, u) <= 1e-6
    assert rel_l2(u_tc, u) > rel_l2(u_32, u)  # the split products are the coarser ones


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_graph_replay_is_bitwise_the_direct_loop(tdlib, precision):
    """The marching loop replayed as a CUDA graph gives the histories of the direct
    loop bitwise; a new load history is captured anew."""
    z, m = load_golden("bar_1x1x4_q2_alpha")
    prec = tdlib.MIXED if precision == "mixed" else tdlib.FP64
    t = np.arange(m.numstep) * m.dt
    amp2 = np.exp(-0.5 * ((t - 10 * m.dt) / (4 * m.dt)) ** 2)
    out = {}
    for graphs in (False, True):
        with tdlib.Context(m) as ctx:
            ctx.set_alpha(0.25, 0.1)
            ctx.set_graphs(graphs)
            ctx.assemble(precision=prec)
            first = ctx.march()
            again = ctx.march()  # replay (or the same direct loop)
            ctx.set_load_history(amp2)
            other = ctx.march()  # a new capture
            out[graphs] = (first, again, other)
    for a, b in zip(out[False], out[True]):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(out[True][0][0], out[True][1][0])
    assert not np.array_equal(out[True][0][0], out[True][2][0])


def test_step_matrices_follow_the_weights(tdlib):
    """The step-distance matrices of the tcgen05 march (B_d, combinations of three
    levels with the averaging weights) are rebuilt when the weights change between
    two marches of one assembly: the second march equals a fresh context's."""
    from tdbem import meshes
    m = meshes.cubed_sphere(4, numstep=90)
    with tdlib.Context(m) as ctx:
        ctx.set_alpha(0.25, 0.1)
        ctx.assemble(precision=tdlib.MIXED)
        ctx.march()
        ctx.set_alpha(0.3, 0.05)
        u1, t1 = ctx.march()
    with tdlib.Context(m) as ctx:
        ctx.set_alpha(0.3, 0.05)
        ctx.assemble(precision=tdlib.MIXED)
        u2, t2 = ctx.march()
    assert np.array_equal(u1, u2) and np.array_equal(t1, t2)
