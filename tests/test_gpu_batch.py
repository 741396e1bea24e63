"""Batched marching (tdbem_march_batch): many load cases on one mesh.

Every case of a batch must give the histories of a plain tdbem_march run with
that case's traction list and load history.  Tolerances: relative L2 error
<= 1e-4 against the plain FP64 GPU form (itself parity-tested against the
oracle at 1e-10) over all steps and dofs of the case; duplicated cases in
different column blocks are bitwise equal; the batch is linear in its loads to
1e-4 of the history norm; the tcgen05 and mma.sync engines agree to 3e-5."""
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


def single(lib, m, trac_row, amp_row, precision, alpha):
    from tdbem import loads
    with lib.Context(m) as ctx:
        ctx.set_alpha(*alpha)
        ctx.set_bc(*loads.single_case_bc(m, trac_row))
        ctx.set_load_history(amp_row)
        ctx.assemble(precision=precision)
        return ctx.march()


def batch(lib, m, trac, amp, alpha, refine=0, engine=0):
    with lib.Context(m) as ctx:
        ctx.set_alpha(*alpha)
        ctx.set_batch_options(engine, refine)
        ctx.assemble(precision=lib.MIXED)
        return ctx.march_batch(trac, amp)


@pytest.fixture(scope="module")
def bar_cases():
    """Bar with a fixed end (UBC columns exchanged), alpha_2 != 0, three loads:
    the input file's own end traction (unit step), the same scaled by -2 under a
    Gaussian pulse, and random tractions on random free dofs."""
    from tdbem import loads
    _, m = load_golden("bar_1x1x4_q2_alpha")
    D = 3 * m.nnd
    n = m.numstep
    rng = np.random.default_rng(7)
    trac = np.zeros((3, D))
    trac[0, m.fbc_dofs] = m.fbc_vals
    trac[1] = -2.0 * trac[0]
    free = np.setdiff1d(np.arange(D), m.ubc_dofs)
    pick = rng.choice(free, 12, replace=False)
    trac[2, pick] = rng.standard_normal(12)
    t = np.arange(n) * m.dt
    amp = np.ones((3, n))
    amp[1] = np.exp(-0.5 * ((t - 20 * m.dt) / (5 * m.dt)) ** 2)
    amp[2] = np.sin(t / (9 * m.dt))
    return m, trac, amp


@pytest.mark.parametrize("engine", [0, 1], ids=["tcgen05", "mma_sync"])
def test_batch_cases_match_single_fp64_bar(tdlib, bar_cases, engine):
    m, trac, amp = bar_cases
    alpha = (0.25, 0.1)
    ub, tb = batch(tdlib, m, trac, amp, alpha, engine=engine)
    assert ub.shape == (m.numstep + 1, 3, 3 * m.nnd)
    for c in range(3):
        u, t = single(tdlib, m, trac[c], amp[c], tdlib.FP64, alpha)
        assert rel_l2(ub[:, c], u) <= TOL_L2, c
        assert rel_l2(tb[:, c], t) <= TOL_L2, c


@pytest.mark.parametrize("engine", [0, 1], ids=["tcgen05", "mma_sync"])
def test_batch_gaussian_patches_sphere(tdlib, engine):
    """Seeded Gaussian pulses on random 4-element patches of a 6x8x8 sphere."""
    from tdbem import loads, meshes
    m = meshes.cubed_sphere(8, numstep=120)
    trac, amp = loads.gaussian_patch_cases(m, 6, seed=0)
    alpha = (0.25, 0.0)
    ub, tb = batch(tdlib, m, trac, amp, alpha, engine=engine)
    for c in (0, 3, 5):
        u, t = single(tdlib, m, trac[c], amp[c], tdlib.FP64, alpha)
        assert rel_l2(ub[:, c], u) <= TOL_L2, c
        assert rel_l2(tb[:, c], t) <= TOL_L2, c


def test_batch_engines_agree(tdlib):
    """tcgen05 (merged levels: the unknowns' history in split-BF16 products, the
    known tractions' part in FP32) and mma.sync (G and H in split-BF16 products) are
    each within ~1e-5 of FP64: the histories agree to 3e-5 of their norm; rows past
    a 128-row tile edge (D = 1158) and 70 cases (two column blocks) included."""
    from tdbem import loads, meshes
    m = meshes.cubed_sphere(8, numstep=60)
    trac, amp = loads.gaussian_patch_cases(m, 70, seed=4, numstep=60)
    u0, _ = batch(tdlib, m, trac, amp, (0.25, 0.0), engine=0)
    u1, _ = batch(tdlib, m, trac, amp, (0.25, 0.0), engine=1)
    assert np.linalg.norm(u0 - u1) <= 3e-5 * np.linalg.norm(u1)
    for c in (0, 63, 64, 69):
        assert np.linalg.norm(u0[:, c] - u1[:, c]) <= 3e-5 * np.linalg.norm(u1[:, c])


@pytest.mark.parametrize("engine", [0, 1], ids=["tcgen05", "mma_sync"])
def test_batch_column_blocks_and_linearity(tdlib, bar_cases, engine):
    """70 cases span two column blocks of 64: cases 64..69 repeat cases 0..5 and
    must come out bitwise equal; case 6 = case 0 + case 2 (same amplitude)."""
    m, trac3, amp3 = bar_cases
    D, n = 3 * m.nnd, m.numstep
    rng = np.random.default_rng(3)
    trac = rng.standard_normal((70, D)) * (rng.random((70, D)) < 0.05)
    amp = np.tile(amp3[2], (70, 1))
    trac[0], trac[2] = trac3[0], trac3[2]
    trac[6] = trac[0] + trac[2]
    trac[64:70] = trac[0:6]
    ub, tb = batch(tdlib, m, trac, amp, (0.25, 0.1), engine=engine)
    assert np.array_equal(ub[:, 64:70], ub[:, 0:6])
    assert np.array_equal(tb[:, 64:70], tb[:, 0:6])
    lin = ub[:, 0] + ub[:, 2]
    assert np.linalg.norm(ub[:, 6] - lin) <= 1e-4 * np.linalg.norm(lin)


def test_batch_refinement(tdlib, bar_cases):
    """Refinement sweeps with the FP32 double-word residual do not lose accuracy."""
    m, trac, amp = bar_cases
    alpha = (0.25, 0.1)
    u, _ = single(tdlib, m, trac[2], amp[2], tdlib.FP64, alpha)
    e = [rel_l2(batch(tdlib, m, trac, amp, alpha, refine=r)[0][:, 2], u) for r in (0, 1, 2)]
    assert max(e) <= TOL_L2
    assert e[2] <= e[0] * 1.5


def test_batch_errors(tdlib, bar_cases):
    m, trac, amp = bar_cases
    with tdlib.Context(m) as ctx:
        ctx.assemble(precision=tdlib.FP64)
        with pytest.raises(tdlib.TdbemError) as ei:
            ctx.march_batch(trac, amp)
        assert ei.value.code == -5  # TDBEM_ERR_UNSUPPORTED: FP32 levels needed
    with tdlib.Context(m) as ctx:
        with pytest.raises(tdlib.TdbemError) as ei:
            ctx.march_batch(trac, amp)
        assert ei.value.code == -6  # TDBEM_ERR_STATE: no levels
