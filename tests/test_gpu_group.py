"""Many meshes at once: grouped assembly and the persistent grouped march.

Grouped assembly runs the same quadrature items as tdbem_assemble_levels in
the same colour order, compiled into another kernel (the compiler may contract
multiply-adds differently), so every level must equal the per-mesh assembly to
1e-13 of the level's max-norm.  The persistent march sums each row's
convolution in another order than the per-mesh kernels, so its histories must
equal per-mesh tdbem_march to the 1e-10 parity bar (per step, max-norm)."""
import numpy as np
import pytest

from conftest import rel_max

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module")
def tdlib():
    import build as b
    b.build()
    from tdbem import lib
    lib.load()
    return lib


def group_models():
    from tdbem import meshes
    ms = [meshes.bar(1, 1, 2, per_unit=1, numstep=40),
          meshes.bar(1, 1, 5, per_unit=2, numstep=70),
          meshes.bar(1, 1, 3, per_unit=3, numstep=55),
          meshes.cubed_sphere(4, numstep=30),
          meshes.bar(1, 1, 8, per_unit=1, numstep=64)]
    setup = [((0.25, 0.0), None), ((0.25, 0.1), "gauss"), ((0.0, 0.0), None),
             ((0.25, 0.0), "sine"), ((0.5, 0.2), None)]
    return ms, setup


def configure(ctx, m, alpha, amp_kind):
    ctx.set_alpha(*alpha)
    if amp_kind:
        t = np.arange(m.numstep) * m.dt
        amp = (np.exp(-0.5 * ((t - 8 * m.dt) / (3 * m.dt)) ** 2) if amp_kind == "gauss"
               else np.sin(t / (5 * m.dt)))
        ctx.set_load_history(amp)


def test_group_levels_and_histories_match_per_mesh(tdlib):
    ms, setup = group_models()
    ref = []
    for m, (alpha, ak) in zip(ms, setup):
        with tdlib.Context(m) as ctx:
            configure(ctx, m, alpha, ak)
            ctx.assemble(precision=tdlib.FP64)
            u, t = ctx.march()
            lv = [(ctx.level(k, 0), ctx.level(k, 1)) for k in (0, 1, ctx.M // 2, ctx.M)]
            ref.append((u, t, lv, ctx.M))
    ctxs = [tdlib.Context(m) for m in ms]
    try:
        for ctx, m, (alpha, ak) in zip(ctxs, ms, setup):
            configure(ctx, m, alpha, ak)
        tdlib.assemble_group(ctxs)
        for ctx, (_, _, lv, M) in zip(ctxs, ref):
            for (G, H), k in zip(lv, (0, 1, M // 2, M)):
                eg, eh = rel_max(ctx.level(k, 0), G), rel_max(ctx.level(k, 1), H)
                assert eg <= 1e-13, f"G level {k}: {eg:.3e}"
                assert eh <= 1e-13, f"H level {k}: {eh:.3e}"
        out = tdlib.march_group(ctxs)
        for (u, t), (ur, tr, _, _) in zip(out, ref):
            assert u.shape == ur.shape
            for s in range(ur.shape[0]):
                if np.abs(ur[s]).max() == 0:
                    assert np.abs(u[s]).max() == 0
                else:
                    assert rel_max(u[s], ur[s]) <= TOL, s
                    assert rel_max(t[s], tr[s]) <= TOL, s
        sh = tdlib.group_shape()
        assert sh["lanes"] in (8, 16, 32) and sh["block"] in (128, 256, 512)
        # a second march reuses the chosen shape and gives bitwise the same histories
        out2 = tdlib.march_group(ctxs)
        for (u, t), (u2, t2) in zip(out, out2):
            assert np.array_equal(u, u2) and np.array_equal(t, t2)
    finally:
        for c in ctxs:
            c.close()


def test_group_errors(tdlib):
    from tdbem import meshes
    m = meshes.bar(1, 1, 2, per_unit=1, numstep=10)
    with tdlib.Context(m) as a, tdlib.Context(m) as b:
        with pytest.raises(tdlib.TdbemError) as ei:
            tdlib.march_group([a, b])
        assert ei.value.code == -6  # TDBEM_ERR_STATE: no levels yet
        with pytest.raises(tdlib.TdbemError):
            tdlib.assemble_group([a, a])
        a.assemble(precision=tdlib.MIXED)
        tdlib.assemble_group([b])
        with pytest.raises(tdlib.TdbemError) as ei:
            tdlib.march_group([a, b])
        assert ei.value.code == -5  # FP64 and mixed levels are not marched together


def test_group_mixed_within_1e4_of_fp64(tdlib):
    """TDBEM_MIXED group (FP32 levels and inverses, one FP64 refinement sweep in the
    persistent march) against each mesh's plain FP64 march: relative L2 error of
    the displacement histories <= 1e-4, as the single-mesh mixed form."""
    ms, setup = group_models()
    keep = [i for i, (alpha, _) in enumerate(setup) if alpha[0] > 0]  # stable alpha only
    ms = [ms[i] for i in keep]
    setup = [setup[i] for i in keep]
    ref = []
    for m, (alpha, ak) in zip(ms, setup):
        with tdlib.Context(m) as ctx:
            configure(ctx, m, alpha, ak)
            ctx.assemble(precision=tdlib.FP64)
            ref.append(ctx.march()[0])
    ctxs = [tdlib.Context(m) for m in ms]
    try:
        for ctx, m, (alpha, ak) in zip(ctxs, ms, setup):
            configure(ctx, m, alpha, ak)
            ctx.set_march_options(refine_sweeps=1)
        tdlib.assemble_group(ctxs, precision=tdlib.MIXED)
        out = tdlib.march_group(ctxs)
        for (u, _), ur in zip(out, ref):
            assert np.linalg.norm(u - ur) <= 1e-4 * np.linalg.norm(ur)
    finally:
        for c in ctxs:
            c.close()
