"""The load-history hook against the oracle.

The reference hard-codes its load amplitude (SolverT::LoadTimeVariation,
SolverT.cpp:379-394: 1 at every step); tdbem_set_load_history replaces it with
amp[s] at solve step s, and the oracle's march takes the same amplitude
(amp[curr - 1] for marching step curr, SetLoad in SolverT.cpp:344-377 scaled).
Here the GPU runs non-constant amplitudes on meshes with prescribed
displacements (UBC columns exchanged) and prescribed tractions, alpha = (0.25,
0.1), and is compared with the oracle's march over the oracle's levels:

* plain FP64 (tdbem_march): 1e-10 per step, max|u - u_oracle| / max|u_oracle|
  (likewise t), the oracle in its exact-zero mode;
* mixed batched (tdbem_march_batch), each case against the oracle's march of
  that case's traction list and amplitude: relative L2 error <= 1e-4 over all
  steps and dofs (the mixed form's bar).
"""
import dataclasses

import numpy as np
import pytest

from conftest import load_golden, rel_max

pytestmark = pytest.mark.gpu

TOL = 1e-10
TOL_L2 = 1e-4
ALPHA = (0.25, 0.1)


@pytest.fixture(scope="module")
def tdlib():
    import build as b
    b.build()
    from tdbem import lib
    lib.load()
    return lib


def amplitudes(n, dt):
    t = np.arange(n) * dt
    ramp = np.minimum(1.0, t / (12 * dt))
    gauss = np.exp(-0.5 * ((t - 25 * dt) / (5 * dt)) ** 2)
    return {"ramp": ramp, "gauss": gauss}


@pytest.fixture(scope="module")
def bar(oracle_mod):
    _, m = load_golden("bar_1x1x4_q2_alpha")
    assert len(m.ubc_dofs) > 0 and len(m.fbc_dofs) > 0
    o = oracle_mod.Oracle(m, clean=True)
    G, H = o.assemble_levels()
    return m, o, G, H


def check_steps(u, uo, what):
    for s in range(uo.shape[0]):
        if np.abs(uo[s]).max() == 0:
            assert np.abs(u[s]).max() == 0, f"{what} step {s}"
            continue
        e = rel_max(u[s], uo[s])
        assert e <= TOL, f"{what} step {s}: {e:.3e} > {TOL:.1e}"


@pytest.mark.parametrize("shape", ["ramp", "gauss"])
def test_fp64_march_with_load_history_matches_oracle(tdlib, bar, shape):
    m, o, G, H = bar
    amp = amplitudes(m.numstep, m.dt)[shape]
    uo, to = o.march(G, H, *ALPHA, amp=amp)
    with tdlib.Context(m) as ctx:
        ctx.set_alpha(*ALPHA)
        ctx.set_load_history(amp)
        ctx.assemble()
        u, t = ctx.march()
    assert np.abs(uo).max() > 0
    check_steps(u, uo, f"u ({shape})")
    check_steps(t, to, f"t ({shape})")


def test_fp64_stepwise_march_with_load_history_matches_oracle(tdlib, bar):
    """The stepwise form (tdbem_march_begin / tdbem_march_step, the drop-in's
    Solve per step) reads the same hook."""
    m, o, G, H = bar
    amp = amplitudes(m.numstep, m.dt)["gauss"]
    n = 60
    uo, to = o.march(G, H, *ALPHA, amp=amp[:n], numstep=n)
    with tdlib.Context(m) as ctx:
        ctx.set_alpha(*ALPHA)
        ctx.set_load_history(amp[:n])
        ctx.assemble(n)
        ctx.march_begin(n)
        rows = [ctx.march_step(s) for s in range(1, n + 1)]
    u = np.stack([r[0] for r in rows])  # step s copies history s - 1
    t = np.stack([r[1] for r in rows])
    check_steps(u, uo[:n], "u stepwise")
    check_steps(t, to[:n], "t stepwise")


def test_batch_cases_with_load_histories_match_oracle(tdlib, bar, oracle_mod):
    """Two cases of one mixed batch: the input's end traction under a ramp and
    random tractions on free dofs under a Gaussian pulse, each against the
    oracle's FP64 march of that case alone."""
    from tdbem import loads
    m, o, G, H = bar
    D = 3 * m.nnd
    n = m.numstep
    amps = amplitudes(n, m.dt)
    trac = np.zeros((2, D))
    trac[0, m.fbc_dofs] = m.fbc_vals
    free = np.setdiff1d(np.arange(D), m.ubc_dofs)
    pick = np.random.default_rng(11).choice(free, 10, replace=False)
    trac[1, pick] = np.random.default_rng(12).standard_normal(10)
    amp = np.stack([amps["ramp"], amps["gauss"]])
    with tdlib.Context(m) as ctx:
        ctx.set_alpha(*ALPHA)
        ctx.assemble(precision=tdlib.MIXED)
        ub, tb = ctx.march_batch(trac, amp)
    for c in range(2):
        ud, uv, fd, fv = loads.single_case_bc(m, trac[c])
        mc = dataclasses.replace(m, ubc_dofs=ud, ubc_vals=uv, fbc_dofs=fd, fbc_vals=fv)
        uo, to = oracle_mod.Oracle(mc, clean=True).march(G, H, *ALPHA, amp=amp[c])
        eu = np.linalg.norm(ub[:, c] - uo) / np.linalg.norm(uo)
        et = np.linalg.norm(tb[:, c] - to) / np.linalg.norm(to)
        assert eu <= TOL_L2, f"case {c}: u rel L2 {eu:.2e}"
        assert et <= TOL_L2, f"case {c}: t rel L2 {et:.2e}"
