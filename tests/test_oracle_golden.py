"""The oracle (C restatement) against the reference's own outputs.

Golden fixtures were produced by tests/golden/make_golden.py, which runs the
reference sources unmodified (built against a single-rank dense PETSc/MPI
stand-in).  With -ffp-contract=off the restatement reproduces them bit for bit;
the tolerance below only absorbs a different libm on another host."""
import numpy as np
import pytest

from conftest import golden_cases, load_golden, rel_max

TOL = 1e-12


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_matches_reference(name, oracle_mod):
    z, m = load_golden(name)
    o = oracle_mod.Oracle(m)
    M = o.max_step()
    assert M == int(z["M"])
    G, H = o.assemble_levels(M)
    w = np.random.default_rng(int(z["seed"])).standard_normal(o.D)
    assert rel_max(G @ w, z["G_w"]) <= TOL
    assert rel_max(H @ w, z["H_w"]) <= TOL
    assert rel_max(np.einsum("d,kde->ke", w, G), z["w_G"]) <= TOL
    assert rel_max(np.einsum("d,kde->ke", w, H), z["w_H"]) <= TOL
    if "G" in z:
        assert rel_max(G, z["G"]) <= TOL and rel_max(H, z["H"]) <= TOL
    u, t = o.march(G, H, float(z["a1"]), float(z["a2"]))
    d = z["dofs"]
    for s in range(u.shape[0]):
        assert rel_max(u[s, d], z["u"][s]) <= TOL, f"u step {s}"
        assert rel_max(t[s, d], z["t"][s]) <= TOL, f"t step {s}"


def test_gh_driver_row_split_equals_full(oracle_mod):
    """The reference's MPI row split: G_H_Driver on node ranges gives the rows of the full call."""
    z, m = load_golden("ref_bar1")
    o = oracle_mod.Oracle(m, nthreads=2)
    full = o.gh_driver(2 * m.dt, m.dt)
    top = o.gh_driver(2 * m.dt, m.dt, 0, 9)
    bot = o.gh_driver(2 * m.dt, m.dt, 10, m.nnd - 1)
    for f, a, b in zip(full, top, bot):
        assert np.array_equal(f, np.vstack([a, b]))


def test_levels_are_step_placements(oracle_mod):
    """Level k = I(k dt) + J((k+1) dt) (SolverStepLinearT.cpp:58-97)."""
    z, m = load_golden("ref_bar1")
    o = oracle_mod.Oracle(m)
    M = o.max_step()
    G, H = o.assemble_levels(M)
    parts = [o.gh_driver(n * m.dt, m.dt) for n in range(1, M + 1)]
    assert np.array_equal(G[0], parts[0][1])
    for k in range(1, M):
        assert np.array_equal(G[k], parts[k - 1][0] + parts[k][1])
        assert np.array_equal(H[k], parts[k - 1][2] + parts[k][3])
    assert np.array_equal(G[M], parts[M - 1][0])


def test_alpha_range_is_rejected(oracle_mod):
    z, m = load_golden("ref_halfspace_plane_1e")
    o = oracle_mod.Oracle(m)
    G, H = o.assemble_levels()
    with pytest.raises(RuntimeError):
        o.march(G, H, 0.8, 0.5)


@pytest.mark.parametrize("name", ["ref_bar1", "sphere_6x4x4", "bar_1x1x4_q2"])
def test_reference_roundoff_floor(name, oracle_mod):
    """The reference leaves round-off where the step response is identically zero.

    The exact-zero oracle differs from the reference only there: by less than 1e-7
    of each level's max norm, and not at all on the first two levels (no quadrature
    point has been passed by both fronts yet)."""
    z, m = load_golden(name)
    G, H = oracle_mod.Oracle(m).assemble_levels()
    Gc, Hc = oracle_mod.Oracle(m, clean=True).assemble_levels()
    for k in range(len(G)):
        assert rel_max(Gc[k], G[k]) < 1e-7 and rel_max(Hc[k], H[k]) < 1e-7
    assert np.array_equal(G[:2], Gc[:2]) and np.array_equal(H[:2], Hc[:2])


def test_oracle_matches_reference_rows_at_benchmark_size(oracle_mod):
    """G_H_Driver row blocks of the 6x16x16 cubed-sphere cavity (D = 4614): the
    reference's own rows (projected on the fixture's seeded vector) at steps 1, 2,
    M/2 and M, for node blocks at the start, middle and end of the node list."""
    z, m = load_golden("rows_sphere_6x16x16")
    o = oracle_mod.Oracle(m)
    w = np.random.default_rng(int(z["seed"])).standard_normal(o.D)
    i = 0
    for lo, hi in z["blocks"]:
        for st in z["steps"]:
            got = o.gh_driver(int(st) * m.dt, m.dt, int(lo), int(hi))
            for b in range(4):
                assert rel_max(got[b] @ w, z["rows_w"][i][b]) <= TOL, f"rows {lo} step {st}"
                assert np.abs(got[b]).max() == z["rows_absmax"][i][b]
            i += 1
