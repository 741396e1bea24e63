"""The two-region solver (SolverMRT) in the oracle, against the reference's own
outputs, and the region-split form of its history sum.

Fixtures come from tests/golden/make_golden.py, which runs SolverMRT.cpp
unmodified (oracle/ref_mrt_driver.cpp): the reference's Layer_B_test0 /
Layer_U_test0 pair and a bar split into two materials (max_step below and above
the regions' MaxStep).  The oracle reproduces them bit for bit; the tolerance
only absorbs a different libm on another host.

The GPU marches the combined system region by region: with u_r, t_r the
displacement and traction histories of region r rebuilt from the combined
unknowns (region 2 sees the interface traction with the opposite sign),
    G_DB^f tg^m - H_DB^f x^m  =  G_r^f t_r^m - H_r^f u_r^m   on region r's rows,
so the history sum needs only the regions' own levels.  The last test checks
that identity on the oracle's levels.
"""
import numpy as np
import pytest

from conftest import load_mrt_golden, mrt_golden_cases, rel_max

TOL = 1e-12


@pytest.mark.parametrize("name", mrt_golden_cases())
def test_mrt_oracle_matches_reference(name, oracle_mod):
    z, m1, m2 = load_mrt_golden(name)
    mr = oracle_mod.MultiRegion(m1, m2, int(z["max_step"]))
    assert (mr.N, mr.NG) == (int(z["N"]), int(z["NG"]))
    GG, HH = mr.assemble_levels()
    rng = np.random.default_rng(int(z["seed"]))
    wg, wh, wr = rng.standard_normal(mr.NG), rng.standard_normal(mr.N), rng.standard_normal(mr.N)
    assert rel_max(GG @ wg, z["G_w"]) <= TOL
    assert rel_max(HH @ wh, z["H_w"]) <= TOL
    assert rel_max(np.einsum("d,kde->ke", wr, GG), z["w_G"]) <= TOL
    assert rel_max(np.einsum("d,kde->ke", wr, HH), z["w_H"]) <= TOL
    X, u1, u2 = mr.march(GG, HH)
    ns = int(z["numstep"])
    for s in range(ns + 1):
        assert rel_max(X[s], z["x"][s]) <= TOL, f"x step {s}"
    # ExtractField stores step n-1 while solving step n: the last row stays zero
    for s in range(ns):
        assert rel_max(u1[s], z["u1"][s]) <= TOL, f"u1 step {s}"
        assert rel_max(u2[s], z["u2"][s]) <= TOL, f"u2 step {s}"
    assert not z["u1"][ns].any() and not z["u2"][ns].any()


def test_interface_matching_and_layout(oracle_mod):
    z, m1, m2 = load_mrt_golden("mrt_bar_2x2")
    mr = oracle_mod.MultiRegion(m1, m2)
    # every region-2 interface node sits on its region-1 partner
    np.testing.assert_allclose(m2.coords[m2.interface], m1.coords[m1.interface[mr.match]],
                               atol=1e-12)
    # displacement columns: a permutation within each region, the interface shared
    assert len(set(mr.ucol[0])) == mr.D1 and len(set(mr.ucol[1])) == mr.D2
    shared = set(mr.ucol[0]) & set(mr.ucol[1])
    assert shared == set(mr.NI1 + mr.NI2 + np.arange(mr.NZ))
    assert mr.N == mr.NI1 + mr.NI2 + 2 * mr.NZ


def test_interface_mismatch_is_refused(oracle_mod):
    z, m1, m2 = load_mrt_golden("mrt_bar_2x2")
    m2.coords = m2.coords.copy()
    m2.coords[m2.interface[3], 0] += 1e-3
    with pytest.raises(ValueError, match="no match"):
        oracle_mod.MultiRegion(m1, m2)


@pytest.mark.parametrize("name", ["mrt_layer_test0", "mrt_bar_2x2_long"])
def test_region_split_history_equals_combined(name, oracle_mod):
    z, m1, m2 = load_mrt_golden(name)
    mr = oracle_mod.MultiRegion(m1, m2, int(z["max_step"]), clean=True)
    (G1, H1), (G2, H2) = mr.region_levels()
    GG, HH = mr.combine(G1, H1, G2, H2)
    X, _, _ = mr.march(GG, HH)
    load = mr.loads(X.shape[0] - 1)
    L = GG.shape[0] - 1
    regions = ((G1, H1, slice(0, mr.D1)), (G2, H2, slice(mr.D1, mr.N)))
    inter = (mr.int1, mr.int2)
    H0inv = np.linalg.inv(HH[0])
    for n in range(1, X.shape[0]):
        rhs_c = GG[0] @ load[n]
        for f in range(1, min(n, L) + 1):
            tg = load[n - f] if n - f > 0 else np.zeros(mr.NG)
            rhs_c += GG[f] @ tg - HH[f] @ X[n - f]
        rhs_r = np.zeros(mr.N)
        for r, (G, H, rows) in enumerate(regions):
            D = G.shape[1]

            def hist(m):
                u = X[m, mr.ucol[r]]
                t = np.zeros(D)
                if m > 0:
                    t[inter[r]] = load[m, mr.gcol[r]]
                ifc = mr.tcol[r] >= 0
                t[ifc] = mr.tsign[r] * X[m, mr.tcol[r][ifc]]
                return u, t

            tl = np.zeros(D)
            tl[inter[r]] = load[n, mr.gcol[r]]
            acc = G[0] @ tl
            for f in range(1, min(n, L) + 1):
                u, t = hist(n - f)
                acc += G[f] @ t - H[f] @ u
            rhs_r[rows] = acc
        assert rel_max(rhs_r, rhs_c) <= 1e-12, f"step {n}"
        assert rel_max(H0inv @ rhs_r, X[n]) <= 1e-9, f"step {n}"
