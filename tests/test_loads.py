"""Load-case generation for batched marching (host only)."""
import numpy as np

from tdbem import loads, meshes
from conftest import load_golden


def test_gaussian_patch_cases_seeded_and_shaped():
    m = meshes.cubed_sphere(4, numstep=80)
    tr, amp = loads.gaussian_patch_cases(m, 5, seed=0)
    tr2, amp2 = loads.gaussian_patch_cases(m, 5, seed=0)
    assert tr.shape == (5, 3 * m.nnd) and amp.shape == (5, 80)
    assert np.array_equal(tr, tr2) and np.array_equal(amp, amp2)
    tr3, _ = loads.gaussian_patch_cases(m, 5, seed=1)
    assert not np.array_equal(tr, tr3)
    for c in range(5):
        nodes = np.flatnonzero(np.abs(tr[c]).reshape(-1, 3).sum(1) > 0)
        assert len(nodes) == 9  # 2 x 2 patch of quads
        v = tr[c].reshape(-1, 3)[nodes]
        assert np.allclose(np.linalg.norm(v, axis=1), 1.0)
        # pulse peak after the onset window: t0 + 3 w with t0 <= 50 dt, w = 5 dt
        k = int(np.argmax(np.abs(amp[c])))
        assert 15 <= k <= 65


def test_single_case_bc_drops_prescribed_dofs():
    _, m = load_golden("bar_1x1x4_q2_alpha")
    D = 3 * m.nnd
    row = np.zeros(D)
    row[m.ubc_dofs[:3]] = 5.0
    row[m.fbc_dofs] = m.fbc_vals
    ud, uv, fd, fv = loads.single_case_bc(m, row)
    assert np.array_equal(ud, m.ubc_dofs)
    assert set(fd) == set(int(d) for d in m.fbc_dofs if d not in set(m.ubc_dofs))
    assert np.allclose(row[fd], fv)
