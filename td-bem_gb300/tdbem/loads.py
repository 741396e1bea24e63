"""Load cases for batched marching: per-case traction vectors and amplitudes.

A load case of ``Context.march_batch`` is a traction vector over the dofs
(cases x D) and an amplitude per step (cases x numstep).  The reference applies
one load per run, a traction list from the input file scaled by
``SolverT::LoadTimeVariation`` (SolverT.cpp:379-394, a unit step); a batch of
cases is the same marching run once per load.

:func:`gaussian_patch_cases` builds the batched workload: each case loads one
random patch of four elements around a node shared by exactly four elements
with a unit traction along the patch's mean element normal, at every node of
the patch, and a Gaussian pulse in time,
``amp(t) = A exp(-((t - t0 - 3 w) / w)^2 / 2)`` with standard deviation
``w = width * dt``, onset ``t0 ~ U[0, onset_max * dt]`` and ``A ~ N(0, 1)``,
all from one seeded generator.
"""
from __future__ import annotations

import numpy as np

from .inputfile import Model


def element_normals(m: Model) -> np.ndarray:
    """Unit normal (p1 - p0) x (p3 - p0) of every quad (nel x 3)."""
    p = m.coords[m.ien]
    n = np.cross(p[:, 1] - p[:, 0], p[:, 3] - p[:, 0])
    return n / np.linalg.norm(n, axis=1, keepdims=True)


def patch_centres(m: Model) -> np.ndarray:
    """Nodes shared by exactly four elements (centres of 2 x 2 patches)."""
    count = np.bincount(m.ien.ravel(), minlength=m.nnd)
    return np.flatnonzero(count == 4)


def gaussian_patch_cases(m: Model, ncases: int, seed: int = 0, width: float = 5.0,
                         onset_max: float = 50.0, numstep: int | None = None):
    """(traction[ncases, D], amp[ncases, numstep]) of seeded Gaussian patch pulses."""
    n = m.numstep if numstep is None else numstep
    rng = np.random.default_rng(seed)
    centres = patch_centres(m)
    if len(centres) == 0:
        raise ValueError("mesh has no node shared by exactly four elements")
    normals = element_normals(m)
    D = 3 * m.nnd
    traction = np.zeros((ncases, D))
    amp = np.zeros((ncases, n))
    t = np.arange(n) * m.dt
    w = width * m.dt
    for c in range(ncases):
        node = int(rng.choice(centres))
        elems = np.flatnonzero((m.ien == node).any(axis=1))
        nvec = normals[elems].mean(axis=0)
        nvec /= np.linalg.norm(nvec)
        for a in np.unique(m.ien[elems].ravel()):
            traction[c, 3 * a:3 * a + 3] = nvec
        t0 = rng.uniform(0.0, onset_max * m.dt)
        A = rng.standard_normal()
        amp[c] = A * np.exp(-0.5 * ((t - t0 - 3.0 * w) / w) ** 2)
    return traction, amp


def single_case_bc(m: Model, traction_row: np.ndarray):
    """Boundary-condition lists that make one batch case a plain ``tdbem_march`` run.

    The model's prescribed displacements stay; the case's traction becomes the
    traction list (every non-zero entry off the prescribed-displacement dofs)."""
    ubc = set(int(d) for d in m.ubc_dofs)
    dofs = [d for d in np.flatnonzero(traction_row) if int(d) not in ubc]
    return (np.asarray(m.ubc_dofs, dtype=np.int32), np.asarray(m.ubc_vals, dtype=np.float64),
            np.asarray(dofs, dtype=np.int32), np.asarray(traction_row[dofs], dtype=np.float64))
