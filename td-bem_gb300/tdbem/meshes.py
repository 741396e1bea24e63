"""Synthetic surface meshes for the benchmark workloads, written as Models.

* :func:`bar` -- prismatic bar, 4-node quads, one end fixed and a unit
  Heaviside normal traction on the other (the layout of the reference's
  ``geometry/Bar_1.txt``: outward normals, u = 0 on every dof of the fixed
  end's nodes, traction on the axial dof of the loaded end's nodes).
* :func:`cubed_sphere` -- spherical cavity in a full space (``if_ext = 1``),
  equiangular cubed-sphere quads with normals pointing into the cavity like
  the reference's ``geometry/SphericalCavity_*.txt``, uniform internal
  pressure p: traction ``t = p * x / |x|`` on every dof.
* :func:`halfspace_cavity` -- box-truncated half-space with a spherical
  cavity: a square free-surface patch at z = 0 (normals +z, out of the solid)
  over a cubed-sphere cavity at depth d (normals into the cavity), internal
  pressure on the cavity, the patch traction-free.

* :func:`two_region_bar` -- a bar split across its axis into two regions of
  different material (the multi-region solver's setting, formulation = 3):
  each region a closed box surface, the shared face listed as the interface of
  both, a normal traction on the far end of region 2, no prescribed
  displacements (the two-region solver has none).

The mesh size h of a cubed sphere is the equiangular arc spacing
``radius * (pi/2) / n``; the time step is ``dt = beta * h / c_p``.
"""
from __future__ import annotations

import numpy as np

from .inputfile import Model


def material_for(mu: float = 1.0, nu: float = 0.25, rho: float = 1.0):
    """Young's modulus giving shear modulus mu at Poisson ratio nu."""
    return 2.0 * mu * (1.0 + nu), nu, rho


def _orient(coords, ien, outward_of):
    """Reorder each quad so that (p1-p0) x (p3-p0) agrees with outward_of(centroid)."""
    out = ien.copy()
    for e, q in enumerate(ien):
        p = coords[q]
        n = np.cross(p[1] - p[0], p[3] - p[0])
        if np.dot(n, outward_of(p.mean(0))) < 0:
            out[e] = q[[0, 3, 2, 1]]
    return out


def bar(lx: float = 1.0, ly: float = 1.0, lz: float = 4.0, per_unit: int = 2,
        mu: float = 1.0, nu: float = 0.25, rho: float = 1.0, beta: float = 0.6,
        numstep: int = 200, traction: float = 1.0) -> Model:
    """Surface mesh of a lx x ly x lz bar along z, quads at per_unit per unit length."""
    nx, ny, nz = (int(round(l * per_unit)) for l in (lx, ly, lz))
    grid = {}
    coords = []

    def node(i, j, k):
        key = (i, j, k)
        if key not in grid:
            grid[key] = len(coords)
            coords.append((lx * i / nx, ly * j / ny, lz * k / nz))
        return grid[key]

    quads = []
    normals = []
    # lateral faces x=0, x=lx, y=0, y=ly and the two end caps
    for (fixed, val, a, b, na, nb, nvec) in (
            ("x", 0, "y", "z", ny, nz, (-1, 0, 0)), ("x", nx, "y", "z", ny, nz, (1, 0, 0)),
            ("y", 0, "x", "z", nx, nz, (0, -1, 0)), ("y", ny, "x", "z", nx, nz, (0, 1, 0)),
            ("z", 0, "x", "y", nx, ny, (0, 0, -1)), ("z", nz, "x", "y", nx, ny, (0, 0, 1))):
        for ia in range(na):
            for ib in range(nb):
                ids = []
                for (da, db) in ((0, 0), (1, 0), (1, 1), (0, 1)):
                    idx = {fixed: val, a: ia + da, b: ib + db}
                    ids.append(node(idx["x"], idx["y"], idx["z"]))
                quads.append(ids)
                normals.append(nvec)
    coords = np.array(coords, float)
    ien = np.array(quads, np.int32)
    for e in range(len(ien)):
        p = coords[ien[e]]
        if np.dot(np.cross(p[1] - p[0], p[3] - p[0]), normals[e]) < 0:
            ien[e] = ien[e][[0, 3, 2, 1]]
    E, nu_, rho_ = material_for(mu, nu, rho)
    m = Model(coords=coords, ien=ien, etype=1, E=E, nu=nu_, rho=rho_, numstep=numstep)
    _, _, cp, _ = m.material()
    m.dt = beta * (1.0 / per_unit) / cp
    z = coords[:, 2]
    fixed_nodes = np.nonzero(np.isclose(z, 0.0))[0]
    loaded = np.nonzero(np.isclose(z, lz))[0]
    m.ubc_dofs = np.array([3 * n + d for n in fixed_nodes for d in range(3)], np.int32)
    m.ubc_vals = np.zeros(len(m.ubc_dofs))
    m.fbc_dofs = np.array([3 * n + 2 for n in loaded], np.int32)
    m.fbc_vals = np.full(len(m.fbc_dofs), float(traction))
    return m


def two_region_bar(per_unit: int = 2, l1: float = 2.0, l2: float = 2.0, width: float = 1.0,
                   mu=(7.95e9, 1.59e10), nu=(0.25, 0.25), rho=(2650.0, 2650.0),
                   beta: float = 0.6, numstep: int = 20, traction: float = 1.0):
    """Regions 1 (0 <= z <= l1) and 2 (l1 <= z <= l1 + l2) of a width x width bar.

    The default material (c_p = 3000 m/s in region 1) puts the time step near
    1e-4 s, the scale of the two-region solver's built-in load pulse
    p0 t exp(-2000 t).  dt = beta h / c_p of region 1, shared by both regions."""
    m1 = bar(width, width, l1, per_unit, mu[0], nu[0], rho[0], beta, numstep, traction)
    m2 = bar(width, width, l2, per_unit, mu[1], nu[1], rho[1], beta, numstep, traction)
    m2.coords = m2.coords + np.array([0.0, 0.0, l1])
    m2.dt = m1.dt
    for m in (m1, m2):
        m.formulation = 3
        m.ubc_dofs = np.zeros(0, np.int32)
        m.ubc_vals = np.zeros(0)
    m1.interface = np.nonzero(np.isclose(m1.coords[:, 2], l1))[0].astype(np.int32)
    m2.interface = np.nonzero(np.isclose(m2.coords[:, 2], l1))[0].astype(np.int32)
    m1.fbc_dofs = np.zeros(0, np.int32)
    m1.fbc_vals = np.zeros(0)
    return m1, m2


def cubed_sphere(n: int = 16, radius: float = 1.0, mu: float = 1.0, nu: float = 0.25,
                 rho: float = 1.0, beta: float = 0.6, numstep: int = 400,
                 pressure: float = 1.0) -> Model:
    """Equiangular cubed sphere with 6*n*n quads and 6*n*n+2 nodes, if_ext = 1."""
    ang = np.linspace(-np.pi / 4, np.pi / 4, n + 1)
    t = np.tan(ang)
    faces = [  # (axis, sign) of each cube face; (u, v) span the other two axes
        (0, 1), (0, -1), (1, 1), (1, -1), (2, 1), (2, -1)]
    key_to_id = {}
    coords = []
    quads = []
    for axis, sign in faces:
        others = [d for d in range(3) if d != axis]
        ids = np.zeros((n + 1, n + 1), np.int64)
        for i in range(n + 1):
            for j in range(n + 1):
                p = np.zeros(3)
                p[axis] = sign
                p[others[0]] = t[i]
                p[others[1]] = t[j]
                p = radius * p / np.linalg.norm(p)
                key = tuple(np.round(p, 10))
                if key not in key_to_id:
                    key_to_id[key] = len(coords)
                    coords.append(p)
                ids[i, j] = key_to_id[key]
        for i in range(n):
            for j in range(n):
                quads.append([ids[i, j], ids[i + 1, j], ids[i + 1, j + 1], ids[i, j + 1]])
    coords = np.array(coords, float)
    ien = np.array(quads, np.int32)
    # normals into the cavity (toward the centre), as the reference's cavity meshes
    ien = _orient(coords, ien, lambda c: -c)
    E, nu_, rho_ = material_for(mu, nu, rho)
    m = Model(coords=coords, ien=ien, etype=1, E=E, nu=nu_, rho=rho_, numstep=numstep,
              if_ext=1)
    _, _, cp, _ = m.material()
    h = radius * (np.pi / 2) / n
    m.dt = beta * h / cp
    rhat = coords / np.linalg.norm(coords, axis=1, keepdims=True)
    m.fbc_dofs = np.arange(3 * len(coords), dtype=np.int32)
    m.fbc_vals = (pressure * rhat).reshape(-1).astype(float)
    return m


def _cubed_sphere_surface(n: int, radius: float, centre=(0.0, 0.0, 0.0)):
    ang = np.linspace(-np.pi / 4, np.pi / 4, n + 1)
    t = np.tan(ang)
    key_to_id, coords, quads = {}, [], []
    for axis, sign in ((0, 1), (0, -1), (1, 1), (1, -1), (2, 1), (2, -1)):
        others = [d for d in range(3) if d != axis]
        ids = np.zeros((n + 1, n + 1), np.int64)
        for i in range(n + 1):
            for j in range(n + 1):
                p = np.zeros(3)
                p[axis] = sign
                p[others[0]] = t[i]
                p[others[1]] = t[j]
                p = radius * p / np.linalg.norm(p)
                key = tuple(np.round(p, 10))
                if key not in key_to_id:
                    key_to_id[key] = len(coords)
                    coords.append(p)
                ids[i, j] = key_to_id[key]
        for i in range(n):
            for j in range(n):
                quads.append([ids[i, j], ids[i + 1, j], ids[i + 1, j + 1], ids[i, j + 1]])
    coords = np.array(coords, float)
    ien = np.array(quads, np.int32)
    ien = _orient(coords, ien, lambda c: -c)  # into the cavity
    return coords + np.asarray(centre, float), ien


def halfspace_cavity(depth: float = 3.0, patch: float = 10.0, per_unit: int = 1,
                     n_sphere: int = 6, radius: float = 1.0, mu: float = 1.0, nu: float = 0.25,
                     rho: float = 1.0, beta: float = 0.6, numstep: int = 200,
                     pressure: float = 1.0) -> Model:
    """Cavity of radius ``radius`` centred at depth ``depth`` under a ``patch`` x
    ``patch`` free-surface square meshed at ``per_unit`` quads per unit length."""
    ns = int(round(patch * per_unit))
    xs = np.linspace(-patch / 2, patch / 2, ns + 1)
    grid = np.array([(x, y, 0.0) for y in xs for x in xs])
    quads = [[j * (ns + 1) + i, j * (ns + 1) + i + 1, (j + 1) * (ns + 1) + i + 1,
              (j + 1) * (ns + 1) + i] for j in range(ns) for i in range(ns)]
    ien_s = _orient(grid, np.array(quads, np.int32), lambda c: np.array([0.0, 0.0, 1.0]))
    c_sph, ien_c = _cubed_sphere_surface(n_sphere, radius, (0.0, 0.0, -depth))
    coords = np.vstack([grid, c_sph])
    ien = np.vstack([ien_s, ien_c + len(grid)]).astype(np.int32)
    E, nu_, rho_ = material_for(mu, nu, rho)
    m = Model(coords=coords, ien=ien, etype=1, E=E, nu=nu_, rho=rho_, numstep=numstep,
              if_ext=1)
    _, _, cp, _ = m.material()
    h = min(1.0 / per_unit, radius * (np.pi / 2) / n_sphere)
    m.dt = beta * h / cp
    rel = c_sph - np.array([0.0, 0.0, -depth])
    rhat = rel / np.linalg.norm(rel, axis=1, keepdims=True)
    nodes = np.arange(len(grid), len(coords))
    m.fbc_dofs = np.array([3 * a + d for a in nodes for d in range(3)], np.int32)
    m.fbc_vals = (pressure * rhat).reshape(-1).astype(float)
    return m


def sphere_cavity_closed_form(t: np.ndarray, radius: float = 1.0, mu: float = 1.0,
                              nu: float = 0.25, rho: float = 1.0, p: float = 1.0) -> np.ndarray:
    """Radial wall displacement u_r(a, t) of a spherical cavity under step pressure p H(t).

    With the P-wave potential phi = f(tau)/r, tau = t - (r - a)/c_p and
    sigma_rr(a) = -p H(t):  f'' + (4 c_s^2/(c_p a)) f' + (4 c_s^2/a^2) f = -p a H(t)/rho
    and u_r(a, t) = -f'/(c_p a) - f/a^2.  Static limit p a / (4 mu)."""
    lam = 2 * mu * nu / (1 - 2 * nu)
    cp = np.sqrt((lam + 2 * mu) / rho)
    cs = np.sqrt(mu / rho)
    a = radius
    b1 = 4 * cs ** 2 / (cp * a)
    b0 = 4 * cs ** 2 / a ** 2
    zeta = b1 / 2
    omega = np.sqrt(b0 - zeta ** 2)
    fs = -p * a / (rho * b0)  # particular solution
    t = np.asarray(t, float)
    e = np.exp(-zeta * t)
    f = fs * (1 - e * (np.cos(omega * t) + (zeta / omega) * np.sin(omega * t)))
    fp = fs * e * (zeta ** 2 / omega + omega) * np.sin(omega * t)
    u = -fp / (cp * a) - f / a ** 2
    return np.where(t > 0, u, 0.0)
