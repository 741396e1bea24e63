"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE).

The oracle is a C restatement of the reference's assembly and marching
(tdbem_oracle.c, each function citing the reference file:line it follows).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the product never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class OrcModel(ctypes.Structure):
    _fields_ = [("nnd", ctypes.c_int), ("nel", ctypes.c_int), ("etype", ctypes.c_int),
                ("coords", _dp), ("ien", _ip), ("E", ctypes.c_double),
                ("nu", ctypes.c_double), ("rho", ctypes.c_double), ("dt", ctypes.c_double),
                ("nq", ctypes.c_int), ("if_ext", ctypes.c_int)]


def build(force: bool = False) -> str:
    """Compile the oracle with the committed Makefile (plain C, gcc)."""
    src = os.path.join(HERE, "tdbem_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_max_step.argtypes = [ctypes.POINTER(OrcModel)]
        L.orc_gh_driver.argtypes = [ctypes.POINTER(OrcModel), ctypes.c_double, ctypes.c_double,
                                    ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp, ctypes.c_int]
        L.orc_assemble_levels.argtypes = [ctypes.POINTER(OrcModel), ctypes.c_int, ctypes.c_int,
                                          _dp, _dp, ctypes.c_int]
        march_args = [ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_int, _ip, _dp, ctypes.c_int,
                      _ip, _dp, _dp, ctypes.c_double, ctypes.c_double]
        L.orc_march.argtypes = march_args + [ctypes.c_int, _dp, _dp, ctypes.c_int]
        L.orc_march_range.argtypes = march_args + [ctypes.c_int, ctypes.c_int, _dp, _dp,
                                                   ctypes.c_int]
        L.orc_lu_factor.argtypes = [ctypes.c_int, _dp, ctypes.c_int]
        L.orc_mrt_amplitude.argtypes = [ctypes.c_int, ctypes.c_double]
        L.orc_mrt_amplitude.restype = ctypes.c_double
        L.orc_mrt_march.argtypes = [ctypes.c_int] * 3 + [_dp, _dp, _dp, ctypes.c_int, _dp,
                                                         ctypes.c_int]
        L.orc_green_step_linear.argtypes = [ctypes.c_double] * 3 + [_dp, _dp, ctypes.c_double,
                                                                    ctypes.c_double] + [_dp] * 5
        L.orc_element_gh.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_double, _dp, _dp,
                                     ctypes.c_double, ctypes.c_double, ctypes.c_int] + [_dp] * 6
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


class _Clean:
    """Context manager setting orc_clean_passed_waves (exact zero step response once
    both wave fronts have passed a quadrature point, instead of the reference's
    round-off there)."""

    def __init__(self, on):
        self.on = on

    def __enter__(self):
        self.flag = ctypes.c_int.in_dll(lib(), "orc_clean_passed_waves")
        self.old = self.flag.value
        self.flag.value = 1 if self.on else 0

    def __exit__(self, *a):
        self.flag.value = self.old


class Oracle:
    """Oracle handle bound to one Model (tdbem.inputfile.Model).

    clean=False reproduces the reference's arithmetic bit for bit; clean=True
    replaces the step response by its exact value 0 wherever both wave fronts
    have passed the quadrature point at both evaluation times (the reference
    leaves round-off there)."""

    def __init__(self, model, nthreads: int = 0, clean: bool = False):
        self.clean = clean
        self.m = model
        self.coords = np.ascontiguousarray(model.coords, np.float64)
        self.ien = np.ascontiguousarray(model.ien, np.int32)
        self.st = OrcModel(model.nnd, model.nel, model.etype, _d(self.coords), _i(self.ien),
                           model.E, model.nu, model.rho, model.dt, model.nq, model.if_ext)
        self.nthreads = nthreads or (os.cpu_count() or 1)

    @property
    def D(self) -> int:
        return 3 * self.m.nnd

    def max_step(self) -> int:
        return lib().orc_max_step(ctypes.byref(self.st))

    def gh_driver(self, t, t_1, node_lo=0, node_hi=None):
        hi = self.m.nnd - 1 if node_hi is None else node_hi
        rows = 3 * (hi - node_lo + 1)
        outs = [np.zeros((rows, self.D)) for _ in range(4)]
        with _Clean(self.clean):
            rc = lib().orc_gh_driver(ctypes.byref(self.st), t, t_1, node_lo, hi,
                                     *[_d(o) for o in outs], self.nthreads)
        if rc:
            raise RuntimeError(f"orc_gh_driver failed ({rc})")
        return outs  # G_I, G_J, H_I, H_J

    def assemble_levels(self, M=None, nsteps=None):
        M = self.max_step() if M is None else M
        nsteps = self.m.numstep if nsteps is None else nsteps
        G = np.zeros((M + 1, self.D, self.D))
        H = np.zeros((M + 1, self.D, self.D))
        with _Clean(self.clean):
            rc = lib().orc_assemble_levels(ctypes.byref(self.st), M, nsteps, _d(G), _d(H),
                                           self.nthreads)
        if rc:
            raise RuntimeError(f"orc_assemble_levels failed ({rc})")
        return G, H

    def march(self, G, H, a1=0.0, a2=0.0, amp=None, numstep=None):
        m = self.m
        numstep = m.numstep if numstep is None else numstep
        M = G.shape[0] - 1
        u = np.zeros((numstep + 1, self.D))
        t = np.zeros((numstep + 1, self.D))
        ud = np.ascontiguousarray(m.ubc_dofs, np.int32)
        uv = np.ascontiguousarray(m.ubc_vals, np.float64)
        fd = np.ascontiguousarray(m.fbc_dofs, np.int32)
        fv = np.ascontiguousarray(m.fbc_vals, np.float64)
        ap = None if amp is None else _d(np.ascontiguousarray(amp, np.float64))
        rc = lib().orc_march(self.D, M, _d(np.ascontiguousarray(G)), _d(np.ascontiguousarray(H)),
                             len(ud), _i(ud), _d(uv), len(fd), _i(fd), _d(fv), ap, a1, a2,
                             numstep, _d(u), _d(t), self.nthreads)
        if rc:
            raise RuntimeError(f"orc_march failed ({rc})")
        return u, t


class MultiRegion:
    """Two-region solver, restated from SolverMRT (SolverMRT.cpp).

    Region r's model m_r lists its interface nodes (m_r.interface, 0-based); the
    interface of region 2 is matched to region 1's node by node (coordinates
    within 1e-10, the first match, SolverMRT.cpp:458-494).  The unknowns of the
    combined system are, in this order (LocalIndexing / InterfaceIndexing,
    SolverMRT.cpp:158-566):
      the interior displacements of region 1, of region 2 (interior nodes in
      ascending order), the interface displacements and the interface tractions
      of region 1 (interface-list order);
    its rows are region 1's collocation dofs, then region 2's; the known vector
    holds the interior tractions of both regions.  Region 2 sees the interface
    traction with the opposite sign.  Levels k = 0..max_step are the regions'
    levels (I(k) + J(k+1), level max_step = I(max_step)) placed by
    Assemble_GH_R1/R2 (SolverMRT.cpp:663-847, UpdateGHLinear 850-949), for the
    steps the marching loop reaches (n <= min(max_step, numstep)); marching
    is Solve_Direct (1028-1097) with SetLoad's load (867-966): the FBC values at
    interior dofs times p0 t exp(-2000 t), or times amp[n] when a load history is
    given.  Displacements of region r at step n (ExtractField, 1261-1309) are
    the combined unknowns mapped back to its dofs."""

    def __init__(self, m1, m2, max_step: int = 10, clean: bool = False, nthreads: int = 0):
        self.r = (Oracle(m1, nthreads, clean), Oracle(m2, nthreads, clean))
        self.L = int(max_step)
        self.nthreads = self.r[0].nthreads
        self._index(m1, m2)

    def _index(self, m1, m2):
        if1 = np.asarray(m1.interface, np.int64)
        if2 = np.asarray(m2.interface, np.int64)
        if len(if1) != len(if2):
            raise ValueError("the regions list different numbers of interface nodes")
        nz = len(if1)

        def dofs(nodes):
            return (3 * np.asarray(nodes, np.int64)[:, None] + np.arange(3)).reshape(-1)

        def interior(m, iface):
            lab = np.zeros(m.nnd, bool)
            lab[iface] = True
            return np.nonzero(~lab)[0]

        self.int1, self.int2 = dofs(interior(m1, if1)), dofs(interior(m2, if2))
        self.ifc1, self.ifc2 = dofs(if1), dofs(if2)
        x1, x2 = m1.coords, m2.coords
        match = np.empty(nz, np.int64)
        for ni in range(nz):
            p = x2[if2[ni]]
            found = -1
            for nj in range(nz):
                q = x1[if1[nj]]
                r = np.sqrt((q[0] - p[0]) * (q[0] - p[0]) + (q[1] - p[1]) * (q[1] - p[1]) +
                            (q[2] - p[2]) * (q[2] - p[2]))
                if r < 1e-10:
                    found = nj
                    break
            if found < 0:
                raise ValueError(f"interface node {ni} of region 2 has no match in region 1")
            match[ni] = found
        self.match = match
        self.d2to1 = dofs(match)
        self.D1, self.D2 = 3 * m1.nnd, 3 * m2.nnd
        self.NI1, self.NI2, self.NZ = len(self.int1), len(self.int2), 3 * nz
        self.N = self.D1 + self.D2
        self.NG = self.NI1 + self.NI2
        base_z = self.NI1 + self.NI2
        base_t = base_z + self.NZ
        # region-local dof -> combined column of its displacement; of its traction
        # (interface dofs only; -1 elsewhere) and that traction's sign
        self.ucol = (np.empty(self.D1, np.int64), np.empty(self.D2, np.int64))
        self.tcol = (np.full(self.D1, -1, np.int64), np.full(self.D2, -1, np.int64))
        self.tsign = (1.0, -1.0)
        self.ucol[0][self.int1] = np.arange(self.NI1)
        self.ucol[0][self.ifc1] = base_z + np.arange(self.NZ)
        self.tcol[0][self.ifc1] = base_t + np.arange(self.NZ)
        self.ucol[1][self.int2] = self.NI1 + np.arange(self.NI2)
        self.ucol[1][self.ifc2] = base_z + self.d2to1
        self.tcol[1][self.ifc2] = base_t + self.d2to1
        self.gcol = (np.arange(self.NI1), self.NI1 + np.arange(self.NI2))

    def region_levels(self, numstep=None):
        """Each region's levels 0..max_step: G_H_Driver runs for the steps
        1..min(max_step, numstep) of the marching loop, so level k holds
        I(k) + J(k+1) up to that step and zeros beyond."""
        numstep = self.r[0].m.numstep if numstep is None else numstep
        return [o.assemble_levels(M=self.L, nsteps=min(self.L, numstep)) for o in self.r]

    def combine(self, G1, H1, G2, H2):
        """Assemble_GH_R1 / Assemble_GH_R2 for every level: (L+1) x N x NG and
        (L+1) x N x N."""
        L1 = G1.shape[0]
        GG = np.zeros((L1, self.N, self.NG))
        HH = np.zeros((L1, self.N, self.N))
        rows = (slice(0, self.D1), slice(self.D1, self.N))
        ints = (self.int1, self.int2)
        ifcs = (self.ifc1, self.ifc2)
        base_z = self.NI1 + self.NI2
        zc = (base_z + np.arange(self.NZ), base_z + self.d2to1)
        for r, (G, H) in enumerate(((G1, H1), (G2, H2))):
            rw = rows[r]
            GG[:, rw, self.gcol[r]] = G[:, :, ints[r]]
            HH[:, rw, self.ucol[r][ints[r]]] = H[:, :, ints[r]]
            HH[:, rw, zc[r]] = H[:, :, ifcs[r]]
            # region 1 moves -G_z to the left, region 2 +G_z (its traction is -t_z)
            HH[:, rw, self.NZ + zc[r]] = -self.tsign[r] * G[:, :, ifcs[r]]
        return GG, HH

    def assemble_levels(self, numstep=None):
        (G1, H1), (G2, H2) = self.region_levels(numstep)
        return self.combine(G1, H1, G2, H2)

    def loads(self, numstep, amp=None):
        """fLoad of every step (row n, row 0 zero): interior FBC values x amplitude."""
        dt = self.r[0].m.dt
        out = np.zeros((numstep + 1, self.NG))
        for n in range(1, numstep + 1):
            a = lib().orc_mrt_amplitude(n, dt) if amp is None else (
                float(amp[n]) if n < len(amp) else 0.0)
            for r, o in enumerate(self.r):
                loc = np.zeros(3 * o.m.nnd)
                for d, v in zip(o.m.fbc_dofs, o.m.fbc_vals):
                    loc[d] = v * a
                out[n, self.gcol[r]] = loc[(self.int1, self.int2)[r]]
        return out

    def march(self, GG, HH, numstep=None, amp=None):
        """Combined unknowns x^n (n = 0..numstep) and the region displacements."""
        numstep = self.r[0].m.numstep if numstep is None else numstep
        load = np.ascontiguousarray(self.loads(numstep, amp))
        X = np.zeros((numstep + 1, self.N))
        L = GG.shape[0] - 1
        rc = lib().orc_mrt_march(self.N, self.NG, L, _d(np.ascontiguousarray(GG)),
                                 _d(np.ascontiguousarray(HH)), _d(load), numstep, _d(X),
                                 self.nthreads)
        if rc:
            raise RuntimeError(f"orc_mrt_march failed ({rc})")
        return X, X[:, self.ucol[0]], X[:, self.ucol[1]]


def lu_factor(A, nthreads=0):
    A = np.ascontiguousarray(A, np.float64)
    rc = lib().orc_lu_factor(A.shape[0], _d(A), nthreads or (os.cpu_count() or 1))
    if rc:
        raise RuntimeError(f"orc_lu_factor failed ({rc})")


def march_range(D, M, G, H, ubc_dofs, ubc_vals, fbc_dofs, fbc_vals, a1, a2, step_lo, step_hi,
                u, t, amp=None, nthreads=0):
    ud = np.ascontiguousarray(ubc_dofs, np.int32)
    uv = np.ascontiguousarray(ubc_vals, np.float64)
    fd = np.ascontiguousarray(fbc_dofs, np.int32)
    fv = np.ascontiguousarray(fbc_vals, np.float64)
    ap = None if amp is None else _d(np.ascontiguousarray(amp, np.float64))
    rc = lib().orc_march_range(D, M, _d(G), _d(H), len(ud), _i(ud), _d(uv), len(fd), _i(fd),
                               _d(fv), ap, a1, a2, step_lo, step_hi, _d(u), _d(t),
                               nthreads or (os.cpu_count() or 1))
    if rc:
        raise RuntimeError(f"orc_march_range failed ({rc})")


def green_step_linear(E, nu, rho, direction, normal, t, t_1):
    outs = [np.zeros(9) for _ in range(5)]
    lib().orc_green_step_linear(E, nu, rho, _d(np.ascontiguousarray(direction, float)),
                                _d(np.ascontiguousarray(normal, float)), t, t_1,
                                *[_d(o) for o in outs])
    return [o.reshape(3, 3) for o in outs]


def element_gh(etype, nq, E, nu, rho, coords, colloc, t, t_1, singular=-1):
    ennd = 4 if etype == 1 else 8
    outs = [np.zeros(9 * ennd) for _ in range(4)] + [np.zeros(9), np.zeros(9)]
    rc = lib().orc_element_gh(etype, nq, E, nu, rho, _d(np.ascontiguousarray(coords, float)),
                              _d(np.ascontiguousarray(colloc, float)), t, t_1, singular,
                              *[_d(o) for o in outs])
    if rc:
        raise RuntimeError("orc_element_gh failed")
    return [o.reshape(3, -1) for o in outs]
