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
