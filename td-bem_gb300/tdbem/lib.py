"""ctypes binding of the C ABI in include/tdbem.h (libtdbem.so).

Fails loudly when the library is missing or no CUDA device is present; there
is no CPU path.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "_build", "libtdbem.so")

FP64 = 0
MIXED = 1

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)

# Every symbol include/tdbem.h declares, with its ctypes signature.
SIGNATURES = {
    "tdbem_last_error": (ctypes.c_char_p, []),
    "tdbem_version": (ctypes.c_char_p, []),
    "tdbem_ctx_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                                        ctypes.c_int, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_void_p)]),
    "tdbem_ctx_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "tdbem_element_gh": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_int, _dp, _dp, _dp, _ip, _dp, _dp, _dp, _dp,
                                        _dp, _dp]),
    "tdbem_max_step": (ctypes.c_int, [ctypes.c_void_p, _ip]),
    "tdbem_num_dof": (ctypes.c_int, [ctypes.c_void_p, _ip]),
    "tdbem_get_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]),
    "tdbem_gh_driver": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       _dp, _dp, _dp, _dp]),
    "tdbem_gh_driver_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                               ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_void_p]),
    "tdbem_assemble_levels": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "tdbem_get_level": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp]),
    "tdbem_set_bc": (ctypes.c_int, [ctypes.c_void_p, _ip, _dp, ctypes.c_int, _ip, _dp,
                                    ctypes.c_int]),
    "tdbem_set_alpha": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double]),
    "tdbem_set_load_history": (ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.c_int]),
    "tdbem_march": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, _dp]),
    "tdbem_march_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp, _dp,
                                         _dp, _dp]),
    "tdbem_history_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p),
                                            ctypes.POINTER(ctypes.c_void_p)]),
    "tdbem_level_bytes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_size_t)]),
    "tdbem_last_timings": (ctypes.c_int, [ctypes.c_void_p, _dp]),
    "tdbem_set_profiling": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "tdbem_kernel_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_longlong), _dp, _dp, _dp]),
    "tdbem_launch_count": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "tdbem_set_march_options": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "tdbem_set_batch_options": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "tdbem_set_graphs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "tdbem_set_pipeline_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "tdbem_inverse_report": (ctypes.c_int, [ctypes.c_void_p, _dp, _ip, _ip]),
    "tdbem_invert": (ctypes.c_int, [ctypes.c_int, _dp, ctypes.c_int, _dp, _dp, _ip]),
    "tdbem_set_march_engine": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "tdbem_assemble_group": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, _ip,
                                            ctypes.c_int]),
    "tdbem_march_group": (ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, _ip,
                                         ctypes.POINTER(_dp), ctypes.POINTER(_dp)]),
    "tdbem_group_shape": (ctypes.c_int, [_ip, _ip, _ip]),
    "tdbem_update_gh_linear": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_int, _dp, _dp, _dp, _dp]),
    "tdbem_march_begin": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "tdbem_march_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, _dp]),
    "tdbem_export_levels": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "tdbem_import_levels": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "tdbem_write_gh": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      _dp]),
    "tdbem_footprint": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                                       ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_size_t)]),
    "tdbem_server_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_size_t, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_void_p)]),
    "tdbem_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.POINTER(ctypes.c_longlong)]),
    "tdbem_server_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_longlong, ctypes.c_double,
                                         _ip]),
    "tdbem_server_result": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_longlong, _dp, _dp, _dp]),
    "tdbem_server_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t),
                                          ctypes.POINTER(ctypes.c_size_t), _ip, _ip,
                                          ctypes.POINTER(ctypes.c_longlong)]),
    "tdbem_server_march_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong),
                                                 ctypes.POINTER(ctypes.c_longlong),
                                                 ctypes.POINTER(ctypes.c_double)]),
    "tdbem_server_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "tdbem_cached_memory": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]),
    "tdbem_release_cached_memory": (ctypes.c_int, [ctypes.c_int,
                                                    ctypes.POINTER(ctypes.c_size_t)]),
    "tdbem_mrt_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, _ip, _ip, ctypes.c_int,
                                        ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "tdbem_mrt_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "tdbem_mrt_size": (ctypes.c_int, [ctypes.c_void_p, _ip, _ip]),
    "tdbem_mrt_columns": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _ip, _ip]),
    "tdbem_mrt_set_load_history": (ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.c_int]),
    "tdbem_mrt_set_refine": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "tdbem_mrt_assemble": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "tdbem_mrt_march": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _dp, _dp, _dp]),
    "tdbem_mrt_begin": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "tdbem_mrt_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _dp, _dp, _dp]),
}

KERNEL_CLASSES = {0: "assemble", 1: "conv", 2: "factor", 3: "solve", 4: "assemble_f32",
                  5: "conv_block", 6: "aux", 7: "conv_batch", 8: "solve_batch"}


class Mesh(ctypes.Structure):
    _fields_ = [("nnd", ctypes.c_int), ("nel", ctypes.c_int), ("etype", ctypes.c_int),
                ("coords", _dp), ("ien", _ip)]


class Material(ctypes.Structure):
    _fields_ = [("E", ctypes.c_double), ("nu", ctypes.c_double), ("rho", ctypes.c_double)]


class Request(ctypes.Structure):
    _fields_ = [("mesh", Mesh), ("mat", Material), ("dt", ctypes.c_double), ("nq", ctypes.c_int),
                ("if_ext", ctypes.c_int), ("ubc_dofs", _ip), ("ubc_vals", _dp),
                ("n_u", ctypes.c_int), ("fbc_dofs", _ip), ("fbc_vals", _dp),
                ("n_f", ctypes.c_int), ("alpha1", ctypes.c_double), ("alpha2", ctypes.c_double),
                ("amp", _dp), ("numstep", ctypes.c_int), ("precision", ctypes.c_int)]


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = 0, 1, 2, 3
ENGINE_TCGEN05, ENGINE_MMA_SYNC, ENGINE_FP32 = 0, 1, 2


def _ctx_array(ctxs):
    arr = (ctypes.c_void_p * len(ctxs))()
    for i, c in enumerate(ctxs):
        arr[i] = c.h.value if isinstance(c.h, ctypes.c_void_p) else c.h
    return arr


def assemble_group(ctxs, nsteps=None, precision: int = FP64):
    """Levels of several contexts together (tdbem_assemble_group)."""
    ns = [c.model.numstep for c in ctxs] if nsteps is None else list(nsteps)
    n_arr = np.ascontiguousarray(ns, np.int32)
    _check(load().tdbem_assemble_group(_ctx_array(ctxs), len(ctxs), _i(n_arr), precision))


def march_group(ctxs, numsteps=None, to_host: bool = True):
    """March several FP64 contexts in one persistent launch; [(u, t)] per context."""
    ns = [c.model.numstep for c in ctxs] if numsteps is None else list(numsteps)
    n_arr = np.ascontiguousarray(ns, np.int32)
    outs = [(np.empty((k + 1, c.D)), np.empty((k + 1, c.D))) for c, k in zip(ctxs, ns)]
    U = (_dp * len(ctxs))(*[_d(u) for u, _ in outs])
    T = (_dp * len(ctxs))(*[_d(t) for _, t in outs])
    if to_host:
        _check(load().tdbem_march_group(_ctx_array(ctxs), len(ctxs), _i(n_arr), U, T))
        return outs
    _check(load().tdbem_march_group(_ctx_array(ctxs), len(ctxs), _i(n_arr), None, None))
    return None


def group_shape():
    a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _check(load().tdbem_group_shape(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
    return {"lanes": a.value, "block": b.value, "blocks_per_sm": c.value}


def element_gh(etype: int, nq: int, E: float, nu: float, rho: float, t_1: float, colloc,
               coords, t, singular):
    """TDElementStepLinearT's element blocks of n (collocation point, element) pairs
    in one launch (tdbem_element_gh).  colloc (n, 3), coords (n, ennd, 3), t (n,),
    singular (n,) (-1: FormGH_Regular).  Returns GE_1, GE_2, HE_1, HE_2 of shape
    (n, 3, 3 ennd) and C_1, C_2 of shape (n, 3, 3)."""
    ennd = 4 if etype == 1 else 8
    xc = np.ascontiguousarray(colloc, np.float64).reshape(-1, 3)
    n = xc.shape[0]
    en = np.ascontiguousarray(coords, np.float64).reshape(n, ennd, 3)
    tt = np.ascontiguousarray(np.broadcast_to(np.asarray(t, np.float64), (n,)))
    sg = np.ascontiguousarray(np.broadcast_to(np.asarray(singular, np.int32), (n,)))
    outs = [np.empty((n, 3, 3 * ennd)) for _ in range(4)] + [np.empty((n, 3, 3)) for _ in range(2)]
    _check(load().tdbem_element_gh(etype, nq, E, nu, rho, t_1, n, _d(xc), _d(en), _d(tt), _i(sg),
                                   *[_d(o) for o in outs]))
    return outs


def invert(A, precision: int = FP64):
    """X = A^-1 on the device (tdbem_invert): returns X, the FP32 inverse's probe
    residual and whether its pivot search fell back to the full panel."""
    a = np.ascontiguousarray(A, np.float64)
    n = a.shape[0]
    x = np.empty_like(a)
    probe = ctypes.c_double()
    full = ctypes.c_int()
    _check(load().tdbem_invert(n, _d(a), precision, _d(x), ctypes.byref(probe),
                               ctypes.byref(full)))
    return x, probe.value, full.value


def cached_memory(device: int = -1) -> int:
    """Device bytes the library keeps for reuse (tdbem_cached_memory)."""
    b = ctypes.c_size_t()
    _check(load().tdbem_cached_memory(device, ctypes.byref(b)))
    return b.value


def release_cached_memory(device: int = -1) -> int:
    """Free the device memory the library keeps for reuse; returns the bytes freed."""
    b = ctypes.c_size_t()
    _check(load().tdbem_release_cached_memory(device, ctypes.byref(b)))
    return b.value


def write_gh(prefix: str, step: int, data) -> None:
    """SolverT::WriteGH's <prefix><step>.txt for a row block (tdbem_write_gh)."""
    a = np.ascontiguousarray(data, np.float64)
    _check(load().tdbem_write_gh(prefix.encode(), step, a.shape[0], a.shape[1], _d(a)))


def footprint(model, precision: int = 1, numstep: Optional[int] = None) -> int:
    """Device bytes a solve of ``model`` needs (tdbem_footprint)."""
    c = np.ascontiguousarray(model.coords, np.float64)
    e = np.ascontiguousarray(model.ien, np.int32)
    mesh = Mesh(model.nnd, model.nel, model.etype, _d(c), _i(e))
    mat = Material(model.E, model.nu, model.rho)
    b = ctypes.c_size_t()
    _check(load().tdbem_footprint(ctypes.byref(mesh), ctypes.byref(mat), model.dt, model.nq,
                                  model.numstep if numstep is None else numstep, precision,
                                  ctypes.byref(b)))
    return b.value


class Server:
    """Continuous-batching server of transient solves (tdbem_server_*)."""

    def __init__(self, device: int = 0, budget_bytes: int = 0, slots: int = 4):
        h = ctypes.c_void_p()
        _check(load().tdbem_server_create(device, budget_bytes, slots, ctypes.byref(h)))
        self.h = h
        self._meta = {}

    def submit(self, model, alpha=(0.25, 0.0), amp=None, precision: int = 1) -> int:
        keep = [np.ascontiguousarray(model.coords, np.float64),
                np.ascontiguousarray(model.ien, np.int32),
                np.ascontiguousarray(model.ubc_dofs, np.int32),
                np.ascontiguousarray(model.ubc_vals, np.float64),
                np.ascontiguousarray(model.fbc_dofs, np.int32),
                np.ascontiguousarray(model.fbc_vals, np.float64)]
        a = None if amp is None else np.ascontiguousarray(amp, np.float64)
        if a is not None and len(a) < model.numstep:
            raise ValueError("amp needs numstep values")
        req = Request(Mesh(model.nnd, model.nel, model.etype, _d(keep[0]), _i(keep[1])),
                      Material(model.E, model.nu, model.rho), model.dt, model.nq, model.if_ext,
                      _i(keep[2]), _d(keep[3]), len(keep[2]), _i(keep[4]), _d(keep[5]),
                      len(keep[4]), alpha[0], alpha[1], None if a is None else _d(a),
                      model.numstep, precision)
        rid = ctypes.c_longlong()
        _check(load().tdbem_server_submit(self.h, ctypes.byref(req), ctypes.byref(rid)))
        self._meta[rid.value] = (model.numstep, 3 * model.nnd)
        return rid.value

    def wait(self, rid: int, timeout: float = -1.0) -> int:
        st = ctypes.c_int()
        _check(load().tdbem_server_wait(self.h, rid, timeout, ctypes.byref(st)))
        return st.value

    def result(self, rid: int):
        """(u, t, {queued_s, run_s, latency_s}) of a finished request."""
        n, D = self._meta.pop(rid)
        u = np.empty((n + 1, D))
        t = np.empty((n + 1, D))
        times = np.zeros(3)
        _check(load().tdbem_server_result(self.h, rid, _d(u), _d(t), _d(times)))
        return u, t, {"queued_s": times[0], "run_s": times[1], "latency_s": times[2]}

    def stats(self):
        used, budget = ctypes.c_size_t(), ctypes.c_size_t()
        act, q, done = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
        _check(load().tdbem_server_stats(self.h, ctypes.byref(used), ctypes.byref(budget),
                                         ctypes.byref(act), ctypes.byref(q), ctypes.byref(done)))
        return {"used_bytes": used.value, "budget_bytes": budget.value, "active": act.value,
                "queued": q.value, "completed": done.value}

    def march_stats(self):
        """Grouped march launches, solve-steps they advanced, mean resident solves."""
        n, st, mr = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_double()
        _check(load().tdbem_server_march_stats(self.h, ctypes.byref(n), ctypes.byref(st),
                                               ctypes.byref(mr)))
        return {"launches": n.value, "solve_steps": st.value, "mean_resident": mr.value}

    def close(self):
        if self.h:
            load().tdbem_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class TdbemError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"tdbem error {code}: {msg}")
        self.code = code


_lib = None


def load(path: Optional[str] = None):
    """Load libtdbem.so (built by td-bem_gb300/build.py); raise if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise FileNotFoundError(f"{p} is missing: run td-bem_gb300/build.py (no CPU fallback)")
    L = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _check(rc: int):
    if rc != 0:
        raise TdbemError(rc, load().tdbem_last_error().decode())


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


class Context:
    """One tdbem_ctx: a mesh + material + time step on the current CUDA device."""

    def __init__(self, model, nq: Optional[int] = None):
        L = load()
        self.model = model
        self._coords = np.ascontiguousarray(model.coords, np.float64)
        self._ien = np.ascontiguousarray(model.ien, np.int32)
        mesh = Mesh(model.nnd, model.nel, model.etype, _d(self._coords), _i(self._ien))
        mat = Material(model.E, model.nu, model.rho)
        h = ctypes.c_void_p()
        _check(L.tdbem_ctx_create(ctypes.byref(mesh), ctypes.byref(mat), model.dt,
                                  nq or model.nq, model.if_ext, ctypes.byref(h)))
        self.h = h
        self.D = 3 * model.nnd
        m = ctypes.c_int()
        _check(L.tdbem_max_step(h, ctypes.byref(m)))
        self.M = m.value
        self.set_bc(model.ubc_dofs, model.ubc_vals, model.fbc_dofs, model.fbc_vals)

    def close(self):
        if getattr(self, "h", None):
            load().tdbem_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def stream(self) -> int:
        s = ctypes.c_void_p()
        _check(load().tdbem_get_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    def set_bc(self, ubc_dofs, ubc_vals, fbc_dofs, fbc_vals):
        self._ud = np.ascontiguousarray(ubc_dofs, np.int32)
        self._uv = np.ascontiguousarray(ubc_vals, np.float64)
        self._fd = np.ascontiguousarray(fbc_dofs, np.int32)
        self._fv = np.ascontiguousarray(fbc_vals, np.float64)
        _check(load().tdbem_set_bc(self.h, _i(self._ud), _d(self._uv), len(self._ud),
                                   _i(self._fd), _d(self._fv), len(self._fd)))

    def set_alpha(self, a1: float, a2: float):
        _check(load().tdbem_set_alpha(self.h, a1, a2))

    def set_march_options(self, block_steps: int = 0, refine_sweeps: int = 0):
        """Time-block steps of the mixed march (0: the engine's default, 32 with
        ENGINE_TCGEN05 and 8 with ENGINE_FP32) and FP64 refinement sweeps per solve."""
        _check(load().tdbem_set_march_options(self.h, block_steps, refine_sweeps))

    def set_march_engine(self, engine: int):
        """ENGINE_TCGEN05 (default: merged levels, split-BF16 tensor-core products, ~1e-5
        of FP64) or ENGINE_FP32 (FP32 products on the CUDA cores, ~2e-7)."""
        _check(load().tdbem_set_march_engine(self.h, engine))

    def set_graphs(self, on: bool):
        _check(load().tdbem_set_graphs(self.h, 1 if on else 0))

    def set_pipeline_wait(self, seconds: float):
        """Limit of each pipeline wait of the tcgen05 convolution (0: the default, 2 s)."""
        _check(load().tdbem_set_pipeline_wait(self.h, seconds))

    def inverse_report(self):
        """(probe residuals, full-search flags, step-2 Richardson sweeps) of the FP32
        inverses of the mixed march."""
        p = (ctypes.c_double * 2)()
        f = (ctypes.c_int * 2)()
        k = ctypes.c_int()
        _check(load().tdbem_inverse_report(self.h, p, f, ctypes.byref(k)))
        return list(p), list(f), k.value

    def set_batch_options(self, engine: int = 0, refine_sweeps: int = 0):
        _check(load().tdbem_set_batch_options(self.h, engine, refine_sweeps))

    def set_load_history(self, amp):
        self._amp = np.ascontiguousarray(amp, np.float64)
        _check(load().tdbem_set_load_history(self.h, _d(self._amp), len(self._amp)))

    def assemble(self, nsteps: Optional[int] = None, precision: int = FP64):
        ns = self.model.numstep if nsteps is None else nsteps
        _check(load().tdbem_assemble_levels(self.h, ns, precision))

    def level(self, k: int, which: int) -> np.ndarray:
        out = np.empty((self.D, self.D))
        _check(load().tdbem_get_level(self.h, k, which, _d(out)))
        return out

    def levels(self):
        G = np.stack([self.level(k, 0) for k in range(self.M + 1)])
        H = np.stack([self.level(k, 1) for k in range(self.M + 1)])
        return G, H

    def gh_driver(self, step: int, node_lo: int = 0, node_hi: Optional[int] = None):
        hi = self.model.nnd - 1 if node_hi is None else node_hi
        rows = 3 * (hi - node_lo + 1)
        outs = [np.empty((rows, self.D)) for _ in range(4)]
        _check(load().tdbem_gh_driver(self.h, step, node_lo, hi, *[_d(o) for o in outs]))
        return outs  # G_I, G_J, H_I, H_J

    def march(self, numstep: Optional[int] = None, to_host: bool = True):
        n = self.model.numstep if numstep is None else numstep
        if to_host:
            u = np.empty((n + 1, self.D))
            t = np.empty((n + 1, self.D))
            _check(load().tdbem_march(self.h, n, _d(u), _d(t)))
            return u, t
        _check(load().tdbem_march(self.h, n, None, None))
        return None

    def march_batch(self, traction, amp=None, numstep: Optional[int] = None,
                    to_host: bool = True):
        """March every load case of ``traction`` (cases x D) at once.

        ``amp`` (cases x numstep) scales case c's traction at step s; None means
        a unit step load.  Returns u, t of shape (numstep + 1, cases, D)."""
        n = self.model.numstep if numstep is None else numstep
        tr = np.ascontiguousarray(traction, dtype=np.float64)
        if tr.ndim != 2 or tr.shape[1] != self.D:
            raise ValueError(f"traction must be (cases, {self.D})")
        nc = tr.shape[0]
        a = None
        if amp is not None:
            a = np.ascontiguousarray(amp, dtype=np.float64)
            if a.shape != (nc, n):
                raise ValueError(f"amp must be ({nc}, {n})")
        if to_host:
            u = np.empty((n + 1, nc, self.D))
            t = np.empty((n + 1, nc, self.D))
            _check(load().tdbem_march_batch(self.h, n, nc, _d(tr), None if a is None else _d(a),
                                            _d(u), _d(t)))
            return u, t
        _check(load().tdbem_march_batch(self.h, n, nc, _d(tr), None if a is None else _d(a),
                                        None, None))
        return None

    def update_gh_linear(self, step: int, G_I, G_J, H_I, H_J, node_lo: int = 0):
        blocks = [np.ascontiguousarray(x, np.float64) for x in (G_I, G_J, H_I, H_J)]
        rows = blocks[0].shape[0]
        hi = node_lo + rows // 3 - 1
        _check(load().tdbem_update_gh_linear(self.h, step, node_lo, hi, *[_d(b) for b in blocks]))

    def march_begin(self, numstep: Optional[int] = None):
        n = self.model.numstep if numstep is None else numstep
        _check(load().tdbem_march_begin(self.h, n))

    def march_step(self, curr_step: int):
        u = np.empty(self.D)
        t = np.empty(self.D)
        _check(load().tdbem_march_step(self.h, curr_step, _d(u), _d(t)))
        return u, t

    def export_levels(self, path: str):
        _check(load().tdbem_export_levels(self.h, path.encode()))

    def import_levels(self, path: str):
        _check(load().tdbem_import_levels(self.h, path.encode()))

    def timings(self):
        out = np.zeros(3)
        _check(load().tdbem_last_timings(self.h, _d(out)))
        return {"assemble_ms": out[0], "factor_ms": out[1], "march_ms": out[2]}

    def set_profiling(self, on: bool):
        _check(load().tdbem_set_profiling(self.h, 1 if on else 0))

    def kernel_stats(self):
        out = {}
        for k, name in KERNEL_CLASSES.items():
            n = ctypes.c_longlong()
            ms, by, fl = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
            _check(load().tdbem_kernel_stats(self.h, k, ctypes.byref(n), ctypes.byref(ms),
                                             ctypes.byref(by), ctypes.byref(fl)))
            out[name] = {"launches": n.value, "ms": ms.value, "bytes": by.value,
                         "flops": fl.value}
        return out

    def launch_count(self) -> int:
        n = ctypes.c_longlong()
        _check(load().tdbem_launch_count(self.h, ctypes.byref(n)))
        return n.value

    def level_bytes(self, precision: int = FP64) -> int:
        b = ctypes.c_size_t()
        _check(load().tdbem_level_bytes(self.h, precision, ctypes.byref(b)))
        return b.value


class MultiRegion:
    """Two-region solver (tdbem_mrt_*, SolverMRT): region models m1, m2 with their
    interface lists (model.interface, 0-based), max_step levels (SolverMRT's
    SetMaxStep; the reference's default 10).  Each region gets its own Context
    (its FBC list gives its loads)."""

    def __init__(self, m1, m2, max_step: int = 10, iface1=None, iface2=None):
        L = load()
        self.regions = (Context(m1), Context(m2))
        i1 = np.ascontiguousarray(m1.interface if iface1 is None else iface1, np.int32)
        i2 = np.ascontiguousarray(m2.interface if iface2 is None else iface2, np.int32)
        if len(i1) != len(i2):
            self.close()
            raise ValueError("the regions list different numbers of interface nodes")
        h = ctypes.c_void_p()
        try:
            _check(L.tdbem_mrt_create(self.regions[0].h, self.regions[1].h, _i(i1), _i(i2),
                                      len(i1), max_step, ctypes.byref(h)))
        except Exception:
            self.close()
            raise
        self.h = h
        self.numstep = m1.numstep
        n, ng = ctypes.c_int(), ctypes.c_int()
        _check(L.tdbem_mrt_size(h, ctypes.byref(n), ctypes.byref(ng)))
        self.N, self.NG = n.value, ng.value
        self.D = (self.regions[0].D, self.regions[1].D)

    def columns(self, region: int):
        u = np.zeros(self.D[region - 1], np.int32)
        t = np.zeros(self.D[region - 1], np.int32)
        _check(load().tdbem_mrt_columns(self.h, region, _i(u), _i(t)))
        return u, t

    def set_load_history(self, amp):
        a = np.ascontiguousarray(np.zeros(0) if amp is None else amp, np.float64)
        self._amp = a
        _check(load().tdbem_mrt_set_load_history(self.h, _d(a), len(a)))

    def set_refine(self, refine: int):
        _check(load().tdbem_mrt_set_refine(self.h, refine))

    def assemble(self, numstep: Optional[int] = None):
        _check(load().tdbem_mrt_assemble(self.h, numstep or self.numstep))

    def march(self, numstep: Optional[int] = None):
        """Combined unknowns x and (u1, t1, u2, t2), numstep + 1 rows each."""
        n = numstep or self.numstep
        x = np.zeros((n + 1, self.N))
        out = [np.zeros((n + 1, d)) for d in (self.D[0], self.D[0], self.D[1], self.D[1])]
        _check(load().tdbem_mrt_march(self.h, n, _d(x), *[_d(o) for o in out]))
        return x, out[0], out[1], out[2], out[3]

    def begin(self, numstep: Optional[int] = None):
        self._steps = numstep or self.numstep
        _check(load().tdbem_mrt_begin(self.h, self._steps))

    def step(self, curr_step: int):
        """Solve step curr_step from the placed levels; x, u1, t1, u2, t2 of that step."""
        out = [np.zeros(k) for k in (self.N, self.D[0], self.D[0], self.D[1], self.D[1])]
        _check(load().tdbem_mrt_step(self.h, curr_step, *[_d(o) for o in out]))
        return tuple(out)

    def close(self):
        if getattr(self, "h", None):
            load().tdbem_mrt_destroy(self.h)
            self.h = None
        for c in getattr(self, "regions", ()):
            c.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

