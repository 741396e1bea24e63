"""Serving workload: a seeded Poisson stream of transient solves and its driver.

:func:`request_mix` draws the stream: arrivals with exponential gaps at a
given rate, each request one of

* a bar 1 x 1 x L, L ~ U{2..8}, 2 or 3 quads per unit length (one end fixed,
  unit axial traction on the other), redrawn until it has >= 300 DOF;
* a cavity sphere 6 x n x n, n ~ U{8..20} (internal pressure);
* a box-truncated half-space cavity: sphere of radius 1 at depth 3 under a
  10 x 10 free-surface patch at 1 quad per unit, cavity 6 x n x n, n ~ U{4..8};

with 100..400 steps and a Heaviside (amp = 1) or Gaussian-pulse load
(``exp(-((t - 3w) / w)^2 / 2)``, w = 5 dt), alpha = (0.25, 0).

:func:`run_stream` submits each request at its arrival time to a
:class:`tdbem.lib.Server`, waits for all of them and returns per-request
latency, queueing and run times with the stream's DOF*steps/s.
"""
from __future__ import annotations

import time

import numpy as np

from . import meshes


def _bar(rng, numstep):
    while True:
        L = int(rng.integers(2, 9))
        p = int(rng.integers(2, 4))
        m = meshes.bar(1, 1, L, per_unit=p, numstep=numstep)
        if 3 * m.nnd >= 300:
            return m, f"bar_1x1x{L}_q{p}"


def request_mix(n: int, rate_hz: float, seed: int = 0, kinds=("bar", "sphere", "halfspace"),
                sphere_range=(8, 20), steps_range=(100, 400)):
    """List of requests {arrival_s, name, model, amp} in arrival order."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for _ in range(n):
        t += rng.exponential(1.0 / rate_hz)
        kind = kinds[int(rng.integers(0, len(kinds)))]
        numstep = int(rng.integers(steps_range[0], steps_range[1] + 1))
        if kind == "bar":
            m, name = _bar(rng, numstep)
        elif kind == "sphere":
            k = int(rng.integers(sphere_range[0], sphere_range[1] + 1))
            m, name = meshes.cubed_sphere(k, numstep=numstep), f"sphere_6x{k}x{k}"
        else:
            k = int(rng.integers(4, 9))
            m = meshes.halfspace_cavity(depth=3.0, patch=10.0, per_unit=1, n_sphere=k,
                                        numstep=numstep)
            name = f"halfspace_cavity_6x{k}x{k}"
        amp = None
        if rng.random() < 0.5:
            w = 5.0 * m.dt
            tt = np.arange(numstep) * m.dt
            amp = np.exp(-0.5 * ((tt - 3.0 * w) / w) ** 2)
            name += "_gauss"
        out.append({"arrival_s": t, "name": name, "model": m, "amp": amp,
                    "dof": 3 * m.nnd, "steps": numstep})
    return out


def run_stream(server, reqs, alpha=(0.25, 0.0), precision: int = 1, keep_results: bool = False):
    """Submit every request at its arrival time, wait for all; per-request records."""
    t0 = time.perf_counter()
    ids = []
    for r in reqs:
        delay = r["arrival_s"] - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        ids.append(server.submit(r["model"], alpha=alpha, amp=r["amp"], precision=precision))
    recs = []
    for r, rid in zip(reqs, ids):
        server.wait(rid)
        u, t, times = server.result(rid)
        rec = {"name": r["name"], "dof": r["dof"], "steps": r["steps"], **times}
        if keep_results:
            rec["u"], rec["t"] = u, t
        recs.append(rec)
    wall = time.perf_counter() - t0
    lat = np.array([x["latency_s"] for x in recs])
    total = float(sum(x["dof"] * x["steps"] for x in recs))
    return {"records": recs, "wall_s": wall, "dof_steps": total,
            "dof_steps_per_s": total / wall,
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_queued_s": float(np.mean([x["queued_s"] for x in recs]))}
