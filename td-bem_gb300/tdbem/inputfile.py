"""Reader and writer for the TD-BEM keyword input format.

The format is the reference's (InputT.cpp:84-994): one keyword per line,
tokens separated by any of `` \\t=;,`` (InputT.cpp:21), integer values parsed
with C ``atoi`` and reals with ``atof``.  ``nodes`` and ``IEN`` are followed
by ``nnd`` / ``nel`` lines; ``UBC_dof``, ``UBC_values``, ``FBC_dof`` and
``FBC_values`` read lines until their count is reached.  Node ids and dof ids
are 1-based in the file and 0-based in memory (InputT.cpp:529, 747, 856).
An unknown keyword is an error (InputT.cpp:130-136).

The same format is parsed natively by the C++ host (csrc/host/input.cpp);
this module exists for tests, mesh generators and the benchmark.
"""
from __future__ import annotations

import dataclasses
import re
from typing import List, Optional

import numpy as np

_DELIM = re.compile(r"[ \t=;,]+")


def _tokens(line: str) -> List[str]:
    return [t for t in _DELIM.split(line.rstrip("\r\n")) if t]


def c_atoi(tok: str) -> int:
    """C atoi: optional sign and leading digits, 0 when there are none."""
    m = re.match(r"\s*([+-]?\d+)", tok)
    return int(m.group(1)) if m else 0


def c_atof(tok: str) -> float:
    """C atof on the longest leading decimal floating-point prefix."""
    m = re.match(r"\s*([+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?)", tok)
    return float(m.group(1)) if m else 0.0


@dataclasses.dataclass
class Model:
    """Everything ModelManagerT holds for the main path (ModelManagerT.h:16-196)."""

    coords: np.ndarray  # nnd x 3 float64
    ien: np.ndarray  # nel x ennd int32, 0-based
    etype: int = 1  # 1 = Q4, 2 = Q8
    E: float = 1.0
    nu: float = 0.0
    rho: float = 1.0
    dt: float = 0.0
    numstep: int = 1
    nq: int = 6
    if_ext: int = 0
    formulation: int = 1
    interpolation: int = 1
    sd: int = 3
    ubc_dofs: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
    ubc_vals: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    fbc_dofs: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
    fbc_vals: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    interface: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
    # auxiliary mesh of a multi-region input (formulation = 3); read, not used by the path
    etype_aux: int = 1
    coords_aux: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 3)))
    ien_aux: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 4), np.int32))

    @property
    def nnd(self) -> int:
        return int(self.coords.shape[0])

    @property
    def nel(self) -> int:
        return int(self.ien.shape[0])

    @property
    def ennd(self) -> int:
        return 4 if self.etype == 1 else 8

    @property
    def ndof(self) -> int:
        return 3 * self.nnd

    def material(self):
        """(mu, lambda, c_p, c_s) as GreenFunctionT::WaveSpeed (GreenFunctionT.cpp:76-84)."""
        mu = self.E / (2 * (1 + self.nu))
        lam = self.E * self.nu / ((1 + self.nu) * (1 - 2 * self.nu))
        return mu, lam, np.sqrt((lam + 2 * mu) / self.rho), np.sqrt(mu / self.rho)

    def max_step(self) -> int:
        """SolverT::ComputeMaxStep (SolverT.cpp:211-250)."""
        _, _, _, cs = self.material()
        x = self.coords
        dmax = 0.0
        for i in range(self.nnd - 1):
            d = np.sqrt(((x[i + 1:] - x[i]) ** 2).sum(1)).max()
            dmax = max(dmax, d)
        return int(np.ceil(dmax / (cs * self.dt)) + 1)


class InputError(ValueError):
    pass


def _read_list(lines, i, count, conv):
    out = []
    while len(out) < count:
        i += 1
        if i >= len(lines):
            raise InputError("unexpected end of file in a dof/value list")
        toks = _tokens(lines[i])
        if not toks:
            raise InputError(f"line {i + 1}: empty line inside a dof/value list")
        for t in toks:
            if len(out) < count:
                out.append(conv(t))
    return i, out


def parse(text: str) -> Model:
    """Parse the reference input format (InputT::ReadInput, InputT.cpp:84-144)."""
    lines = text.splitlines()
    kv = dict(formulation=1, interpolation=1, numstep=1, dt=0.0, nq=6, E=1.0, nu=0.0,
              density=1.0, sd=3, if_ext=0, nnd=0, nel=0, EType=1)
    ennd = 4
    coords = None
    ien = None
    ubc_num = fbc_num = num_if = 0
    ubc_d: List[int] = []
    ubc_v: List[float] = []
    fbc_d: List[int] = []
    fbc_v: List[float] = []
    iface: List[int] = []
    ints = {"formulation", "numstep", "sd", "if_ext", "nnd", "nel"}
    reals = {"dt", "E", "nu", "density"}
    nnd_aux = nel_aux = 0
    etype_aux, ennd_aux = 1, 4
    coords_aux = np.zeros((0, 3))
    ien_aux = np.zeros((0, 4), np.int32)
    i = 0
    while i < len(lines):
        toks = _tokens(lines[i])
        if not toks:
            i += 1
            continue
        k = toks[0]
        val = toks[1] if len(toks) > 1 else None
        if k in ints or k in reals or k in ("interpolation", "nq", "EType", "UBC_num",
                                           "FBC_num", "num_interface"):
            if val is None:
                raise InputError(f"line {i + 1}: {k} is not set properly")
        if k in ints:
            kv[k] = c_atoi(val)
        elif k in reals:
            kv[k] = c_atof(val)
        elif k in ("interpolation", "nq"):
            kv[k] = int(c_atof(val))  # int member assigned from atof (InputT.cpp:239, 262)
        elif k == "EType":
            kv[k] = c_atoi(val)
            if kv[k] == 1:
                ennd = 4
            elif kv[k] == 2:
                ennd = 8
            else:
                raise InputError("unsupported element type")
        elif k == "nodes":
            n = kv["nnd"]
            coords = np.zeros((n, 3))
            for nid in range(n):
                i += 1
                t = _tokens(lines[i]) if i < len(lines) else []
                if len(t) < 3:
                    raise InputError(f"line {i + 1}: node {nid + 1} needs 3 coordinates")
                coords[nid] = [c_atof(t[0]), c_atof(t[1]), c_atof(t[2])]
        elif k == "IEN":
            n = kv["nel"]
            ien = np.zeros((n, ennd), np.int32)
            for eid in range(n):
                i += 1
                t = _tokens(lines[i]) if i < len(lines) else []
                if len(t) < ennd:
                    raise InputError(f"line {i + 1}: element {eid + 1} needs {ennd} nodes")
                ien[eid] = [c_atoi(x) - 1 for x in t[:ennd]]
        elif k == "UBC_num":
            ubc_num = c_atoi(val)
        elif k == "UBC_dof":
            i, ubc_d = _read_list(lines, i, ubc_num, lambda t: c_atoi(t) - 1)
        elif k == "UBC_values":
            i, ubc_v = _read_list(lines, i, ubc_num, c_atof)
        elif k == "FBC_num":
            fbc_num = c_atoi(val)
        elif k == "FBC_dof":
            i, fbc_d = _read_list(lines, i, fbc_num, lambda t: c_atoi(t) - 1)
        elif k == "FBC_values":
            i, fbc_v = _read_list(lines, i, fbc_num, c_atof)
        elif k == "num_interface":
            num_if = c_atoi(val)
        elif k == "interface":
            i, iface = _read_list(lines, i, num_if, lambda t: c_atoi(t) - 1)
        elif kv["formulation"] == 3 and k in ("nnd_aux", "etype_aux", "nel_aux"):
            # InputT::ReadGeometry_Aux (InputT.cpp:548-693), read only when formulation = 3
            if val is None:
                raise InputError(f"line {i + 1}: {k} is not set properly")
            if k == "nnd_aux":
                nnd_aux = c_atoi(val)
            elif k == "nel_aux":
                nel_aux = c_atoi(val)
            else:
                etype_aux = c_atoi(val)
                if etype_aux == 1:
                    ennd_aux = 4
                elif kv["EType"] == 2:  # the reference tests the main EType here (:599)
                    ennd_aux = 8
                else:
                    raise InputError("unsupported element type")
        elif kv["formulation"] == 3 and k == "nodes_aux":
            coords_aux = np.zeros((nnd_aux, 3))
            for nid in range(nnd_aux):
                i += 1
                t = _tokens(lines[i]) if i < len(lines) else []
                if len(t) < 3:
                    raise InputError(f"line {i + 1}: aux node {nid + 1} needs 3 coordinates")
                coords_aux[nid] = [c_atof(t[0]), c_atof(t[1]), c_atof(t[2])]
        elif kv["formulation"] == 3 and k == "IEN_aux":
            ien_aux = np.zeros((nel_aux, ennd_aux), np.int32)
            for eid in range(nel_aux):
                i += 1
                t = _tokens(lines[i]) if i < len(lines) else []
                if len(t) < ennd_aux:
                    raise InputError(f"line {i + 1}: aux element {eid + 1} needs "
                                     f"{ennd_aux} nodes")
                ien_aux[eid] = [c_atoi(x) - 1 for x in t[:ennd_aux]]
        else:
            raise InputError(f"line {i + 1}: unaccepted key word {k!r}")
        i += 1
    if coords is None or ien is None:
        raise InputError("input has no nodes or no IEN block")
    if len(ubc_d) != ubc_num or len(ubc_v) != ubc_num:
        raise InputError("UBC_dof / UBC_values do not match UBC_num")
    if len(fbc_d) != fbc_num or len(fbc_v) != fbc_num:
        raise InputError("FBC_dof / FBC_values do not match FBC_num")
    return Model(coords=coords, ien=ien, etype=kv["EType"], E=kv["E"], nu=kv["nu"],
                 rho=kv["density"], dt=kv["dt"], numstep=kv["numstep"], nq=kv["nq"],
                 if_ext=kv["if_ext"], formulation=kv["formulation"],
                 interpolation=kv["interpolation"], sd=kv["sd"],
                 ubc_dofs=np.array(ubc_d, np.int32), ubc_vals=np.array(ubc_v, float),
                 fbc_dofs=np.array(fbc_d, np.int32), fbc_vals=np.array(fbc_v, float),
                 interface=np.array(iface, np.int32), etype_aux=etype_aux,
                 coords_aux=coords_aux, ien_aux=ien_aux)


def read(path: str) -> Model:
    with open(path) as f:
        return parse(f.read())


def _rows(vals, fmt, per_line=8):
    vals = list(vals)
    return "\n".join(", ".join(fmt(v) for v in vals[k:k + per_line])
                     for k in range(0, len(vals), per_line))


def dumps(m: Model) -> str:
    """Write a Model in the reference input format (round-trips through parse)."""
    r = repr
    out = [f"formulation={m.formulation};"] if m.formulation != 1 else []
    out += [f"numstep={m.numstep};", f"dt={r(float(m.dt))};",
           f"interpolation={m.interpolation};", f"nq={m.nq};", "",
           f"E={r(float(m.E))};", f"nu={r(float(m.nu))};", f"density={r(float(m.rho))};", "",
           f"sd={m.sd};", f"nnd={m.nnd};", f"EType={m.etype};", f"nel={m.nel};", "",
           f"if_ext={m.if_ext};", "", "nodes="]
    out += [f"{r(float(x))}, {r(float(y))}, {r(float(z))}" for x, y, z in m.coords]
    out += ["", "IEN="]
    out += [", ".join(str(int(v) + 1) for v in row) for row in m.ien]
    out += ["", f"UBC_num={len(m.ubc_dofs)};"]
    if len(m.ubc_dofs):
        out += ["UBC_dof=", _rows(m.ubc_dofs, lambda v: str(int(v) + 1)),
                "UBC_values=", _rows(m.ubc_vals, lambda v: r(float(v)))]
    out += ["", f"FBC_num={len(m.fbc_dofs)};"]
    if len(m.fbc_dofs):
        out += ["FBC_dof=", _rows(m.fbc_dofs, lambda v: str(int(v) + 1)),
                "FBC_values=", _rows(m.fbc_vals, lambda v: r(float(v)))]
    if len(m.interface):
        out += ["", f"num_interface={len(m.interface)};", "interface=",
                _rows(m.interface, lambda v: str(int(v) + 1))]
    return "\n".join(out) + "\n"


def write(m: Model, path: str) -> None:
    with open(path, "w") as f:
        f.write(dumps(m))


def load_history_side_file(path: str, nsteps: int) -> Optional[np.ndarray]:
    """Optional per-step load amplitude, one value per line (step 0..nsteps-1).

    The reference hard-wires a Heaviside amplitude (SolverT.cpp:379-394) and
    rejects unknown keywords, so a load history lives beside the input file."""
    vals = [c_atof(t) for line in open(path) for t in _tokens(line)]
    if len(vals) < nsteps:
        raise InputError(f"load history has {len(vals)} values, {nsteps} needed")
    return np.array(vals[:nsteps], float)
