"""The element interface (TDElementT / TDElementStepLinearT) against the oracle.

tdbem_element_gh evaluates FormGH_Regular / FormGH_Singular(node) followed by
GetGHLinear (TDElementStepLinearT.cpp:28-626) for a batch of independent
(collocation point, element) pairs in one launch; the C++ class TDElementGpuT
queues the pairs of the reference's per-element call sequence and evaluates them
that way.  Each pair's blocks GE_1, GE_2, HE_1, HE_2 (3 x 3 ennd) and C_1, C_2
(3 x 3) are compared with the oracle's element restatement (orc_element_gh, in
its exact-zero mode) at 1e-10 relative to the block's max-norm: regular 4-node
elements near and far from the point, each singular corner of a 4-node element,
8-node elements regular and singular at a corner and at a midside node, at the
first step (C term) and later times."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden, rel_max

pytestmark = pytest.mark.gpu

TOL = 1e-10
NAMES = ["GE_1", "GE_2", "HE_1", "HE_2", "C_1", "C_2"]


@pytest.fixture(scope="module")
def tdlib():
    import build as b
    b.build()
    from tdbem import lib
    lib.load()
    return lib


def mesh_pairs(m, rng, count, steps):
    """(colloc, coords, t, singular) of pairs drawn from a mesh: every singular
    (node, element) incidence of a few nodes, plus random regular pairs, each at a
    step drawn from `steps`; the singular node is the element's last node within
    r^2 < 1e-9 of the point, as G_H_Driver picks it (ElastoDynamicsT.cpp:166-175)."""
    ennd = m.ien.shape[1]
    xc, en, tt, sg = [], [], [], []
    nodes = rng.choice(m.nnd, size=min(count, m.nnd), replace=False)
    for c in nodes:
        for e in np.flatnonzero((m.ien == c).any(axis=1)):
            pos = np.flatnonzero(m.ien[e] == c)
            xc.append(m.coords[c])
            en.append(m.coords[m.ien[e]])
            tt.append(m.dt * rng.choice(steps))
            sg.append(int(pos[-1]))
        for e in rng.choice(m.nel, size=3, replace=False):
            if (m.ien[e] == c).any():
                continue
            xc.append(m.coords[c])
            en.append(m.coords[m.ien[e]])
            tt.append(m.dt * rng.choice(steps))
            sg.append(-1)
    return (np.array(xc), np.array(en).reshape(-1, ennd, 3), np.array(tt),
            np.array(sg, np.int32))


def oracle_blocks(oracle_mod, m, xc, en, tt, sg):
    with oracle_mod._Clean(True):
        return [oracle_mod.element_gh(m.etype, m.nq, m.E, m.nu, m.rho, en[i], xc[i], tt[i],
                                      m.dt, int(sg[i])) for i in range(len(sg))]


def check(got, ref, what):
    """got: the six arrays of n pairs; ref: per pair, the oracle's six blocks."""
    for i, r in enumerate(ref):
        for k in range(6):
            g = got[k][i].reshape(r[k].shape)
            e = rel_max(g, r[k])
            assert e <= TOL, f"{what} pair {i} {NAMES[k]}: {e:.3e}"


@pytest.mark.parametrize("name", ["ref_spherical_cavity_1_40", "ref_bar1", "ref_bar2"])
def test_element_batch_matches_oracle(tdlib, oracle_mod, name):
    z, m = load_golden(name)
    rng = np.random.default_rng(5)
    xc, en, tt, sg = mesh_pairs(m, rng, 12, [1, 1, 2, 3, 7])
    assert (sg >= 0).any() and (sg < 0).any() and (tt == m.dt).any()
    if m.etype == 2:
        assert (sg >= 4).any() and ((sg >= 0) & (sg < 4)).any()  # midside and corner
    got = tdlib.element_gh(m.etype, m.nq, m.E, m.nu, m.rho, m.dt, xc, en, tt, sg)
    ref = oracle_blocks(oracle_mod, m, xc, en, tt, sg)
    check(got, ref, name)
    # C term: the Kelvin part at t == t_1 only
    assert np.abs(got[4][tt != m.dt]).max() == 0
    assert np.abs(got[4][tt == m.dt]).max() > 0


def test_element_every_singular_corner(tdlib, oracle_mod):
    """A single quad with the point at each of its corners in turn (the four Duffy
    corner maps), and a point just off the element (regular, near-singular)."""
    z, m = load_golden("ref_bar1")
    quad = m.coords[m.ien[3]]
    xc = np.vstack([quad, quad.mean(0) + [0.0, 0.0, 0.05]])
    en = np.repeat(quad[None], 5, axis=0)
    sg = np.array([0, 1, 2, 3, -1], np.int32)
    for step in (1, 2, 5):
        tt = np.full(5, step * m.dt)
        got = tdlib.element_gh(1, m.nq, m.E, m.nu, m.rho, m.dt, xc, en, tt, sg)
        check(got, oracle_blocks(oracle_mod, m, xc, en, tt, sg), f"step {step}")


def test_element_rejects_bad_input(tdlib):
    z, m = load_golden("ref_bar1")
    quad = m.coords[m.ien[0]][None]
    with pytest.raises(tdlib.TdbemError):
        tdlib.element_gh(1, m.nq, m.E, m.nu, m.rho, m.dt, m.coords[:1], quad, [m.dt], [4])
    L = tdlib.load()
    one = np.zeros(64)
    sg = np.full(1, -1, np.int32)
    d = one.ctypes.data_as(tdlib._dp)
    assert L.tdbem_element_gh(3, m.nq, m.E, m.nu, m.rho, m.dt, 1, d, d, d,
                              sg.ctypes.data_as(tdlib._ip), d, d, d, d, d, d) == -1
    with pytest.raises(tdlib.TdbemError):
        tdlib.element_gh(1, 7, m.E, m.nu, m.rho, m.dt, m.coords[:1], quad, [m.dt], [-1])


@pytest.fixture(scope="module")
def driver(tdlib, tmp_path_factory):
    """tests/cpp/element_driver.cpp built against include/ and the library."""
    out = str(tmp_path_factory.mktemp("cpp") / "element_driver")
    libdir = os.path.join(ROOT, "td-bem_gb300", "_build")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "element_driver.cpp"), "-L" + libdir,
                    "-ltdbem", "-Wl,-rpath," + libdir, "-o", out], check=True)
    return out


@pytest.mark.parametrize("mode", [0, 1], ids=["read_each", "batched"])
@pytest.mark.parametrize("name", ["ref_bar1", "ref_bar2"])
def test_tdelement_gpu_class_matches_oracle(driver, oracle_mod, name, mode):
    """TDElementGpuT through the reference's call sequence: read after every
    FormGH (one launch per element) or form every element first (one launch)."""
    z, m = load_golden(name)
    rng = np.random.default_rng(9)
    xc, en, tt, sg = mesh_pairs(m, rng, 6, [1, 2, 4])
    n = len(sg)
    lines = [f"{m.etype} {m.nq} {float(m.E)!r} {float(m.nu)!r} {float(m.rho)!r} {mode} {n}"]
    for i in range(n):
        vals = [repr(float(tt[i])), repr(float(m.dt)), str(int(sg[i]))]
        vals += [repr(float(v)) for v in xc[i]] + [repr(float(v)) for v in en[i].ravel()]
        lines.append(" ".join(vals))
    r = subprocess.run([driver], input="\n".join(lines) + "\n", capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rows = [np.array(list(map(float, ln.split()))) for ln in r.stdout.strip().split("\n")]
    assert len(rows) == 6 * n
    ennd = 4 if m.etype == 1 else 8
    got = [np.stack([rows[6 * i + k] for i in range(n)]) for k in range(6)]
    got = [g.reshape(n, 3, -1) for g in got]
    assert got[0].shape[2] == 3 * ennd
    check(got, oracle_blocks(oracle_mod, m, xc, en, tt, sg), f"{name} mode {mode}")
