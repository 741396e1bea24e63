"""The C++ drop-in layer and the level checkpoint on the GPU.

tdbem_run follows main.cpp with the host classes (G_H_Driver -> GetGHLinear ->
UpdateGHLinear -> Solve per step) or, with --fast, assembles every level and
marches in one call; both must give the clean oracle's histories to 1e-10
(the parity bar of the plain FP64 form), and displacement.txt must carry them
as RecordResult prints them.  A level checkpoint must restore levels that
march to bitwise the same histories; the stepwise C ABI must equal the
whole-run march bitwise."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden, rel_max

pytestmark = pytest.mark.gpu

TOL = 1e-10
RUN = os.path.join(ROOT, "td-bem_gb300", "_build", "tdbem_run")
CASES = ["ref_bar1_alpha", "bar_1x1x4_q2_alpha", "ref_halfspace_plane_1e", "ref_bar2_alpha"]


@pytest.fixture(scope="module")
def tdlib():
    import build as b
    b.build()
    from tdbem import lib
    lib.load()
    return lib


@pytest.fixture(scope="module")
def oracle_cache(oracle_mod):
    cache = {}

    def get(name):
        if name not in cache:
            z, m = load_golden(name)
            o = oracle_mod.Oracle(m, clean=True)
            G, H = o.assemble_levels()
            u, t = o.march(G, H, float(z["a1"]), float(z["a2"]))
            cache[name] = (z, m, u, t)
        return cache[name]

    return get


def read_dump(path):
    with open(path, "rb") as f:
        n, D = np.frombuffer(f.read(8), np.int32)
        a = np.frombuffer(f.read(), np.float64)
    return a[:(n + 1) * D].reshape(n + 1, D), a[(n + 1) * D:].reshape(n + 1, D)


def check_steps(u, uo, what):
    for s in range(uo.shape[0]):
        if np.abs(uo[s]).max() == 0:
            assert np.abs(u[s]).max() == 0, f"{what} step {s}"
        else:
            assert rel_max(u[s], uo[s]) <= TOL, f"{what} step {s}: {rel_max(u[s], uo[s]):.3e}"


@pytest.mark.parametrize("mode", ["stepwise", "fast"])
@pytest.mark.parametrize("name", CASES)
def test_tdbem_run_matches_oracle(tdlib, oracle_cache, name, mode, tmp_path):
    z, m, uo, to = oracle_cache(name)
    (tmp_path / "input.txt").write_text(str(z["input_text"]))
    (tmp_path / "alpha.txt").write_text(f"{float(z['a1'])!r} {float(z['a2'])!r}\n")
    cmd = [RUN, "input.txt", "--dump", "hist.bin"] + (["--fast"] if mode == "fast" else [])
    r = subprocess.run(cmd, cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    u, t = read_dump(tmp_path / "hist.bin")
    assert u.shape == uo.shape
    check_steps(u, uo, "u")
    check_steps(t, to, "t")
    rows = np.loadtxt(tmp_path / "displacement.txt", comments="%")
    n = int(z["numstep"])
    assert rows.shape == (n, 4)
    assert np.allclose(rows[:, 0], m.dt * np.arange(n), rtol=1e-5, atol=1e-12)
    assert np.allclose(rows[:, 2], u[:n, 2], rtol=1e-5, atol=1e-12 * np.abs(u).max())
    assert np.allclose(rows[:, 3], t[:n, 2], rtol=1e-5, atol=1e-12 * np.abs(t).max())


def test_tdbem_run_write_gh(tdlib, oracle_cache, tmp_path):
    """--write-gh writes main.cpp's step matrices in SolverT::WriteGH's format."""
    z, m, _, _ = oracle_cache("ref_bar1_alpha")
    (tmp_path / "input.txt").write_text(str(z["input_text"]))
    r = subprocess.run([RUN, "input.txt", "--alpha", "0", "0", "--write-gh", "gh_"],
                       cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    with tdlib.Context(m) as ctx:
        GI, GJ, HI, HJ = ctx.gh_driver(2)
    # main.cpp: G1_step <- G_1 (the J part), G2_step <- G_0 (the I part), step - 1
    for fname, ref in (("gh_G1_step1.txt", GJ), ("gh_G2_step1.txt", GI),
                       ("gh_H1_step1.txt", HJ), ("gh_H2_step1.txt", HI)):
        a = np.loadtxt(tmp_path / fname)
        assert a.shape == ref.shape
        assert np.allclose(a, ref, rtol=1e-5, atol=0)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_level_checkpoint_roundtrip(tdlib, prec, tmp_path):
    _, m = load_golden("bar_1x1x4_q2_alpha")
    p = tdlib.FP64 if prec == "fp64" else tdlib.MIXED
    path = str(tmp_path / "levels.bin")
    with tdlib.Context(m) as ctx:
        ctx.set_alpha(0.25, 0.1)
        ctx.assemble(precision=p)
        u, t = ctx.march()
        lv = ctx.level(3, 1)
        ctx.export_levels(path)
    with tdlib.Context(m) as c2:
        c2.set_alpha(0.25, 0.1)
        c2.import_levels(path)
        u2, t2 = c2.march()
        assert np.array_equal(c2.level(3, 1), lv)
    assert np.array_equal(u, u2) and np.array_equal(t, t2)


def test_checkpoint_of_another_mesh_is_refused(tdlib, tmp_path):
    from tdbem import meshes
    _, m = load_golden("bar_1x1x4_q2_alpha")
    path = str(tmp_path / "levels.bin")
    with tdlib.Context(m) as ctx:
        ctx.assemble(precision=tdlib.FP64, nsteps=3)
        ctx.export_levels(path)
    with tdlib.Context(meshes.cubed_sphere(4, numstep=10)) as c2:
        with pytest.raises(tdlib.TdbemError) as ei:
            c2.import_levels(path)
        assert ei.value.code == -1 and "checkpoint is for" in str(ei.value)
    (tmp_path / "junk.bin").write_bytes(b"not a checkpoint at all" * 4)
    with tdlib.Context(m) as c3:
        with pytest.raises(tdlib.TdbemError):
            c3.import_levels(str(tmp_path / "junk.bin"))


def test_stepwise_abi_equals_whole_run(tdlib):
    """tdbem_update_gh_linear from tdbem_gh_driver blocks + tdbem_march_step give
    the histories of tdbem_assemble_levels + tdbem_march to the 1e-10 parity bar
    (the level sums I + J are formed in another order: about 1e-12 here), and
    march_step on assembled levels equals tdbem_march bitwise."""
    _, m = load_golden("bar_1x1x4_q2_alpha")
    n = m.numstep
    with tdlib.Context(m) as ctx:
        ctx.set_alpha(0.25, 0.1)
        ctx.assemble(precision=tdlib.FP64)
        u, t = ctx.march()
        ctx.march_begin(n)
        for s in range(1, n + 1):
            us, ts = ctx.march_step(s)
            assert np.array_equal(us, u[s - 1]) and np.array_equal(ts, t[s - 1])
    with tdlib.Context(m) as c2:
        c2.set_alpha(0.25, 0.1)
        c2.march_begin(n)
        for s in range(1, n + 1):
            if s <= c2.M:
                c2.update_gh_linear(s, *c2.gh_driver(s))
            us, _ = c2.march_step(s)
            assert rel_max(us, u[s - 1]) <= TOL or np.abs(u[s - 1]).max() == 0


@pytest.mark.parametrize("mode", ["stepwise", "fast"])
@pytest.mark.parametrize("name", ["mrt_layer_test0", "mrt_bar_2x2_long"])
def test_tdbem_run_two_regions_matches_oracle(tdlib, oracle_mod, name, mode, tmp_path):
    """tdbem_run --region2: SolverMRGpuT in main()'s per-step pattern for two
    regions (ElastoDynamicsGpuT on each region, UpdateGHLinear with both
    regions' blocks, Solve), or the whole run (--fast); the combined unknowns
    against the oracle's SolverMRT at 1e-10 per step (displacements and
    interface tractions apart), RecordResult's lines from region 2's history."""
    from conftest import load_mrt_golden
    z, m1, m2 = load_mrt_golden(name)
    L = int(z["max_step"])
    mr = oracle_mod.MultiRegion(m1, m2, L, clean=True)
    GG, HH = mr.assemble_levels()
    Xo, _, u2o = mr.march(GG, HH)
    (tmp_path / "r1.txt").write_text(str(z["input_text_1"]))
    (tmp_path / "r2.txt").write_text(str(z["input_text_2"]))
    cmd = [RUN, "r1.txt", "--region2", "r2.txt", "--max-step", str(L), "--dump", "x.bin"]
    r = subprocess.run(cmd + (["--fast"] if mode == "fast" else []), cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    with open(tmp_path / "x.bin", "rb") as f:
        n, N = np.frombuffer(f.read(8), np.int32)
        X = np.frombuffer(f.read(), np.float64).reshape(n + 1, N)
    assert X.shape == Xo.shape
    k = mr.NI1 + mr.NI2 + mr.NZ
    check_steps(X[:, :k], Xo[:, :k], "x displacements")
    check_steps(X[:, k:], Xo[:, k:], "x interface tractions")
    rows = np.loadtxt(tmp_path / "displacement.txt")
    dof = 137 if mr.D2 > 137 else 2
    assert rows.shape == (n, 2)
    assert np.allclose(rows[:, 0], m1.dt * np.arange(n), rtol=1e-5, atol=1e-15)
    assert np.allclose(rows[:, 1], u2o[:n, dof], rtol=1e-5, atol=1e-12 * np.abs(u2o).max())


def test_device_memory_kept_for_the_next_context(tdlib):
    """Buffers of a destroyed context stay allocated for the next one (devmem.cu): a
    second context of the same mesh takes them (nothing new kept afterwards beyond
    what the first left) and gives bitwise the same solve; releasing frees them."""
    from tdbem import meshes
    m = meshes.cubed_sphere(4, numstep=40)
    tdlib.release_cached_memory()
    assert tdlib.cached_memory() == 0
    outs = []
    kept = []
    for _ in range(2):
        with tdlib.Context(m) as ctx:
            ctx.set_alpha(0.25, 0.0)
            ctx.assemble(precision=tdlib.MIXED)
            outs.append(ctx.march())
            if kept:  # the second context runs on the blocks the first one left
                assert tdlib.cached_memory() < kept[0]
        kept.append(tdlib.cached_memory())
    assert kept[0] > 0 and kept[1] == kept[0]
    assert all(np.array_equal(a, b) for a, b in zip(outs[0], outs[1]))
    assert tdlib.release_cached_memory() == kept[1]
    assert tdlib.cached_memory() == 0
