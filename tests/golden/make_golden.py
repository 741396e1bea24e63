"""Generate the golden fixtures that pin the oracle to the TD-BEM reference.

Run here (where the reference sources are):  python tests/golden/make_golden.py

It builds the reference's own sources, unmodified, against the single-rank
dense PETSc/MPI stand-in (oracle/Makefile.ref -> oracle/_ref/ref_driver), runs
the reference's main-loop sequence on each case and stores, per case, an .npz
holding: the input text it ran, alpha, the level count, seeded random
projections of every G/H level (G_k @ w and w @ G_k; the full levels for the
tiny cases) and the u/t histories (every dof for small meshes, a fixed subset
of dofs otherwise).  Tests rebuild the model from the stored text, so they
need neither the reference nor this script at run time.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "td-bem_gb300"))
from tdbem import inputfile, meshes  # noqa: E402

# the reference checkout: $TDBEM_REFERENCE, else a checkout beside this repository
REF_ROOT = os.environ.get("TDBEM_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))
OUT = os.path.join(ROOT, "tests", "golden")
SEED = 20151022


def projection_vector(D: int) -> np.ndarray:
    return np.random.default_rng(SEED).standard_normal(D)


def build_reference() -> str:
    subprocess.run(["make", "-s", "-f", "oracle/Makefile.ref", f"REF_SRC={REF_ROOT}/src", "-j8"],
                   cwd=ROOT, check=True)
    return os.path.join(ROOT, "oracle", "_ref", "ref_driver")


def run_case(driver, name, text, a1=0.0, a2=0.0, full_levels=False, dof_stride=1):
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "input.txt")
        with open(path, "w") as f:
            f.write(text)
        prefix = os.path.join(tmp, "out")
        subprocess.run([driver, path, repr(a1), repr(a2), prefix], cwd=tmp, check=True,
                       stdout=subprocess.DEVNULL)
        D, M, ns = map(int, open(prefix + ".meta").read().split())
        G = np.fromfile(prefix + ".G").reshape(M + 1, D, D)
        H = np.fromfile(prefix + ".H").reshape(M + 1, D, D)
        u = np.fromfile(prefix + ".u").reshape(ns + 1, D)
        t = np.fromfile(prefix + ".t").reshape(ns + 1, D)
    w = projection_vector(D)
    dofs = np.arange(0, D, dof_stride, dtype=np.int32)
    rec = dict(input_text=np.array(text), a1=a1, a2=a2, D=D, M=M, numstep=ns, seed=SEED,
               G_w=G @ w, H_w=H @ w, w_G=np.einsum("d,kde->ke", w, G),
               w_H=np.einsum("d,kde->ke", w, H), G_absmax=np.abs(G).max(axis=(1, 2)),
               H_absmax=np.abs(H).max(axis=(1, 2)), dofs=dofs, u=u[:, dofs], t=t[:, dofs])
    if full_levels:
        rec.update(G=G, H=H)
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **rec)
    print(f"{name}: D={D} M={M} steps={ns}")


def run_rows_case(driver, name, text, blocks, steps):
    """G_H_Driver row blocks of a mesh too large for a full level dump: for each
    (node block, step) the reference's four row blocks (G_1, G_2, H_1, H_2) projected
    on the seeded vector (rows @ w) plus each block's max-norm."""
    m = inputfile.parse(text)
    D = 3 * m.nnd
    w = projection_vector(D)
    proj, amax = [], []
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "input.txt")
        with open(path, "w") as f:
            f.write(text)
        prefix = os.path.join(tmp, "out")
        for lo, hi in blocks:
            for st in steps:
                subprocess.run([driver, path, "--rows", str(lo), str(hi), str(st), prefix],
                               cwd=tmp, check=True, stdout=subprocess.DEVNULL)
                r = np.fromfile(prefix + ".rows").reshape(4, 3 * (hi - lo + 1), D)
                proj.append(r @ w)
                amax.append(np.abs(r).max(axis=(1, 2)))
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), input_text=np.array(text),
                        seed=SEED, blocks=np.array(blocks, np.int32),
                        steps=np.array(steps, np.int32), rows_w=np.array(proj),
                        rows_absmax=np.array(amax))
    print(f"{name}: D={D} blocks={blocks} steps={steps}")


def run_mrt_case(name, text1, text2, max_step):
    """Two-region case through the reference's SolverMRT (oracle/ref_mrt_driver.cpp)."""
    driver = os.path.join(ROOT, "oracle", "_ref", "ref_mrt_driver")
    with tempfile.TemporaryDirectory() as tmp:
        paths = [os.path.join(tmp, f"region{r}.txt") for r in (1, 2)]
        for p, t in zip(paths, (text1, text2)):
            with open(p, "w") as f:
                f.write(t)
        prefix = os.path.join(tmp, "out")
        subprocess.run([driver, *paths, str(max_step), prefix], cwd=tmp, check=True,
                       stdout=subprocess.DEVNULL)
        N, NG, D1, D2, L, ns = map(int, open(prefix + ".meta").read().split())
        G = np.fromfile(prefix + ".G").reshape(L + 1, N, NG)
        H = np.fromfile(prefix + ".H").reshape(L + 1, N, N)
        x = np.fromfile(prefix + ".x").reshape(ns + 1, N)
        u1 = np.fromfile(prefix + ".u1").reshape(ns + 1, D1)
        u2 = np.fromfile(prefix + ".u2").reshape(ns + 1, D2)
    rng = np.random.default_rng(SEED)
    wg, wh, wr = rng.standard_normal(NG), rng.standard_normal(N), rng.standard_normal(N)
    rec = dict(input_text_1=np.array(text1), input_text_2=np.array(text2), max_step=L,
               numstep=ns, N=N, NG=NG, seed=SEED, G_w=G @ wg, H_w=H @ wh,
               w_G=np.einsum("d,kde->ke", wr, G), w_H=np.einsum("d,kde->ke", wr, H),
               x=x, u1=u1, u2=u2)
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **rec)
    print(f"{name}: N={N} NG={NG} L={L} steps={ns}")


def main():
    """All cases, or only those named on the command line."""
    only = set(sys.argv[1:])
    driver = build_reference()
    geo = os.path.join(REF_ROOT, "geometry")
    if only:
        global run_case
        full = run_case

        def run_case(drv, name, *a, **k):  # noqa: F811
            if name in only:
                full(drv, name, *a, **k)
    bar1 = open(os.path.join(geo, "Bar_1.txt")).read()
    run_case(driver, "ref_bar1", bar1, full_levels=True)
    run_case(driver, "ref_bar1_alpha", bar1, a1=0.25, a2=0.25)
    run_case(driver, "ref_halfspace_plane_1e",
             open(os.path.join(geo, "HalfSpacePlane_1E.txt")).read(), full_levels=True)
    # The 1x1x4 bar at 2 quads per unit length, 200 steps (the CPU-runnable workload).
    bar = meshes.bar(1, 1, 4, per_unit=2, numstep=200)
    run_case(driver, "bar_1x1x4_q2", inputfile.dumps(bar))
    bar.numstep = 60
    run_case(driver, "bar_1x1x4_q2_alpha", inputfile.dumps(bar), a1=0.25, a2=0.1)
    # A coarse cubed-sphere cavity (6x4x4 quads), if_ext = 1, uniform pressure.
    sph = meshes.cubed_sphere(4, numstep=80)
    run_case(driver, "sphere_6x4x4", inputfile.dumps(sph))
    # The reference's own spherical cavity mesh, first 40 steps, every 4th dof.
    cav = open(os.path.join(geo, "SphericalCavity_1.txt")).read().replace(
        "numstep=200;", "numstep=40;")
    run_case(driver, "ref_spherical_cavity_1_40", cav, dof_stride=4)
    # The reference's 8-node (Q8) bar: serendipity shapes, singular sub-elements.
    bar2 = open(os.path.join(geo, "Bar_2.txt")).read()
    run_case(driver, "ref_bar2", bar2)
    run_case(driver, "ref_bar2_alpha", bar2, a1=0.25, a2=0.1)
    # Row blocks (start, middle, end of the node list) of the benchmark's 6x16x16
    # cubed-sphere cavity (D = 4614), too large for a full level dump.
    sph16 = meshes.cubed_sphere(16)
    nnd = sph16.nnd
    rows_blocks = [(0, 3), (nnd // 2, nnd // 2 + 3), (nnd - 4, nnd - 1)]
    if not only or "rows_sphere_6x16x16" in only:
        run_rows_case(driver, "rows_sphere_6x16x16", inputfile.dumps(sph16), rows_blocks,
                      [1, 2, 30, 60])
    # Two-region solver (SolverMRT): the reference's layer pair, and a bar split into
    # two materials with the history truncated (max_step 10 < MaxStep of region 1) or
    # longer than both regions' MaxStep.
    if not only or any(n.startswith("mrt_") for n in only):
        def mrt(name, *a):
            if not only or name in only:
                run_mrt_case(name, *a)

        lay = [open(os.path.join(geo, f)).read() for f in ("Layer_B_test0.txt",
                                                         "Layer_U_test0.txt")]
        mrt("mrt_layer_test0", lay[0], lay[1], 10)
        m1, m2 = meshes.two_region_bar(beta=0.6, numstep=20)
        mrt("mrt_bar_2x2", inputfile.dumps(m1), inputfile.dumps(m2), 10)
        m1, m2 = meshes.two_region_bar(beta=1.0, numstep=16)
        mrt("mrt_bar_2x2_long", inputfile.dumps(m1), inputfile.dumps(m2), 24)


if __name__ == "__main__":
    main()
