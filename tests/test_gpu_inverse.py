"""The H^0 inverse (csrc/inverse.cu) on its own and inside the mixed march.

KSPSolve (SolverStepLinearT.cpp:503-504) is replaced by an explicit inverse of the
column-exchanged LHS: blocked Gauss-Jordan with partial pivoting, FP64 for the
plain form and FP32 for the mixed form.  The FP32 inverse first searches each
panel's pivots in its diagonal block only; a zero pivot there, or a probe
residual max |A (X v) - v| / max |v| above 1e-5, makes it start again with the
full partial-pivoting search.  Checked here:

* FP64 against numpy's inverse (1e-11 relative);
* FP32 on a diagonally dominant matrix: no fallback, residual <= 1e-5;
* FP32 on matrices whose diagonal blocks are zero or tiny (the block search
  cannot pivot there): the fallback runs and the residual is <= 1e-5;
* the FP32 inverses the mixed march makes for the sphere and for a bar with
  prescribed displacements (columns of G exchanged into the LHS): residual
  <= 1e-5, with no fallback on the sphere.
All trailing updates are the library's own kernels (no cuBLAS)."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tdlib():
    import build as b
    b.build()
    from tdbem import lib
    lib.load()
    return lib


def residual(A, X):
    return np.abs(A @ X - np.eye(A.shape[0])).max()


def test_fp64_inverse_matches_numpy(tdlib):
    rng = np.random.default_rng(1)
    n = 301
    A = rng.standard_normal((n, n)) + n ** 0.5 * np.eye(n)
    X, probe, full = tdlib.invert(A, tdlib.FP64)
    ref = np.linalg.inv(A)
    assert np.abs(X - ref).max() / np.abs(ref).max() <= 1e-11
    assert full == 1


def test_fp32_inverse_dominant_no_fallback(tdlib):
    rng = np.random.default_rng(2)
    n = 517
    A = rng.standard_normal((n, n)) + 4 * n ** 0.5 * np.eye(n)
    X, probe, full = tdlib.invert(A, tdlib.MIXED)
    assert full == 0
    assert probe <= 1e-5
    assert residual(A, X) <= 1e-5


@pytest.mark.parametrize("scale", [0.0, 1e-7], ids=["zero_blocks", "tiny_blocks"])
def test_fp32_inverse_falls_back_to_full_search(tdlib, scale):
    """[[s R1, B], [C, s R2]] with dominant B, C: the diagonal blocks hold no usable
    pivot, the full search finds them in the other half of each column."""
    rng = np.random.default_rng(3)
    h = 192
    n = 2 * h
    B = rng.standard_normal((h, h)) + 4 * h ** 0.5 * np.eye(h)
    C = rng.standard_normal((h, h)) + 4 * h ** 0.5 * np.eye(h)
    A = np.block([[scale * rng.standard_normal((h, h)), B],
                  [C, scale * rng.standard_normal((h, h))]])
    X, probe, full = tdlib.invert(A, tdlib.MIXED)
    assert full == 1
    assert probe <= 1e-5
    assert residual(A, X) <= 1e-5


def test_singular_matrix_is_reported(tdlib):
    A = np.ones((70, 70))
    with pytest.raises(tdlib.TdbemError) as e:
        tdlib.invert(A, tdlib.FP64)
    assert e.value.code == -4


@pytest.mark.parametrize("case", ["sphere", "bar_ubc"])
def test_march_inverses_pass_the_probe(tdlib, case):
    from tdbem import meshes
    if case == "sphere":
        m = meshes.cubed_sphere(8, numstep=20)
    else:
        _, m = load_golden("bar_1x1x4_q2_alpha")
    with tdlib.Context(m) as ctx:
        ctx.set_alpha(0.25, 0.1)
        ctx.assemble(precision=tdlib.MIXED)
        ctx.march(20)
        probe, full, k2 = ctx.inverse_report()
    print(f"{case}: probe {probe}, full search {full}, step-2 Richardson sweeps {k2}")
    assert max(probe) <= 1e-5
    # alpha_1 = 0.25: the step-2 LHS differs from the later one and is solved with
    # Richardson sweeps (contraction ~0.35 on the sphere, ~0.6 on the bar)
    assert 0 < k2 <= 50
    if case == "sphere":
        assert full == [0, 0]


def test_step2_richardson_matches_fp64(tdlib):
    """The mixed march with the step-2 solve by Richardson sweeps stays within 1e-4
    (relative L2) of the plain FP64 march, and its first solved step within 1e-5."""
    from tdbem import meshes
    m = meshes.cubed_sphere(8, numstep=60)
    out = {}
    for prec in (tdlib.FP64, tdlib.MIXED):
        with tdlib.Context(m) as ctx:
            ctx.set_alpha(0.25, 0.1)
            ctx.set_march_engine(tdlib.ENGINE_FP32)
            ctx.assemble(precision=prec)
            out[prec] = ctx.march()
            if prec == tdlib.MIXED:
                assert ctx.inverse_report()[2] > 0
    u64, u32 = out[tdlib.FP64][0], out[tdlib.MIXED][0]
    assert np.linalg.norm(u32 - u64) / np.linalg.norm(u64) <= 1e-4
    assert np.abs(u32[1] - u64[1]).max() / np.abs(u64[1]).max() <= 1e-5
