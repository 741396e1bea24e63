"""Serving on the host: the request stream, the footprint estimate and the
server's refusal without a GPU (no CPU fallback)."""
import numpy as np
import pytest

from tdbem import meshes, serve


@pytest.fixture(scope="module")
def tdlib():
    import build as b
    b.build()
    from tdbem import lib
    lib.load()
    return lib


def test_request_mix_seeded():
    a = serve.request_mix(12, rate_hz=4.0, seed=5)
    b = serve.request_mix(12, rate_hz=4.0, seed=5)
    assert [r["name"] for r in a] == [r["name"] for r in b]
    assert [r["arrival_s"] for r in a] == [r["arrival_s"] for r in b]
    arr = np.array([r["arrival_s"] for r in a])
    assert np.all(np.diff(arr) > 0)
    for r in a:
        assert 300 <= r["dof"] <= 8000
        assert 100 <= r["steps"] <= 400
        assert r["amp"] is None or len(r["amp"]) == r["steps"]
    kinds = {r["name"].split("_")[0] for r in serve.request_mix(40, 4.0, seed=1)}
    assert kinds == {"bar", "sphere", "halfspace"}


def test_footprint_counts_the_level_store(tdlib):
    m = meshes.cubed_sphere(8, numstep=200)
    M = m.max_step()
    D = 3 * m.nnd
    f64 = tdlib.footprint(m, tdlib.FP64)
    f32 = tdlib.footprint(m, tdlib.MIXED)
    levels64 = 2 * (M + 1) * D * D * 8
    assert levels64 < f64 < 1.3 * levels64
    # FP32 levels and, for the tcgen05 march, the merged BF16 hi/lo planes of the levels
    # and of the 31 step-distance matrices (rows of D rounded up to 64)
    ldb = (D + 63) // 64 * 64
    store32 = 2 * (M + 1) * D * D * 4
    planes = (M + 1 + 31) * D * ldb * 4
    assert store32 + planes < f32 < 1.3 * (store32 + planes)
    # more steps: longer histories, same levels
    assert tdlib.footprint(m, tdlib.MIXED, numstep=400) > f32


def test_footprint_of_the_bench_sphere(tdlib):
    """The 1538-node sphere: the largest node distance is searched over 1.2 M pairs on
    several host threads; the level store follows the mesh's max step (60)."""
    m = meshes.cubed_sphere(16, numstep=400)
    M = m.max_step()
    D = 3 * m.nnd
    assert M == 60
    levels64 = 2 * (M + 1) * D * D * 8
    f64 = tdlib.footprint(m, tdlib.FP64)
    assert levels64 < f64 < 1.3 * levels64


def test_halfspace_cavity_mesh():
    m = meshes.halfspace_cavity(n_sphere=4)
    assert m.nnd == 121 + 6 * 16 + 2 and m.nel == 100 + 6 * 16
    assert m.if_ext == 1
    # patch normals point up (+z), cavity normals toward the cavity centre
    p = m.coords[m.ien]
    n = np.cross(p[:, 1] - p[:, 0], p[:, 3] - p[:, 0])
    assert np.all(n[:100, 2] > 0)
    c = p[100:].mean(1) - np.array([0, 0, -3.0])
    assert np.all(np.einsum("ij,ij->i", n[100:], c) < 0)


def test_server_refuses_without_gpu(tdlib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(tdlib.TdbemError):
        tdlib.Server(0, 0, 2)
