"""The refit oracle on the CPU.  Refitting a buffer to the positions it was
built from must give the builder's own boxes back: bit for bit for the SAH
builder (whose node boxes are unions with -0 written as +0, as the refit
computes them), and up to the sign of zero for the reference builder
(partition() of source/bvh.cpp, whose unions keep glm::min's choice of
zero).  Then the transform restatement on known answers."""
import numpy as np
import pytest

from artemis_gb300 import kgr
from oracle import refit_ref


def soup(n, seed):
    """Random triangles with coordinates that include exact zeros of both signs."""
    rng = np.random.default_rng(seed)
    p = rng.uniform(-1, 1, (3 * n, 3)).astype(np.float32)
    p[rng.random(p.shape) < 0.05] = np.float32(0.0)
    p[rng.random(p.shape) < 0.05] = np.float32(-0.0)
    return p, np.arange(3 * n, dtype=np.uint32).reshape(n, 3)


@pytest.mark.parametrize("max_leaf", [1, 4])
def test_refit_of_sah_buffer_is_identity(max_leaf):
    g = kgr.Generated("box4k", 3)
    bvh = kgr.bvh_build_host(g.positions, g.indices, kgr.BUILDER_SAH, max_leaf)
    tris = np.concatenate([g.indices, g.material_indices[:, None]], axis=1)
    out = refit_ref.refit_threaded(bvh, g.positions, tris)
    assert np.array_equal(out.view(np.uint32), bvh.view(np.uint32))


def test_refit_of_sah_buffer_with_signed_zeros():
    p, idx = soup(3000, 7)
    bvh = kgr.bvh_build_host(p, idx, kgr.BUILDER_SAH, 4)
    out = refit_ref.refit_threaded(bvh, p, np.concatenate([idx, np.zeros((len(idx), 1), np.uint32)], axis=1))
    assert np.array_equal(out.view(np.uint32), bvh.view(np.uint32))


def test_refit_of_reference_builder_buffer():
    p, idx = soup(2000, 8)
    bvh = kgr.bvh_build_host(p, idx, kgr.BUILDER_KOBRA, 1)
    out = refit_ref.refit_threaded(bvh, p, np.concatenate([idx, np.zeros((len(idx), 1), np.uint32)], axis=1))
    canon = lambda a: (a + np.float32(0.0)).view(np.uint32)
    assert np.array_equal(canon(out), canon(bvh))
    # headers and links untouched
    assert np.array_equal(out[0::3].view(np.uint32), bvh[0::3].view(np.uint32))


def test_transform_points_known_answers():
    p = np.array([[1.0, 2.0, 3.0], [-0.0, 0.5, -4.0]], np.float32)
    T = np.eye(4, dtype=np.float32)
    T[:3, 3] = [10.0, -1.0, 0.25]
    np.testing.assert_array_equal(refit_ref.transform_points(T, p, 1.0), p + T[:3, 3])
    np.testing.assert_array_equal(refit_ref.transform_points(T, p, 0.0), p + np.float32(0.0))
    R = np.array([[0, -1, 0, 0], [1, 0, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]], np.float32)  # 90 deg about z
    np.testing.assert_array_equal(refit_ref.transform_points(R, p, 1.0),
                                  np.array([[-2.0, 1.0, 3.0], [-0.5, 0.0, -4.0]], np.float32))


def test_gather_face_normals_take_the_last_triangle():
    p = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float32)
    idx = np.array([[0, 1, 2], [0, 3, 1]], np.uint32)  # vertex 0 and 1 in both: the second wins
    mats = np.zeros((1, 16), np.float32)
    pos, nrm, tris, lights = refit_ref.gather([dict(positions=p, indices=idx)], mats)
    second = refit_ref.face_normals(p, idx[1:].astype(np.int64))[0]
    first = refit_ref.face_normals(p, idx[:1].astype(np.int64))[0]
    np.testing.assert_array_equal(nrm[0], second)
    np.testing.assert_array_equal(nrm[1], second)
    np.testing.assert_array_equal(nrm[2], first)
    np.testing.assert_array_equal(nrm[3], second)
    assert len(lights) == 0 and tris.shape == (2, 4)
