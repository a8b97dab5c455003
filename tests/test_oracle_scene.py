"""The oracle's own scene inputs (oracle/scene_ref.cpp) against the
product's: the CPU reference arm of the benchmark builds its scene, BVH,
lights and camera from these without loading the product library, so they
must give the same bits.

- procedural scenes: every array equal bit for bit (box scene of the ReSTIR
  DI configuration with its generator seed 0x4B4F4252, the small terrain,
  and the 1.16M-triangle terrain of the path-tracing configuration);
- the SAH builder (leaves <= 4): the oracle's threaded buffer equals the
  product's host builder's bit for bit -- an independent check of the
  product builder, since each is written on its own;
- triangle lights: {a, b - a, c - a, emission} of the emissive triangles in
  order, against a NumPy restatement;
- the camera frame of uvw_frame (include/camera.hpp:45-63) against the
  product's kgr_camera_setup."""
import numpy as np
import pytest

from artemis_gb300 import kgr
from oracle import pyoracle

FIELDS = ("positions", "normals", "indices", "material_indices", "materials_raw", "eye", "target")


def same_bits(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("name,seed", [("box4k", 0x4B4F4252), ("box4k", 1), ("box64", 3), ("terrain_s", 1),
                                       ("terrain", 1)])
def test_generator_matches_product(name, seed):
    a = kgr.Generated(name, seed)
    b = pyoracle.GeneratedScene(name, seed)
    for k in FIELDS:
        assert same_bits(getattr(a, k), getattr(b, k)), k
    assert a.fov == b.fov


@pytest.mark.parametrize("name,seed,leaf", [("box4k", 0x4B4F4252, 4), ("box64", 3, 1), ("box64", 3, 8),
                                            ("terrain_s", 1, 4)])
def test_sah_builder_matches_product(name, seed, leaf):
    g = pyoracle.GeneratedScene(name, seed)
    want = kgr.bvh_build_host(g.positions, g.indices, kgr.BUILDER_SAH, leaf)
    got = g.sah_bvh(leaf)
    assert same_bits(got, want)
    # one leaf record per triangle, each triangle exactly once
    leaf_rows = got[0::3][:, 0] == 1.0
    objects = got[0::3][leaf_rows, 1].view(np.int32)
    assert np.array_equal(np.sort(objects), np.arange(len(g.indices)))


def test_sah_builder_degenerate_inputs():
    # identical triangles (every centroid equal: split by index) and an empty list
    pos = np.tile(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), (17, 1))
    idx = np.arange(len(pos), dtype=np.uint32).reshape(-1, 3)
    want = kgr.bvh_build_host(pos, idx, kgr.BUILDER_SAH, 4)
    n = pyoracle.lib().oracle_build_sah(pyoracle.ptr(pos), pyoracle.ptr(idx), len(idx), 4, None, 0)
    got = np.zeros((n, 4), np.float32)
    pyoracle.lib().oracle_build_sah(pyoracle.ptr(pos), pyoracle.ptr(idx), len(idx), 4, pyoracle.ptr(got), n)
    assert same_bits(got, want)
    assert pyoracle.lib().oracle_build_sah(pyoracle.ptr(pos), pyoracle.ptr(idx), 0, 4, None, 0) == 0


def test_lights_in_triangle_order():
    g = pyoracle.GeneratedScene("box4k", 0x4B4F4252)
    em = g.materials_raw[g.material_indices, 6:9]
    lit = np.nonzero(em.max(axis=1) > 0)[0]
    p = g.positions[g.indices[lit]]
    want = np.concatenate([p[:, 0], p[:, 1] - p[:, 0], p[:, 2] - p[:, 0], em[lit]], axis=1).astype(np.float32)
    got = g.lights()
    assert len(got) == 128
    assert same_bits(got, want)


@pytest.mark.parametrize("aspect", [1.0, 16 / 9, 0.5])
def test_camera_matches_product(aspect):
    g = pyoracle.GeneratedScene("terrain_s", 1)
    want = kgr.camera_dict(kgr.camera(g.eye, g.target, g.fov, aspect))
    got = pyoracle.camera(g.eye, g.target, g.fov, aspect)
    for k in ("center", "ax_u", "ax_v", "ax_w"):
        assert same_bits(np.float32(got[k]), np.float32(want[k])), k
