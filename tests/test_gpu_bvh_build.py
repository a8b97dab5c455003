"""The GPU binned-SAH builder (bvh_gpu.cu) against the host one
(bvh_build.cpp): the serialised bvh.cpp buffer, and with it every layout
built from the tree, is the same bit for bit -- on the procedural scenes,
for several leaf sizes, and on degenerate input (all centroids equal, so
every split falls back to splitting by index; a scene smaller than one
chunk).  Build times are printed."""
import time

import numpy as np
import pytest

from artemis_gb300 import kgr

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def scene_pair(positions, indices, materials_raw, max_leaf, **kw):
    gpu = kgr.Scene(positions, indices, materials_raw, builder=kgr.BUILDER_SAH, max_leaf=max_leaf, **kw)
    host = kgr.Scene(positions, indices, materials_raw, builder=kgr.BUILDER_SAH_HOST, max_leaf=max_leaf, **kw)
    return gpu, host


@pytest.mark.parametrize("name", ["box4k", "terrain_s", "terrain"])
def test_gpu_builder_equals_host_builder(name):
    g = kgr.Generated(name, 1)
    gpu, host = scene_pair(g.positions, g.indices, g.materials_raw, 4, normals=g.normals,
                           material_indices=g.material_indices)
    a, b = gpu.bvh(), host.bvh()
    assert a.shape == b.shape
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    ia, ib = gpu.info(), host.info()
    assert (ia.fast_node_count, ia.wide_node_count, ia.wide_max_stack) == \
        (ib.fast_node_count, ib.wide_node_count, ib.wide_max_stack)
    # the host entry point (kgr_bvh_build_host) gives the same buffer
    assert np.array_equal(kgr.bvh_build_host(g.positions, g.indices).view(np.uint32), a.view(np.uint32))
    print(f"{name}: {len(g.indices)} triangles, build {ia.build_ms:.1f} ms on the GPU, {ib.build_ms:.1f} ms on the host")


@pytest.mark.parametrize("max_leaf", [1, 2, 8])
def test_leaf_sizes(max_leaf):
    g = kgr.Generated("terrain_s", 2)
    gpu, host = scene_pair(g.positions, g.indices, g.materials_raw, max_leaf, normals=g.normals,
                           material_indices=g.material_indices)
    assert np.array_equal(gpu.bvh().view(np.uint32), host.bvh().view(np.uint32))


@pytest.mark.parametrize("count", [3, 100, 1000, 5000])
def test_degenerate_identical_triangles(count):
    g = kgr.Generated("box4k", 1)
    tri = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]], np.float32)
    positions = np.tile(tri, (count, 1))
    indices = np.arange(3 * count, dtype=np.uint32).reshape(count, 3)
    gpu, host = scene_pair(positions, indices, g.materials_raw, 4,
                           material_indices=np.zeros(count, np.uint32))
    assert np.array_equal(gpu.bvh().view(np.uint32), host.bvh().view(np.uint32))
