"""GPU traversal parity: hit primitive ids, distances and barycentrics of
the device layouts (fast BVH2, wide BVH4, compressed BVH8, threaded) against the oracle's GLSL threaded walk
(shaders/rt/modules/bvh.glsl:52-99) on the same rays -- bit for bit -- and
occlusion flags of the any-hit walk (amadeus_common.cuh:190-212)."""
import numpy as np
import pytest

from artemis_gb300 import kgr
from tests import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def gpu_closest(sc, rays, layout):
    r = torch.from_numpy(rays).cuda()
    h = torch.zeros((len(rays), 4), dtype=torch.float32, device="cuda")
    sc.trace_closest(r.data_ptr(), len(rays), h.data_ptr(), layout)
    torch.cuda.synchronize()
    return h.cpu().numpy()


def gpu_any(sc, rays, layout):
    r = torch.from_numpy(rays).cuda()
    o = torch.zeros(len(rays), dtype=torch.int32, device="cuda")
    sc.trace_any(r.data_ptr(), len(rays), o.data_ptr(), layout)
    torch.cuda.synchronize()
    return o.cpu().numpy().astype(np.uint32)


def assert_hits_equal(gpu, ref):
    assert gpu.shape == ref.shape
    bad = np.nonzero(np.any(gpu.view(np.uint32) != ref.view(np.uint32), axis=1))[0]
    assert len(bad) == 0, f"{len(bad)} of {len(gpu)} rays differ, first {bad[:5]}: {gpu[bad[:3]]} vs {ref[bad[:3]]}"


@pytest.fixture(scope="module")
def box4k():
    return helpers.both("box4k", 1)


@pytest.mark.parametrize("layout", [kgr.LAYOUT_FAST, kgr.LAYOUT_THREADED, kgr.LAYOUT_WIDE, kgr.LAYOUT_CW8])
def test_camera_rays_bit_exact(box4k, layout):
    g, sc, osc = box4k
    cam = kgr.camera(g.eye, g.target, g.fov, 1.0)
    rays = helpers.camera_rays(cam, 256, 256)
    ref, _ = osc.trace_closest(rays)
    got = gpu_closest(sc, rays, layout)
    assert_hits_equal(got, ref["raw"])
    assert (ref["prim"] >= 0).all()


@pytest.mark.parametrize("layout", [kgr.LAYOUT_FAST, kgr.LAYOUT_THREADED, kgr.LAYOUT_WIDE, kgr.LAYOUT_CW8])
def test_random_rays_bit_exact(box4k, layout):
    g, sc, osc = box4k
    rays = helpers.random_rays(g, 50000, 11)
    ref, _ = osc.trace_closest(rays)
    assert_hits_equal(gpu_closest(sc, rays, layout), ref["raw"])


@pytest.mark.parametrize("layout", [kgr.LAYOUT_FAST, kgr.LAYOUT_THREADED, kgr.LAYOUT_WIDE, kgr.LAYOUT_CW8])
def test_any_hit_bit_exact(box4k, layout):
    g, sc, osc = box4k
    rays = helpers.random_rays(g, 50000, 12)
    hits, _ = osc.trace_closest(rays)
    # shadow-style segments ending before, at and after the closest hit
    t = np.where(hits["prim"] >= 0, hits["t"], 3.0).astype(np.float32)
    rays[:, 7] = t * np.random.default_rng(3).choice([0.5, 1.0, 2.0], len(rays)).astype(np.float32)
    ref, _ = osc.trace_any(rays)
    got = gpu_any(sc, rays, layout)
    np.testing.assert_array_equal(got, ref)
    assert 0.2 < ref.mean() < 0.9


def test_reference_builder_buffer_drops_in(box4k):
    """A buffer serialised by the reference builder (partition/serialize,
    one primitive per leaf) is accepted as-is and traced identically."""
    g, _, _ = box4k
    kob = kgr.bvh_build_host(g.positions, g.indices, kgr.BUILDER_KOBRA)
    sc = kgr.Scene.from_generated(g, bvh=kob)
    osc = helpers.oracle_scene(g, kob, sc.lights())
    rays = np.concatenate([helpers.random_rays(g, 20000, 13),
                           helpers.camera_rays(kgr.camera(g.eye, g.target, g.fov, 1.0), 128, 128)])
    ref, _ = osc.trace_closest(rays)
    for layout in (kgr.LAYOUT_FAST, kgr.LAYOUT_THREADED, kgr.LAYOUT_WIDE, kgr.LAYOUT_CW8):
        assert_hits_equal(gpu_closest(sc, rays, layout), ref["raw"])


def test_host_buffer_entry_points(box4k):
    g, sc, osc = box4k
    rays = helpers.random_rays(g, 4096, 14)
    ref, _ = osc.trace_closest(rays)
    assert_hits_equal(sc.trace_closest_host(rays), ref["raw"])
    occ_ref, _ = osc.trace_any(rays)
    np.testing.assert_array_equal(sc.trace_any_host(rays), occ_ref)


def test_edge_cases(box4k):
    """Empty batch, rays with zero direction components, origins on box
    planes, tmax = 0 and NaN directions."""
    g, sc, osc = box4k
    sc.trace_closest_host(np.zeros((0, 8), np.float32))
    rays = np.zeros((8, 8), np.float32)
    rays[:, 4:7] = [[0, 0, -1], [0, 1, 0], [1, 0, 0], [0, 0, 1], [0, -1, 0], [-1, 0, 0], [0, 0, -1], [np.nan, 0, 1]]
    rays[:, 0:3] = [[0, 0, 0], [0.5, 0, 0.5], [-2, 0, 0], [0, 0, 2], [1.5, 1.5, 1.5], [0, -1.9, 0], [0, 0, 0], [0, 0, 0]]
    rays[:, 7] = [np.inf] * 6 + [0.0, np.inf]
    ref, _ = osc.trace_closest(rays)
    for layout in (kgr.LAYOUT_FAST, kgr.LAYOUT_THREADED, kgr.LAYOUT_WIDE, kgr.LAYOUT_CW8):
        assert_hits_equal(sc.trace_closest_host(rays, layout), ref["raw"])
    assert ref["prim"][6] == -1


@pytest.mark.parametrize("name", ["terrain_s"])
def test_terrain_fast_equals_threaded(name):
    """On a 0.25M-triangle scene the fast and wide layouts agree with the
    threaded walk on the GPU, and all with the oracle on a subset."""
    g, sc, osc = helpers.both(name, 1)
    cam = kgr.camera(g.eye, g.target, g.fov, 16 / 9)
    rays = np.concatenate([helpers.camera_rays(cam, 320, 180), helpers.random_rays(g, 40000, 15)])
    fast = gpu_closest(sc, rays, kgr.LAYOUT_FAST)
    thr = gpu_closest(sc, rays, kgr.LAYOUT_THREADED)
    wide = gpu_closest(sc, rays, kgr.LAYOUT_WIDE)
    cw8 = gpu_closest(sc, rays, kgr.LAYOUT_CW8)
    assert_hits_equal(fast, thr)
    assert_hits_equal(wide, thr)
    assert_hits_equal(cw8, thr)
    ref, _ = osc.trace_closest(rays[::7])
    assert_hits_equal(fast[::7], ref["raw"])


@pytest.mark.parametrize("name", ["box4k", "terrain_s", "terrain"])
def test_wide_layout_is_built(name):
    """The wide layout exists for the benchmark scenes and its worst-case
    walk fits the 64-entry traversal stack."""
    g = kgr.Generated(name, 1)
    sc = kgr.Scene.from_generated(g)
    info = sc.info()
    assert info.wide_node_count > 0
    assert 0 < info.wide_max_stack < 64
    assert info.wide_node_count < info.fast_node_count


@pytest.mark.parametrize("name", ["box4k", "terrain_s", "terrain"])
def test_compressed_layout_is_built(name):
    """The compressed eight-child layout exists for the benchmark scenes:
    about a third of the fast layout's node count, a shallow tree, 80 bytes
    a node, every triangle record once."""
    g = kgr.Generated(name, 1)
    sc = kgr.Scene.from_generated(g)
    info = sc.info()
    assert info.cw8_node_count > 0
    assert info.cw8_node_count * 2 < info.fast_node_count
    assert 0 < info.cw8_depth <= 15
    nodes = sc.array(kgr.ARRAY_CW8_NODES)
    assert len(nodes) == 80 * info.cw8_node_count
    tris = sc.array(kgr.ARRAY_CW8_TRIANGLES).view(np.float32).reshape(-1, 12)
    assert len(tris) == info.triangle_count
    ranks = np.sort(tris[:, 7].view(np.int32))
    np.testing.assert_array_equal(ranks, np.arange(info.triangle_count))
    sc.close()


def test_compressed_layout_grazing_and_axis_rays():
    """Rays along the axes and grazing the terrain (origins just above the
    surface, nearly horizontal): the quantised boxes still cull
    conservatively, so every hit equals the threaded walk's."""
    g, sc, osc = helpers.both("terrain_s", 1)
    rng = np.random.default_rng(21)
    n = 30000
    o = np.stack([rng.uniform(-1.9, 1.9, n), rng.uniform(-0.4, 0.2, n), rng.uniform(-1.9, 1.9, n)], 1)
    d = np.stack([rng.normal(size=n), rng.normal(scale=0.02, size=n), rng.normal(size=n)], 1)
    axis = rng.integers(0, 6, n // 5)
    d[: n // 5] = 0
    d[np.arange(n // 5), axis % 3] = np.where(axis < 3, 1.0, -1.0)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3], rays[:, 4:7], rays[:, 7] = o, d, np.inf
    thr = gpu_closest(sc, rays, kgr.LAYOUT_THREADED)
    assert_hits_equal(gpu_closest(sc, rays, kgr.LAYOUT_CW8), thr)
    ref, _ = osc.trace_closest(rays[::5])
    assert_hits_equal(thr[::5], ref["raw"])
    occ = gpu_any(sc, rays, kgr.LAYOUT_CW8)
    np.testing.assert_array_equal(occ, gpu_any(sc, rays, kgr.LAYOUT_THREADED))
    sc.close()
