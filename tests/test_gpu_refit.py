"""Refit on the GPU (kgr_scene_set_transforms, kgr_scene_refit) against the
refit oracle and against scenes created from scratch.

A three-mesh scene split out of the box4k scene: mesh 0 with normals and no
model, mesh 1 without normals (face normals) under a rotation, mesh 2 the
emissive ceiling under a translation, so moving it moves the lights.
Checked bit for bit:
- a refit to the current transforms or positions changes nothing: every
  layout, vertex and light stays identical to what scene creation built;
- after new transforms, vertices, normals and lights equal those of a scene
  created with the new transforms, and the threaded buffer equals the
  oracle's refit of the old buffer (refit_ref.refit_threaded);
- traversal on every layout and a path-traced frame equal the oracle's on
  the refitted buffer;
- the same for deformed positions given on the device, and for scenes made
  from a caller's buffer (the reference builder's, and chained leaves)."""
import numpy as np
import pytest

from artemis_gb300 import kgr
from oracle import pyoracle, refit_ref
from tests import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ARRAYS = [kgr.ARRAY_THREADED, kgr.ARRAY_FAST_NODES, kgr.ARRAY_WIDE_NODES, kgr.ARRAY_TRIANGLE_RECORDS]
LAYOUTS = [kgr.LAYOUT_FAST, kgr.LAYOUT_THREADED, kgr.LAYOUT_WIDE]


def rot_y(deg, scale=1.0, t=(0.0, 0.0, 0.0)):
    a = np.radians(deg)
    m = np.eye(4, dtype=np.float32)
    m[0, 0], m[0, 2], m[2, 0], m[2, 2] = np.cos(a), np.sin(a), -np.sin(a), np.cos(a)
    m[:3, :3] *= np.float32(scale)
    m[:3, 3] = t
    return m


def translate(t):
    m = np.eye(4, dtype=np.float32)
    m[:3, 3] = t
    return m


M0 = {1: rot_y(10.0, 1.0, (0.1, 0.0, 0.0)), 2: translate((0.0, -0.05, 0.0))}
M1 = {1: rot_y(35.0, 0.9, (-0.2, 0.1, 0.3)), 2: translate((0.3, -0.1, 0.2))}


def split_meshes(g, models):
    T = len(g.indices)
    emissive = g.materials["emission"].max(axis=1) > 0
    lit = emissive[g.material_indices]
    parts = [np.nonzero(~lit & (np.arange(T) % 2 == 0))[0], np.nonzero(~lit & (np.arange(T) % 2 == 1))[0],
             np.nonzero(lit)[0]]
    meshes = []
    for k, ids in enumerate(parts):
        verts, inv = np.unique(g.indices[ids].ravel(), return_inverse=True)
        meshes.append(dict(positions=g.positions[verts], normals=None if k == 1 else g.normals[verts],
                           indices=inv.reshape(-1, 3).astype(np.uint32), material_indices=g.material_indices[ids],
                           model=models.get(k)))
    return meshes


@pytest.fixture(scope="module")
def gen():
    return kgr.Generated("box4k", 1)


def snapshot(sc):
    p, n = sc.vertices()
    return [sc.array(a) for a in ARRAYS] + [p.view(np.uint32), n.view(np.uint32), sc.lights().view(np.uint32)]


def assert_snapshots_equal(a, b):
    names = ["threaded", "fast nodes", "wide nodes", "triangle records", "positions", "normals", "lights"]
    for name, x, y in zip(names, a, b):
        assert x.shape == y.shape and np.array_equal(x, y), f"{name} differ"


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


def check_traversal(g, sc, osc, seed):
    cam = kgr.camera(g.eye, g.target, g.fov, 1.0)
    rays = np.concatenate([helpers.camera_rays(cam, 128, 128), helpers.random_rays(g, 30000, seed)])
    ref, _ = osc.trace_closest(rays)
    assert (ref["prim"] >= 0).mean() > 0.5
    short = rays.copy()
    short[:, 7] = 0.7
    occ, _ = osc.trace_any(short)
    for layout in LAYOUTS:
        got = gpu_closest(sc, rays, layout)
        bad = np.nonzero(np.any(got.view(np.uint32) != ref["raw"].view(np.uint32), axis=1))[0]
        assert len(bad) == 0, f"layout {layout}: {len(bad)} of {len(rays)} hits differ"
        assert np.array_equal(gpu_any(sc, short, layout), occ), f"layout {layout}: occlusion differs"


def oracle_of(sc, g, tris):
    p, n = sc.vertices()
    return pyoracle.Scene(p, n, tris, g.materials_raw, sc.lights(), sc.bvh())


def test_refit_to_same_transforms_changes_nothing(gen):
    sc = kgr.Scene(None, None, gen.materials_raw, meshes=split_meshes(gen, M0))
    before = snapshot(sc)
    sc.set_transforms([1, 2], [M0[1], M0[2]])
    assert_snapshots_equal(before, snapshot(sc))
    sc.set_transforms([], [])  # every mesh at its current model
    assert_snapshots_equal(before, snapshot(sc))
    p, _ = sc.vertices()
    d = torch.from_numpy(p).cuda()
    sc.refit(d.data_ptr())
    assert_snapshots_equal(before, snapshot(sc))
    sc.close()


@pytest.mark.parametrize("builder", [kgr.BUILDER_SAH, kgr.BUILDER_SAH_HOST])
def test_new_transforms_match_a_new_scene_and_the_oracle(gen, builder):
    meshes1 = split_meshes(gen, M1)
    sc = kgr.Scene(None, None, gen.materials_raw, meshes=split_meshes(gen, M0), builder=builder)
    bvh0 = sc.bvh()
    sc.set_transforms([1, 2], [M1[1], M1[2]])
    fresh = kgr.Scene(None, None, gen.materials_raw, meshes=meshes1)
    pos, nrm, tris, lights = refit_ref.gather(meshes1, gen.materials_raw)
    p, n = sc.vertices()
    fp, fn = fresh.vertices()
    assert np.array_equal(p.view(np.uint32), fp.view(np.uint32))
    assert np.array_equal(n.view(np.uint32), fn.view(np.uint32))
    assert np.array_equal(p.view(np.uint32), pos.view(np.uint32))
    assert np.array_equal(n.view(np.uint32), nrm.view(np.uint32))
    assert np.array_equal(sc.lights().view(np.uint32), fresh.lights().view(np.uint32))
    assert np.array_equal(sc.lights().view(np.uint32), lights.view(np.uint32))
    assert len(lights) == 128 and not np.array_equal(lights, refit_ref.gather(split_meshes(gen, M0),
                                                                               gen.materials_raw)[3])
    want = refit_ref.refit_threaded(bvh0, pos, tris)
    assert np.array_equal(sc.bvh().view(np.uint32), want.view(np.uint32))
    check_traversal(gen, sc, oracle_of(sc, gen, tris), 5)
    sc.close()
    fresh.close()


def test_path_traced_frame_after_refit_matches_oracle(gen):
    sc = kgr.Scene(None, None, gen.materials_raw, meshes=split_meshes(gen, M0))
    sc.set_transforms([1, 2], [M1[1], M1[2]])
    _, _, tris, _ = refit_ref.gather(split_meshes(gen, M1), gen.materials_raw)
    osc = oracle_of(sc, gen, tris)
    W = H = 64
    cam = kgr.camera(gen.eye, gen.target, gen.fov, 1.0)
    bufs = helpers.device_buffers(torch, W * H)
    att = kgr.Attachment("path_tracer")
    att.attach(W, H)
    att.load()
    att.set_option("spp", 2)
    att.set_option("russian_roulette", True)
    for layout in ("fast", "wide"):
        att.set_option("layout", layout)
        att.render(helpers.launch(cam, W, H, bufs, frame=0, max_depth=5), sc)
        torch.cuda.synchronize()
        ref = [np.zeros((W * H, 4), np.float32) for _ in range(4)]
        pyoracle.render_pt(osc, helpers.oracle_params(cam, W, H, max_depth=5, spp=2, frame=0, russian_roulette=1),
                           ref)
        got = bufs[0].cpu().numpy()
        exact = np.all(got.view(np.uint32) == ref[0].view(np.uint32), axis=1).mean()
        assert exact >= 0.99, f"{layout}: {exact}"
        assert got[:, :3].mean() > 0.01
    att.close()
    sc.close()


def test_refit_with_device_positions(gen):
    meshes = split_meshes(gen, M0)
    sc = kgr.Scene(None, None, gen.materials_raw, meshes=meshes)
    bvh0 = sc.bvh()
    p0, n0 = sc.vertices()
    k = np.arange(len(p0), dtype=np.float32)
    wob = (p0 + np.float32(0.04) * np.sin(k * np.float32(0.37))[:, None].astype(np.float32)).astype(np.float32)
    d = torch.from_numpy(wob).cuda()
    sc.refit(d.data_ptr())
    # expected: positions as given; own normals kept; mesh 1's face normals from the new positions
    sizes = [len(m["positions"]) for m in meshes]
    off = np.concatenate([[0], np.cumsum(sizes)])
    parts = []
    for i, m in enumerate(meshes):
        sl = slice(off[i], off[i + 1])
        parts.append(dict(positions=wob[sl], normals=None if m["normals"] is None else n0[sl],
                          indices=m["indices"], material_indices=m["material_indices"]))
    pos, nrm, tris, lights = refit_ref.gather(parts, gen.materials_raw)
    p, n = sc.vertices()
    assert np.array_equal(p.view(np.uint32), pos.view(np.uint32))
    assert np.array_equal(n.view(np.uint32), nrm.view(np.uint32))
    assert np.array_equal(sc.lights().view(np.uint32), lights.view(np.uint32))
    assert np.array_equal(sc.bvh().view(np.uint32), refit_ref.refit_threaded(bvh0, pos, tris).view(np.uint32))
    check_traversal(gen, sc, oracle_of(sc, gen, tris), 6)
    # normals given too
    n2 = (n0 * np.float32(-1.0)).astype(np.float32)
    dn = torch.from_numpy(n2).cuda()
    sc.refit(d.data_ptr(), dn.data_ptr())
    _, n = sc.vertices()
    own = np.concatenate([np.full(s, m["normals"] is not None) for s, m in zip(sizes, meshes)])
    assert np.array_equal(n[own].view(np.uint32), n2[own].view(np.uint32))
    assert np.array_equal(n[~own].view(np.uint32), nrm[~own].view(np.uint32))
    sc.close()


@pytest.mark.parametrize("builder,max_leaf", [(kgr.BUILDER_KOBRA, 1), (kgr.BUILDER_SAH, 4)])
def test_refit_of_a_caller_buffer(gen, builder, max_leaf):
    meshes0 = split_meshes(gen, M0)
    pos0, _, tris0, _ = refit_ref.gather(meshes0, gen.materials_raw)
    buf = kgr.bvh_build_host(pos0, tris0[:, :3], builder, max_leaf)
    sc = kgr.Scene(None, None, gen.materials_raw, meshes=meshes0, bvh=buf)
    sc.set_transforms([1, 2], [M1[1], M1[2]])
    pos, _, tris, _ = refit_ref.gather(split_meshes(gen, M1), gen.materials_raw)
    assert np.array_equal(sc.bvh().view(np.uint32), refit_ref.refit_threaded(buf, pos, tris).view(np.uint32))
    check_traversal(gen, sc, oracle_of(sc, gen, tris), 7)
    sc.close()


def test_refit_time_terrain():
    g = kgr.Generated("terrain", 1)
    sc = kgr.Scene.from_generated(g)
    d = torch.from_numpy(np.ascontiguousarray(g.positions)).cuda()
    dn = torch.from_numpy(np.ascontiguousarray(g.normals)).cuda()
    before = [sc.array(a) for a in ARRAYS]
    sc.refit(d.data_ptr(), dn.data_ptr())
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n = 10
    e0.record()
    for _ in range(n):
        sc.refit(d.data_ptr(), dn.data_ptr(), stream=torch.cuda.current_stream().cuda_stream)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / n
    info = sc.info()
    print(f"refit terrain ({info.triangle_count} tris, {info.fast_node_count} fast nodes): {ms:.3f} ms; "
          f"build {info.build_ms:.1f} ms")
    for a, b in zip(before, [sc.array(a) for a in ARRAYS]):
        assert np.array_equal(a, b)
    sc.close()


def test_refit_of_a_one_triangle_scene():
    """The root is a leaf: the fast layout's single node keeps its empty right
    slot, there is no wide layout, and the threaded buffer is one record."""
    mats = np.zeros((1, 16), np.float32)
    mats[0, 0:3] = 0.5
    mats[0, 15:16].view(np.int32)[0] = 4
    tri = dict(positions=np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32),
               normals=np.array([[0, 0, 1]] * 3, np.float32), indices=np.array([[0, 1, 2]], np.uint32))
    sc = kgr.Scene(None, None, mats, meshes=[dict(tri)])
    assert sc.info().wide_node_count == 0 and sc.info().fast_node_count == 1
    before = snapshot(sc)
    sc.set_transforms([0], [translate((0.0, 0.0, 0.0))])
    after = snapshot(sc)
    # an identity model re-derives every vertex (x + 0 == x here) and box
    for name, a, b in zip(("threaded", "fast", "wide", "tris"), before[:4], after[:4]):
        assert np.array_equal(a, b), name
    m = rot_y(30.0, 2.0, (0.5, -0.25, 1.0))
    sc.set_transforms([0], [m])
    pos, nrm, tris, _ = refit_ref.gather([dict(tri, model=m)], mats)
    p, _ = sc.vertices()
    assert np.array_equal(p.view(np.uint32), pos.view(np.uint32))
    assert np.array_equal(sc.bvh().view(np.uint32), refit_ref.refit_threaded(before[0].view(np.float32).reshape(-1, 4),
                                                                            pos, tris).view(np.uint32))
    # toward the triangle from three sides, then away from it (misses)
    toward = np.array([[0, 0, 3], [0, 3, 0], [3, 0, 0]], np.float32)
    rays = np.zeros((6, 8), np.float32)
    c = pos.mean(axis=0)
    rays[:, 0:3] = c + np.concatenate([toward, toward])
    rays[:3, 4:7] = -toward / 3.0
    rays[3:, 4:7] = toward / 3.0
    rays[:, 7] = np.inf
    osc = pyoracle.Scene(pos, nrm, tris, mats, sc.lights(), sc.bvh())
    ref, _ = osc.trace_closest(rays)
    assert (ref["prim"][3:] < 0).all()
    short = rays.copy()
    short[:, 7] = 3.5
    occ, _ = osc.trace_any(short)
    assert occ[:3].any() and not occ[3:].any()
    for layout in (kgr.LAYOUT_FAST, kgr.LAYOUT_THREADED):
        assert np.array_equal(gpu_closest(sc, rays, layout).view(np.uint32), ref["raw"].view(np.uint32))
        assert np.array_equal(gpu_any(sc, short, layout), occ)
    sc.close()


def test_refit_requantises_the_compressed_layout(gen):
    """The compressed layout is refitted in place: its nodes are requantised
    from the refitted boxes by the builder's own rules, its triangle records
    move with the vertices, and every hit stays equal to the threaded walk
    and the oracle on the moved scene."""
    sc = kgr.Scene(None, None, gen.materials_raw, meshes=split_meshes(gen, M0))
    n = sc.info().cw8_node_count
    assert n > 0
    before = sc.array(kgr.ARRAY_CW8_NODES).copy()
    sc.set_transforms([1, 2], [M1[1], M1[2]])
    assert sc.info().cw8_node_count == n
    after = sc.array(kgr.ARRAY_CW8_NODES)
    assert not np.array_equal(before, after)
    # the slots, child and triangle bases do not move
    b16, a16 = before.view(np.uint32).reshape(n, 20), after.view(np.uint32).reshape(n, 20)
    np.testing.assert_array_equal(b16[:, 4:8], a16[:, 4:8])
    np.testing.assert_array_equal(b16[:, 3] >> 24, a16[:, 3] >> 24)
    _, _, tris, _ = refit_ref.gather(split_meshes(gen, M1), gen.materials_raw)
    osc = oracle_of(sc, gen, tris)
    cam = kgr.camera(gen.eye, gen.target, gen.fov, 1.0)
    rays = np.concatenate([helpers.camera_rays(cam, 96, 96), helpers.random_rays(gen, 20000, 9)])
    ref, _ = osc.trace_closest(rays)
    got = gpu_closest(sc, rays, kgr.LAYOUT_CW8)
    assert np.array_equal(got.view(np.uint32), ref["raw"].view(np.uint32))
    short = rays.copy()
    short[:, 7] = 0.7
    occ, _ = osc.trace_any(short)
    assert np.array_equal(gpu_any(sc, short, kgr.LAYOUT_CW8), occ)
    # back to the creation transforms: the nodes come back bit for bit
    sc.set_transforms([1, 2], [M0[1], M0[2]])
    assert np.array_equal(sc.array(kgr.ARRAY_CW8_NODES), before)
    sc.close()
