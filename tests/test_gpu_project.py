"""A Kobra project rendered on the GPU: the scene read by kgr_project_* and
created from its meshes equals the oracle's reading of the same files (world
vertices and lights bit for bit), a path-traced frame from the project's own
camera equals the oracle's render, and moving an entity through
kgr_scene_set_transforms gives the scene a fresh load of the moved project
gives."""
import numpy as np
import pytest

from artemis_gb300 import kgr
from oracle import project_ref, pyoracle, refit_ref
from tests import helpers
from tests.test_project import box_entities

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def write(tmp, ents, mats):
    kgr.write_project(tmp, {"Main": ents}, mats)
    return tmp


def world(d):
    ents, meshes, mats, _ = project_ref.read_scene(d, "Main.kobra")
    pos, nrm, tris, lights = refit_ref.gather(meshes, mats)
    return ents, pos, nrm, tris, lights, mats


def test_project_scene_renders_like_the_oracle(tmp_path):
    g = kgr.Generated("box4k", 1)
    ents, mats = box_entities(g)
    d = write(str(tmp_path / "p"), ents, mats)
    ps = kgr.Project(d).read_scene(0)
    sc = kgr.Scene.from_project(ps)
    oents, pos, nrm, tris, lights, omats = world(d)
    p, n = sc.vertices()
    assert np.array_equal(p.view(np.uint32), pos.view(np.uint32))
    assert np.array_equal(n.view(np.uint32), nrm.view(np.uint32))
    assert np.array_equal(sc.lights().view(np.uint32), lights.view(np.uint32)) and len(lights) == 128
    osc = pyoracle.Scene(pos, nrm, tris, omats, sc.lights(), sc.bvh())
    W, H = 96, 64
    cam = ps.camera(aspect=W / H)
    bufs = helpers.device_buffers(torch, W * H)
    att = kgr.Attachment("path_tracer")
    att.attach(W, H)
    att.load()
    att.set_option("spp", 2)
    att.render(helpers.launch(cam, W, H, bufs, frame=0, max_depth=4), sc)
    torch.cuda.synchronize()
    ref = [np.zeros((W * H, 4), np.float32) for _ in range(4)]
    pyoracle.render_pt(osc, helpers.oracle_params(cam, W, H, max_depth=4, spp=2, frame=0), ref)
    got = bufs[0].cpu().numpy()
    exact = np.all(got.view(np.uint32) == ref[0].view(np.uint32), axis=1).mean()
    print(f"project frame: exact {exact:.6f}, mean {got[:, :3].mean():.4f}")
    assert exact >= 0.99 and got[:, :3].mean() > 0.01
    att.close()
    sc.close()


def test_moving_an_entity_equals_a_fresh_load(tmp_path):
    g = kgr.Generated("box4k", 1)
    ents, mats = box_entities(g)
    d0 = write(str(tmp_path / "a"), ents, mats)
    ps = kgr.Project(d0).read_scene(0)
    sc = kgr.Scene.from_project(ps)
    obj = ps.entities()[1]
    moved = dict(ents[1], position=(-0.25, 0.125, 0.0), rotation=(0.0, 75.0, -10.0), scale=(1.0, 1.0, 0.5))
    m = kgr.transform_matrix(moved["position"], moved["rotation"], moved["scale"])
    ids = list(range(obj["mesh_first"], obj["mesh_first"] + obj["mesh_count"]))
    sc.set_transforms(ids, [m] * len(ids))
    d1 = write(str(tmp_path / "b"), [ents[0], moved] + ents[2:], mats)
    fresh = kgr.Scene.from_project(kgr.Project(d1).read_scene(0))
    for a, b in zip(sc.vertices(), fresh.vertices()):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.array_equal(sc.lights().view(np.uint32), fresh.lights().view(np.uint32))
    _, pos, nrm, tris, lights, omats = world(d1)
    osc = pyoracle.Scene(pos, nrm, tris, omats, sc.lights(), sc.bvh())
    rays = helpers.random_rays(g, 20000, 3)
    ref, _ = osc.trace_closest(rays)
    r = torch.from_numpy(rays).cuda()
    for layout in (kgr.LAYOUT_FAST, kgr.LAYOUT_WIDE, kgr.LAYOUT_THREADED):
        h = torch.zeros((len(rays), 4), dtype=torch.float32, device="cuda")
        sc.trace_closest(r.data_ptr(), len(rays), h.data_ptr(), layout)
        torch.cuda.synchronize()
        assert np.array_equal(h.cpu().numpy().view(np.uint32), ref["raw"].view(np.uint32))
    sc.close()
    fresh.close()
