"""Reading Kobra projects on the host (kgr_project_*), against the project
oracle (oracle/project_ref.py) on projects written in the layout
Project::save produces: every vertex, index, material, model matrix and
camera frame bit for bit.  Edge cases the reference's loader has: comments,
entities without a transform, an entity with a mesh that is not
renderable, a submesh whose cache file is missing, materials shared by
name, an unknown element type, a @materials list."""
import os

import numpy as np
import pytest

from artemis_gb300 import kgr
from oracle import project_ref


def box_entities(g):
    """box4k split into entities: ground (no transform), objects (moved),
    lights (emissive), a hidden mesh, a camera."""
    T = len(g.indices)
    lit = (g.materials["emission"].max(axis=1) > 0)[g.material_indices]
    ids_obj = np.nonzero(~lit)[0]
    half = len(ids_obj) // 2

    def sub(ids, mat_of):
        out = []
        for m in np.unique(g.material_indices[ids]):
            sel = ids[g.material_indices[ids] == m]
            verts, inv = np.unique(g.indices[sel].ravel(), return_inverse=True)
            out.append(dict(positions=g.positions[verts], normals=g.normals[verts],
                            indices=inv.reshape(-1, 3).astype(np.uint32), material=mat_of(m)))
        return out

    name = lambda m: "mat%d" % m
    ents = [
        dict(name="ground", position=(0, 0, 0), rotation=(0, 0, 0), scale=(1, 1, 1),
             submeshes=sub(ids_obj[:half], name)),
        dict(name="objects", position=(0.125, -0.25, 0.5), rotation=(12.5, -30, 5), scale=(0.75, 1.25, 1),
             submeshes=sub(ids_obj[half:], name)),
        dict(name="lights", position=(0, -0.0625, 0), rotation=(0, 0, 0), scale=(1, 1, 1),
             submeshes=sub(np.nonzero(lit)[0], name)),
        dict(name="hidden", position=(5, 5, 5), submeshes=sub(ids_obj[:10], name), renderable=False),
        dict(name="main camera", position=list(g.eye), rotation=(-0.05, 0.1, 0.0), camera=(float(g.fov), 1.5)),
    ]
    assert T == sum(len(s["indices"]) for e in ents[:3] for s in e["submeshes"])
    mats = {}
    for m in range(len(g.materials)):
        r = g.materials[m]
        mats["mat%d" % m] = dict(diffuse=r["diffuse"], specular=r["specular"], emission=r["emission"],
                                 roughness=float(r["roughness"]), refraction=float(r["refraction"]),
                                 type=int(g.materials_raw[m, 15:16].view(np.int32)[0]))
    return ents, mats


@pytest.fixture(scope="module")
def project_dir(tmp_path_factory):
    g = kgr.Generated("box4k", 1)
    d = str(tmp_path_factory.mktemp("kobra_project"))
    ents, mats = box_entities(g)
    # a listed submesh whose cache file is absent
    ents[1]["submeshes"].append(dict(positions=None, normals=None, indices=None, material="mat0"))
    kgr.write_project(d, {"Main": ents, "Empty": []}, mats)
    # comments, an unknown element, a @materials list (the reference parses, never saves these)
    path = os.path.join(d, "Main.kobra")
    text = open(path).read()
    text = "# a comment\n@materials\n.list 2\n\tmat0.mat\n\tmat1.mat\n@unknown thing\n" + text
    open(path, "w").write(text)
    return d, g


def test_project_file(project_dir):
    d, _ = project_dir
    p = kgr.Project(d)
    assert p.scene_files() == ["Main.kobra", "Empty.kobra"] == project_ref.read_project(d)
    p.close()


def test_scene_matches_oracle(project_dir):
    d, g = project_dir
    p = kgr.Project(d)
    s = p.read_scene(0)
    info = s.info()
    ents, meshes, mats, missing = project_ref.read_scene(d, "Main.kobra")
    assert info.entity_count == len(ents) == 5
    assert info.mesh_count == len(meshes) and info.missing_meshes == missing == 1
    assert info.triangle_count == len(g.indices)
    got = s.meshes()
    for a, b in zip(got, meshes):
        for k in ("positions", "normals", "indices", "material_indices", "model"):
            assert np.array_equal(np.asarray(a[k]).view(np.uint32), np.asarray(b[k]).view(np.uint32)), k
    assert np.array_equal(s.materials_raw().view(np.uint32), mats.view(np.uint32))
    assert info.material_count == len(mats) == len(g.materials)
    e = s.entities()
    assert [x["name"] for x in e] == ["ground", "objects", "lights", "hidden", "main camera"]
    assert e[3]["mesh_count"] == 0 and not e[3]["renderable"]
    for x, y in zip(e, ents):
        assert np.array_equal(x["model"].view(np.uint32), y["model"].view(np.uint32))
        assert (x["mesh_first"], x["mesh_count"]) == (y["mesh_first"], y["mesh_count"])
    assert info.camera_entity == 4
    cam = s.camera()
    c = ents[4]
    want = project_ref.camera_frame(c["position"], c["rotation"], *c["camera"])
    for got_v, key in zip(want, ("center", "ax_u", "ax_v", "ax_w")):
        assert np.array_equal(np.array(getattr(cam.camera, key)[:], np.float32).view(np.uint32),
                              got_v.view(np.uint32)), key
    s.close()
    p.close()


def test_materials_read_back(project_dir):
    d, g = project_dir
    s = kgr.Project(d).read_scene(0)
    m = s.materials_raw()
    # %f keeps six decimals: equal to the generated materials within that
    np.testing.assert_allclose(m[:, 0:9], g.materials_raw[:, 0:9], atol=5e-7)
    np.testing.assert_allclose(m[:, 13:15], g.materials_raw[:, 13:15], atol=5e-7)
    assert np.array_equal(m[:, 15].view(np.int32), g.materials_raw[:, 15].view(np.int32))


def test_empty_scene_and_errors(project_dir, tmp_path):
    d, _ = project_dir
    s = kgr.Project(d).read_scene(1)
    info = s.info()
    assert info.entity_count == 0 and info.mesh_count == 0 and info.material_count == 1
    assert info.camera_entity == -1
    with pytest.raises(kgr.KgrError):
        kgr.Project(str(tmp_path))  # no project.den
    os.makedirs(tmp_path / "p", exist_ok=True)
    (tmp_path / "p" / "project.den").write_text("@scenes 1\nMissing.kobra\n")
    with pytest.raises(kgr.KgrError):
        kgr.Project(str(tmp_path / "p"))
    # a material file that does not exist
    q = tmp_path / "q"
    kgr.write_project(str(q), {"S": [dict(name="a", submeshes=[dict(positions=np.zeros((3, 3)), normals=np.zeros((3, 3)),
                                                                    indices=np.arange(3).reshape(1, 3),
                                                                    material="nope")])]}, {})
    with pytest.raises(kgr.KgrError):
        kgr.Project(str(q)).read_scene(0)


def test_transform_matrix_known_answers():
    m = kgr.transform_matrix([1, 2, 3], [0, 90, 0], [2, 2, 2])
    p = m @ np.array([1, 0, 0, 1], np.float32)
    np.testing.assert_allclose(p[:3], [1, 2, 1], atol=1e-6)  # x -> -z under +90 about y, scaled by 2
    np.testing.assert_array_equal(kgr.transform_matrix([0, 0, 0], [0, 0, 0], [1, 1, 1]), np.eye(4, dtype=np.float32))
    for args in (([0.5, -1, 2], [10, 20, 30], [1, 2, 3]), ([0, 0, 0], [-45, 0, 90], [1, 1, 1])):
        want = project_ref.transform_matrix(*args).T
        assert np.array_equal(kgr.transform_matrix(*args).view(np.uint32), want.view(np.uint32))
