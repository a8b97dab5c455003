"""Host-side checks that need no GPU: the C ABI loads and exports every
function include/kgr.h declares, the option surface behaves like the
reference's AttachmentRTX, and the host BVH builders produce what the oracle
and the threaded-walk semantics require."""
import os
import re

import numpy as np
import pytest

from artemis_gb300 import kgr
from oracle import pyoracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header="kgr.h"):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(kgr_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = kgr.lib()
    names = declared_functions("kgr.h") + declared_functions("kgr_serve.h")
    assert len(names) >= 45
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert L.kgr_abi_version() == 5


def test_status_strings():
    assert kgr.lib().kgr_status_string(0) == b"ok"
    assert kgr.lib().kgr_status_string(7) == b"malformed BVH"


def test_attachment_options_without_device():
    a = kgr.Attachment("path_tracer")
    # defaults
    assert a.get_option("spp") == 1
    assert a.get_option("russian_roulette") is False
    assert a.get_option("layout") == "fast"
    a.set_option("russian_roulette", True)
    a.set_option("spp", 4)
    a.set_option("layout", "threaded")
    assert a.get_option("russian_roulette") is True
    assert a.get_option("spp") == 4
    assert a.get_option("layout") == "threaded"
    # unknown names are ignored, as the reference's set_option does; get
    # returns the default-constructed variant (int 0)
    a.set_option("no_such_option", 3)
    assert a.get_option("no_such_option") == 0
    # a known name with the wrong type is rejected
    with pytest.raises(kgr.KgrError) as e:
        a.set_option("spp", 2.5)
    assert e.value.status == 11
    with pytest.raises(kgr.KgrError):
        a.set_option("layout", "bogus")
    # render before attach/load
    with pytest.raises(kgr.KgrError) as e:
        kgr.check(kgr.lib().kgr_render(a.handle, None, None, None))
    assert e.value.status in (1, 5)
    a.close()


def test_unknown_kind_and_plugin_export():
    with pytest.raises(kgr.KgrError):
        kgr.Attachment("no_such_kind")
    r = kgr.lib().kgr_load_attachment(b"path_tracer")
    assert r.name == b"Path Tracer" and r.ptr
    kgr.lib().kgr_destroy(r.ptr)
    r = kgr.lib().kgr_load_attachment(b"bogus")
    assert r.name is None and not r.ptr


def test_scene_create_reports_missing_device():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    g = kgr.Generated("tiny", 0)
    with pytest.raises(kgr.KgrError) as e:
        kgr.Scene.from_generated(g)
    assert e.value.status == 13


@pytest.mark.parametrize("name,seed", [("tiny", 0), ("box64", 3), ("box4k", 1)])
def test_kobra_builder_matches_oracle_restatement(name, seed):
    """The product's partition()/serialize() (source/bvh.cpp:102-260) gives
    the same buffer, bit for bit, as the oracle's line-by-line restatement."""
    g = kgr.Generated(name, seed)
    prod = kgr.bvh_build_host(g.positions, g.indices, kgr.BUILDER_KOBRA)
    sc = pyoracle.Scene(g.positions, g.normals, g.tris4(), g.materials_raw, np.zeros((0, 12), np.float32), prod)
    ref = pyoracle.build_kobra_bvh(sc.triangle_boxes())
    np.testing.assert_array_equal(ref.view(np.uint32), prod.view(np.uint32))


def leaf_objects(bvh):
    obj = bvh[0::3, 1].view(np.int32)
    return obj[obj != -1]


@pytest.mark.parametrize("max_leaf", [1, 4, 8])
def test_sah_threaded_layout_invariants(max_leaf):
    g = kgr.Generated("box4k", 2)
    b = kgr.bvh_build_host(g.positions, g.indices, kgr.BUILDER_SAH, max_leaf)
    assert len(b) % 3 == 0
    objs = leaf_objects(b)
    assert sorted(objs.tolist()) == list(range(len(g.indices)))
    hdr = b[0::3]
    leaf = hdr[:, 1].view(np.int32) != -1
    # leaf flag float 1.0 on leaves, 0.0 on internal records (bvh.cpp:242)
    assert np.all(hdr[leaf, 0] == 1.0) and np.all(hdr[~leaf, 0] == 0.0)
    links = hdr[:, 2:4].view(np.int32)
    assert np.all((links == -1) | ((links >= 0) & (links < len(b)) & (links % 3 == 0)))
    # internal boxes contain the boxes of the records below them
    pos = g.positions
    for r in np.nonzero(~leaf)[0][:200]:
        lo, hi = b[3 * r + 1, :3], b[3 * r + 2, :3]
        node, end = int(links[r, 0]), int(links[r, 1])
        while node != end:
            h = b[node]
            o = int(h[1:2].view(np.int32)[0])
            if o != -1:
                tri = pos[g.indices[o]]
                assert np.all(tri >= lo) and np.all(tri <= hi)
            node = int(h[3:4].view(np.int32)[0])
    # chains of at most max_leaf records
    if max_leaf == 1:
        assert np.sum(~leaf) == len(g.indices) - 1


def _rays_through(g, n, rng):
    o = rng.uniform(-1.8, 1.8, (n, 3)).astype(np.float32)
    tgt = g.positions[g.indices[rng.integers(0, len(g.indices), n)]].mean(axis=1)
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3], rays[:, 4:7], rays[:, 7] = o, d, np.inf
    return rays


@pytest.mark.parametrize("builder,max_leaf", [(kgr.BUILDER_SAH, 4), (kgr.BUILDER_KOBRA, 1)])
def test_threaded_walk_equals_brute_force(builder, max_leaf):
    """The GLSL walk over either builder's layout returns the nearest
    triangle, ties resolved to the first one in walk order."""
    g = kgr.Generated("box4k", 5)
    b = kgr.bvh_build_host(g.positions, g.indices, builder, max_leaf)
    sc = pyoracle.Scene(g.positions, g.normals, g.tris4(), g.materials_raw, np.zeros((0, 12), np.float32), b)
    rays = _rays_through(g, 3000, np.random.default_rng(0))
    hits, st = sc.trace_closest(rays)
    brute = sc.trace_brute(rays)
    np.testing.assert_array_equal(hits["raw"].view(np.uint32), brute["raw"].view(np.uint32))
    assert (hits["prim"] >= 0).mean() > 0.99
    assert st.internal_visits > 0 and st.leaf_visits > 0


def test_oracle_any_hit_agrees_with_closest():
    g = kgr.Generated("box4k", 6)
    b = kgr.bvh_build_host(g.positions, g.indices)
    sc = pyoracle.Scene(g.positions, g.normals, g.tris4(), g.materials_raw, np.zeros((0, 12), np.float32), b)
    rays = _rays_through(g, 2000, np.random.default_rng(1))
    hits, _ = sc.trace_closest(rays)
    rays2 = rays.copy()
    rays2[:, 7] = np.where(hits["prim"] >= 0, hits["t"] * 1.01, 1.0)
    occ, _ = sc.trace_any(rays2)
    assert np.all(occ[hits["prim"] >= 0] == 1)
    rays2[:, 7] = np.where(hits["prim"] >= 0, hits["t"] * 0.99, 1.0)
    occ, _ = sc.trace_any(rays2)
    assert np.all(occ[hits["prim"] >= 0] == 0)


def test_generator_is_deterministic():
    a = kgr.Generated("box4k", 7)
    b = kgr.Generated("box4k", 7)
    c = kgr.Generated("box4k", 8)
    assert np.array_equal(a.positions, b.positions)
    assert not np.array_equal(a.positions, c.positions)
    assert len(a.indices) == 12 + 4096 + 128
    emissive = (a.materials["emission"].max(axis=1) > 0)[a.material_indices]
    assert emissive.sum() == 128
