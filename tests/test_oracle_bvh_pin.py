"""The Kobra BVH builder -- the oracle's restatement and the product's host
builder -- against the reference's own source/bvh.cpp, on the CPU.

tests/golden/reference_bvh.json holds what serialize(partition(boxes)) of
source/bvh.cpp:102-260, compiled unmodified on the host by
oracle/ref_bvh.cpp, builds: for the triangle boxes of three procedural
scenes, the SHA-256 of the threaded buffer; for small seeded box sets at
the builder's edges (one to three boxes, identical boxes, boxes of zero
extent in one axis or all three, a row of boxes, a thousand random boxes),
the boxes and the buffer in full.  Both builders must give the buffer bit
for bit."""
import hashlib
import json
import os

import numpy as np
import pytest

from artemis_gb300 import kgr
from oracle import pyoracle

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "reference_bvh.json")) as f:
    FIXTURE = json.load(f)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


def scene_boxes(g):
    osc = pyoracle.Scene(g.positions, g.normals, g.tris4(), g.materials_raw, g.lights(), np.zeros((0, 4), np.float32))
    return osc.triangle_boxes()


@pytest.mark.parametrize("case", FIXTURE["scenes"], ids=lambda c: c["scene"])
def test_oracle_builder_matches_reference_on_scenes(case):
    g = pyoracle.GeneratedScene(case["scene"], case["seed"])
    boxes = scene_boxes(g)
    assert len(boxes) == case["boxes"] and sha(boxes) == case["boxes_sha256"]
    bvh = pyoracle.build_kobra_bvh(boxes)
    assert len(bvh) == case["rows"]
    assert sha(bvh) == case["bvh_sha256"]


@pytest.mark.parametrize("case", FIXTURE["scenes"], ids=lambda c: c["scene"])
def test_product_builder_matches_reference_on_scenes(case):
    g = kgr.Generated(case["scene"], case["seed"])
    bvh = kgr.bvh_build_host(g.positions, g.indices, kgr.BUILDER_KOBRA)
    assert len(bvh) == case["rows"]
    assert sha(bvh) == case["bvh_sha256"]


@pytest.mark.parametrize("case", FIXTURE["box_sets"], ids=lambda c: c["name"])
def test_oracle_builder_matches_reference_on_box_sets(case):
    boxes = np.asarray(case["boxes"], np.uint32).view(np.float32).reshape(-1, 6)
    ref = np.asarray(case["bvh"], np.uint32).reshape(-1, 4)
    bvh = pyoracle.build_kobra_bvh(boxes)
    np.testing.assert_array_equal(bvh.view(np.uint32), ref)


def test_box_sets_cover_the_edges():
    """Every leaf of the reference's buffer holds one box and every box is
    in one leaf; the identical and point sets are in the fixture."""
    names = {c["name"] for c in FIXTURE["box_sets"]}
    assert {"one", "identical", "points", "flat", "row"} <= names
    for c in FIXTURE["box_sets"]:
        ref = np.asarray(c["bvh"], np.uint32).reshape(-1, 4)
        obj = ref[0::3, 1].view(np.int32)
        n = len(c["boxes"])
        assert sorted(obj[obj != -1].tolist()) == list(range(n))
