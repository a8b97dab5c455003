"""The oracle's threaded-BVH walk against the reference's own traversal
shaders, on the CPU.

tests/golden/reference_traversal.json holds, for three procedural scenes
and their oracle-built BVHs (SAH with leaves of up to four triangles, and
the restated bvh.cpp builder), the closest object and distance that trace()
of shaders/rt/modules/bvh.glsl -- with bbox.glsl, intersect.glsl, ray.glsl
and primitives.glsl, compiled unmodified as C++ by oracle/ref_glsl.cpp --
returns for camera rays, random rays and edge cases (directions with zero
components, axis-aligned rays, origins inside the scene box).  The oracle's
walk (oracle_trace_closest) must return the same object and the same
distance, bit for bit; the GPU walks are compared with the oracle by the
-m gpu traversal tests."""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import pyoracle

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "reference_traversal.json")) as f:
    FIXTURE = json.load(f)


def oracle_bvh(g, builder, max_leaf):
    if builder == "sah":
        return g.sah_bvh(max_leaf)
    osc = pyoracle.Scene(g.positions, g.normals, g.tris4(), g.materials_raw, g.lights(), np.zeros((0, 4), np.float32))
    return pyoracle.build_kobra_bvh(osc.triangle_boxes())


@pytest.mark.parametrize("case", FIXTURE["scenes"], ids=lambda c: f"{c['scene']}-{c['builder']}")
def test_oracle_walk_matches_reference_shaders(case):
    g = pyoracle.GeneratedScene(case["scene"], case["seed"])
    bvh = oracle_bvh(g, case["builder"], case["max_leaf"])
    digest = hashlib.sha256(np.ascontiguousarray(bvh, np.float32).tobytes()).hexdigest()
    assert digest == case["bvh_sha256"], "the oracle no longer builds the fixture's BVH"
    osc = pyoracle.Scene(g.positions, g.normals, g.tris4(), g.materials_raw, g.lights(), bvh)
    r6 = np.asarray(case["rays"], np.uint32).view(np.float32).reshape(-1, 6)
    rays = np.zeros((len(r6), 8), np.float32)
    rays[:, 0:3], rays[:, 4:7], rays[:, 7] = r6[:, 0:3], r6[:, 3:6], np.inf
    hits, _ = osc.trace_closest(rays)
    want = np.asarray(case["hits"], np.int64)
    prim = np.asarray(hits["prim"], np.int64)
    t_bits = np.asarray(hits["t"], np.float32).view(np.uint32).astype(np.int64)
    hit = want[:, 0] >= 0
    print(f"{case['scene']} ({case['builder']}): {len(want)} rays, {hit.sum()} hits")
    np.testing.assert_array_equal(prim, want[:, 0])
    np.testing.assert_array_equal(t_bits[hit], want[hit, 1])
    assert hit.sum() > len(want) // 2


@pytest.mark.parametrize("case", FIXTURE["scenes"], ids=lambda c: f"{c['scene']}-{c['builder']}")
def test_oracle_any_hit_matches_reference_shaders(case):
    """A ray is occluded on (0, tmax) exactly when the shaders' closest hit
    lies below tmax: with tmax just under and just over each closest
    distance, the oracle's any-hit walk (oracle_trace_any) must answer no
    and yes."""
    g = pyoracle.GeneratedScene(case["scene"], case["seed"])
    bvh = oracle_bvh(g, case["builder"], case["max_leaf"])
    osc = pyoracle.Scene(g.positions, g.normals, g.tris4(), g.materials_raw, g.lights(), bvh)
    r6 = np.asarray(case["rays"], np.uint32).view(np.float32).reshape(-1, 6)
    want = np.asarray(case["hits"], np.int64)
    hit = want[:, 0] >= 0
    t = want[hit, 1].astype(np.uint32).view(np.float32)
    for scale, expect in ((np.float32(0.999), False), (np.float32(1.001), True)):
        rays = np.zeros((hit.sum(), 8), np.float32)
        rays[:, 0:3], rays[:, 4:7], rays[:, 7] = r6[hit, 0:3], r6[hit, 3:6], t * scale
        occ, _ = osc.trace_any(rays)
        assert np.all(np.asarray(occ, bool) == expect), scale
