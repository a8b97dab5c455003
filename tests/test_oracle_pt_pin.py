"""The oracle's path tracer against the reference's own path-tracer
programs, on the CPU.

tests/golden/reference_pt.json holds one sample of every pixel of small
images rendered by the reference's __closesthit__ and __miss__ programs
(source/optix/amadeus_path_tracer.cu with source/optix/amadeus_common.cuh,
include/cuda/brdf.cuh and include/optix/lighting.cuh), compiled unmodified
on the host by oracle/ref_pt.cpp: the Lambertian box scene and the
50%-GGX terrain, depths 0 to 6, with and without an environment map
(linear and point filtering) and quad lights.  The harness finds hits with the oracle's
walk and takes each pixel's PCG seed from the pixel index and frame, as the
benchmark configurations do; everything else -- make_ray, the shading
normal and position, the material, next-event estimation over the
triangle and quad lights and the map, the BSDF sample, the recursion with its depth
test and the miss program -- is the reference's code.

The oracle (oracle_render_pt, Russian roulette off: the reference's
amadeus path tracer has none) must give the same radiance: bit for bit up
to depth 1, where a path has at most two vertices and both sides sum the
same terms in the same order; at depth 2 and beyond within 1e-6 relative,
since the reference adds the terms recursively (direct + T * indirect from
the deepest vertex back) and the oracle in path order (L += beta * direct).
The GPU path tracer equals the oracle bit for bit (the -m gpu suite), so
this also pins the kernels."""
import json
import os

import numpy as np
import pytest

from oracle import pyoracle

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "reference_pt.json")) as f:
    FIXTURE = json.load(f)

REL_TOL = 1e-6  # recursive against running sums of the same float terms


def oracle_image(case):
    g = pyoracle.GeneratedScene(case["scene"], case["seed"])
    env = None
    if "env" in case:
        env = np.asarray(case["env"], np.uint32).view(np.float32).reshape(case["env_shape"])
    quads = None
    if "quads" in case:
        quads = np.asarray(case["quads"], np.uint32).view(np.float32).reshape(-1, 12)
    osc = pyoracle.Scene(g.positions, g.normals, g.tris4(), g.materials_raw, g.lights(), g.sah_bvh(4), quads=quads,
                         env=env, env_filter=case.get("env_filter", 0))
    W, H = case["width"], case["height"]
    cam = pyoracle.camera(g.eye, g.target, g.fov, W / H)
    p = pyoracle.render_params(W, H, cam, max_depth=case["max_depth"], spp=1, frame=case["frame"],
                               russian_roulette=0)
    c, _ = pyoracle.render_pt(osc, p)
    return c[0][:, :3]


def case_id(c):
    env = (f"-env{c['env_filter']}" if "env" in c else "") + ("-quads" if "quads" in c else "")
    return f"{c['scene']}-d{c['max_depth']}-f{c['frame']}{env}"


@pytest.mark.parametrize("case", FIXTURE["cases"], ids=case_id)
def test_oracle_path_tracer_matches_reference_programs(case):
    ref = np.asarray(case["radiance"], np.uint32).view(np.float32).reshape(-1, 3)
    img = oracle_image(case)
    assert img.shape == ref.shape
    exact = np.all(img.view(np.uint32) == ref.view(np.uint32), axis=1)
    if case["max_depth"] <= 1:
        assert exact.all(), f"{(~exact).sum()} pixels differ"
    rel = np.abs(img - ref) / np.maximum(np.maximum(np.abs(img), np.abs(ref)), 1e-6)
    print(f"{case_id(case)}: {exact.mean():.4f} of pixels bit-exact, max relative difference {rel.max():.3g}")
    assert rel.max() <= REL_TOL


def test_fixture_covers_the_cases():
    """GGX and Lambertian scenes, several depths, both filters of the map,
    and images that are not black."""
    ids = {case_id(c) for c in FIXTURE["cases"]}
    assert any("terrain_s" in i for i in ids) and any("box4k" in i for i in ids)
    assert {c.get("env_filter") for c in FIXTURE["cases"]} >= {None, 0, 1}
    assert max(c["max_depth"] for c in FIXTURE["cases"]) >= 3
    for c in FIXTURE["cases"]:
        ref = np.asarray(c["radiance"], np.uint32).view(np.float32)
        assert np.isfinite(ref).all() and ref.max() > 0


def test_roulette_keeps_the_mean():
    """Russian roulette is not in the reference's amadeus path tracer; the
    option follows its naive path tracer (naive_path_tracer.cu:294-303):
    past depth 2 a path ends with probability q = 1 - min(max(0.05, beta.y),
    1) and survivors are divided by 1 - q.  Its uniform is fract(seed.x),
    the last value the BSDF sample drew, so it is not independent of the
    bounce direction.  On the box scene at depth 8 (1024 samples of 16 x 16
    pixels) the image mean stays within 2% of the image without roulette,
    with fewer bounce rays."""
    g = pyoracle.GeneratedScene("box4k", 1)
    osc = pyoracle.Scene(g.positions, g.normals, g.tris4(), g.materials_raw, g.lights(), g.sah_bvh(4))
    W = H = 16
    cam = pyoracle.camera(g.eye, g.target, g.fov, 1.0)
    run = lambda rr: pyoracle.render_pt(osc, pyoracle.render_params(W, H, cam, max_depth=8, spp=1024, frame=0,
                                                                     russian_roulette=rr, rr_start_depth=3))
    (plain, _, _, _), st_plain = run(0)
    (rr, _, _, _), st_rr = run(1)
    print(f"mean {plain[:, :3].mean():.5f} without roulette, {rr[:, :3].mean():.5f} with; "
          f"bounce rays {st_plain.bounce_rays} -> {st_rr.bounce_rays}")
    assert abs(rr[:, :3].mean() / plain[:, :3].mean() - 1) < 0.02
    assert st_rr.bounce_rays < 0.9 * st_plain.bounce_rays
