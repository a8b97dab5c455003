"""The oracle's ReSTIR DI against the reference's own ReSTIR DI programs,
on the CPU.

tests/golden/reference_restir.json holds what the reference's programs
(source/optix/amadeus_restir.cu: RIS over 32 candidates in
__closesthit__initial, __raygen__temporal with the M-cap of 200,
__raygen__spatial with five neighbours over 30 pixels, run twice with the
reservoir swaps of include/amadeus/restir.cuh:254-303) compute when
compiled unmodified on the host by oracle/ref_restir.cpp: the colour after
two or three frames of a still camera, and the reservoirs the next frame
would reuse (selected point, w, W, M), on the box scene and the 50%-GGX
terrain, depths 0 to 2, with and without an environment map and quad
lights.  The harness
finds hits with the oracle's walk and takes the pixel's PCG seeds from the
pixel index and frame (the RIS reservoir's seed, which the reference draws
from std::random_device at allocation, with the oracle's salt); the rest is
the reference's code.

The oracle (oracle_render_restir with the reference's constants) must give
the same reservoirs bit for bit, and the same colour bit for bit at depth 0;
with an indirect bounce the path part of the initial pass sums its terms in
path order where the reference recurses, so the colour agrees within 1e-6
relative.  The GPU's ReSTIR DI equals the oracle (the -m gpu suite), so this
also pins the kernels."""
import json
import os

import numpy as np
import pytest

from oracle import pyoracle

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "reference_restir.json")) as f:
    FIXTURE = json.load(f)

REL_TOL = 1e-6  # the path part's recursive against running sums


def case_id(c):
    env = (f"-env{c['env_filter']}" if "env" in c else "") + ("-quads" if "quads" in c else "")
    return f"{c['scene']}-d{c['max_depth']}-{c['frames']}frames{env}"


def oracle_run(case):
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
    n = W * H
    state = pyoracle.RestirBuffers(n)
    bufs = [np.zeros((n, 4), np.float32) for _ in range(4)]
    for f in range(case["frames"]):
        p = pyoracle.render_params(W, H, cam, max_depth=case["max_depth"], spp=1, frame=f, samples=f,
                                   accumulate=int(f > 0), candidates=32, temporal=1, temporal_mcap=200,
                                   spatial_passes=2, spatial_neighbors=5, spatial_radius=30)
        pyoracle.render_restir(osc, p, state, bufs)
    return bufs[0], state.arrays


@pytest.mark.parametrize("case", FIXTURE["cases"], ids=case_id)
def test_oracle_restir_matches_reference_programs(case):
    color, A = oracle_run(case)
    ref_color = np.asarray(case["color"], np.uint32).view(np.float32).reshape(-1, 4)
    res = np.asarray(case["reservoirs"], np.uint32).view(np.float32).reshape(-1, 6)
    # reservoirs: bit for bit
    np.testing.assert_array_equal(res[:, 5].astype(np.int32), A["prev_M"])
    np.testing.assert_array_equal(res[:, 4].view(np.uint32), A["prev_W"].view(np.uint32))
    np.testing.assert_array_equal(res[:, 3].view(np.uint32), A["prev_w"].view(np.uint32))
    valid = A["prev_M"] > 0
    assert valid.mean() > 0.5
    np.testing.assert_array_equal(res[valid, :3].view(np.uint32), A["prev_point"][valid].view(np.uint32))
    # colour
    exact = np.all(color.view(np.uint32) == ref_color.view(np.uint32), axis=1)
    if case["max_depth"] == 0:
        assert exact.all(), f"{(~exact).sum()} pixels differ"
    rel = np.abs(color - ref_color) / np.maximum(np.maximum(np.abs(color), np.abs(ref_color)), 1e-6)
    print(f"{case_id(case)}: colour {exact.mean():.4f} bit-exact, max relative difference {rel.max():.3g}; "
          f"reservoirs equal on {valid.sum()} non-empty pixels")
    assert rel.max() <= REL_TOL
