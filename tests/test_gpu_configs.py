"""Parity on the benchmark configurations themselves, as configured.

- Plain path tracing at 1920x1080, 4 spp, depth 8, Russian roulette from
  depth 3, on the 1.16M-triangle terrain (50% Lambertian, 50% GGX with
  roughness in [0.05, 0.8]; 1024 emissive triangles): the GPU renders the
  whole frame, the oracle renders bands of rows of it (top, middle, bottom),
  on all three layouts.  This is where the GPU's GGX shading
  (brdf.cuh:335-434 and the Lambert/GGX mixture of eval(), :437-589) meets
  the oracle.
- ReSTIR DI exactly at 256x256: the box scene with generator seed
  0x4B4F4252, 32 candidates, temporal reuse with M-cap 20, one spatial pass
  of 5 neighbours over 30 px (amadeus_restir.cu:82-559).
- ReSTIR GI on a GGX scene (the 0.26M-triangle terrain), so rough GGX
  reconnection vertices and the bounded reconnection Jacobian are exercised.

Tolerance (stated in each test): >= 99.9% of pixels within 1e-4 relative in
FP32 radiance; DI selected samples equal on >= 99.9% of pixels.  The exact
bit-equal fraction is printed beside it."""
import math

import numpy as np
import pytest

from artemis_gb300 import kgr
from oracle import pyoracle
from tests import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RTOL = 1e-4


def rel_ok(a, b, rtol=RTOL, atol=1e-6):
    return np.abs(a - b) <= rtol * np.maximum(np.abs(a), np.abs(b)) + atol


def exact_rows(a, b):
    return np.all(a.view(np.uint32) == b.view(np.uint32), axis=1)


W2, H2 = 1920, 1080
BANDS = ((0, 24), (528, 552), (1056, 1080))


@pytest.fixture(scope="module")
def terrain():
    g, sc, osc = helpers.both("terrain", 1)
    yield g, sc, osc
    sc.close()


@pytest.fixture(scope="module")
def terrain_oracle_bands(terrain):
    """Oracle colour and AOVs of the 4-spp frame, rows of BANDS only."""
    g, sc, osc = terrain
    cam = kgr.camera(g.eye, g.target, g.fov, W2 / H2)
    ref = [np.zeros((W2 * H2, 4), np.float32) for _ in range(4)]
    for r0, r1 in BANDS:
        p = helpers.oracle_params(cam, W2, H2, max_depth=8, spp=4, frame=0, samples=0, accumulate=0,
                                  russian_roulette=1, rr_start_depth=3, row_begin=r0, row_end=r1)
        pyoracle.render_pt(osc, p, ref)
    return cam, ref


def band_rows():
    return np.concatenate([np.arange(r0 * W2, r1 * W2) for r0, r1 in BANDS])


@pytest.mark.parametrize("layout", ["fast", "wide", "cw8", "threaded"])
def test_pt_terrain_1080p_4spp_ggx_matches_oracle(terrain, terrain_oracle_bands, layout):
    """C2 as configured; tolerance 1e-4 relative on >= 99.9% of band pixels."""
    g, sc, osc = terrain
    cam, ref = terrain_oracle_bands
    bufs = helpers.device_buffers(torch, W2 * H2)
    att = kgr.Attachment("path_tracer")
    att.attach(W2, H2)
    att.load()
    for k, v in {"spp": 4, "russian_roulette": True, "rr_start_depth": 3, "layout": layout}.items():
        att.set_option(k, v)
    att.render(helpers.launch(cam, W2, H2, bufs, max_depth=8, frame=0, samples=0), sc)
    torch.cuda.synchronize()
    st = att.stats()
    att.close()
    rows = band_rows()
    out = [b.cpu().numpy()[rows] for b in bufs]
    want = [r[rows] for r in ref]
    exact = exact_rows(out[0], want[0]).mean()
    close = np.all(rel_ok(out[0], want[0]), axis=1).mean()
    print(f"C2 PT {layout}: {len(rows)} band pixels, colour exact {exact:.6f}, within 1e-4 {close:.6f}")
    assert close >= 0.999
    for k in (1, 2, 3):
        assert np.all(rel_ok(out[k], want[k]), axis=1).mean() >= 0.999
    # the bands see both material kinds: GGX pixels (specular > 0) are compared
    mats = g.materials_raw.reshape(-1, 16)
    assert (mats[:, 3:6].max(axis=1) > 0).any() and (mats[:, 3:6].max(axis=1) == 0).any()
    assert out[0][:, :3].mean() > 0.01
    assert st.shadow_rays > 0 and st.bounce_rays > 0


def test_pt_terrain_bands_hit_ggx_surfaces(terrain, terrain_oracle_bands):
    """The compared bands really contain GGX surfaces: the primary hits of the
    band pixels, traced on the oracle, land on materials with specular > 0 for
    a sizeable share of pixels."""
    g, sc, osc = terrain
    cam, _ = terrain_oracle_bands
    rays = helpers.camera_rays(cam, W2, H2)[band_rows()]
    hits, _ = osc.trace_closest(rays)
    prim = hits["prim"]
    mat = g.tris4()[prim[prim >= 0], 3]
    spec = g.materials_raw.reshape(-1, 16)[mat, 3:6].max(axis=1)
    share = (spec > 0).mean()
    print(f"band primary hits on GGX materials: {share:.3f} of {len(mat)} hits")
    assert share > 0.2


def test_restir_di_c1_exact_config_matches_oracle():
    """C1 as configured (256x256, seed 0x4B4F4252, 32 candidates, temporal
    M-cap 20, one spatial pass of 5 neighbours over 30 px), two frames so
    temporal reuse has history.  Selected samples equal on >= 99.9% of
    pixels; colour within 1e-4 relative on >= 99.9%."""
    g, sc, osc = helpers.both("box4k", 0x4B4F4252)
    W = H = 256
    opts = {"candidates": 32, "temporal": True, "temporal_mcap": 20, "spatial_passes": 1,
            "spatial_neighbors": 5, "spatial_radius": 30}
    cam = kgr.camera(g.eye, g.target, g.fov, 1.0)
    bufs = helpers.device_buffers(torch, W * H)
    att = kgr.Attachment("restir_di")
    att.attach(W, H)
    att.load()
    for k, v in opts.items():
        att.set_option(k, v)
    n = W * H
    state = pyoracle.RestirBuffers(n)
    ref = [np.zeros((n, 4), np.float32) for _ in range(4)]
    for f in range(2):
        att.render(helpers.launch(cam, W, H, bufs, frame=f, samples=0, accumulate=False, max_depth=2), sc)
        p = helpers.oracle_params(cam, W, H, max_depth=2, spp=1, frame=f, samples=0, accumulate=0, candidates=32,
                                  temporal=1, temporal_mcap=20, spatial_passes=1, spatial_neighbors=5,
                                  spatial_radius=30)
        pyoracle.render_restir(osc, p, state, ref)
    torch.cuda.synchronize()
    res_a = att.debug_copy("reservoir_prev_a", np.zeros((n, 4), np.float32))
    res_b = att.debug_copy("reservoir_prev_b", np.zeros((n, 4), np.float32))
    att.close()
    A = state.arrays
    valid = A["prev_M"] > 0
    same = ((res_a[:, 3].view(np.int32) == A["prev_light"]) & np.all(res_a[:, :3] == A["prev_point"], axis=1))
    color = bufs[0].cpu().numpy()
    exact = exact_rows(color, ref[0]).mean()
    close = np.all(rel_ok(color, ref[0]), axis=1).mean()
    print(f"C1 ReSTIR DI: selection agreement {same[valid].mean():.6f} over {valid.sum()} pixels, "
          f"colour exact {exact:.6f}, within 1e-4 {close:.6f}")
    assert valid.mean() > 0.95
    assert same[valid].mean() >= 0.999
    np.testing.assert_array_equal(res_b[:, 2].view(np.int32), A["prev_M"])
    assert np.all(rel_ok(res_b[:, 1], A["prev_W"]), axis=0).mean() >= 0.999
    assert close >= 0.999
    sc.close()


def orbit(g, f, deg=0.5):
    e = g.eye - g.target
    a = math.radians(deg * f)
    ca, sa = math.cos(a), math.sin(a)
    return np.array([ca * e[0] + sa * e[2], e[1], -sa * e[0] + ca * e[2]], np.float32) + g.target


@pytest.mark.parametrize("layout", ["fast", "cw8", "threaded"])
def test_restir_gi_on_ggx_terrain_matches_oracle(layout):
    """ReSTIR GI with C3's reuse settings (M-cap 30, 3 spatial iterations of
    8 neighbours) on the GGX terrain, three orbit frames, depth 8 with
    Russian roulette from 3.  Colour within 1e-4 relative on >= 99.9% of
    pixels; final reservoirs bit-equal on >= 99.9%."""
    g, sc, osc = helpers.both("terrain_s", 1)
    W, H, frames = 128, 96, 3
    bufs = helpers.device_buffers(torch, W * H)
    att = kgr.Attachment("restir_gi")
    att.attach(W, H)
    att.load()
    opts = {"layout": layout, "candidates": 32, "gi_mcap": 30, "gi_spatial_iterations": 3, "gi_neighbors": 8,
            "russian_roulette": True, "rr_start_depth": 3}
    for k, v in opts.items():
        att.set_option(k, v)
    state = pyoracle.GiState(W * H, temporal=True, mcap=30, iterations=3, neighbors=8, radius=30)
    ocolor = np.zeros((W * H, 4), np.float32)
    prev = None
    for f in range(frames):
        cam = kgr.camera(orbit(g, f), g.target, g.fov, W / H)
        att.render(helpers.launch(cam, W, H, bufs, frame=f, max_depth=8), sc)
        d = kgr.camera_dict(cam)
        if prev is not None:
            d["prev_projection"], d["prev_view"] = prev["projection"], prev["view"]
        p = pyoracle.render_params(W, H, d, max_depth=8, frame=f, russian_roulette=1, rr_start_depth=3,
                                   candidates=32)
        pyoracle.render_gi(osc, p, state, ocolor)
        prev = kgr.camera_dict(cam)
    torch.cuda.synchronize()
    color = bufs[0].cpu().numpy()
    ra = att.debug_copy("gi_reservoir_a", np.zeros((W * H, 4), np.float32))
    rb = att.debug_copy("gi_reservoir_b", np.zeros((W * H, 4), np.float32))
    att.close()
    close = np.all(rel_ok(color, ocolor), axis=1).mean()
    exact = exact_rows(color, ocolor).mean()
    same = exact_rows(ra, state.arrays["res_a"]).mean()
    # reservoirs whose sample sits on a rough GGX vertex (reconnectable, W sign bit clear, L_o > 0)
    live = (rb[:, 3] > 0) & (rb[:, :3].max(axis=1) > 0)
    print(f"GI terrain {layout}: colour exact {exact:.6f}, within 1e-4 {close:.6f}, reservoirs equal {same:.6f}, "
          f"live reconnectable samples {live.mean():.3f}")
    assert close >= 0.999
    assert same >= 0.999
    assert np.all(rel_ok(rb, state.arrays["res_b"]), axis=1).mean() >= 0.999
    assert live.mean() > 0.05
    assert color[:, :3].mean() > 0.01
    sc.close()
