"""Quad lights and the environment map, the two light sources of
ArmadaLaunchInfo besides emissive triangles, on the GPU against the oracle.

- Ld (amadeus_common.cuh:256-286) picks uniformly over quads + triangles +
  the environment; Ld_light (lighting.cuh:149-174) for a quad samples the
  parallelogram without reflection; Ld_Environment (amadeus_common.cuh:
  215-254) samples a direction and reads the map at (u, v).
- The path tracer's miss program reads the map at (u, 1 - v)
  (amadeus_path_tracer.cu:204-220), ReSTIR's at (u, v)
  (amadeus_restir.cu:561-578); the ray past the last vertex is cast, since
  the miss program has no depth test.
- ReSTIR DI's sample_direct (amadeus_common.cuh:301-377) draws quad,
  triangle and environment samples; the targets drop the light cosine and
  1/d^2 for the environment (type 2).

The map is read by the texture unit (tex2D<float4>); the oracle follows the
texture-fetching rules of the CUDA programming guide (the coordinate in
fixed point, weights with 8 fractional bits rounded half up).  Point
sampling agrees on every lookup; linear filtering on nearly all, the rest
within a fraction of one weight step, since the guide does not fix how the
hardware combines the weights.  A smooth map keeps that difference far
below the tolerance of the renders.  Tolerance: >= 99.9% of pixels within 1e-4 relative in FP32
radiance, >= 99.9% equal DI selections."""
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


def smooth_sky(w=64, h=32):
    """A smooth sky: brighter towards v = 1 and around one azimuth, coloured."""
    u = (np.arange(w) + 0.5) / w
    v = (np.arange(h) + 0.5) / h
    U, V = np.meshgrid(u, v)
    base = 0.2 + 1.5 * V ** 2 + 0.6 * np.exp(-((U - 0.3) ** 2) / 0.02) * V
    tex = np.stack([base * 0.9, base * 1.0, base * 1.2, np.ones_like(base)], axis=-1)
    return tex.astype(np.float32)


def blocky_sky(w=16, h=8, seed=3):
    """Point-sampled map with distinct texels."""
    rng = np.random.default_rng(seed)
    t = rng.uniform(0.1, 2.0, (h, w, 4)).astype(np.float32)
    t[..., 3] = 1.0
    return t


def quads_above():
    """Three quad lights above the terrain, facing down and sideways."""
    q = np.array([[-1.0, 1.6, -1.0, 0.5, 0, 0, 0, 0, 0.5, 4.0, 3.5, 3.0],
                  [0.4, 1.5, 0.2, 0.4, 0, 0, 0, 0, 0.6, 2.0, 2.5, 3.0],
                  [1.5, 0.3, -1.0, 0, 0.3, 0, 0, 0, 0.5, 6.0, 6.0, 6.0]], np.float32)
    return q


@pytest.fixture(scope="module")
def terrain_s():
    g, sc, osc = helpers.both("terrain_s", 1)
    yield g, sc, osc
    sc.close()


def oracle_scene_with(g, sc, quads, env, env_filter):
    return pyoracle.Scene(g.positions, g.normals, g.tris4(), g.materials_raw, sc.lights(), sc.bvh(),
                          quads=quads, env=env, env_filter=env_filter)


def render_pt(g, sc, W, H, layout, quads, env, opts, frames=1, max_depth=3):
    cam = kgr.camera(g.eye, g.target, g.fov, W / H)
    bufs = helpers.device_buffers(torch, W * H)
    dq = torch.from_numpy(quads).cuda() if quads is not None else None
    att = kgr.Attachment("path_tracer")
    att.attach(W, H)
    att.load()
    for k, v in opts.items():
        att.set_option(k, v)
    att.set_option("layout", layout)
    for f in range(frames):
        info = helpers.launch(cam, W, H, bufs, frame=f, samples=f * opts.get("spp", 1), accumulate=f > 0,
                              max_depth=max_depth)
        if dq is not None:
            kgr.set_quad_lights(info, dq.data_ptr(), len(quads))
        if env is not None:
            env.attach_to(info)
        att.render(info, sc)
    torch.cuda.synchronize()
    att.close()
    return cam, [b.cpu().numpy() for b in bufs]


@pytest.mark.parametrize("layout", ["fast", "cw8", "threaded"])
@pytest.mark.parametrize("what", ["quads+env", "env", "quads"])
def test_path_tracer_quads_and_environment_match_oracle(terrain_s, layout, what):
    g, sc, _ = terrain_s
    W, H = 128, 96
    quads = quads_above() if "quads" in what else None
    tex = smooth_sky() if "env" in what else None
    env = kgr.Environment(tex, kgr.FILTER_LINEAR) if tex is not None else None
    opts = {"spp": 2, "russian_roulette": True, "rr_start_depth": 1}
    cam, out = render_pt(g, sc, W, H, layout, quads, env, opts, frames=2)
    osc = oracle_scene_with(g, sc, quads, tex, kgr.FILTER_LINEAR)
    ref = [np.zeros((W * H, 4), np.float32) for _ in range(4)]
    for f in range(2):
        p = helpers.oracle_params(cam, W, H, max_depth=3, spp=2, frame=f, samples=2 * f, accumulate=int(f > 0),
                                  russian_roulette=1, rr_start_depth=1)
        pyoracle.render_pt(osc, p, ref)
    color, ocolor = out[0], ref[0]
    exact = np.all(color.view(np.uint32) == ocolor.view(np.uint32), axis=1).mean()
    close = np.all(rel_ok(color, ocolor), axis=1).mean()
    print(f"PT {what} {layout}: exact {exact:.6f}, within 1e-4 {close:.6f}")
    assert close >= 0.999
    for k in (1, 2, 3):
        assert np.all(rel_ok(out[k], ref[k]), axis=1).mean() >= 0.999
    if env is not None:
        env.close()


def test_environment_changes_the_image(terrain_s):
    """The sky is seen directly (pixels that miss the terrain take the map at
    (u, 1 - v)) and lights the terrain; quads add light."""
    g, sc, _ = terrain_s
    W, H = 64, 48
    opts = {"spp": 1}  # one camera ray a pixel, the same in both renders
    _, plain = render_pt(g, sc, W, H, "fast", None, None, opts)
    env = kgr.Environment(smooth_sky(), kgr.FILTER_LINEAR)
    _, lit = render_pt(g, sc, W, H, "fast", quads_above(), env, opts)
    env.close()
    miss = plain[3][:, :3].max(axis=1) == 0  # no primary hit: position AOV stays 0
    assert miss.any()
    assert np.all(plain[0][miss, :3] == 0)
    assert np.all(lit[0][miss, :3] > 0.1)
    assert lit[0][~miss, :3].mean() > plain[0][~miss, :3].mean()


@pytest.mark.parametrize("filt", [kgr.FILTER_LINEAR, kgr.FILTER_POINT])
def test_environment_lookups_follow_the_texture_rules(filt):
    """kgr_environment_sample against the oracle's reading of the texture
    rules, at random coordinates (wrap addressing included)."""
    tex = smooth_sky() if filt == kgr.FILTER_LINEAR else blocky_sky()
    env = kgr.Environment(tex, filt)
    rng = np.random.default_rng(7)
    uv = rng.uniform(-0.5, 1.5, (20000, 2)).astype(np.float32)
    d_uv = torch.from_numpy(uv).cuda()
    out = torch.zeros((len(uv), 4), dtype=torch.float32, device="cuda")
    env.sample(d_uv.data_ptr(), len(uv), out.data_ptr())
    torch.cuda.synchronize()
    got = out.cpu().numpy()[:, :3]
    want = pyoracle.env_lookup(tex, uv, filt)
    exact = np.all(got == want, axis=1).mean()
    close = np.all(rel_ok(got, want), axis=1).mean()
    worst = float((np.abs(got - want) / np.maximum(np.abs(want), 1e-6)).max())
    print(f"texture lookups filter={filt}: exact {exact:.6f}, within 1e-4 {close:.6f}, max rel {worst:.2e}")
    if filt == kgr.FILTER_POINT:
        # the texel a coordinate falls in: every lookup equal
        assert exact == 1.0
    else:
        # the hardware's bilinear weights are 8-bit fixed point; the guide
        # does not fix the arithmetic of their products and sums, so a few
        # lookups differ by a fraction of one weight step of this smooth map
        assert close >= 0.995
        assert worst <= 2e-3
    env.close()


@pytest.mark.parametrize("layout", ["fast", "threaded"])
def test_restir_di_quads_and_environment_match_oracle(terrain_s, layout):
    g, sc, _ = terrain_s
    W, H = 96, 72
    quads = quads_above()
    tex = smooth_sky()
    env = kgr.Environment(tex, kgr.FILTER_LINEAR)
    dq = torch.from_numpy(quads).cuda()
    cam = kgr.camera(g.eye, g.target, g.fov, W / H)
    bufs = helpers.device_buffers(torch, W * H)
    att = kgr.Attachment("restir_di")
    att.attach(W, H)
    att.load()
    opts = {"candidates": 32, "temporal": True, "temporal_mcap": 20, "spatial_passes": 1, "spatial_neighbors": 5,
            "spatial_radius": 30, "layout": layout}
    for k, v in opts.items():
        att.set_option(k, v)
    n = W * H
    osc = oracle_scene_with(g, sc, quads, tex, kgr.FILTER_LINEAR)
    state = pyoracle.RestirBuffers(n)
    ref = [np.zeros((n, 4), np.float32) for _ in range(4)]
    for f in range(2):
        info = helpers.launch(cam, W, H, bufs, frame=f, samples=0, accumulate=False, max_depth=2)
        kgr.set_quad_lights(info, dq.data_ptr(), len(quads))
        env.attach_to(info)
        att.render(info, sc)
        p = helpers.oracle_params(cam, W, H, max_depth=2, spp=1, frame=f, samples=0, accumulate=0, candidates=32,
                                  temporal=1, temporal_mcap=20, spatial_passes=1, spatial_neighbors=5,
                                  spatial_radius=30)
        pyoracle.render_restir(osc, p, state, ref)
    torch.cuda.synchronize()
    res_a = att.debug_copy("reservoir_prev_a", np.zeros((n, 4), np.float32))
    res_b = att.debug_copy("reservoir_prev_b", np.zeros((n, 4), np.float32))
    att.close()
    env.close()
    A = state.arrays
    light = res_a[:, 3].view(np.int32)
    valid = A["prev_M"] > 0
    same = (light == A["prev_light"]) & np.all(res_a[:, :3] == A["prev_point"], axis=1)
    kinds = {"quad": (light >= 0) & (light < len(quads)), "triangle": light >= len(quads), "environment": light < -1}
    color = bufs[0].cpu().numpy()
    close = np.all(rel_ok(color, ref[0]), axis=1).mean()
    exact = np.all(color.view(np.uint32) == ref[0].view(np.uint32), axis=1).mean()
    print(f"ReSTIR DI quads+env {layout}: selection agreement {same[valid].mean():.6f}, colour exact {exact:.6f}, "
          f"within 1e-4 {close:.6f}; selected " + ", ".join(f"{k} {v[valid].mean():.3f}" for k, v in kinds.items()))
    assert valid.mean() > 0.5
    assert same[valid].mean() >= 0.999
    np.testing.assert_array_equal(res_b[:, 2].view(np.int32), A["prev_M"])
    assert np.all(rel_ok(res_b[:, 1], A["prev_W"])[valid]) or rel_ok(res_b[:, 1], A["prev_W"])[valid].mean() >= 0.999
    assert close >= 0.999
    for k in ("quad", "environment"):
        assert kinds[k][valid].mean() > 0.01, k


def test_consumers_without_extra_lights_refuse_them(terrain_s):
    """ReSTIR GI and the radiance cache light with the scene's triangles
    only: a launch with quads or an environment map is refused."""
    g, sc, _ = terrain_s
    W = H = 32
    env = kgr.Environment(smooth_sky(), kgr.FILTER_LINEAR)
    cam = kgr.camera(g.eye, g.target, g.fov, 1.0)
    bufs = helpers.device_buffers(torch, W * H)
    for kind, opts in (("restir_gi", {}), ("path_tracer", {"cache": True})):
        att = kgr.Attachment(kind)
        att.attach(W, H)
        att.load()
        for k, v in opts.items():
            att.set_option(k, v)
        info = env.attach_to(helpers.launch(cam, W, H, bufs, max_depth=2))
        assert kgr.lib().kgr_render(att.handle, __import__("ctypes").byref(info), sc.handle, None) == 4
        att.close()
    env.close()
