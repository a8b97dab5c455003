"""Parity of the "mamba" attachment -- the editor's default GI mode
(Mamba::render, editor/mamba.cu:941-1312; editor/optix/mamba_shader.cu;
editor/optix/probe.cuh; editor/mamba_kernels.cu) -- with the oracle's
restatement (oracle_mamba_*, oracle/oracle.cpp).

Each case renders six frames: three from one camera (samples 0, 1, 2), then
the camera moves (samples back to 0, the temporal pass reprojects) and three
more.  Every frame's image, and after the last frame every buffer of the
state -- G-buffer, current and previous reservoirs, accumulated direct
light, secondary rays, Sobel, probe raster, groups, and the whole probe
table (lookup-table headers, refs, hashes, cell and probe positions,
probe normals, bin radiance sums in fixed point, counts and depth stamps)
-- are compared bit for bit.  Tolerance: exact (integer, index and hash
work; float arithmetic in the same order on both sides)."""
import numpy as np
import pytest

from artemis_gb300 import kgr
from oracle import pyoracle
from tests import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

W, H = 128, 96
MAX_PROBES, MAX_LUTS = 1 << 14, 16
FRAMES = 6


def orbit(g, deg):
    e = np.asarray(g.eye, np.float64) - np.asarray(g.target, np.float64)
    a = np.radians(deg)
    ca, sa = np.cos(a), np.sin(a)
    return (np.array([ca * e[0] + sa * e[2], e[1], -sa * e[0] + ca * e[2]]) + g.target).astype(np.float32)


def blocky_sky(w=16, h=8, seed=5):
    rng = np.random.default_rng(seed)
    t = rng.uniform(0.1, 1.5, (h, w, 4)).astype(np.float32)
    t[..., 3] = 1.0
    return t


def same(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def first_difference(a, b):
    """(number of differing rows, the first few) of two equally shaped arrays."""
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    if a.shape != b.shape:
        return ("shape", a.shape, b.shape)
    av = a.reshape(a.shape[0], -1).view(np.uint8)
    bv = b.reshape(b.shape[0], -1).view(np.uint8)
    rows = np.nonzero(np.any(av != bv, axis=1))[0]
    return len(rows), rows[:5].tolist()


def run(name, layout, flags, sky=None, frames=FRAMES, compare_every_frame=True, size=(W, H),
        tables=(MAX_PROBES, MAX_LUTS)):
    """Renders `frames` frames on the GPU and the oracle; returns the two
    attachments' final buffers and the per-frame colour agreement."""
    W, H = size
    max_probes, max_luts = tables
    g, sc, osc = helpers.both(name, 1)
    env = None
    if sky is not None:
        env = kgr.Environment(sky, kgr.FILTER_POINT)
        osc = pyoracle.Scene(g.positions, g.normals, g.tris4(), g.materials_raw, sc.lights(), sc.bvh(), env=sky,
                             env_filter=kgr.FILTER_POINT)
    att = kgr.Attachment("mamba")
    att.attach(W, H)
    for k, v in {**flags, "layout": layout, "max_probes": max_probes, "max_luts": max_luts}.items():
        att.set_option(k, v)
    att.load()
    om = pyoracle.Mamba(W, H, max_probes, max_luts)
    bufs = helpers.device_buffers(torch, W * H)
    oflags = {k: int(v) for k, v in flags.items()}
    prev = None
    colors = []
    for f in range(frames):
        moved = f >= 3
        eye = orbit(g, 4.0) if moved else g.eye
        samples = f - 3 if moved else f
        cam = kgr.camera(eye, g.target, g.fov, W / H)
        info = helpers.launch(cam, W, H, bufs, samples=samples)
        info.time = 0.25 * f
        if env is not None:
            env.attach_to(info)
        att.render(info, sc)
        d = kgr.camera_dict(cam)
        ocolor, _ = om.frame(osc, pyoracle.mamba_params(W, H, d, prev=prev, time=0.25 * f, samples=samples, **oflags))
        prev = d
        if compare_every_frame or f == frames - 1:
            torch.cuda.synchronize()
            colors.append((bufs[0].cpu().numpy(), ocolor.copy()))
    torch.cuda.synchronize()
    out = {}
    for name_, (dt, w) in pyoracle.MAMBA_BUFFERS.items():
        ob = om.buffer(name_)
        gb = np.zeros_like(ob)
        att.debug_copy("mamba_" + name_, gb)
        out[name_] = (gb, ob)
    att.close()
    om.close()
    if env is not None:
        env.close()
    sc.close()
    return out, colors


def check(out, colors, label):
    for f, (gc, oc) in enumerate(colors):
        exact = np.all(gc.view(np.uint32) == oc.view(np.uint32), axis=1).mean()
        print(f"{label} frame {f}: colour exact {exact:.6f}, mean {gc[:, :3].mean():.5f}")
        assert same(gc, oc), f"frame {f}: {first_difference(gc, oc)}"
    bad = {k: first_difference(*v) for k, v in out.items() if not same(*v)}
    assert not bad, f"buffers differ: {bad}"
    counters = out["counters"][0].ravel()
    print(f"{label}: {counters[0]} probes, {counters[1]} lookup tables, "
          f"{int(out['bin_n'][0].sum())} splats, raster coverage {out['raster'][0].mean():.3f}")
    return counters


DIRECT = {"direct_lighting": True, "temporal_reuse": True, "spatial_reuse": True}


@pytest.mark.parametrize("flags", [
    {},
    {"direct_lighting": True},
    {"direct_lighting": True, "temporal_reuse": True},
    {"direct_lighting": True, "spatial_reuse": True},
    DIRECT,
], ids=["irradiance", "direct", "direct+temporal", "direct+spatial", "direct+temporal+spatial"])
def test_mamba_box_scene_matches_oracle(flags):
    out, colors = run("box4k", "fast", flags)
    counters = check(out, colors, f"box4k {sorted(flags)}")
    assert counters[0] > 10 and counters[1] >= 2
    assert colors[-1][0][:, :3].mean() > 0.01


def test_mamba_1080p_terrain_matches_oracle():
    """The benchmark's configuration as configured: 1920x1080 on the
    1.16M-triangle terrain (half GGX), direct lighting with temporal and
    spatial reuse, three frames with the state carried; every buffer bit
    for bit."""
    out, colors = run("terrain", "fast", DIRECT, frames=3, compare_every_frame=False, size=(1920, 1080),
                      tables=(1 << 16, 64))
    counters = check(out, colors, "terrain 1080p")
    assert counters[0] > 100


@pytest.mark.parametrize("layout", ["fast", "cw8", "threaded"])
def test_mamba_ggx_terrain_matches_oracle(layout):
    """The 0.26M-triangle terrain: half its materials GGX, so the secondary
    rays' BSDF samples, the probe gather's BRDF/pdf and the reservoirs'
    targets take the GGX lobe."""
    out, colors = run("terrain_s", layout, DIRECT)
    counters = check(out, colors, f"terrain_s {layout}")
    assert counters[0] > 10
    mats = out["s_hit_mat"][0]
    assert len(np.unique(mats)) > 1


def test_mamba_environment_matches_oracle():
    """A point-sampled environment map: the sky is one more light of
    sample_light, the secondary rays' misses read it, and so do the final
    gather's background pixels (sky_at, editor/optix/common.cuh:18-31)."""
    out, colors = run("terrain_s", "fast", DIRECT, sky=blocky_sky())
    check(out, colors, "terrain_s sky")
    gc = colors[-1][0]
    g_index = out["g_index"][0]
    assert (g_index == -1).any() and gc[g_index == -1, :3].max() > 0.05
    sky_lights = out["res_r1"][0][:, 3] != 0
    assert sky_lights.any()


@pytest.mark.parametrize("view", ["indirect_lighting", "render_probes", "render_probe_radiance"])
def test_mamba_debug_views_match_oracle(view):
    """The other switches of Mamba::options (editor/mamba.cuh:60-67): the
    secondary radiance instead of the probes, and the probe indicator and
    probe radiance overlays of raster_probes."""
    out, colors = run("box4k", "fast", {"direct_lighting": True, view: True}, frames=4)
    check(out, colors, f"box4k {view}")


def test_mamba_refuses_quad_lights():
    g, sc, _ = helpers.both("box64", 3)
    att = kgr.Attachment("mamba")
    att.attach(32, 32)
    att.set_option("max_probes", 256)
    att.set_option("max_luts", 4)
    att.load()
    bufs = helpers.device_buffers(torch, 32 * 32)
    info = helpers.launch(kgr.camera(g.eye, g.target, g.fov, 1.0), 32, 32, bufs)
    q = torch.zeros((1, 12), dtype=torch.float32, device="cuda")
    kgr.set_quad_lights(info, q.data_ptr(), 1)
    with pytest.raises(kgr.KgrError) as e:
        att.render(info, sc)
    assert e.value.status == 4  # KGR_ERR_UNSUPPORTED
    att.close()
    sc.close()


def test_mamba_stage_times_and_launches():
    g, sc, _ = helpers.both("box4k", 1)
    att = kgr.Attachment("mamba")
    att.attach(W, H)
    for k, v in {**DIRECT, "profile": True, "max_probes": MAX_PROBES, "max_luts": MAX_LUTS}.items():
        att.set_option(k, v)
    att.load()
    bufs = helpers.device_buffers(torch, W * H)
    cam = kgr.camera(g.eye, g.target, g.fov, W / H)
    for f in range(3):
        att.render(helpers.launch(cam, W, H, bufs, samples=f), sc)
    t = att.stage_times()
    for k in ("generate", "trace_closest", "restir_primary", "restir_temporal", "restir_spatial",
              "restir_temporal_vis", "restir_spatial_vis", "mamba_secondary", "mamba_gather", "mamba_probes",
              "mamba_final"):
        assert t[k][1] > 0 and t[k][0] > 0.0, k
    # G-buffer 3, primary 3, temporal 3 (2 rays + merge; spatial follows), spatial 5,
    # secondary 1, splat 2, Sobel + raster + collapse + allocation 5, final gather 1
    assert att.stats().kernel_launches == 23
    att.close()
    sc.close()


def test_mamba_reset_history_restarts_the_state():
    """reset_history clears the reservoirs, the direct light, the secondary
    records and the probe table: three frames after a reset equal three
    frames of a fresh attachment, buffers included."""
    g, sc, _ = helpers.both("box4k", 1)
    cam = kgr.camera(g.eye, g.target, g.fov, W / H)

    def frames(att, bufs, n):
        for f in range(n):
            info = helpers.launch(cam, W, H, bufs, samples=f)
            info.time = 0.25 * f
            att.render(info, sc)
        torch.cuda.synchronize()
        return bufs[0].cpu().numpy()

    def make():
        att = kgr.Attachment("mamba")
        att.attach(W, H)
        for k, v in {**DIRECT, "max_probes": MAX_PROBES, "max_luts": MAX_LUTS}.items():
            att.set_option(k, v)
        att.load()
        return att

    a, b = make(), make()
    ba, bb = helpers.device_buffers(torch, W * H), helpers.device_buffers(torch, W * H)
    frames(a, ba, 3)
    a.set_option("reset_history", True)
    ca = frames(a, ba, 3)
    cb = frames(b, bb, 3)
    assert same(ca, cb)
    for name in ("bin_le", "bin_n", "refs", "probe_pos", "res_r3", "prev_r3", "direct_le", "s_le", "raster"):
        dt, w = pyoracle.MAMBA_BUFFERS[name]
        n = pyoracle.Mamba(W, H, MAX_PROBES, MAX_LUTS)
        ref = n.buffer(name)
        n.close()
        xa, xb = np.zeros_like(ref), np.zeros_like(ref)
        a.debug_copy("mamba_" + name, xa)
        b.debug_copy("mamba_" + name, xb)
        assert same(xa, xb), name
    a.close()
    b.close()
    sc.close()


def test_mamba_full_tables_match_oracle():
    """A table of 16 probes fills in the first frame: the later allocations
    find no probe left (a second-level slot is then not claimed), and the
    frames stay bit-exact with the oracle's."""
    out, colors = run("box4k", "fast", DIRECT, frames=4, tables=(16, 2))
    counters = check(out, colors, "box4k 16 probes")
    assert counters[0] == 16 and counters[1] == 2
