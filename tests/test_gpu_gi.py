"""ReSTIR GI on the GPU against the oracle's restatement of the same
specification: three frames of an orbiting camera (temporal reuse through
reprojection), 3 spatial iterations of 8 neighbours.  Tolerance: colour
within 1e-4 relative on >= 99.9% of pixels, final reservoirs equal."""
import math

import numpy as np
import pytest

from artemis_gb300 import kgr
from oracle import pyoracle
from tests import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def orbit(g, f, deg=0.5):
    e = g.eye - g.target
    a = math.radians(deg * f)
    ca, sa = math.cos(a), math.sin(a)
    eye = np.array([ca * e[0] + sa * e[2], e[1], -sa * e[0] + ca * e[2]], np.float32) + g.target
    return eye


def rel_ok(a, b, rtol=1e-4, atol=1e-6):
    return np.abs(a - b) <= rtol * np.maximum(np.abs(a), np.abs(b)) + atol


# 16 neighbours: the most an iteration allows, every neighbour slot in use
@pytest.mark.parametrize("layout,neighbors", [("fast", 8), ("threaded", 8), ("wide", 8), ("fast", 16)])
def test_restir_gi_matches_oracle(layout, neighbors):
    g, sc, osc = helpers.both("box4k", 1)
    W, H, frames = 64, 64, 3
    bufs = helpers.device_buffers(torch, W * H)
    att = kgr.Attachment("restir_gi")
    att.attach(W, H)
    att.load()
    att.set_option("layout", layout)
    att.set_option("gi_neighbors", neighbors)
    state = pyoracle.GiState(W * H, temporal=True, mcap=30, iterations=3, neighbors=neighbors, radius=30)
    ocolor = np.zeros((W * H, 4), np.float32)
    prev = None
    for f in range(frames):
        cam = kgr.camera(orbit(g, f), g.target, g.fov, 1.0)
        att.render(helpers.launch(cam, W, H, bufs, frame=f, max_depth=2), sc)
        d = kgr.camera_dict(cam)
        if prev is not None:
            d["prev_projection"], d["prev_view"] = prev["projection"], prev["view"]
        p = pyoracle.render_params(W, H, d, max_depth=2, frame=f)
        pyoracle.render_gi(osc, p, state, ocolor)
        prev = kgr.camera_dict(cam)
    torch.cuda.synchronize()
    color = bufs[0].cpu().numpy()
    close = np.all(rel_ok(color, ocolor), axis=1).mean()
    exact = np.all(color.view(np.uint32) == ocolor.view(np.uint32), axis=1).mean()
    ra = att.debug_copy("gi_reservoir_a", np.zeros((W * H, 4), np.float32))
    rb = att.debug_copy("gi_reservoir_b", np.zeros((W * H, 4), np.float32))
    same = np.all(ra.view(np.uint32) == state.arrays["res_a"].view(np.uint32), axis=1).mean()
    print(f"GI {layout}/{neighbors}: colour exact {exact:.6f}, within 1e-4 {close:.6f}, reservoirs equal {same:.6f}")
    assert close >= 0.999
    assert same >= 0.999
    assert np.all(rel_ok(rb, state.arrays["res_b"]), axis=1).mean() >= 0.999
    assert color[:, :3].mean() > 0.01
    att.close()
