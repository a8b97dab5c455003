"""kgr_render_pt_noalloc: a path-traced frame for callers that cannot
allocate device memory when they render (a host that fixes its device memory
at start-up and hands it out itself).  Its scratch is a
fixed array inside the library, so this checks, through the C ABI, that two
calls in a row each give the same image as the path-tracer attachment (the
existing entry point) within the 1e-4 relative tolerance of the parity
tests, and that a request beyond the 65536-path limit is refused cleanly.

Kept in its own file that sorts last, so a run that stops at the first
failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from artemis_gb300 import kgr
from tests import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

RTOL = 1e-4


def close(a, b):
    return np.abs(a - b) <= RTOL * np.maximum(np.abs(a), np.abs(b)) + 1e-6


def attachment_frame(g, sc, W, H, spp, frame):
    cam = kgr.camera(g.eye, g.target, g.fov, W / H)
    bufs = helpers.device_buffers(torch, W * H)
    att = kgr.Attachment("path_tracer")
    att.attach(W, H)
    att.load()
    att.set_option("spp", spp)
    att.set_option("russian_roulette", True)
    att.set_option("rr_start_depth", 2)
    att.render(helpers.launch(cam, W, H, bufs, max_depth=5, frame=frame), sc)
    torch.cuda.synchronize()
    att.close()
    return [b.cpu().numpy() for b in bufs]


def noalloc_frame(g, sc, W, H, spp, frame):
    cam = kgr.camera(g.eye, g.target, g.fov, W / H)
    bufs = helpers.device_buffers(torch, W * H)
    info = helpers.launch(cam, W, H, bufs, max_depth=5, frame=frame)
    kgr.check(kgr.lib().kgr_render_pt_noalloc(sc.handle, ctypes.byref(info), spp, 1, 2, None))
    torch.cuda.synchronize()
    return [b.cpu().numpy() for b in bufs]


def test_noalloc_matches_attachment_two_calls_in_a_row():
    g = kgr.Generated("box4k", 1)
    sc = kgr.Scene.from_generated(g)
    W, H, spp = 96, 96, 4  # 36864 paths, within the 65536-path limit
    for frame in (0, 1):
        want = attachment_frame(g, sc, W, H, spp, frame)
        got = noalloc_frame(g, sc, W, H, spp, frame)
        for k in range(4):
            assert np.all(close(got[k], want[k]), axis=1).mean() == 1.0, (frame, k)
        assert want[0][:, :3].mean() > 0.01
    sc.close()


def test_noalloc_rejects_requests_over_the_limit():
    g = kgr.Generated("box64", 3)
    sc = kgr.Scene.from_generated(g)
    W, H = 256, 256
    cam = kgr.camera(g.eye, g.target, g.fov, 1.0)
    bufs = helpers.device_buffers(torch, W * H)
    info = helpers.launch(cam, W, H, bufs, max_depth=3)
    status = kgr.lib().kgr_render_pt_noalloc(sc.handle, ctypes.byref(info), 2, 0, 3, None)
    assert status == 1
    assert b"65536" in kgr.lib().kgr_last_error()
    # extents that are not whole numbers in [1, 65536] are refused before any
    # conversion or launch (-256 x -256 would otherwise wrap to 65536 paths)
    for res in ((-256.0, -256.0), (float("nan"), 16.0), (16.5, 16.0), (0.0, 8.0), (1e30, 1.0)):
        bad = helpers.launch(cam, W, H, bufs, max_depth=3)
        bad.resolution[0], bad.resolution[1] = res
        assert kgr.lib().kgr_render_pt_noalloc(sc.handle, ctypes.byref(bad), 1, 0, 3, None) == 1, res
    # the largest allowed request still works after the refusal
    kgr.check(kgr.lib().kgr_render_pt_noalloc(sc.handle, ctypes.byref(info), 1, 0, 3, None))
    torch.cuda.synchronize()
    assert np.isfinite(bufs[0].cpu().numpy()).all()
    sc.close()
