"""The autotuner: every traversal launch shape (layout fast or wide, shadow
kernel, block size, occupancy) renders the same image, so tuning changes speed only --
the frame after kgr_autotune is bit-identical to the frame before it, for an
attachment and for the batcher; options still override the tuned shape."""
import numpy as np
import pytest

from artemis_gb300 import kgr
from tests import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["path_tracer", "restir_di"])
def test_attachment_autotune_keeps_the_image(kind):
    g, sc, _ = helpers.both("box4k", 1)
    W = H = 96
    cam = kgr.camera(g.eye, g.target, g.fov, 1.0)
    bufs = helpers.device_buffers(torch, W * H)
    att = kgr.Attachment(kind)
    att.attach(W, H)
    att.load()
    if kind == "path_tracer":
        att.set_option("spp", 2)
    else:
        att.set_option("temporal", False)
    att.set_option("russian_roulette", True)
    info = helpers.launch(cam, W, H, bufs, frame=5, max_depth=4)
    assert att.trace_tune() == {"layout": "fast", "shadow": "grid", "block": 128, "occupancy": 0}
    att.render(info, sc)
    torch.cuda.synchronize()
    before = bufs[0].clone()
    res = att.autotune(info, sc, frames=2)
    assert res["candidates"] == 24  # fast and wide x 2 shadow kernels x 3 block sizes x 2 occupancies
    assert 0 < res["best_ms"] <= res["default_ms"]
    assert att.trace_tune() == res["best"]
    att.render(info, sc)
    torch.cuda.synchronize()
    assert torch.equal(bufs[0].view(torch.int32), before.view(torch.int32))
    # options override the tuned shape field by field
    att.set_option("trace_block", 64)
    att.set_option("layout", "fast")
    t = att.trace_tune()
    assert t["block"] == 64 and t["layout"] == "fast" and t["shadow"] == res["best"]["shadow"]
    att.close()


def test_batcher_autotune_keeps_the_image():
    g, sc, _ = helpers.both("box4k", 1)
    dims = [(64, 48), (40, 40)]
    outs = [torch.zeros((w * h, 4), dtype=torch.float32, device="cuda") for w, h in dims]
    jobs = [kgr.batch_job(kgr.camera(g.eye, g.target, g.fov, w / h), w, h, 3, o.data_ptr(), frame=7)
            for (w, h), o in zip(dims, outs)]
    b = kgr.Batcher(1 << 16, 8)
    b.render(sc, jobs, max_depth=4)
    torch.cuda.synchronize()
    before = [o.clone() for o in outs]
    res = b.autotune(sc, jobs, frames=2, max_depth=4)
    assert res["candidates"] == 24 and 0 < res["best_ms"] <= res["default_ms"]
    layout = {"fast": kgr.LAYOUT_FAST, "wide": kgr.LAYOUT_WIDE}[res["best"]["layout"]]
    b.render(sc, jobs, max_depth=4, layout=layout)
    torch.cuda.synchronize()
    for o, ref in zip(outs, before):
        assert torch.equal(o.view(torch.int32), ref.view(torch.int32))
    b.close()
