"""The autotuner: every traversal launch shape (layout fast, wide or cw8, shadow
kernel, block size, occupancy, shared-memory stack entries) renders the same image, so tuning changes speed only --
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
    assert att.trace_tune() == {"layout": "fast", "shadow": "persistent", "block": 128, "occupancy": 0, "stack": 0}
    att.render(info, sc)
    torch.cuda.synchronize()
    before = bufs[0].clone()
    res = att.autotune(info, sc, frames=2)
    # fast, wide and cw8 x 2 shadow kernels x 3 block sizes x 2 occupancies, then the best with 8
    # and 16 shared-memory stack entries
    assert res["candidates"] == 38
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
    assert res["candidates"] == 38 and 0 < res["best_ms"] <= res["default_ms"]
    layout = {"fast": kgr.LAYOUT_FAST, "wide": kgr.LAYOUT_WIDE, "cw8": kgr.LAYOUT_CW8}[res["best"]["layout"]]
    b.render(sc, jobs, max_depth=4, layout=layout)
    torch.cuda.synchronize()
    for o, ref in zip(outs, before):
        assert torch.equal(o.view(torch.int32), ref.view(torch.int32))
    b.close()


@pytest.mark.parametrize("layout", ["fast", "wide"])
@pytest.mark.parametrize("shadow", ["grid", "persistent"])
def test_shared_memory_stacks_keep_the_image(layout, shadow):
    """trace_stack 8 and 16 keep the top of each traversal stack in shared
    memory and spill deeper entries to local memory (the terrain's walks go
    deeper than 8 entries); every pixel and AOV stays bit-identical."""
    g, sc, _ = helpers.both("terrain_s", 1)
    assert sc.info().wide_max_stack > 16
    W, H = 160, 96
    cam = kgr.camera(g.eye, g.target, g.fov, W / H)
    out = {}
    for k in (0, 8, 16):
        bufs = helpers.device_buffers(torch, W * H)
        att = kgr.Attachment("path_tracer")
        att.attach(W, H)
        att.load()
        att.set_option("spp", 3)
        att.set_option("russian_roulette", True)
        att.set_option("layout", layout)
        att.set_option("trace_shadow", shadow)
        att.set_option("trace_stack", k)
        assert att.trace_tune()["stack"] == k
        att.render(helpers.launch(cam, W, H, bufs, frame=2, max_depth=6), sc)
        torch.cuda.synchronize()
        out[k] = [b.cpu().numpy() for b in bufs]
        att.close()
    for k in (8, 16):
        for a, b in zip(out[0], out[k]):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_batcher_shared_memory_stack_keeps_the_image():
    g, sc, _ = helpers.both("terrain_s", 1)
    dims = [(96, 64), (50, 40)]
    res = {}
    for k in (0, 16):
        outs = [torch.zeros((w * h, 4), dtype=torch.float32, device="cuda") for w, h in dims]
        jobs = [kgr.batch_job(kgr.camera(g.eye, g.target, g.fov, w / h), w, h, 2, o.data_ptr(), frame=3)
                for (w, h), o in zip(dims, outs)]
        b = kgr.Batcher(1 << 15, 4)
        b.set_tune(shadow=kgr.TRACE_PERSISTENT, block=64, occupancy=1, stack=k)
        for _ in range(3):  # eager, capture, replay
            b.render(sc, jobs, max_depth=5)
        torch.cuda.synchronize()
        res[k] = [o.cpu().numpy() for o in outs]
        b.close()
    for a, b in zip(res[0], res[16]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
