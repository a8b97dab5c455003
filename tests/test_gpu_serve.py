"""The render server: a request gives the same image alone and in a mix of
other requests (bit for bit, and equal to the attachment's render);
admission keeps the admitted buffers within the memory budget; bad requests
are refused at submission without disturbing the others; waits time out;
a ReSTIR DI request equals the attachment's frames from a fresh history."""
import numpy as np
import pytest

from artemis_gb300 import kgr
from tests import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DEPTH = 6


def attachment_render(sc, g, w, h, spp, frame, eye, kind="path_tracer", rr=True, frames=1):
    cam = kgr.camera(eye, g.target, g.fov, w / h)
    bufs = helpers.device_buffers(torch, w * h)
    att = kgr.Attachment(kind)
    att.attach(w, h)
    att.load()
    if kind == "path_tracer":
        att.set_option("spp", spp)
    att.set_option("russian_roulette", rr)
    att.set_option("rr_start_depth", 3)
    for i in range(frames):
        att.render(helpers.launch(cam, w, h, bufs, frame=frame + i, max_depth=DEPTH, accumulate=i > 0, samples=i), sc)
    torch.cuda.synchronize()
    att.close()
    return bufs[0].cpu().numpy()


def eye_of(g, i):
    return (np.array(g.eye, np.float32) + np.float32(0.05) * i).tolist()


@pytest.mark.parametrize("policy,autotune", [(kgr.SCHEDULE_FCFS, False), (kgr.SCHEDULE_FAIR, False),
                                             (kgr.SCHEDULE_FAIR, True)])
def test_same_image_alone_and_in_the_mix(policy, autotune):
    """Under either scheduling policy, with or without per-scene tuning of
    the traversal launch shape, a request gives the same image alone, in a
    mix, and as the attachment renders it."""
    g, sc, _ = helpers.both("box4k", 1)
    w, h, spp, frame = 80, 60, 5, 11
    srv = kgr.Server(path_capacity=1 << 15, max_jobs=8, spp_per_tick=2, policy=policy, autotune=autotune)
    sid = srv.add_scene(sc)
    alone = np.zeros((w * h, 4), np.float32)
    r = srv.wait(srv.submit(sid, w, h, spp, eye_of(g, 0), g.target, g.fov, alone, max_depth=DEPTH, frame=frame),
                 60000.0)
    assert r.status == 0 and r.done and r.ticks == 3
    # the same request among others of other sizes, spp and cameras
    mix = [(64, 64, 3), (120, 20, 7), (w, h, spp), (33, 17, 1), (100, 90, 4), (48, 48, 9)]
    outs, ids = [], []
    for i, (mw, mh, ms) in enumerate(mix):
        out = np.zeros((mw * mh, 4), np.float32)
        same = (mw, mh, ms) == (w, h, spp)
        ids.append(srv.submit(sid, mw, mh, ms, eye_of(g, 0 if same else i + 1), g.target, g.fov, out,
                              max_depth=DEPTH, frame=frame if same else i))
        outs.append(out)
    res = [srv.wait(i, 60000.0) for i in ids]
    assert all(x.status == 0 for x in res)
    st = srv.stats()
    assert st.completed == 1 + len(mix) and st.failed == 0
    assert st.mean_jobs_per_tick > 1.0  # requests shared ticks
    assert st.latency_p99_ms >= st.latency_p50_ms > 0.0
    srv.close()
    in_mix = outs[2]
    assert np.array_equal(alone, in_mix)
    ref = attachment_render(sc, g, w, h, spp, frame, eye_of(g, 0))
    assert np.array_equal(alone, ref)
    for (mw, mh, ms), out, i in zip(mix, outs, range(len(mix))):
        if (mw, mh, ms) != (w, h, spp):
            assert np.array_equal(out, attachment_render(sc, g, mw, mh, ms, i, eye_of(g, i + 1)))


def test_admission_stays_within_budget():
    g, sc, _ = helpers.both("box64", 1)
    w, h = 64, 48
    budget = w * h * 16 * 2 + 100  # two requests' accumulation buffers
    srv = kgr.Server(path_capacity=1 << 15, max_jobs=8, spp_per_tick=1, memory_budget=budget)
    sid = srv.add_scene(sc)
    outs = [np.zeros((w * h, 4), np.float32) for _ in range(6)]
    ids = [srv.submit(sid, w, h, 3, eye_of(g, i), g.target, g.fov, outs[i], max_depth=DEPTH, frame=i)
           for i in range(6)]
    res = [srv.wait(i, 60000.0) for i in ids]
    st = srv.stats()
    srv.close()
    assert all(r.status == 0 for r in res)
    assert 0 < st.peak_budget_bytes <= budget
    assert max(r.queue_ms for r in res) > 0.0  # later requests waited for budget
    for i in range(6):
        assert np.array_equal(outs[i], attachment_render(sc, g, w, h, 3, i, eye_of(g, i)))


def test_bad_requests_are_refused_and_others_finish():
    g, sc, _ = helpers.both("box64", 1)
    srv = kgr.Server(path_capacity=4096, max_jobs=4, memory_budget=1 << 20)
    sid = srv.add_scene(sc)
    out = np.zeros((32 * 32, 4), np.float32)
    ok = srv.submit(sid, 32, 32, 2, g.eye, g.target, g.fov, out, max_depth=DEPTH)
    for kw in ({"scene_id": sid + 5}, {"width": 0}, {"width": 128, "height": 64}, {"spp": 0},
               {"width": 300, "height": 300}):
        args = dict(scene_id=sid, width=32, height=32, spp=1)
        args.update(kw)
        with pytest.raises(kgr.KgrError):
            srv.submit(args["scene_id"], args["width"], args["height"], args["spp"], g.eye, g.target, g.fov,
                       max_depth=DEPTH)
    assert srv.wait(ok, 60000.0).status == 0
    # a wait that cannot be satisfied in time reports KGR_ERR_TIMEOUT
    big = srv.submit(sid, 64, 64, 64, g.eye, g.target, g.fov, max_depth=DEPTH)
    with pytest.raises(kgr.KgrError) as e:
        srv.wait(big, 0.0)
    assert e.value.status == 9
    assert srv.wait(big, 120000.0).status == 0
    srv.close()
    assert np.array_equal(out, attachment_render(sc, g, 32, 32, 2, 0, g.eye))


def test_shutdown_fails_unfinished_requests_without_hanging():
    g, sc, _ = helpers.both("box64", 1)
    srv = kgr.Server(path_capacity=4096, max_jobs=2, spp_per_tick=1)
    sid = srv.add_scene(sc)
    for i in range(20):
        srv.submit(sid, 64, 64, 16, eye_of(g, i), g.target, g.fov, max_depth=DEPTH, frame=i)
    srv.close()  # returns once the device work in flight is done


def test_restir_request_equals_attachment_frames():
    g, sc, _ = helpers.both("box4k", 1)
    w, h, frames, frame = 72, 56, 3, 4
    srv = kgr.Server(path_capacity=1 << 15, max_jobs=4)
    sid = srv.add_scene(sc)
    outs = []
    for _ in range(2):  # the second request reuses the resident attachment
        out = np.zeros((w * h, 4), np.float32)
        r = srv.wait(srv.submit(sid, w, h, frames, g.eye, g.target, g.fov, out, kind=kgr.REQUEST_RESTIR_DI,
                                max_depth=DEPTH, frame=frame, russian_roulette=False), 60000.0)
        assert r.status == 0
        outs.append(out)
    srv.close()
    ref = attachment_render(sc, g, w, h, 1, frame, g.eye, kind="restir_di", rr=False, frames=frames)
    assert np.array_equal(outs[0], ref)
    assert np.array_equal(outs[1], ref)


def test_fair_policy_serves_small_requests_beside_a_large_one():
    """Processor sharing: small requests submitted behind a large one finish
    first; under FCFS the large one holds the ticks until it is done."""
    g, sc, _ = helpers.both("box4k", 1)
    lat = {}
    for policy in (kgr.SCHEDULE_FCFS, kgr.SCHEDULE_FAIR):
        srv = kgr.Server(path_capacity=1 << 16, max_jobs=8, spp_per_tick=2, policy=policy)
        sid = srv.add_scene(sc)
        big = srv.submit(sid, 256, 256, 16, g.eye, g.target, g.fov, max_depth=DEPTH, frame=1)
        small = [srv.submit(sid, 32, 32, 2, eye_of(g, i), g.target, g.fov, max_depth=DEPTH, frame=2 + i)
                 for i in range(4)]
        rb = srv.wait(big, 120000.0)
        rs = [srv.wait(i, 120000.0) for i in small]
        srv.close()
        assert rb.status == 0 and all(r.status == 0 for r in rs)
        lat[policy] = (rb.latency_ms, max(r.latency_ms for r in rs))
    # FCFS: the small requests wait for the large one; FAIR: they do not
    assert lat[kgr.SCHEDULE_FCFS][1] >= 0.5 * lat[kgr.SCHEDULE_FCFS][0]
    assert lat[kgr.SCHEDULE_FAIR][1] < 0.5 * lat[kgr.SCHEDULE_FAIR][0]
