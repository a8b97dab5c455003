"""Batched path tracing: images of different sizes, cameras, frames and
sample slices in one shared wavefront frame give, bit for bit, what the
path_tracer attachment renders for each alone -- also when a job's samples
are spread over several frames, and when the frame is a CUDA graph replay."""
import numpy as np
import pytest

from artemis_gb300 import kgr
from tests import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

DEPTH = 6


def cam_for(g, i, w, h):
    eye = np.array(g.eye, np.float32) + np.float32(0.07) * i
    return kgr.camera(eye, g.target, g.fov, w / h)


def single(sc, cam, w, h, spp, frame):
    bufs = helpers.device_buffers(torch, w * h)
    att = kgr.Attachment("path_tracer")
    att.attach(w, h)
    att.load()
    att.set_option("spp", spp)
    att.set_option("russian_roulette", True)
    att.set_option("rr_start_depth", 3)
    att.render(helpers.launch(cam, w, h, bufs, frame=frame, max_depth=DEPTH), sc)
    torch.cuda.synchronize()
    att.close()
    return [b.cpu().numpy() for b in bufs]


SPECS = [(64, 48, 3, 5), (40, 40, 1, 9), (96, 30, 2, 0), (17, 23, 4, 2)]  # width, height, spp, frame


def job_buffers(w, h):
    return helpers.device_buffers(torch, w * h)


def test_batch_equals_single_renders():
    g, sc, _ = helpers.both("box4k", 1)
    cams = [cam_for(g, i, w, h) for i, (w, h, _, _) in enumerate(SPECS)]
    bufs = [job_buffers(w, h) for (w, h, _, _) in SPECS]
    jobs = [kgr.batch_job(cams[i], w, h, spp, *[b.data_ptr() for b in bufs[i][:1]], frame=f,
                          normal=bufs[i][1].data_ptr(), albedo=bufs[i][2].data_ptr(), position=bufs[i][3].data_ptr())
            for i, (w, h, spp, f) in enumerate(SPECS)]
    b = kgr.Batcher(1 << 16, 16)
    b.render(sc, jobs, max_depth=DEPTH, use_graph=False)
    torch.cuda.synchronize()
    counts = b.ray_counts()
    assert counts[0] == sum(w * h * s for (w, h, s, _) in SPECS)
    for i, (w, h, spp, f) in enumerate(SPECS):
        ref = single(sc, cams[i], w, h, spp, f)
        got = [x.cpu().numpy() for x in bufs[i]]
        for k in range(4):
            assert np.array_equal(got[k], ref[k]), (i, k)
    b.close()


def test_sample_slices_over_frames_equal_one_render():
    g, sc, _ = helpers.both("box4k", 1)
    w, h, spp, frame = 64, 48, 4, 3
    cam = cam_for(g, 0, w, h)
    other_cam = cam_for(g, 3, 40, 40)
    out = job_buffers(w, h)
    other = job_buffers(40, 40)
    b = kgr.Batcher(1 << 16, 8)
    for s0, k in ((0, 1), (1, 2), (3, 1)):
        jobs = [kgr.batch_job(other_cam, 40, 40, 2, other[0].data_ptr(), frame=7),
                kgr.batch_job(cam, w, h, spp, out[0].data_ptr(), sample_begin=s0, sample_count=k, frame=frame)]
        b.render(sc, jobs, max_depth=DEPTH, use_graph=False)
    torch.cuda.synchronize()
    ref = single(sc, cam, w, h, spp, frame)
    assert np.array_equal(out[0].cpu().numpy(), ref[0])
    b.close()


def test_graph_replay_equals_eager_and_replays():
    g, sc, _ = helpers.both("box4k", 1)
    cams = [cam_for(g, i, w, h) for i, (w, h, _, _) in enumerate(SPECS)]
    eager = [job_buffers(w, h) for (w, h, _, _) in SPECS]
    graph = [job_buffers(w, h) for (w, h, _, _) in SPECS]

    def jobs_for(bufs):
        return [kgr.batch_job(cams[i], w, h, spp, bufs[i][0].data_ptr(), frame=f)
                for i, (w, h, spp, f) in enumerate(SPECS)]

    b = kgr.Batcher(1 << 16, 16)
    b.render(sc, jobs_for(eager), max_depth=DEPTH, use_graph=False)
    replayed = []
    for _ in range(3):  # eager, capture + replay, replay
        b.render(sc, jobs_for(graph), max_depth=DEPTH, use_graph=True)
        replayed.append(b.launch_info()[1])
    torch.cuda.synchronize()
    assert replayed == [False, True, True]
    for i in range(len(SPECS)):
        assert np.array_equal(eager[i][0].cpu().numpy(), graph[i][0].cpu().numpy()), i
    # a different mix replays the same graph
    mix = [kgr.batch_job(cams[1], 40, 40, 1, graph[1][0].data_ptr(), frame=9)]
    b.render(sc, mix, max_depth=DEPTH, use_graph=True)
    torch.cuda.synchronize()
    assert b.launch_info()[1]
    assert np.array_equal(graph[1][0].cpu().numpy(), eager[1][0].cpu().numpy())
    b.close()


def test_capacity_and_argument_errors():
    g, sc, _ = helpers.both("box64", 1)
    cam = cam_for(g, 0, 32, 32)
    out = job_buffers(32, 32)
    b = kgr.Batcher(1000, 2)
    with pytest.raises(kgr.KgrError) as e:
        b.render(sc, [kgr.batch_job(cam, 32, 32, 1, out[0].data_ptr())])
    assert e.value.status == 8  # KGR_ERR_BUDGET
    with pytest.raises(kgr.KgrError) as e:
        b.render(sc, [kgr.batch_job(cam, 8, 8, 2, out[0].data_ptr(), sample_begin=1, sample_count=2)])
    assert e.value.status == 1
    with pytest.raises(kgr.KgrError):
        b.render(sc, [kgr.batch_job(cam, 8, 8, 1, out[0].data_ptr())] * 3)
    b.close()
