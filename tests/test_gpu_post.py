"""Tonemapping and denoising on the GPU.  kgr_tonemap against the oracle's
restatement of include/cuda/color.cuh: ACES bit for bit; sRGB within one
8-bit step (powf's last bit differs between the device and the host C
library; at least 99% of channels equal).  The denoiser against its NumPy
restatement (rtol 1e-4: expf/powf ulps through five passes), and on a
path-traced frame: the denoised 4-spp image is closer to the 1024-spp
reference than the raw one."""
import numpy as np
import pytest

from artemis_gb300 import kgr
from oracle import post_ref, pyoracle
from tests import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [kgr.TONEMAP_ACES, kgr.TONEMAP_SRGB])
def test_tonemap_matches_oracle(mode):
    rng = np.random.default_rng(mode)
    h, w = 23, 37  # not multiples of the 16 x 16 block
    hdr = np.zeros((h, w, 4), np.float32)
    hdr[..., :3] = (10.0 ** rng.uniform(-4, 2, (h, w, 3))).astype(np.float32)
    hdr[0, 0, :3] = [0.0, 0.0031308, 1e6]
    d_hdr = torch.from_numpy(hdr).cuda()
    d_ldr = torch.zeros((h, w), dtype=torch.int32, device="cuda")
    kgr.tonemap(d_hdr.data_ptr(), d_ldr.data_ptr(), w, h, mode)
    got = d_ldr.cpu().numpy().view(np.uint32)
    ref = pyoracle.tonemap(hdr, mode)
    if mode == kgr.TONEMAP_ACES:
        np.testing.assert_array_equal(got, ref)
    else:
        ch = lambda a: np.stack([(a >> s) & 0xFF for s in (0, 8, 16, 24)], -1).astype(np.int32)
        diff = np.abs(ch(got) - ch(ref))
        assert diff.max() <= 1 and (diff == 0).mean() >= 0.99


def render_with_aovs(g, sc, w, h, spp, frame):
    cam = kgr.camera(g.eye, g.target, g.fov, w / h)
    bufs = helpers.device_buffers(torch, w * h)
    att = kgr.Attachment("path_tracer")
    att.attach(w, h)
    att.load()
    att.set_option("spp", spp)
    att.set_option("russian_roulette", True)
    att.render(helpers.launch(cam, w, h, bufs, frame=frame, max_depth=6), sc)
    torch.cuda.synchronize()
    att.close()
    return bufs


def result_array(dn, w, h):
    """The denoiser's result buffer (device) as a (w*h, 4) array."""
    return dn.copy_result(np.zeros((w * h, 4), np.float32))


@pytest.mark.parametrize("guides", [kgr.DENOISE_NORMAL | kgr.DENOISE_ALBEDO | kgr.DENOISE_POSITION,
                                    kgr.DENOISE_NORMAL, kgr.DENOISE_NONE])
def test_denoiser_matches_oracle(guides):
    g, sc, _ = helpers.both("box4k", 1)
    w, h = 72, 56
    bufs = render_with_aovs(g, sc, w, h, 2, 3)
    dn = kgr.Denoiser(w, h, guides)
    dn.denoise(bufs[0].data_ptr(), bufs[1].data_ptr(), bufs[2].data_ptr(), bufs[3].data_ptr())
    torch.cuda.synchronize()
    cpu = [b.cpu().numpy().reshape(h, w, 4) for b in bufs]
    got = result_array(dn, w, h).reshape(h, w, 4)
    ref = post_ref.denoise(cpu[0], cpu[1], cpu[2], cpu[3], guides)
    np.testing.assert_allclose(got, ref, rtol=1e-4, atol=1e-6)
    dn.close()


def test_denoising_lowers_relmse():
    g, sc, _ = helpers.both("box4k", 1)
    w, h = 128, 128
    ref = np.zeros((w * h, 3))
    n_ref = 64
    for f in range(n_ref):
        ref += render_with_aovs(g, sc, w, h, 16, 1000 + f)[0].cpu().numpy()[:, :3]
    ref /= n_ref
    bufs = render_with_aovs(g, sc, w, h, 4, 7)
    dn = kgr.Denoiser(w, h)
    dn.denoise(bufs[0].data_ptr(), bufs[1].data_ptr(), bufs[2].data_ptr(), bufs[3].data_ptr())
    rel = lambda x: float(np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2)))
    raw, den = rel(bufs[0].cpu().numpy()[:, :3]), rel(result_array(dn, w, h)[:, :3])
    print(f"relMSE 4 spp: raw {raw:.4f}, denoised {den:.4f}")
    assert den < 0.5 * raw
    dn.close()
