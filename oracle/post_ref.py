"""NumPy restatement of the denoiser of artemis_gb300/csrc/post.cu (the
edge-avoiding a-trous filter of Dammertz et al. 2010 with this project's
edge-stopping functions).  TEST INFRASTRUCTURE: only tests/ import it.

The reference has no counterpart to restate -- its denoiser is the closed
OptiX AI denoiser (source/layers/denoiser.cu:9-149) -- so this follows the
kernel's own specification: the same taps in the same order, float32
arithmetic, so that the GPU result agrees to the last few ulps of expf/powf.
"""
import numpy as np

H1 = np.array([1 / 16, 1 / 4, 3 / 8, 1 / 4, 1 / 16], np.float32)
NORMAL, ALBEDO, POSITION = 1, 2, 4


def _lum(c):
    return np.float32(0.2126) * c[..., 0] + np.float32(0.7152) * c[..., 1] + np.float32(0.0722) * c[..., 2]


def _albedo_div(a):
    return np.where(a[..., :3] > np.float32(1e-3), a[..., :3], np.float32(1.0)).astype(np.float32)


def denoise(color, normal, albedo, position, guides, iterations=5, sigma_color=1.0, normal_power=64.0,
            sigma_position=0.2):
    """color, normal, albedo, position: float32 (H, W, 4).  Returns (H, W, 4)."""
    f32 = np.float32
    c = np.ascontiguousarray(color, f32).copy()
    n = np.ascontiguousarray(normal, f32)[..., :3]
    x = np.ascontiguousarray(position, f32)[..., :3]
    h, w = c.shape[:2]
    hit = np.any(n != 0, axis=-1)
    cur = c[..., :3].copy()
    if guides & ALBEDO:
        cur = (cur / _albedo_div(albedo)).astype(f32)
    for i in range(iterations):
        step = 1 << i
        sc = f32(sigma_color) * f32(1.0 / (1 << i))
        lp = _lum(cur)
        acc = np.zeros_like(cur)
        wsum = np.zeros((h, w), f32)
        for dy in range(-2, 3):
            for dx in range(-2, 3):
                oy, ox = dy * step, dx * step
                ys, xs = np.arange(h) + oy, np.arange(w) + ox
                vy, vx = (ys >= 0) & (ys < h), (xs >= 0) & (xs < w)
                yq, xq = np.clip(ys, 0, h - 1), np.clip(xs, 0, w - 1)
                valid = vy[:, None] & vx[None, :]
                cq = cur[yq][:, xq]
                nq = n[yq][:, xq]
                hq = hit[yq][:, xq]
                valid = valid & (hq == hit)
                wt = np.full((h, w), H1[dx + 2] * H1[dy + 2], f32)
                lq = _lum(cq)
                wt = wt * np.exp(-np.abs(lp - lq) / (sc * f32(0.5) * (lp + lq) + f32(1e-4))).astype(f32)
                if guides & NORMAL:
                    cs = n[..., 0] * nq[..., 0] + n[..., 1] * nq[..., 1] + n[..., 2] * nq[..., 2]
                    wn = np.power(np.maximum(cs, f32(0)), f32(normal_power)).astype(f32)
                    wt = np.where(hit, wt * wn, wt)
                if (guides & POSITION) and (dx != 0 or dy != 0):
                    v = x[yq][:, xq] - x
                    ln = np.sqrt((v * v).sum(-1)).astype(f32)
                    d = np.where(ln > 0, np.abs((n * v).sum(-1)) / np.where(ln > 0, ln, f32(1)), f32(0)).astype(f32)
                    wt = np.where(hit, wt * np.exp(-d / f32(sigma_position)).astype(f32), wt)
                wt = np.where(valid, wt, f32(0))
                acc = acc + wt[..., None] * cq
                wsum = wsum + wt
        cur = np.where(wsum[..., None] > 0, acc / np.where(wsum > 0, wsum, f32(1))[..., None], cur).astype(f32)
    if guides & ALBEDO:
        cur = (cur * _albedo_div(albedo)).astype(f32)
    out = c.copy()
    out[..., :3] = cur
    return out
