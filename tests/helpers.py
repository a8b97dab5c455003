"""Shared setup for the parity tests: one procedural scene seen by both the
CUDA path (libkgr, device buffers from torch) and the CPU oracle."""
import numpy as np

from artemis_gb300 import kgr
from oracle import pyoracle


def oracle_scene(g, bvh, lights):
    return pyoracle.Scene(g.positions, g.normals, g.tris4(), g.materials_raw, lights, bvh)


def both(name, seed=1, builder=kgr.BUILDER_SAH, max_leaf=4):
    """(generated scene, device Scene, oracle Scene) with the same BVH."""
    g = kgr.Generated(name, seed)
    sc = kgr.Scene.from_generated(g, builder=builder, max_leaf=max_leaf)
    return g, sc, oracle_scene(g, sc.bvh(), sc.lights())


def camera_rays(cam, width, height, jitter=None):
    """Pinhole rays of make_ray with a fixed -0.5 offset (amadeus_restir.cu:30-65),
    computed with the same float32 operation order."""
    c = cam.camera
    U, V, W = (np.array(x[:], np.float32) for x in (c.ax_u, c.ax_v, c.ax_w))
    ix, iy = np.meshgrid(np.arange(width, dtype=np.float32), np.arange(height, dtype=np.float32))
    ax = (ix.ravel() + np.float32(-0.5)) / np.float32(width)
    ay = (iy.ravel() + np.float32(-0.5)) / np.float32(height)
    dx = np.float32(2.0) * ax - np.float32(1.0)
    dy = np.float32(2.0) * ay - np.float32(1.0)
    d = (dx[:, None] * U + dy[:, None] * V) + W
    d = d * (np.float32(1.0) / np.sqrt((d * d).sum(axis=1, dtype=np.float32)))[:, None]
    rays = np.zeros((len(d), 8), np.float32)
    rays[:, 0:3] = np.array(c.center[:], np.float32)
    rays[:, 4:7] = d
    rays[:, 7] = np.inf
    return rays


def random_rays(g, n, seed, tmax=np.inf):
    rng = np.random.default_rng(seed)
    lo, hi = g.positions.min(axis=0), g.positions.max(axis=0)
    o = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    tgt = g.positions[g.indices[rng.integers(0, len(g.indices), n)]].mean(axis=1)
    d = (tgt - o).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3], rays[:, 4:7], rays[:, 7] = o, d, tmax
    return rays


def device_buffers(torch, n):
    return [torch.zeros((n, 4), dtype=torch.float32, device="cuda") for _ in range(4)]


def launch(cam, width, height, bufs, **kw):
    info = kgr.launch_info(cam, width, height, [b.data_ptr() for b in bufs], **kw)
    return info


def oracle_params(cam, width, height, **kw):
    return pyoracle.render_params(width, height, kgr.camera_dict(cam), **kw)
