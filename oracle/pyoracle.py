"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py.  The product path never loads this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

u32p = ctypes.POINTER(ctypes.c_uint32)
f32p = ctypes.POINTER(ctypes.c_float)


class OracleScene(ctypes.Structure):
    _fields_ = [("positions", ctypes.c_void_p), ("normals", ctypes.c_void_p),
                ("tris", ctypes.c_void_p), ("materials", ctypes.c_void_p),
                ("lights", ctypes.c_void_p), ("bvh", ctypes.c_void_p),
                ("vertex_count", ctypes.c_uint32), ("triangle_count", ctypes.c_uint32),
                ("material_count", ctypes.c_uint32), ("light_count", ctypes.c_uint32),
                ("bvh_vec4_count", ctypes.c_uint32), ("pad", ctypes.c_uint32),
                ("quads", ctypes.c_void_p), ("env", ctypes.c_void_p), ("quad_count", ctypes.c_uint32),
                ("env_width", ctypes.c_uint32), ("env_height", ctypes.c_uint32), ("env_filter", ctypes.c_int32)]


class TraceStats(ctypes.Structure):
    _fields_ = [("internal_visits", ctypes.c_uint64), ("leaf_visits", ctypes.c_uint64),
                ("rays", ctypes.c_uint64)]


class RenderParams(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("center", ctypes.c_float * 3), ("ax_u", ctypes.c_float * 3),
                ("ax_v", ctypes.c_float * 3), ("ax_w", ctypes.c_float * 3),
                ("projection", ctypes.c_float * 16), ("view", ctypes.c_float * 16),
                ("prev_projection", ctypes.c_float * 16), ("prev_view", ctypes.c_float * 16),
                ("max_depth", ctypes.c_int32), ("spp", ctypes.c_int32),
                ("samples", ctypes.c_int32), ("accumulate", ctypes.c_int32),
                ("frame", ctypes.c_uint32), ("russian_roulette", ctypes.c_int32),
                ("rr_start_depth", ctypes.c_int32), ("candidates", ctypes.c_int32),
                ("temporal", ctypes.c_int32), ("temporal_mcap", ctypes.c_int32),
                ("spatial_passes", ctypes.c_int32), ("spatial_neighbors", ctypes.c_int32),
                ("spatial_radius", ctypes.c_int32), ("row_begin", ctypes.c_uint32),
                ("row_end", ctypes.c_uint32), ("threads", ctypes.c_int32)]


class SceneArrays(ctypes.Structure):
    _fields_ = [("positions", ctypes.c_void_p), ("normals", ctypes.c_void_p), ("indices", ctypes.c_void_p),
                ("material_indices", ctypes.c_void_p), ("materials", ctypes.c_void_p),
                ("vertex_count", ctypes.c_uint32), ("triangle_count", ctypes.c_uint32),
                ("material_count", ctypes.c_uint32), ("eye", ctypes.c_float * 3), ("target", ctypes.c_float * 3),
                ("fov_deg", ctypes.c_float)]


class RenderStats(ctypes.Structure):
    _fields_ = [("camera_rays", ctypes.c_uint64), ("bounce_rays", ctypes.c_uint64),
                ("shadow_rays", ctypes.c_uint64)]


class RestirState(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in (
        "cur_light", "cur_point", "cur_w", "cur_W", "cur_M",
        "prev_light", "prev_point", "prev_w", "prev_W", "prev_M",
        "materials", "intermediate", "auxiliary", "cur_env_v", "prev_env_v")]


class GiStateC(ctypes.Structure):
    _fields_ = [("res_a", ctypes.c_void_p), ("res_b", ctypes.c_void_p), ("prev_position", ctypes.c_void_p),
                ("prev_normal", ctypes.c_void_p), ("prev_center", ctypes.c_float * 3),
                ("gi_temporal", ctypes.c_int32), ("gi_mcap", ctypes.c_int32),
                ("gi_spatial_iterations", ctypes.c_int32), ("gi_neighbors", ctypes.c_int32),
                ("gi_radius", ctypes.c_int32), ("gi_confidence_rule", ctypes.c_int32)]


class GiState:
    """Oracle-side ReSTIR GI state carried between frames."""

    def __init__(self, n, temporal=True, mcap=30, iterations=3, neighbors=8, radius=30, confidence_rule=1):
        self.arrays = {k: np.zeros((n, 4), np.float32)
                       for k in ("res_a", "res_b", "prev_position", "prev_normal")}
        self.c = GiStateC(*[ptr(self.arrays[k]) for k in ("res_a", "res_b", "prev_position", "prev_normal")],
                          (ctypes.c_float * 3)(0, 0, 0), int(temporal), mcap, iterations, neighbors, radius,
                          int(confidence_rule))
        self.started = False


def render_gi(scene, params, state, color=None):
    n = params.width * params.height
    if color is None:
        color = np.zeros((n, 4), np.float32)
    direct = np.zeros((n, 4), np.float32)
    if not state.started:
        state.c.prev_center[:] = params.center[:]
        state.started = True
    st = RenderStats()
    lib().oracle_render_gi(ctypes.byref(scene.c), ctypes.byref(params), ctypes.byref(state.c), ptr(color),
                           ptr(direct), ctypes.byref(st))
    return color, direct, st


class MambaParams(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("center", ctypes.c_float * 3), ("ax_u", ctypes.c_float * 3),
                ("ax_v", ctypes.c_float * 3), ("ax_w", ctypes.c_float * 3),
                ("prev_projection", ctypes.c_float * 16), ("prev_view", ctypes.c_float * 16),
                ("time", ctypes.c_float), ("samples", ctypes.c_int32),
                ("direct_lighting", ctypes.c_int32), ("indirect_lighting", ctypes.c_int32),
                ("irradiance", ctypes.c_int32), ("render_probes", ctypes.c_int32),
                ("render_probe_radiance", ctypes.c_int32), ("temporal_reuse", ctypes.c_int32),
                ("spatial_reuse", ctypes.c_int32), ("threads", ctypes.c_int32)]


# dtype and row width of each Mamba buffer (the GPU build's layouts)
MAMBA_BUFFERS = {
    "g_position": (np.float32, 4), "g_normal": (np.float32, 4), "g_index": (np.int32, 1),
    "direct_le": (np.float32, 4), "res_r0": (np.float32, 4), "res_r1": (np.float32, 4),
    "res_r2": (np.float32, 4), "res_r3": (np.float32, 4), "prev_r0": (np.float32, 4),
    "prev_r1": (np.float32, 4), "prev_r2": (np.float32, 4), "prev_r3": (np.float32, 4),
    "s_wi": (np.float32, 4), "s_le": (np.float32, 4), "s_ld": (np.float32, 4), "s_ld_wi": (np.float32, 4),
    "s_hit_x": (np.float32, 4), "s_hit_n": (np.float32, 4), "s_hit_wo": (np.float32, 4),
    "s_hit_mat": (np.int32, 1), "sobel": (np.float32, 1), "raster": (np.float32, 1),
    "raster_indicator": (np.float32, 4), "raster_radiance": (np.float32, 4), "probe_ids": (np.int32, 1),
    "group_probes": (np.int32, 4), "group_sizes": (np.int32, 1), "counters": (np.int32, 2),
    "luts": (np.float32, 8), "refs": (np.int32, 1), "hashes": (np.uint32, 1), "lut_positions": (np.float32, 4),
    "probe_pos": (np.float32, 4), "probe_nrm": (np.float32, 4), "bin_le": (np.uint64, 3),
    "bin_n": (np.uint32, 1), "bin_depth": (np.uint64, 1),
}


class Mamba:
    """Oracle Mamba state (oracle_mamba_*): frame() renders one frame into a
    (W*H, 4) float32 colour array; buffer(name) copies a state buffer."""

    def __init__(self, width, height, max_probes=1 << 20, max_luts=1024):
        self.width, self.height = width, height
        self.h = lib().oracle_mamba_create(width, height, max_probes, max_luts)
        assert self.h

    def frame(self, scene, params, color=None):
        if color is None:
            color = np.zeros((self.width * self.height, 4), np.float32)
        st = RenderStats()
        lib().oracle_mamba_frame(self.h, ctypes.byref(scene.c), ctypes.byref(params), ptr(color), ctypes.byref(st))
        return color, st

    def buffer(self, name):
        dt, w = MAMBA_BUFFERS[name]
        n = lib().oracle_mamba_buffer(self.h, name.encode(), None, 0)
        assert n >= 0, name
        out = np.zeros(n // np.dtype(dt).itemsize, dt)
        lib().oracle_mamba_buffer(self.h, name.encode(), ptr(out), n)
        return out.reshape(-1, w) if w > 1 else out

    def close(self):
        if self.h:
            lib().oracle_mamba_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def mamba_params(width, height, cam, prev=None, time=0.0, samples=0, threads=0, **flags):
    """cam/prev: camera dicts {center, ax_u, ax_v, ax_w, projection, view};
    flags: direct_lighting, indirect_lighting, irradiance, render_probes,
    render_probe_radiance, temporal_reuse, spatial_reuse."""
    prev = prev or cam
    p = MambaParams()
    p.width, p.height = width, height
    for k in ("center", "ax_u", "ax_v", "ax_w"):
        getattr(p, k)[:] = [float(v) for v in cam[k]]
    p.prev_projection[:] = [float(v) for v in np.asarray(prev["projection"], np.float32).ravel()]
    p.prev_view[:] = [float(v) for v in np.asarray(prev["view"], np.float32).ravel()]
    p.time = time
    p.samples = samples
    p.irradiance = 1
    for k, v in flags.items():
        setattr(p, k, int(v))
    p.threads = threads
    return p


def build():
    """Compile liboracle.so with the committed Makefile (g++, -ffp-contract=off)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        L.oracle_build_kobra.restype = ctypes.c_int64
        L.oracle_build_kobra.argtypes = [vp, ctypes.c_uint32, vp, ctypes.c_uint64]
        L.oracle_triangle_boxes.argtypes = [ctypes.POINTER(OracleScene), vp]
        for fn in (L.oracle_trace_closest, L.oracle_trace_any):
            fn.argtypes = [ctypes.POINTER(OracleScene), vp, ctypes.c_uint32, vp,
                           ctypes.POINTER(TraceStats), ctypes.c_int]
        L.oracle_trace_closest_brute.argtypes = [ctypes.POINTER(OracleScene), vp, ctypes.c_uint32, vp]
        L.oracle_render_pt.argtypes = [ctypes.POINTER(OracleScene), ctypes.POINTER(RenderParams),
                                       vp, vp, vp, vp, ctypes.POINTER(RenderStats)]
        L.oracle_render_pt_f64.argtypes = [ctypes.POINTER(OracleScene), ctypes.POINTER(RenderParams),
                                           vp, ctypes.POINTER(RenderStats)]
        L.oracle_render_restir.argtypes = [ctypes.POINTER(OracleScene), ctypes.POINTER(RenderParams),
                                           ctypes.POINTER(RestirState), vp, vp, vp, vp,
                                           ctypes.POINTER(RenderStats)]
        L.oracle_render_gi.argtypes = [ctypes.POINTER(OracleScene), ctypes.POINTER(RenderParams),
                                       ctypes.POINTER(GiStateC), vp, vp, ctypes.POINTER(RenderStats)]
        L.oracle_kat_rng.argtypes = [ctypes.c_float] * 3 + [ctypes.c_int, vp]
        L.oracle_tonemap.argtypes = [vp, vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int]
        L.oracle_env_lookup.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, vp, ctypes.c_uint32, vp]
        L.oracle_generate_scene.restype = ctypes.c_int
        L.oracle_generate_scene.argtypes = [ctypes.c_char_p, ctypes.c_uint64, ctypes.POINTER(vp)]
        L.oracle_generated_view.argtypes = [vp, ctypes.POINTER(SceneArrays)]
        L.oracle_generated_destroy.argtypes = [vp]
        L.oracle_build_sah.restype = ctypes.c_int64
        L.oracle_build_sah.argtypes = [vp, vp, ctypes.c_uint32, ctypes.c_int, vp, ctypes.c_uint64]
        L.oracle_scene_lights.restype = ctypes.c_uint32
        L.oracle_scene_lights.argtypes = [vp, vp, vp, ctypes.c_uint32, vp, vp]
        L.oracle_camera.argtypes = [vp, vp, vp, ctypes.c_float, ctypes.c_float, vp, vp, vp, vp]
        L.oracle_kat_intersect.restype = ctypes.c_float
        L.oracle_kat_intersect.argtypes = [vp] * 6
        L.oracle_kat_sample_light.argtypes = [vp] * 4
        L.oracle_kat_brdf_eval.argtypes = [vp] * 5
        L.oracle_kat_brdf.argtypes = [vp] * 5
        L.oracle_kat_math.argtypes = [vp, ctypes.c_int, vp]
        L.oracle_kat_atan2_asin.argtypes = [vp, vp, ctypes.c_int, vp]
        L.oracle_mamba_create.restype = vp
        L.oracle_mamba_create.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int32, ctypes.c_int32]
        L.oracle_mamba_destroy.argtypes = [vp]
        L.oracle_mamba_frame.argtypes = [vp, ctypes.POINTER(OracleScene), ctypes.POINTER(MambaParams), vp,
                                         ctypes.POINTER(RenderStats)]
        L.oracle_mamba_buffer.restype = ctypes.c_int64
        L.oracle_mamba_buffer.argtypes = [vp, ctypes.c_char_p, vp, ctypes.c_uint64]
        _LIB = L
    return _LIB


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class Scene:
    """Host arrays of one scene, as the oracle reads them.

    positions/normals: (V,3) float32; tris: (T,4) uint32 (i0,i1,i2,material);
    materials: structured kgr_material array as raw float32 (M,16);
    lights: (L,12) float32; bvh: (K,4) float32 threaded layout."""

    def __init__(self, positions, normals, tris, materials, lights, bvh, quads=None, env=None, env_filter=0):
        """quads: (Q,12) float32 {a, ab, ac, intensity}; env: (H,W,4) float32 texels
        of the environment map, env_filter 0 linear / 1 point."""
        self.positions = np.ascontiguousarray(positions, dtype=np.float32)
        self.normals = np.ascontiguousarray(normals, dtype=np.float32)
        self.tris = np.ascontiguousarray(tris, dtype=np.uint32)
        self.materials = np.ascontiguousarray(materials, dtype=np.float32)
        self.lights = np.ascontiguousarray(lights, dtype=np.float32)
        self.bvh = np.ascontiguousarray(bvh, dtype=np.float32)
        self.quads = None if quads is None or len(quads) == 0 else np.ascontiguousarray(quads, np.float32)
        self.env = None if env is None else np.ascontiguousarray(env, np.float32)
        self.c = OracleScene(ptr(self.positions), ptr(self.normals), ptr(self.tris),
                             ptr(self.materials), ptr(self.lights), ptr(self.bvh),
                             len(self.positions), len(self.tris), len(self.materials),
                             len(self.lights), len(self.bvh), 0,
                             ptr(self.quads), ptr(self.env), 0 if self.quads is None else len(self.quads),
                             0 if self.env is None else self.env.shape[1],
                             0 if self.env is None else self.env.shape[0], env_filter)

    def triangle_boxes(self):
        boxes = np.zeros((len(self.tris), 6), np.float32)
        lib().oracle_triangle_boxes(ctypes.byref(self.c), ptr(boxes))
        return boxes

    def trace_closest(self, rays, threads=0):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        hits = np.zeros((len(rays), 4), np.float32)
        st = TraceStats()
        lib().oracle_trace_closest(ctypes.byref(self.c), ptr(rays), len(rays), ptr(hits),
                                   ctypes.byref(st), threads)
        return hits_view(hits), st

    def trace_any(self, rays, threads=0):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        occ = np.zeros(len(rays), np.uint32)
        st = TraceStats()
        lib().oracle_trace_any(ctypes.byref(self.c), ptr(rays), len(rays), ptr(occ),
                               ctypes.byref(st), threads)
        return occ, st

    def trace_brute(self, rays):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        hits = np.zeros((len(rays), 4), np.float32)
        lib().oracle_trace_closest_brute(ctypes.byref(self.c), ptr(rays), len(rays), ptr(hits))
        return hits_view(hits)


def hits_view(raw):
    """(N,4) float32 hit records -> dict of prim (int32), t, b1, b2."""
    raw = np.ascontiguousarray(raw, dtype=np.float32)
    return {"prim": raw[:, 0].view(np.int32).copy(), "t": raw[:, 1].copy(),
            "b1": raw[:, 2].copy(), "b2": raw[:, 3].copy(), "raw": raw}


def build_kobra_bvh(boxes):
    boxes = np.ascontiguousarray(boxes, dtype=np.float32)
    n = len(boxes)
    cap = max(3 * (2 * n), 3)
    out = np.zeros((cap, 4), np.float32)
    cnt = lib().oracle_build_kobra(ptr(boxes), n, ptr(out), cap)
    assert cnt >= 0
    return out[:cnt].copy()


def render_params(width, height, cam, **kw):
    p = RenderParams()
    p.width, p.height = width, height
    for k in ("center", "ax_u", "ax_v", "ax_w"):
        getattr(p, k)[:] = [float(x) for x in cam[k]]
    for k in ("projection", "view"):
        getattr(p, k)[:] = [float(x) for x in cam[k]]
        getattr(p, "prev_" + k)[:] = [float(x) for x in cam.get("prev_" + k, cam[k])]
    defaults = dict(max_depth=2, spp=1, samples=0, accumulate=0, frame=0, russian_roulette=0,
                    rr_start_depth=3, candidates=32, temporal=1, temporal_mcap=200,
                    spatial_passes=2, spatial_neighbors=5, spatial_radius=30,
                    row_begin=0, row_end=0, threads=0)
    defaults.update(kw)
    for k, v in defaults.items():
        setattr(p, k, v)
    return p


def render_pt(scene, params, bufs=None):
    n = params.width * params.height
    if bufs is None:
        bufs = [np.zeros((n, 4), np.float32) for _ in range(4)]
    st = RenderStats()
    lib().oracle_render_pt(ctypes.byref(scene.c), ctypes.byref(params), *[ptr(b) for b in bufs],
                           ctypes.byref(st))
    return bufs, st


def render_pt_f64(scene, params):
    out = np.zeros((params.width * params.height, 3), np.float64)
    st = RenderStats()
    lib().oracle_render_pt_f64(ctypes.byref(scene.c), ctypes.byref(params), ptr(out), ctypes.byref(st))
    return out, st


class RestirBuffers:
    """Oracle-side ReSTIR DI state (32-byte SoA reservoirs + per-pixel data)."""

    def __init__(self, n):
        self.arrays = {
            "cur_light": np.full(n, -1, np.int32), "cur_point": np.zeros((n, 3), np.float32),
            "cur_w": np.zeros(n, np.float32), "cur_W": np.zeros(n, np.float32),
            "cur_M": np.zeros(n, np.int32),
            "prev_light": np.full(n, -1, np.int32), "prev_point": np.zeros((n, 3), np.float32),
            "prev_w": np.zeros(n, np.float32), "prev_W": np.zeros(n, np.float32),
            "prev_M": np.zeros(n, np.int32),
            "materials": np.zeros((n, 16), np.float32),
            "intermediate": np.zeros((n, 4), np.float32), "auxiliary": np.zeros((n, 4), np.float32),
            "cur_env_v": np.zeros(n, np.float32), "prev_env_v": np.zeros(n, np.float32),
        }
        self.c = RestirState(*[ptr(self.arrays[f[0]]) for f in RestirState._fields_])


def render_restir(scene, params, state, bufs=None):
    n = params.width * params.height
    if bufs is None:
        bufs = [np.zeros((n, 4), np.float32) for _ in range(4)]
    st = RenderStats()
    lib().oracle_render_restir(ctypes.byref(scene.c), ctypes.byref(params), ctypes.byref(state.c),
                               *[ptr(b) for b in bufs], ctypes.byref(st))
    return bufs, st


class GeneratedScene:
    """A seeded procedural scene generated by the oracle's own generator
    (scene_ref.cpp), with the same fields as the product's generated scenes:
    positions, normals (V,3) float32; indices (T,3) and material_indices (T,)
    uint32; materials_raw (M,16) float32; eye, target, fov."""

    def __init__(self, name, seed):
        h = ctypes.c_void_p()
        if lib().oracle_generate_scene(name.encode(), seed, ctypes.byref(h)) != 0:
            raise ValueError(f"unknown procedural scene: {name}")
        try:
            v = SceneArrays()
            lib().oracle_generated_view(h, ctypes.byref(v))
            V, T, M = v.vertex_count, v.triangle_count, v.material_count

            def arr(addr, ctype, n):
                return np.ctypeslib.as_array((ctype * n).from_address(addr)).copy()
            self.positions = arr(v.positions, ctypes.c_float, 3 * V).reshape(V, 3)
            self.normals = arr(v.normals, ctypes.c_float, 3 * V).reshape(V, 3)
            self.indices = arr(v.indices, ctypes.c_uint32, 3 * T).reshape(T, 3)
            self.material_indices = arr(v.material_indices, ctypes.c_uint32, T)
            self.materials_raw = arr(v.materials, ctypes.c_float, 16 * M).reshape(M, 16)
            self.eye = np.array(v.eye[:], np.float32)
            self.target = np.array(v.target[:], np.float32)
            self.fov = float(v.fov_deg)
        finally:
            lib().oracle_generated_destroy(h)

    def tris4(self):
        return np.concatenate([self.indices, self.material_indices[:, None]], axis=1).astype(np.uint32)

    def sah_bvh(self, max_leaf=4):
        """Threaded bvh.cpp-layout buffer of the oracle's SAH builder."""
        pos, idx = self.positions, np.ascontiguousarray(self.indices)
        n = lib().oracle_build_sah(ptr(pos), ptr(idx), len(idx), max_leaf, None, 0)
        out = np.zeros((n, 4), np.float32)
        assert lib().oracle_build_sah(ptr(pos), ptr(idx), len(idx), max_leaf, ptr(out), n) == n
        return out

    def lights(self):
        args = [ptr(self.positions), ptr(np.ascontiguousarray(self.indices)), ptr(self.material_indices),
                len(self.indices), ptr(self.materials_raw)]
        n = lib().oracle_scene_lights(*args, None)
        out = np.zeros((n, 12), np.float32)
        lib().oracle_scene_lights(*args, ptr(out))
        return out

    def scene(self, max_leaf=4):
        return Scene(self.positions, self.normals, self.tris4(), self.materials_raw, self.lights(),
                     self.sah_bvh(max_leaf))


def env_lookup(texels, uv, filt=0):
    """The oracle's texture read of an (H, W, 4) map at (N, 2) coordinates -> (N, 3)."""
    t = np.ascontiguousarray(texels, np.float32)
    uv = np.ascontiguousarray(uv, np.float32)
    out = np.zeros((len(uv), 3), np.float32)
    lib().oracle_env_lookup(ptr(t), t.shape[1], t.shape[0], filt, ptr(uv), len(uv), ptr(out))
    return out


def camera(eye, target, fov, aspect, up=(0.0, 1.0, 0.0)):
    """{center, ax_u, ax_v, ax_w} of uvw_frame (include/camera.hpp:45-63)."""
    e, t, u = (np.ascontiguousarray(x, np.float32) for x in (eye, target, up))
    c, U, V, W = (np.zeros(3, np.float32) for _ in range(4))
    lib().oracle_camera(ptr(e), ptr(t), ptr(u), fov, aspect, ptr(c), ptr(U), ptr(V), ptr(W))
    return {"center": c.tolist(), "ax_u": U.tolist(), "ax_v": V.tolist(), "ax_w": W.tolist(),
            "projection": [0.0] * 16, "view": [0.0] * 16}


def tonemap(hdr, mode=0):
    """hdr: float32 (H, W, 4) -> uint32 (H, W), rows bottom to top (color.cuh:84-103)."""
    hdr = np.ascontiguousarray(hdr, np.float32)
    h, w = hdr.shape[:2]
    out = np.zeros((h, w), np.uint32)
    lib().oracle_tonemap(ptr(hdr), ptr(out), w, h, mode)
    return out
