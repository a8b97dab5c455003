"""ctypes binding of libkgr (include/kgr.h).

The Python side is a thin mirror of the C ABI used by the tests and the
benchmark: scenes, traversal calls and the attachment life cycle of the
reference's AttachmentRTX (attach, load, set_option/get_option, render,
unload).  All compute goes through libkgr's CUDA kernels; there is no
Python or CPU fallback.  Device buffers are passed as raw pointers (for
example torch CUDA tensors' data_ptr()).
"""
import ctypes
import os

import numpy as np

from . import build as _build

c_u32, c_i32, c_u64, c_f = ctypes.c_uint32, ctypes.c_int32, ctypes.c_uint64, ctypes.c_float
vp = ctypes.c_void_p

LAYOUT_FAST, LAYOUT_THREADED, LAYOUT_WIDE, LAYOUT_CW8 = 0, 1, 2, 3
TRACE_GRID, TRACE_PERSISTENT = 0, 1
BUILDER_SAH, BUILDER_KOBRA, BUILDER_SAH_HOST = 0, 1, 2
ARRAY_THREADED, ARRAY_FAST_NODES, ARRAY_WIDE_NODES, ARRAY_TRIANGLE_RECORDS = 0, 1, 2, 3
ARRAY_CW8_NODES, ARRAY_CW8_TRIANGLES = 4, 5
VALUE_NONE, VALUE_INT, VALUE_FLOAT, VALUE_BOOL, VALUE_STRING = range(5)


class KgrError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"kgr status {status}: {msg}")
        self.status = status


class Mesh(ctypes.Structure):
    _fields_ = [("positions", vp), ("normals", vp), ("vertex_count", c_u32), ("indices", vp),
                ("material_indices", vp), ("triangle_count", c_u32), ("model", vp)]


class SceneOptions(ctypes.Structure):
    _fields_ = [("builder", c_i32), ("max_leaf_size", c_i32), ("device", c_i32), ("reserved", c_i32)]


class SceneInfo(ctypes.Structure):
    _fields_ = [("vertex_count", c_u32), ("triangle_count", c_u32), ("light_count", c_u32),
                ("material_count", c_u32), ("bvh_vec4_count", c_u32), ("fast_node_count", c_u32),
                ("device_bytes", c_u64), ("build_ms", ctypes.c_double),
                ("bounds_min", c_f * 3), ("bounds_max", c_f * 3),
                ("wide_node_count", c_u32), ("wide_max_stack", c_u32),
                ("cw8_node_count", c_u32), ("cw8_depth", c_u32)]


class TraceTune(ctypes.Structure):
    _fields_ = [("layout", c_i32), ("shadow", c_i32), ("block", c_i32), ("occupancy", c_i32), ("stack", c_i32)]

    def as_dict(self):
        return {"layout": {0: "fast", 1: "threaded", 2: "wide", 3: "cw8"}[self.layout],
                "shadow": {0: "grid", 1: "persistent"}[self.shadow], "block": self.block,
                "occupancy": self.occupancy, "stack": self.stack}


class AutotuneResult(ctypes.Structure):
    _fields_ = [("best", TraceTune), ("best_ms", ctypes.c_double), ("default_ms", ctypes.c_double),
                ("candidates", c_u32), ("reserved", c_u32)]

    def as_dict(self):
        return {"best": self.best.as_dict(), "best_ms": round(self.best_ms, 3),
                "default_ms": round(self.default_ms, 3), "candidates": self.candidates}


class Value(ctypes.Structure):
    _fields_ = [("tag", c_i32), ("i", c_i32), ("f", c_f), ("b", c_i32), ("s", ctypes.c_char_p)]


class Context(ctypes.Structure):
    _fields_ = [("width", c_u32), ("height", c_u32), ("device", c_i32), ("reserved", c_i32)]


class _Camera(ctypes.Structure):
    _fields_ = [("center", c_f * 3), ("ax_u", c_f * 3), ("ax_v", c_f * 3), ("ax_w", c_f * 3),
                ("projection", c_f * 16), ("view", c_f * 16)]


class _Lights(ctypes.Structure):
    _fields_ = [("quad_lights", vp), ("tri_lights", vp), ("quad_count", c_i32), ("tri_count", c_i32)]


class _Buffers(ctypes.Structure):
    _fields_ = [("color", vp), ("normal", vp), ("albedo", vp), ("position", vp)]


class LaunchInfo(ctypes.Structure):
    _fields_ = [("resolution", c_f * 2), ("camera", _Camera), ("lights", _Lights), ("buffers", _Buffers),
                ("materials", vp), ("environment_map", c_u64), ("has_environment_map", c_i32),
                ("accumulate", c_i32), ("time", c_f), ("max_depth", c_i32), ("samples", c_i32), ("frame", c_u32)]


class RenderStats(ctypes.Structure):
    _fields_ = [("camera_rays", c_u64), ("bounce_rays", c_u64), ("shadow_rays", c_u64),
                ("kernel_launches", c_u32), ("reserved", c_u32)]


class GeneratedView(ctypes.Structure):
    _fields_ = [("positions", vp), ("normals", vp), ("vertex_count", c_u32), ("indices", vp),
                ("material_indices", vp), ("triangle_count", c_u32), ("materials", vp),
                ("material_count", c_u32), ("camera_eye", c_f * 3), ("camera_target", c_f * 3),
                ("camera_fov_deg", c_f)]


class PluginRet(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("ptr", vp)]


_LIB = None


def lib():
    """Load libkgr.so, building it first if it is missing."""
    global _LIB
    if _LIB is None:
        path = _build.LIB
        if not os.path.exists(path):
            _build.build()
        L = ctypes.CDLL(path)
        sigs = {
            "kgr_status_string": (ctypes.c_char_p, [c_i32]),
            "kgr_last_error": (ctypes.c_char_p, []),
            "kgr_abi_version": (ctypes.c_int, []),
            "kgr_scene_create": (c_i32, [vp, c_u32, vp, c_u32, vp, vp]),
            "kgr_scene_create_from_bvh": (c_i32, [vp, c_u32, vp, c_u32, vp, c_u32, c_i32, vp]),
            "kgr_scene_info_get": (c_i32, [vp, vp]),
            "kgr_bvh_build_host": (c_i32, [vp, c_u32, vp, c_u32, c_i32, c_i32, vp, c_u32, vp]),
            "kgr_scene_copy_bvh": (c_i32, [vp, vp, c_u32, vp]),
            "kgr_scene_copy_lights": (c_i32, [vp, vp, c_u32, vp]),
            "kgr_scene_copy_vertices": (c_i32, [vp, vp, vp]),
            "kgr_scene_copy_array": (c_i32, [vp, c_i32, vp, c_u64, vp]),
            "kgr_scene_set_transforms": (c_i32, [vp, vp, vp, c_u32, vp]),
            "kgr_scene_refit": (c_i32, [vp, vp, vp, vp]),
            "kgr_scene_destroy": (c_i32, [vp]),
            "kgr_trace_closest": (c_i32, [vp, vp, c_u32, vp, c_i32, vp]),
            "kgr_trace_any": (c_i32, [vp, vp, c_u32, vp, c_i32, vp]),
            "kgr_trace_closest_host": (c_i32, [vp, vp, c_u32, vp, c_i32]),
            "kgr_trace_any_host": (c_i32, [vp, vp, c_u32, vp, c_i32]),
            "kgr_trace_counts": (c_i32, [vp, vp, c_u32, c_i32, vp]),
            "kgr_create": (c_i32, [ctypes.c_char_p, vp]),
            "kgr_attach": (c_i32, [vp, vp]),
            "kgr_load": (c_i32, [vp]),
            "kgr_unload": (c_i32, [vp]),
            "kgr_set_option": (c_i32, [vp, ctypes.c_char_p, vp]),
            "kgr_get_option": (c_i32, [vp, ctypes.c_char_p, vp]),
            "kgr_render": (c_i32, [vp, vp, vp, vp]),
            "kgr_destroy": (c_i32, [vp]),
            "kgr_get_render_stats": (c_i32, [vp, vp]),
            "kgr_debug_copy": (c_i32, [vp, ctypes.c_char_p, vp, c_u64]),
            "kgr_get_stage_times": (c_i32, [vp, vp, vp, c_u32]),
            "kgr_render_pt_noalloc": (c_i32, [vp, vp, c_i32, c_i32, c_i32, vp]),
            "kgr_environment_create": (c_i32, [vp, c_u32, c_u32, c_i32, c_i32, vp]),
            "kgr_environment_texture": (c_i32, [vp, vp]),
            "kgr_environment_sample": (c_i32, [vp, vp, c_u32, vp, vp]),
            "kgr_environment_destroy": (c_i32, [vp]),
            "kgr_mlp_create": (c_i32, [c_i32, c_u64, c_i32, vp]),
            "kgr_mlp_get_weights": (c_i32, [vp, vp]),
            "kgr_mlp_set_weights": (c_i32, [vp, vp]),
            "kgr_mlp_forward": (c_i32, [vp, vp, c_u32, vp, vp]),
            "kgr_mlp_gradients": (c_i32, [vp, vp, vp, c_u32, vp, vp]),
            "kgr_mlp_train_step": (c_i32, [vp, vp, vp, c_u32, c_f, vp]),
            "kgr_mlp_destroy": (c_i32, [vp]),
            "kgr_mlp_set_inference": (c_i32, [vp, c_i32]),
            "kgr_mlp_set_training": (c_i32, [vp, c_i32]),
            "kgr_tonemap": (c_i32, [vp, vp, c_u32, c_u32, c_i32, vp]),
            "kgr_denoiser_create": (c_i32, [c_u32, c_u32, c_i32, c_i32, vp]),
            "kgr_denoise": (c_i32, [vp, vp, vp, vp]),
            "kgr_denoiser_result": (c_i32, [vp, vp]),
            "kgr_denoiser_destroy": (c_i32, [vp]),
            "kgr_denoiser_copy_result": (c_i32, [vp, vp, c_u64]),
            "kgr_mlp_check": (c_i32, [vp]),
            "kgr_mlp_test_wait_timeout": (c_i32, [vp, vp, c_u32, vp, vp]),
            "kgr_get_visit_counts": (c_i32, [vp, vp]),
            "kgr_measure_read_bandwidth": (c_i32, [c_i32, c_u64, c_i32, vp]),
            "kgr_load_attachment": (PluginRet, [ctypes.c_char_p]),
            "kgr_generate_scene": (c_i32, [ctypes.c_char_p, c_u64, vp]),
            "kgr_generated_get": (c_i32, [vp, vp]),
            "kgr_generated_destroy": (c_i32, [vp]),
            "kgr_camera_setup": (c_i32, [vp, vp, vp, c_f, c_f, vp]),
            "kgr_transform_matrix": (c_i32, [vp, vp, vp, vp]),
            "kgr_project_open": (c_i32, [ctypes.c_char_p, vp]),
            "kgr_project_scene_count": (c_i32, [vp, vp]),
            "kgr_project_scene_file": (c_i32, [vp, c_u32, vp]),
            "kgr_project_read_scene": (c_i32, [vp, c_i32, vp]),
            "kgr_project_scene_info_get": (c_i32, [vp, vp]),
            "kgr_project_scene_meshes": (c_i32, [vp, vp, vp, vp, vp]),
            "kgr_project_scene_entity": (c_i32, [vp, c_u32, vp]),
            "kgr_project_scene_camera": (c_i32, [vp, c_u32, c_f, vp]),
            "kgr_project_scene_destroy": (c_i32, [vp]),
            "kgr_project_close": (c_i32, [vp]),
            "kgr_batcher_create": (c_i32, [c_i32, c_u32, c_u32, vp]),
            "kgr_batcher_render": (c_i32, [vp, vp, vp, c_u32, vp, vp]),
            "kgr_batcher_autotune": (c_i32, [vp, vp, vp, c_u32, vp, c_i32, vp, vp]),
            "kgr_batcher_set_tune": (c_i32, [vp, vp]),
            "kgr_autotune": (c_i32, [vp, vp, vp, c_i32, vp, vp]),
            "kgr_get_trace_tune": (c_i32, [vp, vp]),
            "kgr_batcher_ray_counts": (c_i32, [vp, vp]),
            "kgr_batcher_launch_info": (c_i32, [vp, vp, vp]),
            "kgr_batcher_destroy": (c_i32, [vp]),
            "kgr_server_create": (c_i32, [vp, vp]),
            "kgr_server_add_scene": (c_i32, [vp, vp, vp]),
            "kgr_server_submit": (c_i32, [vp, vp, vp]),
            "kgr_server_wait": (c_i32, [vp, c_u64, ctypes.c_double, vp]),
            "kgr_server_stats_get": (c_i32, [vp, vp]),
            "kgr_server_destroy": (c_i32, [vp]),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(L, name)
            fn.restype, fn.argtypes = res, args
        _LIB = L
    return _LIB


def check(status):
    if status != 0:
        msg = lib().kgr_last_error().decode(errors="replace")
        raise KgrError(status, msg)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(vp)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


MATERIAL_DTYPE = np.dtype([("diffuse", "<f4", 3), ("specular", "<f4", 3), ("emission", "<f4", 3),
                           ("ambient", "<f4", 3), ("shininess", "<f4"), ("roughness", "<f4"),
                           ("refraction", "<f4"), ("type", "<i4")])


def bvh_build_host(positions, indices, builder=BUILDER_SAH, max_leaf=4):
    """Threaded bvh.cpp-layout buffer built on the host (no device needed)."""
    pos, idx = _f32(positions), _u32(indices)
    n = c_u32()
    check(lib().kgr_bvh_build_host(_ptr(pos), len(pos), _ptr(idx), len(idx), builder, max_leaf, None, 0,
                                   ctypes.byref(n)))
    out = np.zeros((n.value, 4), np.float32)
    check(lib().kgr_bvh_build_host(_ptr(pos), len(pos), _ptr(idx), len(idx), builder, max_leaf, _ptr(out),
                                   n.value, ctypes.byref(n)))
    return out


class Generated:
    """Host arrays of a procedural scene (copied out of the library)."""

    def __init__(self, name, seed=0):
        h = vp()
        check(lib().kgr_generate_scene(name.encode(), seed, ctypes.byref(h)))
        try:
            v = GeneratedView()
            check(lib().kgr_generated_get(h, ctypes.byref(v)))
            V, T, M = v.vertex_count, v.triangle_count, v.material_count
            self.positions = np.ctypeslib.as_array((c_f * (3 * V)).from_address(v.positions)).reshape(V, 3).copy()
            self.normals = np.ctypeslib.as_array((c_f * (3 * V)).from_address(v.normals)).reshape(V, 3).copy()
            self.indices = np.ctypeslib.as_array((c_u32 * (3 * T)).from_address(v.indices)).reshape(T, 3).copy()
            self.material_indices = np.ctypeslib.as_array((c_u32 * T).from_address(v.material_indices)).copy()
            raw = np.ctypeslib.as_array((c_f * (16 * M)).from_address(v.materials)).copy()
            self.materials = raw.view(MATERIAL_DTYPE)
            self.materials_raw = raw.reshape(M, 16)
            self.eye = np.array(v.camera_eye[:], np.float32)
            self.target = np.array(v.camera_target[:], np.float32)
            self.fov = float(v.camera_fov_deg)
        finally:
            lib().kgr_generated_destroy(h)

    def tris4(self):
        return np.concatenate([self.indices, self.material_indices[:, None]], axis=1).astype(np.uint32)


class Scene:
    """A device-resident scene: triangles, materials, lights and both BVH layouts."""

    def __init__(self, positions, indices, materials_raw, normals=None, material_indices=None,
                 builder=BUILDER_SAH, max_leaf=4, device=-1, bvh=None, meshes=None):
        """One mesh from positions/indices/normals/material_indices, or
        several: meshes = [dict(positions=, indices=, normals=None,
        material_indices=None, model=None (4x4, applied as glm's column-major
        mat4 * vec4, i.e. model @ [p, 1]))]; positions/indices are then None."""
        if meshes is None:
            meshes = [dict(positions=positions, indices=indices, normals=normals,
                           material_indices=material_indices)]
        self._keep = [_f32(materials_raw)]
        arr = (Mesh * len(meshes))()
        for k, m in enumerate(meshes):
            pos, idx = _f32(m["positions"]), _u32(m["indices"])
            nrm = None if m.get("normals") is None else _f32(m["normals"])
            mid = None if m.get("material_indices") is None else _u32(m["material_indices"])
            model = None if m.get("model") is None else _f32(np.asarray(m["model"], np.float32).T)
            self._keep += [pos, idx, nrm, mid, model]
            arr[k] = Mesh(_ptr(pos), _ptr(nrm), len(pos), _ptr(idx), _ptr(mid), len(idx), _ptr(model))
        mats = self._keep[0]
        self.handle = self._create(ctypes.cast(arr, vp), len(meshes), _ptr(mats), len(mats), builder, max_leaf,
                                   device, bvh)

    @staticmethod
    def _create(meshes_ptr, mesh_count, materials_ptr, material_count, builder, max_leaf, device, bvh=None):
        h = vp()
        if bvh is None:
            opt = SceneOptions(builder, max_leaf, device, 0)
            check(lib().kgr_scene_create(meshes_ptr, mesh_count, materials_ptr, material_count, ctypes.byref(opt),
                                         ctypes.byref(h)))
        else:
            b = _f32(bvh)
            check(lib().kgr_scene_create_from_bvh(meshes_ptr, mesh_count, materials_ptr, material_count, _ptr(b),
                                                  len(b), device, ctypes.byref(h)))
        return h

    @classmethod
    def from_project(cls, project_scene, builder=BUILDER_SAH, max_leaf=4, device=-1, bvh=None):
        """A device scene from a ProjectScene's meshes and materials (mesh k of
        the project scene is mesh k here)."""
        ms, n, mats, nm = project_scene.mesh_array()
        self = cls.__new__(cls)
        self._keep = [project_scene]
        self.handle = cls._create(ms, n, mats, nm, builder, max_leaf, device, bvh)
        return self

    @classmethod
    def from_generated(cls, g, **kw):
        return cls(g.positions, g.indices, g.materials_raw, normals=g.normals,
                   material_indices=g.material_indices, **kw)

    def info(self):
        i = SceneInfo()
        check(lib().kgr_scene_info_get(self.handle, ctypes.byref(i)))
        return i

    def bvh(self):
        n = c_u32()
        check(lib().kgr_scene_copy_bvh(self.handle, None, 0, ctypes.byref(n)))
        out = np.zeros((n.value, 4), np.float32)
        check(lib().kgr_scene_copy_bvh(self.handle, _ptr(out), n.value, ctypes.byref(n)))
        return out

    def lights(self):
        n = c_u32()
        check(lib().kgr_scene_copy_lights(self.handle, None, 0, ctypes.byref(n)))
        out = np.zeros((n.value, 12), np.float32)
        check(lib().kgr_scene_copy_lights(self.handle, _ptr(out), n.value, ctypes.byref(n)))
        return out

    def vertices(self):
        """(positions, normals) as (V, 3) float32, read from the device."""
        n = self.info().vertex_count
        p, q = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32)
        check(lib().kgr_scene_copy_vertices(self.handle, _ptr(p), _ptr(q)))
        return p, q

    def array(self, which):
        """Raw bytes (uint8) of one device array: ARRAY_THREADED, ARRAY_FAST_NODES,
        ARRAY_WIDE_NODES, ARRAY_TRIANGLE_RECORDS, ARRAY_CW8_NODES or ARRAY_CW8_TRIANGLES."""
        n = c_u64()
        check(lib().kgr_scene_copy_array(self.handle, which, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, np.uint8)
        check(lib().kgr_scene_copy_array(self.handle, which, _ptr(out), n.value, ctypes.byref(n)))
        return out

    def set_transforms(self, mesh_ids, models, stream=None):
        """New 4x4 model matrices (model @ [p, 1]) for the listed meshes, then a refit."""
        ids = _u32(mesh_ids)
        ms = _f32(np.stack([np.asarray(m, np.float32).T for m in models])) if len(ids) else None
        check(lib().kgr_scene_set_transforms(self.handle, _ptr(ids), _ptr(ms), len(ids), stream))

    def refit(self, positions_ptr, normals_ptr=None, stream=None):
        """New world-space positions (device pointer, 3 floats per vertex), then a refit."""
        check(lib().kgr_scene_refit(self.handle, positions_ptr, normals_ptr, stream))

    def trace_closest(self, rays_ptr, n, hits_ptr, layout=LAYOUT_FAST, stream=None):
        check(lib().kgr_trace_closest(self.handle, rays_ptr, n, hits_ptr, layout, stream))

    def trace_any(self, rays_ptr, n, occ_ptr, layout=LAYOUT_FAST, stream=None):
        check(lib().kgr_trace_any(self.handle, rays_ptr, n, occ_ptr, layout, stream))

    def trace_closest_host(self, rays, layout=LAYOUT_FAST):
        rays = _f32(rays)
        hits = np.zeros((len(rays), 4), np.float32)
        check(lib().kgr_trace_closest_host(self.handle, _ptr(rays), len(rays), _ptr(hits), layout))
        return hits

    def trace_any_host(self, rays, layout=LAYOUT_FAST):
        rays = _f32(rays)
        occ = np.zeros(len(rays), np.uint32)
        check(lib().kgr_trace_any_host(self.handle, _ptr(rays), len(rays), _ptr(occ), layout))
        return occ

    def trace_counts(self, rays_ptr, n, any_hit=False):
        out = (c_u64 * 4)()
        check(lib().kgr_trace_counts(self.handle, rays_ptr, n, 1 if any_hit else 0, out))
        return list(out)

    def close(self):
        if self.handle:
            lib().kgr_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_bandwidth(nbytes, iters, device=-1):
    """GB/s of a streaming read of nbytes, repeated iters times (best of 5)."""
    out = ctypes.c_double()
    check(lib().kgr_measure_read_bandwidth(device, nbytes, iters, ctypes.byref(out)))
    return out.value


def camera(eye, target, fov, aspect, up=(0.0, 1.0, 0.0)):
    """uvw_frame + projection/view matrices filled into a fresh LaunchInfo."""
    info = LaunchInfo()
    e, t, u = _f32(eye), _f32(target), _f32(up)
    check(lib().kgr_camera_setup(_ptr(e), _ptr(t), _ptr(u), fov, aspect, ctypes.byref(info)))
    return info


def camera_dict(info):
    c = info.camera
    return {"center": list(c.center), "ax_u": list(c.ax_u), "ax_v": list(c.ax_v), "ax_w": list(c.ax_w),
            "projection": list(c.projection), "view": list(c.view)}


FILTER_LINEAR, FILTER_POINT = 0, 1


class Environment:
    """kgr_environment: an RGBA float environment map as a CUDA texture
    object (normalised coordinates, wrap addressing; linear filtering as the
    reference's set_envmap makes it, or point sampling)."""

    def __init__(self, rgba, filter=FILTER_LINEAR, device=-1):
        texels = np.ascontiguousarray(rgba, dtype=np.float32)
        assert texels.ndim == 3 and texels.shape[2] == 4, "texels are (height, width, 4)"
        self.height, self.width = texels.shape[:2]
        self.texels = texels
        self.filter = filter
        h = vp()
        check(lib().kgr_environment_create(_ptr(texels), self.width, self.height, filter, device, ctypes.byref(h)))
        self.handle = h
        t = c_u64()
        check(lib().kgr_environment_texture(h, ctypes.byref(t)))
        self.texture = t.value

    def sample(self, uv_ptr, n, out_ptr, stream=None):
        """tex2D<float4> at n (u, v) pairs: device arrays of 2 and 4 floats per entry."""
        check(lib().kgr_environment_sample(self.handle, uv_ptr, n, out_ptr, stream))

    def attach_to(self, info):
        info.environment_map = self.texture
        info.has_environment_map = 1
        return info

    def close(self):
        if self.handle:
            lib().kgr_environment_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_quad_lights(info, quads_ptr, count):
    """Quad lights {a, ab, ac, intensity} (12 floats each, a device array) for a launch."""
    info.lights.quad_lights = quads_ptr
    info.lights.quad_count = count
    return info


TONEMAP_ACES, TONEMAP_SRGB = 0, 1
DENOISE_NONE, DENOISE_NORMAL, DENOISE_ALBEDO, DENOISE_POSITION = 0, 1, 2, 4


def tonemap(hdr_ptr, ldr_ptr, width, height, mode=TONEMAP_ACES, stream=None):
    """kgr_tonemap: float4 HDR (device) -> packed RGBA8 (device), rows bottom to top."""
    check(lib().kgr_tonemap(hdr_ptr, ldr_ptr, width, height, mode, stream))


class DenoiseParams(ctypes.Structure):
    _fields_ = [("iterations", c_i32), ("sigma_color", c_f), ("normal_power", c_f), ("sigma_position", c_f),
                ("reserved", c_i32 * 4)]


class DenoiseInput(ctypes.Structure):
    _fields_ = [("color", vp), ("normal", vp), ("albedo", vp), ("position", vp)]


class Denoiser:
    """kgr_denoiser: the a-trous denoiser over the AOV buffers (device pointers)."""

    def __init__(self, width, height, guides=DENOISE_NORMAL | DENOISE_ALBEDO | DENOISE_POSITION, device=-1):
        h = vp()
        check(lib().kgr_denoiser_create(width, height, guides, device, ctypes.byref(h)))
        self.handle = h

    def denoise(self, color, normal, albedo=None, position=None, iterations=5, sigma_color=1.0, normal_power=64.0,
                sigma_position=0.2, stream=None):
        inp = DenoiseInput(color, normal, albedo, position)
        p = DenoiseParams(iterations, sigma_color, normal_power, sigma_position)
        check(lib().kgr_denoise(self.handle, ctypes.byref(inp), ctypes.byref(p), stream))

    def result(self):
        """Device pointer of the result (float4 per pixel)."""
        r = vp()
        check(lib().kgr_denoiser_result(self.handle, ctypes.byref(r)))
        return r.value

    def copy_result(self, out):
        """Copy the result into a float32 host array of W x H x 4 values."""
        check(lib().kgr_denoiser_copy_result(self.handle, _ptr(out), out.nbytes))
        return out

    def close(self):
        if self.handle:
            lib().kgr_denoiser_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Mlp:
    """kgr_mlp: the radiance-cache network (device pointers for x/out/targets)."""

    def __init__(self, dtype="bf16", seed=0, device=-1):
        h = vp()
        check(lib().kgr_mlp_create(0 if dtype == "bf16" else 1, seed, device, ctypes.byref(h)))
        self.handle, self.dtype = h, dtype

    def weights(self):
        w = np.zeros((6, 64, 64), np.float32)
        check(lib().kgr_mlp_get_weights(self.handle, _ptr(w)))
        return w

    def set_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        check(lib().kgr_mlp_set_weights(self.handle, _ptr(w)))

    def forward(self, x_ptr, n, out_ptr, stream=None):
        check(lib().kgr_mlp_forward(self.handle, x_ptr, n, out_ptr, stream))

    def gradients(self, x_ptr, t_ptr, n):
        g = np.zeros((6, 64, 64), np.float32)
        loss = ctypes.c_float()
        check(lib().kgr_mlp_gradients(self.handle, x_ptr, t_ptr, n, _ptr(g), ctypes.byref(loss)))
        return loss.value, g

    def train_step(self, x_ptr, t_ptr, n, lr=1e-3, stream=None):
        check(lib().kgr_mlp_train_step(self.handle, x_ptr, t_ptr, n, lr, stream))

    def set_inference(self, kernel):
        """"mma" (warp-level mma.sync) or "tcgen05" (tensor memory accumulators)."""
        check(lib().kgr_mlp_set_inference(self.handle, {"mma": 0, "tcgen05": 1}[kernel]))

    def set_training(self, kernel):
        """Gradient kernel: "mma" (warp-level mma.sync) or "tcgen05" (tensor memory accumulators)."""
        check(lib().kgr_mlp_set_training(self.handle, {"mma": 0, "tcgen05": 1}[kernel]))

    def check(self):
        """Raise if a tcgen05 kernel gave up on an mbarrier wait."""
        check(lib().kgr_mlp_check(self.handle))

    def test_wait_timeout(self, x_ptr, n, out_ptr, stream=None):
        """One tcgen05 inference whose loads are withheld, so its waits run out (a test of that path)."""
        check(lib().kgr_mlp_test_wait_timeout(self.handle, x_ptr, n, out_ptr, stream))

    def close(self):
        if self.handle:
            lib().kgr_mlp_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Attachment:
    """kgr_attachment: the AttachmentRTX life cycle over the C ABI."""

    def __init__(self, kind="path_tracer"):
        h = vp()
        check(lib().kgr_create(kind.encode(), ctypes.byref(h)))
        self.handle = h
        self.kind = kind

    def attach(self, width, height, device=-1):
        ctx = Context(width, height, device, 0)
        check(lib().kgr_attach(self.handle, ctypes.byref(ctx)))

    def load(self):
        check(lib().kgr_load(self.handle))

    def unload(self):
        check(lib().kgr_unload(self.handle))

    def set_option(self, name, value):
        v = Value()
        if isinstance(value, bool):
            v.tag, v.b = VALUE_BOOL, int(value)
        elif isinstance(value, int):
            v.tag, v.i = VALUE_INT, value
        elif isinstance(value, float):
            v.tag, v.f = VALUE_FLOAT, value
        elif isinstance(value, str):
            v.tag, v.s = VALUE_STRING, value.encode()
        else:
            raise TypeError(type(value))
        check(lib().kgr_set_option(self.handle, name.encode(), ctypes.byref(v)))

    def get_option(self, name):
        v = Value()
        check(lib().kgr_get_option(self.handle, name.encode(), ctypes.byref(v)))
        if v.tag == VALUE_INT:
            return v.i
        if v.tag == VALUE_FLOAT:
            return v.f
        if v.tag == VALUE_BOOL:
            return bool(v.b)
        if v.tag == VALUE_STRING:
            return v.s.decode()
        return None

    def render(self, info, scene, stream=None):
        check(lib().kgr_render(self.handle, ctypes.byref(info), scene.handle, stream))

    def stats(self):
        s = RenderStats()
        check(lib().kgr_get_render_stats(self.handle, ctypes.byref(s)))
        return s

    def autotune(self, info, scene, frames=3, stream=None):
        """kgr_autotune: time every traversal launch shape on `frames` real
        frames of `info`, keep the fastest; returns the result as a dict."""
        r = AutotuneResult()
        check(lib().kgr_autotune(self.handle, ctypes.byref(info), scene.handle, frames, stream, ctypes.byref(r)))
        return r.as_dict()

    def trace_tune(self):
        t = TraceTune()
        check(lib().kgr_get_trace_tune(self.handle, ctypes.byref(t)))
        return t.as_dict()

    STAGES = ("generate", "trace_closest", "shade", "shadow", "accumulate", "restir_primary",
              "restir_temporal", "restir_spatial", "restir_finalize", "cache_infer", "cache_train",
              "restir_temporal_vis", "restir_spatial_vis", "mamba_secondary", "mamba_gather",
              "mamba_probes", "mamba_final")

    def stage_times(self):
        """{stage: (total ms, launches)} since the last call ("profile" option)."""
        n = len(self.STAGES)
        ms = (ctypes.c_double * n)()
        la = (c_u32 * n)()
        check(lib().kgr_get_stage_times(self.handle, ms, la, n))
        return {s: (ms[i], la[i]) for i, s in enumerate(self.STAGES)}

    def visit_counts(self):
        out = (c_u64 * 4)()
        check(lib().kgr_get_visit_counts(self.handle, out))
        return list(out)

    def debug_copy(self, what, out):
        check(lib().kgr_debug_copy(self.handle, what.encode(), _ptr(out), out.nbytes))
        return out

    def close(self):
        if self.handle:
            lib().kgr_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def launch_info(cam_info, width, height, buffers, max_depth=2, samples=0, accumulate=False, frame=0):
    """Fill a LaunchInfo from a camera LaunchInfo and four device pointers."""
    info = LaunchInfo()
    ctypes.pointer(info)[0] = cam_info
    info.resolution[0], info.resolution[1] = float(width), float(height)
    info.buffers.color, info.buffers.normal, info.buffers.albedo, info.buffers.position = buffers
    info.max_depth = max_depth
    info.samples = samples
    info.accumulate = 1 if accumulate else 0
    info.frame = frame
    return info


# ------------------------------------------------------------ Kobra projects

class ProjectSceneInfo(ctypes.Structure):
    _fields_ = [("entity_count", c_u32), ("mesh_count", c_u32), ("vertex_count", c_u32),
                ("triangle_count", c_u32), ("material_count", c_u32), ("textured_materials", c_u32),
                ("missing_meshes", c_u32), ("camera_entity", c_i32)]


class ProjectEntity(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("position", c_f * 3), ("rotation", c_f * 3), ("scale", c_f * 3),
                ("model", c_f * 16), ("renderable", c_i32), ("has_camera", c_i32), ("fov", c_f), ("aspect", c_f),
                ("mesh_first", c_u32), ("mesh_count", c_u32)]

    def as_dict(self):
        return {"name": self.name.decode(), "position": list(self.position), "rotation": list(self.rotation),
                "scale": list(self.scale), "model": np.array(self.model[:], np.float32).reshape(4, 4).T,
                "renderable": bool(self.renderable), "has_camera": bool(self.has_camera), "fov": self.fov,
                "aspect": self.aspect, "mesh_first": self.mesh_first, "mesh_count": self.mesh_count}


def transform_matrix(position, rotation_deg, scale):
    """Transform::matrix() as a 4x4 array M with M @ [p, 1] the world point."""
    p, r, s_ = _f32(position), _f32(rotation_deg), _f32(scale)
    out = np.zeros(16, np.float32)
    check(lib().kgr_transform_matrix(_ptr(p), _ptr(r), _ptr(s_), _ptr(out)))
    return out.reshape(4, 4).T.copy()


class Project:
    """A Kobra project directory (project.den, .kobra scenes, .cache meshes, assets/*.mat)."""

    def __init__(self, directory):
        h = vp()
        check(lib().kgr_project_open(str(directory).encode(), ctypes.byref(h)))
        self.handle = h

    def scene_files(self):
        n = c_u32()
        check(lib().kgr_project_scene_count(self.handle, ctypes.byref(n)))
        out = []
        for i in range(n.value):
            name = ctypes.c_char_p()
            check(lib().kgr_project_scene_file(self.handle, i, ctypes.byref(name)))
            out.append(name.value.decode())
        return out

    def read_scene(self, index=-1):
        h = vp()
        check(lib().kgr_project_read_scene(self.handle, index, ctypes.byref(h)))
        return ProjectScene(h)

    def close(self):
        if self.handle:
            lib().kgr_project_close(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ProjectScene:
    """Host arrays of one scene read from a project."""

    def __init__(self, handle):
        self.handle = handle

    def info(self):
        i = ProjectSceneInfo()
        check(lib().kgr_project_scene_info_get(self.handle, ctypes.byref(i)))
        return i

    def entities(self):
        out = []
        for k in range(self.info().entity_count):
            e = ProjectEntity()
            check(lib().kgr_project_scene_entity(self.handle, k, ctypes.byref(e)))
            out.append(e.as_dict())
        return out

    def mesh_array(self):
        ms, n, mats, nm = vp(), c_u32(), vp(), c_u32()
        check(lib().kgr_project_scene_meshes(self.handle, ctypes.byref(ms), ctypes.byref(n), ctypes.byref(mats),
                                             ctypes.byref(nm)))
        return ms, n.value, mats, nm.value

    def meshes(self):
        """Each mesh as a dict of numpy copies: positions, normals, indices,
        material_indices (object space) and model (4x4, M @ [p, 1])."""
        ms, n, _, _ = self.mesh_array()
        arr = ctypes.cast(ms, ctypes.POINTER(Mesh))
        out = []
        for k in range(n):
            m = arr[k]
            V, T = m.vertex_count, m.triangle_count
            get = lambda ptr, ct, cnt: np.ctypeslib.as_array((ct * cnt).from_address(ptr)).copy()
            out.append({"positions": get(m.positions, c_f, 3 * V).reshape(V, 3),
                        "normals": get(m.normals, c_f, 3 * V).reshape(V, 3),
                        "indices": get(m.indices, c_u32, 3 * T).reshape(T, 3),
                        "material_indices": get(m.material_indices, c_u32, T),
                        "model": get(m.model, c_f, 16).reshape(4, 4).T.copy()})
        return out

    def materials_raw(self):
        _, _, mats, nm = self.mesh_array()
        return np.ctypeslib.as_array((c_f * (16 * nm)).from_address(mats.value)).reshape(nm, 16).copy()

    def camera(self, entity=None, aspect=0.0):
        """Launch camera of a camera entity (the first one by default)."""
        if entity is None:
            entity = self.info().camera_entity
        info = LaunchInfo()
        check(lib().kgr_project_scene_camera(self.handle, entity, aspect, ctypes.byref(info)))
        return info

    def close(self):
        if self.handle:
            lib().kgr_project_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_project(directory, scenes, materials):
    """Write a Kobra project in the layout Project::save produces
    (source/project.cpp:63-205): .cache/<submesh> files (int32 vertex and
    index counts, 56-byte Vertex records, uint32 indices), assets/<name>.mat
    (the material_fmt text), one <scene>.kobra per scene and project.den.

    scenes: {scene name: [entity]}, entity = dict(name, position, rotation
    (degrees), scale, submeshes=[dict(positions, normals, indices,
    material)], renderable=True, camera=None or (fov, aspect)); a submesh
    whose positions is None is listed but not written (a missing cache
    file).  materials: {name: dict(diffuse, specular, emission, roughness,
    refraction, type)}.  Transforms are written with nine significant
    digits, so they read back exactly."""
    import os
    os.makedirs(os.path.join(directory, ".cache"), exist_ok=True)
    os.makedirs(os.path.join(directory, "assets"), exist_ok=True)
    for name, m in materials.items():
        d, sp, e = (m.get(k, (0.0, 0.0, 0.0)) for k in ("diffuse", "specular", "emission"))
        text = ("name: %s\ndiffuse: %f,%f,%f\nspecular: %f,%f,%f\nemission: %f,%f,%f\nroughness: %f\n"
                "refraction: %f\ntype: %d\nalbedo_texture: \nnormal_texture: \nroughness_texture: " %
                (name, *d, *sp, *e, m.get("roughness", 0.001), m.get("refraction", 1.0), m.get("type", 4)))
        with open(os.path.join(directory, "assets", name + ".mat"), "w") as f:
            f.write(text)
    sid = 0
    g = lambda v: " ".join("%.9g" % float(x) for x in v)
    for scene_name, entities in scenes.items():
        lines = []
        for ent in entities:
            lines.append("")
            lines.append("@entity " + ent["name"])
            lines.append(".transform %s %s %s" % (g(ent.get("position", (0, 0, 0))), g(ent.get("rotation", (0, 0, 0))),
                                                  g(ent.get("scale", (1, 1, 1)))))
            subs = ent.get("submeshes", [])
            if subs:
                lines.append(".mesh %d" % len(subs))
                for sm in subs:
                    fname = "submesh-%d.submesh" % sid
                    sid += 1
                    if sm["positions"] is not None:
                        p = _f32(sm["positions"])
                        n = _f32(sm["normals"])
                        idx = _u32(sm["indices"]).ravel()
                        vert = np.zeros((len(p), 14), np.float32)
                        vert[:, 0:3], vert[:, 3:6] = p, n
                        with open(os.path.join(directory, ".cache", fname), "wb") as f:
                            f.write(np.array([len(p), len(idx)], np.int32).tobytes())
                            f.write(vert.tobytes())
                            f.write(idx.tobytes())
                    lines.append("\t%s, %s.mat" % (fname, sm["material"]))
            if ent.get("renderable", True) and subs:
                lines.append(".renderable")
            if ent.get("camera") is not None:
                lines.append(".camera %s" % g(ent["camera"]))
        with open(os.path.join(directory, scene_name + ".kobra"), "w") as f:
            f.write("\n".join(lines) + "\n")
    with open(os.path.join(directory, "project.den"), "w") as f:
        f.write("@scenes %d\n" % len(scenes) + "".join(s + ".kobra\n" for s in scenes))


# ------------------------------------------------------------ batching / serving (include/kgr_serve.h)

class BatchJob(ctypes.Structure):
    _fields_ = [("width", c_u32), ("height", c_u32), ("spp", c_u32), ("sample_begin", c_u32),
                ("sample_count", c_u32), ("frame", c_u32), ("accumulate", c_i32), ("samples", c_i32),
                ("center", c_f * 3), ("ax_u", c_f * 3), ("ax_v", c_f * 3), ("ax_w", c_f * 3),
                ("color", vp), ("normal", vp), ("albedo", vp), ("position", vp)]


class BatchOptions(ctypes.Structure):
    _fields_ = [("max_depth", c_i32), ("russian_roulette", c_i32), ("rr_start_depth", c_i32), ("layout", c_i32),
                ("use_graph", c_i32), ("reserved", c_i32 * 3)]


REQUEST_PATH_TRACER, REQUEST_RESTIR_DI = 0, 1


class ServerConfig(ctypes.Structure):
    _fields_ = [("device", c_i32), ("path_capacity", c_u32), ("max_jobs", c_u32), ("spp_per_tick", c_u32),
                ("memory_budget", c_u64), ("layout", c_i32), ("use_graph", c_i32), ("autotune", c_i32),
                ("policy", c_i32)]


SCHEDULE_FCFS, SCHEDULE_FAIR = 0, 1


class Request(ctypes.Structure):
    _fields_ = [("scene", c_u32), ("kind", c_i32), ("width", c_u32), ("height", c_u32), ("spp", c_u32),
                ("max_depth", c_u32), ("frame", c_u32), ("russian_roulette", c_i32), ("rr_start_depth", c_i32),
                ("eye", c_f * 3), ("target", c_f * 3), ("fov_deg", c_f), ("host_color", vp)]


class RequestResult(ctypes.Structure):
    _fields_ = [("status", c_i32), ("done", c_i32), ("queue_ms", ctypes.c_double), ("latency_ms", ctypes.c_double),
                ("service_ms", ctypes.c_double), ("ticks", c_u32), ("reserved", c_u32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", c_u64), ("completed", c_u64), ("failed", c_u64), ("rays", c_u64), ("ticks", c_u64),
                ("busy_ms", ctypes.c_double), ("latency_p50_ms", ctypes.c_double),
                ("latency_p90_ms", ctypes.c_double), ("latency_p99_ms", ctypes.c_double),
                ("latency_max_ms", ctypes.c_double), ("mean_jobs_per_tick", ctypes.c_double),
                ("peak_budget_bytes", c_u64), ("graph_replays", c_u64)]


def batch_job(cam_info, width, height, spp, color, sample_begin=0, sample_count=None, frame=0,
              normal=None, albedo=None, position=None):
    """A BatchJob for a camera LaunchInfo (kgr.camera) and device pointers."""
    j = BatchJob()
    j.width, j.height, j.spp, j.frame = width, height, spp, frame
    j.sample_begin = sample_begin
    j.sample_count = spp - sample_begin if sample_count is None else sample_count
    c = cam_info.camera
    j.center[:], j.ax_u[:], j.ax_v[:], j.ax_w[:] = list(c.center), list(c.ax_u), list(c.ax_v), list(c.ax_w)
    j.color, j.normal, j.albedo, j.position = color, normal, albedo, position
    return j


class Batcher:
    """kgr_batcher: several path-traced jobs per shared wavefront frame."""

    def __init__(self, path_capacity, max_jobs=256, device=-1):
        h = vp()
        check(lib().kgr_batcher_create(device, path_capacity, max_jobs, ctypes.byref(h)))
        self.handle = h

    def render(self, scene, jobs, max_depth=8, russian_roulette=True, rr_start_depth=3, layout=LAYOUT_FAST,
               use_graph=True, stream=None):
        arr = (BatchJob * len(jobs))(*jobs)
        opt = BatchOptions(max_depth, 1 if russian_roulette else 0, rr_start_depth, layout, 1 if use_graph else 0)
        check(lib().kgr_batcher_render(self.handle, scene.handle, arr, len(jobs), ctypes.byref(opt), stream))

    def autotune(self, scene, jobs, frames=3, max_depth=8, russian_roulette=True, rr_start_depth=3,
                 use_graph=True, stream=None):
        """kgr_batcher_autotune; returns the result dict (best["layout"] is the
        layout to render with from then on)."""
        arr = (BatchJob * len(jobs))(*jobs)
        opt = BatchOptions(max_depth, 1 if russian_roulette else 0, rr_start_depth, LAYOUT_FAST, 1 if use_graph else 0)
        r = AutotuneResult()
        check(lib().kgr_batcher_autotune(self.handle, scene.handle, arr, len(jobs), ctypes.byref(opt), frames, stream,
                                         ctypes.byref(r)))
        return r.as_dict()

    def set_tune(self, shadow=0, block=128, occupancy=0, stack=0):
        """Launch shape of the traversal stages (the layout is a render argument)."""
        t = TraceTune(LAYOUT_FAST, shadow, block, occupancy, stack)
        check(lib().kgr_batcher_set_tune(self.handle, ctypes.byref(t)))

    def ray_counts(self):
        c = (c_u64 * 3)()
        check(lib().kgr_batcher_ray_counts(self.handle, c))
        return list(c)

    def launch_info(self):
        n, g = c_u32(), c_i32()
        check(lib().kgr_batcher_launch_info(self.handle, ctypes.byref(n), ctypes.byref(g)))
        return n.value, bool(g.value)

    def close(self):
        if self.handle:
            lib().kgr_batcher_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """kgr_server: the render request loop (host thread inside libkgr)."""

    def __init__(self, path_capacity=1 << 24, max_jobs=256, spp_per_tick=0, memory_budget=120 << 30,
                 layout=LAYOUT_FAST, use_graph=True, device=-1, autotune=False, policy=SCHEDULE_FCFS):
        cfg = ServerConfig(device, path_capacity, max_jobs, spp_per_tick, memory_budget, layout,
                           1 if use_graph else 0, 1 if autotune else 0, policy)
        h = vp()
        check(lib().kgr_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.handle = h
        self._keep = {}

    def add_scene(self, scene):
        i = c_u32()
        check(lib().kgr_server_add_scene(self.handle, scene.handle, ctypes.byref(i)))
        self._keep[("scene", i.value)] = scene
        return i.value

    def submit(self, scene_id, width, height, spp, eye, target, fov, out=None, kind=REQUEST_PATH_TRACER,
               max_depth=8, frame=0, russian_roulette=True, rr_start_depth=3):
        """Queue a request; `out` (float32 numpy array of width*height*4, kept
        alive here) receives the image."""
        q = Request(scene_id, kind, width, height, spp, max_depth, frame, 1 if russian_roulette else 0,
                    rr_start_depth)
        q.eye[:], q.target[:], q.fov_deg = list(map(float, eye)), list(map(float, target)), float(fov)
        q.host_color = None if out is None else out.ctypes.data_as(vp)
        rid = c_u64()
        check(lib().kgr_server_submit(self.handle, ctypes.byref(q), ctypes.byref(rid)))
        if out is not None:
            self._keep[rid.value] = out
        return rid.value

    def wait(self, rid, timeout_ms=-1.0):
        """RequestResult of a request; raises KgrError on timeout."""
        r = RequestResult()
        st = lib().kgr_server_wait(self.handle, rid, timeout_ms, ctypes.byref(r))
        if st not in (0,):
            raise KgrError(st, lib().kgr_last_error().decode(errors="replace"))
        self._keep.pop(rid, None)  # the library no longer writes the output array
        return r

    def stats(self):
        s = ServerStats()
        check(lib().kgr_server_stats_get(self.handle, ctypes.byref(s)))
        return s

    def close(self):
        if self.handle:
            lib().kgr_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
