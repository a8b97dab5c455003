"""Kobra project oracle (test infrastructure only): a Python restatement of
how the reference reads a project directory, used by the tests to check the
library's loader (kgr_project_*).

- read_project(): Project::load_project (include/project.hpp:58-92):
  project.den holds "@scenes N" and N scene file names.
- read_scene(): s_load_scene (source/project.cpp:242-560): '#' comments,
  "@entity <name>" elements with ".transform" (nine floats: position,
  rotation in degrees, scale), ".mesh K" plus K lines "<submesh>, <material>",
  ".renderable" and ".camera <fov> <aspect>"; submeshes from .cache/
  (load_mesh, :222-239: int32 counts, 56-byte Vertex records, uint32
  indices), materials from assets/ (load_material,
  source/daemons/material.cpp:37-97), shared by name.
- transform_matrix(): Transform::matrix() (include/transform.hpp:67-72) with
  glm's scalar formulas for quat(euler), mat4_cast, translate, scale and the
  matrix product, in float32, one operation at a time.
- camera_frame(): uvw_frame (include/camera.hpp:45-63) with
  Transform::forward()/up() (transform.hpp:98-112), whose quaternion takes
  the rotation in degrees as if it were radians.
Floats are parsed with the C library's strtof and cosf/sinf/tanf are the C
library's, through ctypes, so the restatement sees the same values as the
compiled loader.
"""
import ctypes
import ctypes.util
import os

import numpy as np

_libc = ctypes.CDLL(ctypes.util.find_library("c"))
_libc.strtof.restype = ctypes.c_float
_libc.strtof.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]
_libm = ctypes.CDLL(ctypes.util.find_library("m"))
for _fn in ("cosf", "sinf", "tanf", "sqrtf"):
    getattr(_libm, _fn).restype = ctypes.c_float
    getattr(_libm, _fn).argtypes = [ctypes.c_float]

f32 = np.float32


def strtof(text):
    return f32(_libc.strtof(text.encode(), None))


def cosf(x):
    return f32(_libm.cosf(float(x)))


def sinf(x):
    return f32(_libm.sinf(float(x)))


def tanf(x):
    return f32(_libm.tanf(float(x)))


def floats(text, n):
    """Up to n floats from whitespace-separated text (missing ones are 0)."""
    toks = text.split()
    return [strtof(toks[k]) if k < len(toks) else f32(0.0) for k in range(n)]


# -------------------------------------------------------------- glm math

def quat_from_euler(e):
    h = f32(0.5)
    cx, cy, cz = cosf(e[0] * h), cosf(e[1] * h), cosf(e[2] * h)
    sx, sy, sz = sinf(e[0] * h), sinf(e[1] * h), sinf(e[2] * h)
    w = cx * cy * cz + sx * sy * sz
    x = sx * cy * cz - cx * sy * sz
    y = cx * sy * cz + sx * cy * sz
    z = cx * cy * sz - sx * sy * cz
    return w, x, y, z


def mat4_cast(q):
    w, x, y, z = q
    one, two = f32(1.0), f32(2.0)
    qxx, qyy, qzz = x * x, y * y, z * z
    qxz, qxy, qyz = x * z, x * y, y * z
    qwx, qwy, qwz = w * x, w * y, w * z
    m = np.zeros((4, 4), np.float32)  # m[col][row]
    m[0][0] = one - two * (qyy + qzz)
    m[0][1] = two * (qxy + qwz)
    m[0][2] = two * (qxz - qwy)
    m[1][0] = two * (qxy - qwz)
    m[1][1] = one - two * (qxx + qzz)
    m[1][2] = two * (qyz + qwx)
    m[2][0] = two * (qxz + qwy)
    m[2][1] = two * (qyz - qwx)
    m[2][2] = one - two * (qxx + qyy)
    m[3][3] = one
    return m


def mul4(a, b):
    r = np.zeros((4, 4), np.float32)
    for i in range(4):
        for row in range(4):
            r[i][row] = ((a[0][row] * b[i][0] + a[1][row] * b[i][1]) + a[2][row] * b[i][2]) + a[3][row] * b[i][3]
    return r


def translate4(m, v):
    r = m.copy()
    for row in range(4):
        r[3][row] = ((m[0][row] * v[0] + m[1][row] * v[1]) + m[2][row] * v[2]) + m[3][row]
    return r


def scale4(m, v):
    r = m.copy()
    for row in range(4):
        r[0][row] = m[0][row] * v[0]
        r[1][row] = m[1][row] * v[1]
        r[2][row] = m[2][row] * v[2]
    return r


def transform_matrix(position, rotation_deg, scale):
    """Column-major (glm) 4x4: m[col][row]."""
    k = f32(0.01745329251994329576923690768489)
    rad = [f32(r) * k for r in rotation_deg]
    eye = np.eye(4, dtype=np.float32)
    p = translate4(eye, [f32(v) for v in position])
    r = mat4_cast(quat_from_euler(rad))
    s = scale4(eye, [f32(v) for v in scale])
    return mul4(mul4(p, r), s)


def _cross(a, b):
    return [a[1] * b[2] - b[1] * a[2], a[2] * b[0] - b[2] * a[0], a[0] * b[1] - b[0] * a[1]]


def _normalize(v):
    d = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]
    inv = f32(1.0) / f32(np.sqrt(d, dtype=np.float32))
    return [v[0] * inv, v[1] * inv, v[2] * inv]


def _rotate(q, v):
    w = q[0]
    qv = [q[1], q[2], q[3]]
    uv = _cross(qv, v)
    uuv = _cross(qv, uv)
    two = f32(2.0)
    return [v[k] + ((uv[k] * w) + uuv[k]) * two for k in range(3)]


def camera_frame(position, rotation, fov, aspect):
    """(center, u, v, w) of uvw_frame for a camera entity."""
    q = quat_from_euler([f32(r) for r in rotation])
    fwd = _normalize(_rotate(q, [f32(0.0), f32(0.0), f32(-1.0)]))
    up = _normalize(_rotate(q, [f32(0.0), f32(1.0), f32(0.0)]))
    eye = [f32(p) for p in position]
    lookat = [eye[k] + fwd[k] for k in range(3)]
    w = [lookat[k] - eye[k] for k in range(3)]
    wlen = f32(np.sqrt((w[0] * w[0] + w[1] * w[1]) + w[2] * w[2], dtype=np.float32))
    u = _normalize(_cross(w, up))
    v = _normalize(_cross(u, w))
    vlen = wlen * tanf(f32(fov) * f32(0.01745329251994329576923690768489) / f32(2.0))
    v = [x * vlen for x in v]
    ulen = vlen * f32(aspect)
    u = [x * ulen for x in u]
    return [np.array(a, np.float32) for a in (eye, u, v, w)]


# -------------------------------------------------------------- files

def read_project(directory):
    toks = open(os.path.join(directory, "project.den")).read().split()
    assert toks[0] == "@scenes"
    n = int(toks[1])
    return toks[2:2 + n]


def read_material(path):
    lines = open(path).read().split("\n") + [""] * 10
    m = np.zeros(16, np.float32)
    m[0:3] = [1.0, 0.0, 1.0]
    m[13], m[14] = f32(0.001), f32(1.0)
    m[15:16].view(np.int32)[0] = 4
    name = lines[0][len("name: "):].split()[0] if lines[0].startswith("name: ") and lines[0][6:].split() else ""
    for k, key, off in ((1, "diffuse: ", 0), (2, "specular: ", 3), (3, "emission: ", 6)):
        if lines[k].startswith(key):
            m[off:off + 3] = [strtof(t) for t in lines[k][len(key):].split(",")[:3]]
    if lines[4].startswith("roughness: "):
        m[13] = strtof(lines[4][11:])
    if lines[5].startswith("refraction: "):
        m[14] = strtof(lines[5][12:])
    if lines[6].startswith("type: "):
        m[15:16].view(np.int32)[0] = int(lines[6][6:].split()[0])
    return name, m


def read_submesh(path):
    if not os.path.exists(path):
        return None
    raw = open(path, "rb").read()
    nv, ni = np.frombuffer(raw[:8], np.int32)
    vert = np.frombuffer(raw[8:8 + 56 * nv], np.float32).reshape(nv, 14)
    idx = np.frombuffer(raw[8 + 56 * nv:8 + 56 * nv + 4 * ni], np.uint32).reshape(-1, 3)
    return vert[:, 0:3].copy(), vert[:, 3:6].copy(), idx.copy()


def read_scene(directory, scene_file):
    """(entities, meshes, materials (M,16) float32, missing): meshes are dicts
    {positions, normals, indices, material_indices, model (4x4, M @ [p,1])}
    for submeshes of renderable entities, in file order."""
    lines = open(os.path.join(directory, scene_file)).read().split("\n")
    if lines and lines[-1] == "":
        lines.pop()
    elements, cur, i = [], None, 0
    while i < len(lines):
        line = lines[i]
        i += 1
        if not line or line[0] == "#":
            continue
        if line[0] == "@":
            kind = line[1:].split()[0] if line[1:].split() else ""
            if kind in ("entity", "materials"):
                cur = {"entity": kind == "entity", "name": line[7:].strip(" \t\r") if kind == "entity" else "",
                       "position": [0, 0, 0], "rotation": [0, 0, 0], "scale": [1, 1, 1], "meshes": [],
                       "renderable": False, "camera": None}
                elements.append(cur)
            continue
        if line[0] != "." or cur is None:
            continue
        field = line[1:]
        if field.startswith("transform"):
            v = floats(field[10:], 9)
            cur["position"], cur["rotation"], cur["scale"] = v[0:3], v[3:6], v[6:9]
        elif field.startswith("mesh"):
            count = int(field[5:])
            cur["meshes"] = []
            for _ in range(count):
                ml = lines[i].lstrip(" \t")
                i += 1
                mesh, _, rest = ml.partition(",")
                cur["meshes"].append((mesh, rest.split()[0] if rest.split() else ""))
        elif field.startswith("renderable"):
            cur["renderable"] = True
        elif field.startswith("list"):
            i += int(field[5:])
        elif field.startswith("camera"):
            fov, aspect = floats(field[7:], 2)
            cur["camera"] = (fov, aspect)
    entities, meshes, mats, by_name, missing = [], [], [], {}, 0
    for el in elements:
        if not el["entity"]:
            continue
        model = transform_matrix(el["position"], el["rotation"], el["scale"]).T.copy()  # row-major M
        first = len(meshes)
        if el["renderable"] and el["meshes"]:
            for mesh, mat in el["meshes"]:
                name, m = read_material(os.path.join(directory, "assets", mat))
                if name not in by_name:
                    by_name[name] = len(mats)
                    mats.append(m)
                sub = read_submesh(os.path.join(directory, ".cache", mesh))
                if sub is None:
                    missing += 1
                    continue
                p, n, idx = sub
                meshes.append({"positions": p, "normals": n, "indices": idx,
                               "material_indices": np.full(len(idx), by_name[name], np.uint32), "model": model})
        entities.append(dict(el, model=model, mesh_first=first, mesh_count=len(meshes) - first))
    return entities, meshes, np.array(mats, np.float32).reshape(-1, 16), missing
