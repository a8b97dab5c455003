"""Refit oracle (test infrastructure only): a NumPy restatement of what
moving geometry does to a scene, used by the tests to check the library's
in-place refit (kgr_scene_set_transforms / kgr_scene_refit).

- gather(): the world-space scene the reference builds from its meshes.
  Vertices are Transform::apply (include/transform.hpp:76-79,
  glm::mat4 * vec4(p, 1), the four column terms summed in order); normals
  are the model applied to vec4(n, 0).  A mesh without normals gets the
  unnormalised face normal e1 x e2 of the last triangle that names the
  vertex.  Emissive triangles become triangle lights {a, b - a, c - a,
  emission} in triangle order, as ArmadaRTX rebuilds them after a transform
  change (source/amadeus/armada.cu:181-198 and :98-153).
- refit_threaded(): the boxes of a threaded buffer in the bvh.cpp layout
  (source/bvh.cpp:213-260) for new vertex positions, with the topology
  unchanged.  A leaf record holds its triangle's box, Submesh::bvh's
  min(p1, min(p2, p3)) per axis with glm::min (include/mesh.hpp:48-78).  An
  internal record holds the union of its subtree, which in the pre-order
  layout is the run of records between it and its miss link; the union is
  taken over the triangle boxes with -0 written as +0, so it is a function
  of the set of values.
All arithmetic is float32, one IEEE operation at a time.
"""
import numpy as np

FLT_MAX = np.float32(np.finfo(np.float32).max)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def transform_points(model, p, w):
    """model @ [p, w] for (N, 3) points, summed column by column in order."""
    M = _f32(model)
    p = _f32(p)
    w = np.float32(w)
    out = np.empty_like(p)
    for i in range(3):
        out[:, i] = ((M[i, 0] * p[:, 0] + M[i, 1] * p[:, 1]) + M[i, 2] * p[:, 2]) + M[i, 3] * w
    return out


def face_normals(positions, tris):
    a, b, c = positions[tris[:, 0]], positions[tris[:, 1]], positions[tris[:, 2]]
    e1, e2 = b - a, c - a
    n = np.empty_like(e1)
    n[:, 0] = e1[:, 1] * e2[:, 2] - e1[:, 2] * e2[:, 1]
    n[:, 1] = e1[:, 2] * e2[:, 0] - e1[:, 0] * e2[:, 2]
    n[:, 2] = e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]
    return n


def gather(meshes, materials_raw):
    """(positions (V,3), normals (V,3), tris (T,4) uint32, lights (L,12)) of
    meshes given as dicts {positions, indices, normals, material_indices, model}
    (model: 4x4, applied as model @ [p, 1]; None = vertices as given)."""
    P, N, T = [], [], []
    vb = 0
    for m in meshes:
        p = _f32(m["positions"])
        model = m.get("model")
        P.append(p.copy() if model is None else transform_points(model, p, 1.0))
        nrm = m.get("normals")
        idx = np.ascontiguousarray(m["indices"], dtype=np.uint32).reshape(-1, 3)
        mid = m.get("material_indices")
        mid = np.zeros(len(idx), np.uint32) if mid is None else np.asarray(mid, np.uint32)
        tris = np.concatenate([idx + np.uint32(vb), mid[:, None]], axis=1).astype(np.uint32)
        if nrm is not None:
            n = _f32(nrm)
            N.append(n.copy() if model is None else transform_points(model, n, 0.0))
        else:
            wp = P[-1]
            n = np.zeros_like(wp)
            if len(idx):
                src = np.full(len(wp), -1, np.int64)
                t_of = np.repeat(np.arange(len(idx)), 3)
                np.maximum.at(src, idx.ravel().astype(np.int64), t_of)
                fn = face_normals(wp, idx.astype(np.int64))
                hit = src >= 0
                n[hit] = fn[src[hit]]
            N.append(n)
        T.append(tris)
        vb += len(p)
    positions = np.concatenate(P) if P else np.zeros((0, 3), np.float32)
    normals = np.concatenate(N) if N else np.zeros((0, 3), np.float32)
    tris = np.concatenate(T) if T else np.zeros((0, 4), np.uint32)
    return positions, normals, tris, lights_of(positions, tris, materials_raw)


def lights_of(positions, tris, materials_raw):
    emission = _f32(materials_raw)[:, 6:9]
    e = emission[tris[:, 3]]
    lit = np.nonzero(np.any(e > 0, axis=1))[0]
    t = tris[lit]
    a, b, c = positions[t[:, 0]], positions[t[:, 1]], positions[t[:, 2]]
    return np.concatenate([a, b - a, c - a, e[lit]], axis=1).astype(np.float32)


def _glm_min(a, b):
    return np.where(b < a, b, a)


def _glm_max(a, b):
    return np.where(a < b, b, a)


def triangle_boxes(positions, tris):
    """Raw Submesh::bvh boxes: (T,3) min and (T,3) max."""
    a, b, c = positions[tris[:, 0]], positions[tris[:, 1]], positions[tris[:, 2]]
    return _glm_min(a, _glm_min(b, c)).astype(np.float32), _glm_max(a, _glm_max(b, c)).astype(np.float32)


def refit_threaded(bvh, positions, tris):
    """The threaded buffer `bvh` ((K,4) float32) with every box recomputed
    from `positions`; headers, links and w components unchanged."""
    out = _f32(bvh).copy()
    R = len(out) // 3
    if R == 0:
        return out
    hdr = out.view(np.int32)
    is_leaf = out[0::3, 0] == np.float32(1.0)
    obj = hdr[0::3, 1]
    miss = hdr[0::3, 3]
    tmn, tmx = triangle_boxes(_f32(positions), np.asarray(tris, np.int64))
    # canonical triangle boxes per record (leaf records only), FLT_MAX elsewhere
    cmn = np.full((R, 3), FLT_MAX, np.float32)
    cmx = np.full((R, 3), -FLT_MAX, np.float32)
    leaf_rec = np.nonzero(is_leaf)[0]
    cmn[leaf_rec] = tmn[obj[leaf_rec]] + np.float32(0.0)
    cmx[leaf_rec] = tmx[obj[leaf_rec]] + np.float32(0.0)
    box_mn = out[1::3, :3]
    box_mx = out[2::3, :3]
    box_mn[leaf_rec] = tmn[obj[leaf_rec]]
    box_mx[leaf_rec] = tmx[obj[leaf_rec]]
    for r in np.nonzero(~is_leaf)[0]:
        end = miss[r] // 3 if miss[r] >= 0 else R
        box_mn[r] = cmn[r + 1:end].min(axis=0)
        box_mx[r] = cmx[r + 1:end].max(axis=0)
    out[1::3, :3] = box_mn
    out[2::3, :3] = box_mx
    return out
