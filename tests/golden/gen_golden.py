"""Regenerate tests/golden/reference_kat.json, reference_traversal.json,
reference_bvh.json, reference_pt.json and reference_restir.json from the
reference's own headers, shaders, builder, path-tracer and ReSTIR DI
programs.

Builds oracle/_ref/ref_kat and oracle/_ref/ref_color_kat (oracle/Makefile,
target `ref`), which compile include/cuda/random.cuh, include/cuda/math.cuh,
include/cuda/brdf.cuh, include/cuda/color.cuh and include/optix/lighting.cuh
of the reference checkout unmodified on the host, runs them and stores their
JSON output.  Builds oracle/_ref/ref_glsl, the traversal shaders
(shaders/rt/modules/{ray,primitives,bbox,intersect,bvh}.glsl) compiled as
C++, runs trace() on two procedural scenes with the oracle's BVHs and stores
each ray's closest object and distance.  Builds oracle/_ref/ref_bvh, the
reference's source/bvh.cpp (partition, serialize) compiled on the host, and
stores the buffer it builds from the triangle boxes of three procedural
scenes (as a SHA-256) and from small hand-made box sets (in full).  Builds
oracle/_ref/ref_pt, the reference's path-tracer programs
(source/optix/amadeus_path_tracer.cu with amadeus_common.cuh) compiled on
the host over the oracle's scene and walk, and stores one sample of each
pixel of small images of two procedural scenes, with and without an
environment map.  Builds oracle/_ref/ref_restir, the reference's ReSTIR DI
programs (source/optix/amadeus_restir.cu) compiled the same way, and stores
the colour after a few frames of a still camera and the reservoirs the
next frame would reuse.  Needs the reference checkout, named by --reference or the
REFERENCE environment variable; the committed JSON is what the tests read, so
this script only runs when the vectors are regenerated.

    python tests/golden/gen_golden.py --reference PATH
"""
import argparse
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("REFERENCE"))
    args = ap.parse_args()
    if not args.reference:
        ap.error("name the reference checkout with --reference or REFERENCE")
    subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "ref",
                           "REFERENCE=" + args.reference])
    out = subprocess.check_output([os.path.join(ROOT, "oracle", "_ref", "ref_kat")])
    data = json.loads(out)
    color = subprocess.check_output([os.path.join(ROOT, "oracle", "_ref", "ref_color_kat")])
    data.update(json.loads(color))
    data["_generated_by"] = "tests/golden/gen_golden.py from the reference headers " \
        "include/cuda/{random,math,brdf,color}.cuh and include/optix/lighting.cuh"
    with open(os.path.join(HERE, "reference_kat.json"), "w") as f:
        json.dump(data, f, indent=0)
    print("wrote", os.path.join(HERE, "reference_kat.json"), file=sys.stderr)
    traversal = {"scenes": [traversal_case(*c) for c in TRAVERSAL_CASES],
                 "_generated_by": "tests/golden/gen_golden.py: trace() of the reference's "
                                  "shaders/rt/modules/bvh.glsl (with bbox.glsl, intersect.glsl, ray.glsl, "
                                  "primitives.glsl) compiled as C++ by oracle/ref_glsl.cpp"}
    with open(os.path.join(HERE, "reference_traversal.json"), "w") as f:
        json.dump(traversal, f, separators=(",", ":"))
    print("wrote", os.path.join(HERE, "reference_traversal.json"), file=sys.stderr)
    bvh = {"scenes": [bvh_scene_case(*c) for c in BVH_SCENES], "box_sets": bvh_box_sets(),
           "_generated_by": "tests/golden/gen_golden.py: serialize(partition(boxes)) of the reference's "
                            "source/bvh.cpp compiled on the host by oracle/ref_bvh.cpp"}
    with open(os.path.join(HERE, "reference_bvh.json"), "w") as f:
        json.dump(bvh, f, separators=(",", ":"))
    print("wrote", os.path.join(HERE, "reference_bvh.json"), file=sys.stderr)
    pt = {"cases": [pt_case(*c) for c in PT_CASES],
          "_generated_by": "tests/golden/gen_golden.py: the reference's __closesthit__ / __miss__ programs "
                           "(source/optix/amadeus_path_tracer.cu, amadeus_common.cuh) compiled on the host by "
                           "oracle/ref_pt.cpp"}
    with open(os.path.join(HERE, "reference_pt.json"), "w") as f:
        json.dump(pt, f, separators=(",", ":"))
    print("wrote", os.path.join(HERE, "reference_pt.json"), file=sys.stderr)
    restir = {"cases": [restir_case(*c) for c in RESTIR_CASES],
              "_generated_by": "tests/golden/gen_golden.py: the reference's ReSTIR DI programs "
                               "(source/optix/amadeus_restir.cu) compiled on the host by oracle/ref_restir.cpp"}
    with open(os.path.join(HERE, "reference_restir.json"), "w") as f:
        json.dump(restir, f, separators=(",", ":"))
    print("wrote", os.path.join(HERE, "reference_restir.json"), file=sys.stderr)


# (scene, generator seed, builder, max leaf size, camera rays per side, random rays)
TRAVERSAL_CASES = [("box4k", 1, "sah", 4, 24, 512), ("box64", 3, "kobra", 1, 24, 512),
                   ("terrain_s", 1, "sah", 4, 24, 512)]


def traversal_rays(g, side, n_random, seed):
    """Camera rays through a side x side grid, seeded random rays between
    random points and triangle centroids, and edge cases: directions with
    zero components, axis-aligned rays, origins inside the scene box."""
    import numpy as np
    from artemis_gb300 import kgr
    rays = []
    cam = kgr.camera_dict(kgr.camera(g.eye, g.target, g.fov, 1.0))
    U, V, W, C = (np.asarray(cam[k], np.float32) for k in ("ax_u", "ax_v", "ax_w", "center"))
    for iy in range(side):
        for ix in range(side):
            u = np.float32(2.0 * (ix + 0.5) / side - 1.0)
            v = np.float32(2.0 * (iy + 0.5) / side - 1.0)
            d = u * U + v * V + W
            d = d / np.float32(np.sqrt(np.float32(d @ d)))
            rays.append(np.concatenate([C, d]))
    rng = np.random.default_rng(seed)
    lo, hi = g.positions.min(axis=0), g.positions.max(axis=0)
    cent = g.positions[g.indices].mean(axis=1)
    for _ in range(n_random):
        o = rng.uniform(lo, hi).astype(np.float32)
        t = cent[rng.integers(0, len(cent))]
        d = (t - o).astype(np.float32)
        d = d / np.float32(np.linalg.norm(d))
        rays.append(np.concatenate([o, d]))
    mid = ((lo + hi) * 0.5).astype(np.float32)
    for axis in range(3):
        for sign in (1.0, -1.0):
            d = np.zeros(3, np.float32)
            d[axis] = sign
            rays.append(np.concatenate([mid, d]))
            rays.append(np.concatenate([C, d]))
    for d in ([1, 1, 0], [0, 1, 1], [1, 0, -1], [0.3, -1, 0], [0, 0, -1]):
        d = np.asarray(d, np.float32)
        d = d / np.float32(np.linalg.norm(d))
        rays.append(np.concatenate([C, d]))
        rays.append(np.concatenate([mid, d]))
    return np.asarray(rays, np.float32)


def traversal_case(name, seed, builder, max_leaf, side, n_random):
    import hashlib
    import numpy as np
    sys.path.insert(0, ROOT)
    from oracle import pyoracle
    g = pyoracle.GeneratedScene(name, seed)
    bvh = build_bvh(g, builder, max_leaf)
    rays = traversal_rays(g, side, n_random, seed)
    tris = np.ascontiguousarray(g.tris4(), np.uint32)
    blob = (np.asarray([len(g.positions), len(tris), len(bvh), len(rays)], np.uint32).tobytes()
            + np.ascontiguousarray(g.positions, np.float32).tobytes() + tris.tobytes()
            + np.ascontiguousarray(bvh, np.float32).tobytes() + rays.tobytes())
    out = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "ref_glsl")], input=blob, capture_output=True,
                         check=True).stdout.decode().split("\n")
    hits = [[int(o), int(t, 16)] for o, t in (line.split() for line in out if line.strip())]
    assert len(hits) == len(rays)
    return {"scene": name, "seed": seed, "builder": builder, "max_leaf": max_leaf,
            "bvh_sha256": hashlib.sha256(np.ascontiguousarray(bvh, np.float32).tobytes()).hexdigest(),
            "rays": rays.view(np.uint32).tolist(), "hits": hits}


def build_bvh(g, builder, max_leaf):
    """The oracle's BVH of a generated scene in the threaded layout: its SAH
    builder, or its restatement of the reference's bvh.cpp builder."""
    from oracle import pyoracle
    if builder == "sah":
        return g.sah_bvh(max_leaf)
    osc = pyoracle.Scene(g.positions, g.normals, g.tris4(), g.materials_raw, g.lights(),
                         __import__("numpy").zeros((0, 4), "float32"))
    return pyoracle.build_kobra_bvh(osc.triangle_boxes())


BVH_SCENES = [("box64", 3), ("box4k", 1), ("terrain_s", 1)]


def reference_bvh(boxes):
    """serialize(partition(boxes)) of the reference's builder, as float32
    rows of 4 (3 per node)."""
    import numpy as np
    boxes = np.ascontiguousarray(boxes, np.float32)
    blob = np.asarray([len(boxes)], np.uint32).tobytes() + boxes.tobytes()
    out = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "ref_bvh")], input=blob, capture_output=True,
                         check=True).stdout
    return np.frombuffer(out, np.float32).reshape(-1, 4)


def bvh_scene_case(name, seed):
    import hashlib
    import numpy as np
    sys.path.insert(0, ROOT)
    from oracle import pyoracle
    g = pyoracle.GeneratedScene(name, seed)
    osc = pyoracle.Scene(g.positions, g.normals, g.tris4(), g.materials_raw, g.lights(), np.zeros((0, 4), np.float32))
    boxes = np.ascontiguousarray(osc.triangle_boxes(), np.float32)
    ref = reference_bvh(boxes)
    return {"scene": name, "seed": seed, "boxes": len(boxes),
            "boxes_sha256": hashlib.sha256(boxes.tobytes()).hexdigest(), "rows": len(ref),
            "bvh_sha256": hashlib.sha256(ref.tobytes()).hexdigest()}


def bvh_box_sets():
    """Seeded box sets at the builder's edges: one, two and three boxes,
    seven identical boxes, boxes flat in y, point boxes, a row of boxes
    along x, and a thousand random boxes."""
    import numpy as np
    rng = np.random.default_rng(5)

    def rnd(n):
        lo = rng.uniform(-5, 5, (n, 3))
        return np.hstack([lo, lo + rng.uniform(0, 1, (n, 3))]).astype(np.float32)
    sets = {"one": rnd(1), "two": rnd(2), "three": rnd(3), "identical": np.tile(rnd(1), (7, 1))}
    flat = rnd(40)
    flat[:, 4] = flat[:, 1]
    pts = rnd(33)
    pts[:, 3:] = pts[:, :3]
    row = np.zeros((50, 6), np.float32)
    row[:, 0] = np.arange(50)
    row[:, 3] = np.arange(50) + 0.5
    row[:, 4:] = 1
    sets.update({"flat": flat, "points": pts, "row": row, "random1000": rnd(1000)})
    return [{"name": k, "boxes": v.view(np.uint32).tolist(), "bvh": reference_bvh(v).view(np.uint32).tolist()}
            for k, v in sets.items()]


# (scene, generator seed, width, height, max depth, frame, environment filter or None, quad lights)
PT_CASES = [("box4k", 1, 24, 24, 1, 0, None, False), ("box4k", 1, 24, 24, 3, 1, None, False),
            ("box4k", 1, 24, 24, 6, 2, None, False), ("terrain_s", 1, 24, 24, 0, 0, None, False),
            ("terrain_s", 1, 24, 24, 3, 1, None, False), ("terrain_s", 1, 24, 24, 2, 0, 0, False),
            ("terrain_s", 1, 24, 24, 1, 3, 1, False), ("terrain_s", 1, 24, 24, 1, 0, None, True),
            ("terrain_s", 1, 24, 24, 2, 1, 0, True)]


def pt_quads():
    """Three quad lights {a, ab, ac, intensity} above and beside the
    terrain."""
    import numpy as np
    return np.array([[-1.0, 1.6, -1.0, 0.5, 0, 0, 0, 0, 0.5, 4.0, 3.5, 3.0],
                     [0.4, 1.5, 0.2, 0.4, 0, 0, 0, 0, 0.6, 2.0, 2.5, 3.0],
                     [1.5, 0.3, -1.0, 0, 0.3, 0, 0, 0, 0.5, 6.0, 6.0, 6.0]], np.float32)


def light_options(case, env_filter, quads, files):
    """The harness options for an environment map and quad lights, their
    temporary files, and the fixture entries that describe them."""
    import tempfile
    import numpy as np
    opts = []
    if env_filter is not None:
        env = pt_environment()
        with tempfile.NamedTemporaryFile(delete=False) as f:
            f.write(np.array([env.shape[1], env.shape[0]], np.uint32).tobytes() + env.tobytes())
            files.append(f.name)
        opts += ["--env", f.name, str(env_filter)]
        case["env"] = env.view(np.uint32).ravel().tolist()
        case["env_shape"] = list(env.shape)
        case["env_filter"] = env_filter
    if quads:
        q = pt_quads()
        with tempfile.NamedTemporaryFile(delete=False) as f:
            f.write(np.array([len(q)], np.uint32).tobytes() + q.tobytes())
            files.append(f.name)
        opts += ["--quads", f.name]
        case["quads"] = q.view(np.uint32).ravel().tolist()
    return opts


def pt_environment():
    """A seeded 32 x 16 RGBA environment map (alpha 1), stored in the
    fixture so that the test does not depend on the generator."""
    import numpy as np
    rng = np.random.default_rng(7)
    env = rng.uniform(0.0, 2.0, (16, 32, 4)).astype(np.float32)
    env[..., 3] = 1.0
    return env


def pt_case(name, seed, w, h, depth, frame, env_filter, quads):
    import numpy as np
    cmd = [os.path.join(ROOT, "oracle", "_ref", "ref_pt"), name, str(seed), str(w), str(h), str(depth), str(frame)]
    case = {"scene": name, "seed": seed, "width": w, "height": h, "max_depth": depth, "frame": frame}
    files = []
    cmd += light_options(case, env_filter, quads, files)
    try:
        out = subprocess.run(cmd, capture_output=True, check=True).stdout
    finally:
        for path in files:
            os.unlink(path)
    img = np.frombuffer(out, np.float32)
    assert len(img) == 3 * w * h
    case["radiance"] = img.view(np.uint32).tolist()
    return case


# (scene, generator seed, width, height, max depth, frames, environment filter or None, quad lights)
RESTIR_CASES = [("box4k", 1, 24, 24, 0, 3, None, False), ("box4k", 1, 24, 24, 2, 3, None, False),
                ("terrain_s", 1, 24, 24, 2, 3, None, False), ("terrain_s", 1, 24, 24, 0, 2, 0, False),
                ("terrain_s", 1, 24, 24, 1, 2, 1, False), ("terrain_s", 1, 24, 24, 0, 2, None, True),
                ("terrain_s", 1, 24, 24, 1, 2, 0, True)]


def restir_case(name, seed, w, h, depth, frames, env_filter, quads):
    import numpy as np
    cmd = [os.path.join(ROOT, "oracle", "_ref", "ref_restir"), name, str(seed), str(w), str(h), str(depth),
           str(frames)]
    case = {"scene": name, "seed": seed, "width": w, "height": h, "max_depth": depth, "frames": frames}
    files = []
    cmd += light_options(case, env_filter, quads, files)
    try:
        out = subprocess.run(cmd, capture_output=True, check=True).stdout
    finally:
        for path in files:
            os.unlink(path)
    a = np.frombuffer(out, np.float32)
    n = w * h
    assert len(a) == frames * n * 4 + n * 6
    case["color"] = a[(frames - 1) * n * 4:frames * n * 4].view(np.uint32).tolist()
    case["reservoirs"] = a[frames * n * 4:].view(np.uint32).tolist()
    return case


if __name__ == "__main__":
    main()
