"""Regenerate tests/golden/reference_kat.json from the reference's own headers.

Builds oracle/_ref/ref_kat and oracle/_ref/ref_color_kat (oracle/Makefile,
target `ref`), which compile include/cuda/random.cuh, include/cuda/math.cuh,
include/cuda/brdf.cuh, include/cuda/color.cuh and include/optix/lighting.cuh
of the reference checkout unmodified on the host, runs them and stores their
JSON output.  Needs the reference checkout, named by --reference or the
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


if __name__ == "__main__":
    main()
