"""Regenerate the golden fixtures in tests/golden/ from the reference tree.

Run where the retrofire reference tree is available: pass its path as the
first argument, or set RETROFIRE_REF (the default is where this build's
container mounts it, /root/reference).  It copies the reference's own golden
images and the expected values written in its unit tests (read as text),
so that the tests can pin the oracle without the reference present:

  core/tests/textured_quad.ppm      (core/tests/rendering.rs:18-60)
  core/triangle.ppm                 (core/examples/hello_tri.rs:1-58)
  raster.rs shared-edge and gradient expected maps (raster.rs:325-401)
  clip.rs all-cases histogram       (clip.rs:714-718)
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_REF = os.environ.get("RETROFIRE_REF", "/root/reference")


def parse_ppm(data):
    # P6 header: magic, width, height, maxval, one whitespace byte
    toks, i = [], 0
    while len(toks) < 4:
        while data[i:i + 1].isspace():
            i += 1
        j = i
        while not data[j:j + 1].isspace():
            j += 1
        toks.append(data[i:j])
        i = j
    i += 1
    assert toks[0] == b"P6", toks
    w, h = int(toks[1]), int(toks[2])
    img = np.frombuffer(data[i:i + w * h * 3], np.uint8).reshape(h, w, 3)
    return img


def raw_string_after(src, fn_name):
    k = src.index("fn " + fn_name)
    m = re.search(r'r"(.*?)";', src[k:], re.S)
    return m.group(1)


def main(ref, out_dir=HERE):
    out = {}
    for name, rel in [("textured_quad", "core/tests/textured_quad.ppm"),
                      ("triangle", "core/triangle.ppm")]:
        img = parse_ppm(open(os.path.join(ref, rel), "rb").read())
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), rgb=img)
    raster = open(os.path.join(ref, "core/src/render/raster.rs")).read()
    out["shared_edge"] = raw_string_after(raster, "shared_edge_should_not_have_gaps_or_overdraw")
    out["gradient"] = raw_string_after(raster, "gradient")
    clip = open(os.path.join(ref, "core/src/render/clip.rs")).read()
    m = re.search(r"out_tris,\s*\[([0-9,\s]+)\]", clip)
    out["clip_histogram"] = [int(x) for x in m.group(1).split(",") if x.strip()]
    out["source"] = "retrofire reference tree; see make_goldens.py docstring"
    with open(os.path.join(out_dir, "reference_vectors.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else DEFAULT_REF)
