"""A small scene with image textures (Standard / Layered) for the tests.

Writes PFM and PPM images next to a generated tiny box scene and swaps the
first shaders' Constant textures for Standard and Layered ones."""
import os
import re

import numpy as np


def write_pfm(path, img, little=True):
    h, w = img.shape[:2]
    grey = img.ndim == 2
    head = ("Pf" if grey else "PF") + "\n%d %d\n%s\n" % (w, h, "-1.0" if little else "1.0")
    rows = img[::-1].astype("<f4" if little else ">f4")  # bottom row first
    with open(path, "wb") as f:
        f.write(head.encode())
        f.write(rows.tobytes())


def write_ppm(path, img8):
    h, w, _ = img8.shape
    with open(path, "wb") as f:
        f.write(b"P6\n# test image\n%d %d\n255\n" % (w, h))
        f.write(img8.astype(np.uint8).tobytes())


def make_texture_scene(mscgpu, out_dir, seed=7):
    y = mscgpu.generate_scene(100, 4321, out_dir)
    rng = np.random.default_rng(seed)
    write_pfm(os.path.join(out_dir, "tex_a.pfm"), rng.uniform(0.1, 0.9, size=(5, 7, 3)).astype(np.float32))
    write_ppm(os.path.join(out_dir, "tex_b.ppm"), rng.integers(0, 256, size=(4, 6, 3)))
    write_pfm(os.path.join(out_dir, "mask.pfm"), rng.uniform(0, 1, size=(3, 3)).astype(np.float32), little=False)
    mscgpu.write_image(os.path.join(out_dir, "tex_c.exr"), rng.uniform(0, 1.5, size=(6, 5, 3)).astype(np.float32))
    text = open(y).read()
    head, scene, ext = text.split("---")
    blocks = list(re.finditer(r"  texture:\n    type: Constant\n    colour: \[[^\]]*\]\n", scene))
    standard = "  texture:\n    type: Standard\n    string: tex_a.pfm\n"
    layered = ("  texture:\n    type: Layered\n    upper:\n      type: Standard\n      string: tex_b.ppm\n"
               "    lower:\n      type: Constant\n      colour: [0.2, 0.3, 0.4]\n"
               "    mask:\n      type: Standard\n      string: mask.pfm\n")
    nested = ("  texture:\n    type: Layered\n    upper:\n      type: Layered\n"
              "      upper:\n        type: Constant\n        colour: [0.9, 0.1, 0.1]\n"
              "      lower:\n        type: Standard\n        string: tex_c.exr\n"
              "      mask:\n        type: Standard\n        string: tex_b.ppm\n"
              "    lower:\n      type: Standard\n      string: tex_b.ppm\n"
              "    mask:\n      type: Constant\n      colour: [0.5, 0.25, 0.75]\n")
    repl = [standard, layered, nested]
    out = []
    last = 0
    for k, b in enumerate(blocks):
        out.append(scene[last:b.start()])
        out.append(repl[k] if k < len(repl) else b.group(0))
        last = b.end()
    out.append(scene[last:])
    path = os.path.join(out_dir, "textured.yaml")
    open(path, "w").write(head + "---" + "".join(out) + "---" + ext)
    return path
