"""Image textures (StandardTexture / LayeredTexture) on the CPU side.

The reference samples images through OpenImageIO (absent here); both sides
restate it as a periodic bilinear lookup between texel centres, t = 0 on the
image's top row.  These tests pin the oracle's image reading and lookup against
an independent numpy restatement, and check that both scene loaders accept the
texture trees and reject unreadable images."""
import os

import numpy as np
import pytest

from texture_scene import make_texture_scene, write_pfm, write_ppm


def _bilinear(img, s, t):
    h, w, _ = img.shape
    s = np.float32(s) - np.floor(np.float32(s))
    t = np.float32(t) - np.floor(np.float32(t))
    x = np.float32(s * np.float32(w) - np.float32(0.5))
    y = np.float32(t * np.float32(h) - np.float32(0.5))
    x0, y0 = int(np.floor(x)), int(np.floor(y))
    fx, fy = np.float32(x - np.float32(x0)), np.float32(y - np.float32(y0))
    x0, y0 = x0 % w, y0 % h
    x1, y1 = (x0 + 1) % w, (y0 + 1) % h
    gx, gy = np.float32(1) - fx, np.float32(1) - fy
    c = lambda yy, xx: img[yy, xx].astype(np.float32)
    return (c(y0, x0) * gx + c(y0, x1) * fx) * gy + (c(y1, x0) * gx + c(y1, x1) * fx) * fy


@pytest.mark.parametrize("kind", ["pfm_le", "pfm_be", "pfm_grey", "ppm8"])
def test_oracle_image_lookup_is_periodic_bilinear(built, tmp_path, kind):
    _, oracle = built
    rng = np.random.default_rng(3)
    if kind == "ppm8":
        raw = rng.integers(0, 256, size=(4, 6, 3))
        img = (raw / np.float32(255)).astype(np.float32)
        path = str(tmp_path / "a.ppm")
        write_ppm(path, raw)
    elif kind == "pfm_grey":
        g = rng.uniform(0, 1, size=(3, 5)).astype(np.float32)
        img = np.repeat(g[:, :, None], 3, axis=2)
        path = str(tmp_path / "g.pfm")
        write_pfm(path, g)
    else:
        img = rng.uniform(0, 2, size=(5, 7, 3)).astype(np.float32)
        path = str(tmp_path / "a.pfm")
        write_pfm(path, img, little=(kind == "pfm_le"))
    s = np.concatenate([rng.uniform(-2, 3, 200), [0, 0.5, 1, 1e-7, -1e-7]]).astype(np.float32)
    t = np.concatenate([rng.uniform(-2, 3, 200), [0, 1, 0.5, 0.999999, 2]]).astype(np.float32)
    got = oracle.image_lookup(path, s, t)
    want = np.array([_bilinear(img, a, b) for a, b in zip(s, t)], np.float32)
    assert np.allclose(got, want, rtol=1e-6, atol=1e-6)


def test_textured_scene_loads_in_both_loaders(built, tmp_path):
    mscgpu, oracle = built
    y = make_texture_scene(mscgpu, str(tmp_path))
    info, tv, _ = mscgpu.scene_load_host(y)
    s = oracle.Scene(y)
    otv, _ = s.triangles_array()
    assert info["triangles"] == s.triangles
    assert np.array_equal(tv.view(np.uint32), otv.view(np.uint32))


def test_unreadable_texture_image_is_rejected(built, tmp_path):
    mscgpu, _ = built
    y = make_texture_scene(mscgpu, str(tmp_path))
    with open(os.path.join(str(tmp_path), "tex_a.pfm"), "wb") as f:
        f.write(b"P3\n1 1\n255\n0 0 0\n")  # ASCII PPM: not a format this build reads
    with pytest.raises(mscgpu.MscError, match="not PFM, binary PPM or OpenEXR"):
        mscgpu.scene_load_host(y)


def test_exr_texture_reads_back_the_written_halves(built, tmp_path):
    """An image written by the product's OpenEXR writer (RGBA half) is read back
    by the texture loader: at texel centres the lookup returns the halves."""
    mscgpu, oracle = built
    rng = np.random.default_rng(11)
    img = rng.uniform(0, 3, size=(4, 7, 3)).astype(np.float32)
    path = str(tmp_path / "t.exr")
    mscgpu.write_image(path, img)
    h, w = img.shape[:2]
    ys, xs = np.mgrid[0:h, 0:w]
    s = ((xs + 0.5) / w).astype(np.float32).ravel()
    t = ((ys + 0.5) / h).astype(np.float32).ravel()
    got = oracle.image_lookup(path, s, t)
    want = img.astype(np.float16).astype(np.float32).reshape(-1, 3)
    assert np.allclose(got, want, rtol=1e-6, atol=1e-7)
