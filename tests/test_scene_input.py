"""Scene input on the CPU: the OBJ readers pinned against the reference's own
tinyobjloader (compiled from its sources into oracle/_ref), and the product's
YAML/OBJ scene assembly against the oracle's independent loader."""
import os

import numpy as np
import pytest

OBJ_CASES = {
    "tri.obj": "v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvt 0 1\nf 1/1 2/2 3/3\n",
    "quad_fan.obj": "v -1 0 -1\nv 1 0 -1\nv 1 0 1\nv -1 0 1\nv 0 2 0\nvt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\n"
                    "f 1/1 2/2 3/3 4/4\nf 1/1 2/2 5/3\nf 4/4 3/3 2/2 1/1 5/1\n",
    "negative.obj": "v 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0\nvt 0 0\nvt 1 1\nf -4/-2 -3/-1 -2/-2\nf -3/-1 -1/-1 -2/-2\n",
    "normals.obj": "v 0 0 0\nv 1 0 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//1 3//1\n",
    "plain.obj": "# a comment\n\nv 0 0 0\n  v 1 0 0\n\tv 0 1 0\nf 1 2 3\n",
    "crlf.obj": "v 0 0 0\r\nv 1 0 0\r\nv 0 1 0\r\nvt 0 0\r\nvt 1 0\r\nvt 0 1\r\nvn 0 0 1\r\n"
                "f 1/1/1 2/2/1 3/3/1\r\n",
    "numbers.obj": "v 1e-3 +2.5E+1 -3.25\nv 12345.678901 -0.000001 7\nv 3. -0 .5\nv 1.5e 2x 4\n"
                   "vt 0.333333333 0.666666667\nf 1/1 2/1 3/1\nf 2/1 3/1 4/1\n",
    "shared.obj": "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\n"
                  "f 1/1 2/2 3/3\nf 1/1 3/3 4/4\nf 1/2 3/3 4/4\n",
}


@pytest.fixture(scope="module")
def obj_dir(tmp_path_factory):
    d = tmp_path_factory.mktemp("objs")
    for name, text in OBJ_CASES.items():
        (d / name).write_bytes(text.encode())
    return d


def _same(a, b):
    for x, y in zip(a, b):
        assert x.shape == y.shape, (x.shape, y.shape)
        assert np.array_equal(x.view(np.uint32) if x.dtype == np.float32 else x,
                              y.view(np.uint32) if y.dtype == np.float32 else y)


@pytest.mark.parametrize("name", sorted(OBJ_CASES))
def test_obj_readers_match_reference_tinyobj(built, obj_dir, name):
    mscgpu, oracle = built
    ref = oracle.ref_tinyobj()
    if ref is None:
        pytest.skip("reference tinyobjloader not compiled (reference sources absent)")
    path = str(obj_dir / name)
    want = oracle.obj_load(path, library=ref)
    _same(oracle.obj_load(path), want)
    _same(mscgpu.obj_load(path), want)


def test_obj_readers_match_reference_on_generated_meshes(built, tiny_scene):
    mscgpu, oracle = built
    ref = oracle.ref_tinyobj()
    if ref is None:
        pytest.skip("reference tinyobjloader not compiled (reference sources absent)")
    d = os.path.dirname(tiny_scene)
    objs = sorted(f for f in os.listdir(d) if f.endswith(".obj"))
    assert objs
    for f in objs:
        path = os.path.join(d, f)
        want = oracle.obj_load(path, library=ref)
        _same(oracle.obj_load(path), want)
        _same(mscgpu.obj_load(path), want)


def test_fan_and_dedup_semantics(built, obj_dir):
    mscgpu, _ = built
    pos, tex, idx = mscgpu.obj_load(str(obj_dir / "quad_fan.obj"))
    # first face (4 verts) -> 2 triangles (0,1,2), (0,2,3); pentagon -> 3 triangles
    assert idx.shape == (1 + 2 + 3, 3)
    assert list(idx[0]) == [0, 1, 2] and list(idx[1]) == [0, 2, 3]
    # vertex 5 with vt 1 differs from (1,1): a new unique vertex
    assert pos.shape[0] == tex.shape[0]


@pytest.mark.parametrize("cfg,scale", [(100, 1.0), (0, 0.25), (1, 0.02), (2, 0.02), (1, 0.3)])
def test_product_scene_matches_oracle_loader(built, scene_dir, cfg, scale):
    mscgpu, oracle = built
    y = mscgpu.generate_scene(cfg, 99, str(scene_dir / ("load%d" % cfg)), scale=scale)
    info, tv, tg = mscgpu.scene_load_host(y)
    s = oracle.Scene(y)
    otv, otg = s.triangles_array()
    assert info["triangles"] == s.triangles and info["lights"] == s.lights
    assert (info["width"], info["height"], info["spp"]) == (s.width, s.height, s.spp)
    assert np.array_equal(tv.view(np.uint32), otv.view(np.uint32))
    assert np.array_equal(tg, otg)


def test_scene_document_order_and_lights(built, tmp_path):
    mscgpu, _ = built
    (tmp_path / "t.obj").write_text(OBJ_CASES["tri.obj"])
    y = tmp_path / "s.yaml"
    y.write_text("""image:
  width: 8
  height: 4
  sample base: 2
camera:
  type: PinHole
  translation: [0, 0, 10]
  rotation: [0, 90, 0]
  focal length: 10
---
light:
  type: Quad
  translation: [0, 3, 0]
  rotation: [0, 0, -90]
  scale: [1, 1]
  intensity: 5
shader:
  type: Lambert
  texture:
    type: Constant
    colour: [0.5, 0.5, 0.5]
  reflectance: 1
object:
  type: Polygon
  filename: t.obj
  translation: [0, 0, 0]
  rotation: [0, 0, 0]
  scale: [1, 1, 1]
  shader: 0
object:   # a repeated key is a second object, as the reference iterates them in order
  type: Polygon
  filename: t.obj
  translation: [5, 0, 0]
  rotation: [0, 0, 0]
  scale: [2, 2, 2]
  shader: 0
""")
    info, tv, tg = mscgpu.scene_load_host(str(y))
    # objects first (geomIDs 0 and 1), then the light's geometry (geomID 2) with its two triangles
    assert info["geometries"] == 3 and info["shaders"] == 2 and info["lights"] == 1
    assert list(tg) == [0, 1, 2, 2]
    assert np.allclose(tv[1, :3], [5, 0, 0]) and np.allclose(tv[1, 3:6], [7, 0, 0])
    assert (info["width"], info["height"], info["spp"]) == (8, 4, 4)


BAD_SCENES = {
    "settings_keys": "settings:\n  min depth: 1\n  max depth: 2\n---\n",
    "camera_type": "camera:\n  type: Fisheye\n  translation: [0,0,0]\n  rotation: [0,0,0]\n  focal length: 5\n---\n",
    "image_keys": "image:\n  width: 4\n  height: 4\n---\n",
    "shader_index": "---\nobject:\n  type: Polygon\n  filename: t.obj\n  translation: [0,0,0]\n"
                    "  rotation: [0,0,0]\n  scale: [1,1,1]\n  shader: 3\n",
    "missing_obj": "---\nshader:\n  type: Lambert\n  texture:\n    type: Constant\n    colour: [1,1,1]\n"
                   "  reflectance: 1\nobject:\n  type: Polygon\n  filename: nope.obj\n  translation: [0,0,0]\n"
                   "  rotation: [0,0,0]\n  scale: [1,1,1]\n  shader: 0\n",
    "one_document": "image:\n  width: 4\n  height: 4\n  sample base: 1\n",
    "bad_indent": "image:\n  width: 4\n   height: 4\n  sample base: 1\n---\n",
}


@pytest.mark.parametrize("name", sorted(BAD_SCENES))
def test_malformed_scenes_are_rejected(built, tmp_path, name):
    mscgpu, _ = built
    (tmp_path / "t.obj").write_text(OBJ_CASES["tri.obj"])
    y = tmp_path / "bad.yaml"
    y.write_text(BAD_SCENES[name])
    with pytest.raises(mscgpu.MscError) as e:
        mscgpu.scene_load_host(str(y))
    assert e.value.code == -2


def test_missing_scene_file_fails_before_any_gpu_call(built, tmp_path):
    mscgpu, _ = built
    with pytest.raises(mscgpu.MscError) as e:
        mscgpu.Pathtracer(str(tmp_path / "absent.yaml"))
    assert e.value.code == -2 and "cannot open" in str(e.value)


def _random_obj(path, records, seed):
    """A large OBJ (several MB, so the reader splits it between workers) of
    random v / vt / vn records and faces of 2-5 corners in every index form,
    with relative (negative) indices and repeated triples."""
    rng = np.random.default_rng(seed)
    lines, nv, nvt, nvn = [], 0, 0, 0

    def idx(n):
        if rng.random() < 0.3:
            return -int(rng.integers(1, min(n, 50) + 1))
        if rng.random() < 0.05:
            return int(rng.integers(1, min(n, 8) + 1))
        return int(rng.integers(1, n + 1))
    for _ in range(records):
        r = rng.random()
        if r < 0.35 or nv < 4:
            lines.append("v %.6f %.6f %.6f" % tuple(rng.uniform(-5, 5, 3)))
            nv += 1
        elif r < 0.45:
            lines.append("vt %.6f %.6f" % tuple(rng.uniform(0, 1, 2)))
            nvt += 1
        elif r < 0.52:
            lines.append("vn %.6f %.6f %.6f" % tuple(rng.uniform(-1, 1, 3)))
            nvn += 1
        elif r < 0.53:
            lines.append("# f 1 2 3")
        else:
            corners = []
            for _ in range(int(rng.choice([2, 3, 3, 4, 5]))):
                t, v = rng.random(), idx(nv)
                if t < 0.25 or (nvt == 0 and nvn == 0):
                    corners.append("%d" % v)
                elif t < 0.5 and nvt:
                    corners.append("%d/%d" % (v, idx(nvt)))
                elif t < 0.75 and nvn:
                    corners.append("%d//%d" % (v, idx(nvn)))
                elif nvt and nvn:
                    corners.append("%d/%d/%d" % (v, idx(nvt), idx(nvn)))
                else:
                    corners.append("%d" % v)
            lines.append("f " + " ".join(corners))
    with open(path, "w", newline="") as f:
        f.write("\r\n".join(lines) + "\r\n")


def test_parallel_obj_reader_matches_reference_on_a_large_file(built, tmp_path):
    """The reader splits files of 1 MB and more between worker threads; the
    result must stay tinyobjloader's (vertex order, fans, relative indices)."""
    mscgpu, oracle = built
    path = str(tmp_path / "large.obj")
    _random_obj(path, 120000, 11)
    assert os.path.getsize(path) > (1 << 20)
    mine = mscgpu.obj_load(path)
    _same(mine, oracle.obj_load(path))
    ref = oracle.ref_tinyobj()
    if ref is not None:
        _same(mine, oracle.obj_load(path, library=ref))
