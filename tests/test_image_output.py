"""Image files of the headless path (the reference's batch mode writes RGBA
half EXR, src/main.cpp:199-213): parsed back here by an independent reader
of the OpenEXR layout and compared with numpy's float16 rounding."""
import ctypes as C
import struct

import numpy as np


def _read_exr(path):
    b = open(path, "rb").read()
    assert struct.unpack_from("<I", b, 0)[0] == 20000630 and struct.unpack_from("<I", b, 4)[0] == 2
    p = 8
    attrs = {}
    while b[p] != 0:
        e = b.index(b"\0", p)
        name = b[p:e].decode()
        p = e + 1
        e = b.index(b"\0", p)
        typ = b[p:e].decode()
        p = e + 1
        size = struct.unpack_from("<i", b, p)[0]
        p += 4
        attrs[name] = (typ, b[p:p + size])
        p += size
    p += 1
    x0, y0, x1, y1 = struct.unpack("<4i", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    assert attrs["compression"][1] == b"\0"
    chans = []
    q = 0
    cl = attrs["channels"][1]
    while cl[q] != 0:
        e = cl.index(b"\0", q)
        chans.append(cl[q:e].decode())
        q = e + 1 + 16
    offsets = struct.unpack_from("<%dQ" % h, b, p)
    img = {}
    for y, off in enumerate(offsets):
        yy, size = struct.unpack_from("<ii", b, off)
        assert yy == y and size == w * len(chans) * 2
        data = np.frombuffer(b, np.float16, w * len(chans), off + 8).reshape(len(chans), w)
        for c, name in enumerate(chans):
            img.setdefault(name, np.zeros((h, w), np.float16))[y] = data[c]
    return chans, img


def test_exr_rgba_half_round_trip(built, tmp_path):
    mscgpu, _ = built
    lib = mscgpu.load_library()
    lib.msc_write_image_file.argtypes = [C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_float)]
    rng = np.random.default_rng(3)
    h, w = 7, 13
    rgb = (rng.standard_normal((h, w, 3)) * np.array([1.0, 300.0, 1e-5])).astype(np.float32)
    rgb[0, 0] = [70000.0, 65519.0, 6e-8]  # overflow to inf, largest finite, subnormal
    rgb[0, 1] = [np.inf, -0.0, 2.0 ** -25]
    path = str(tmp_path / "img.exr")
    assert lib.msc_write_image_file(path.encode(), w, h, rgb.ctypes.data_as(C.POINTER(C.c_float))) == 0
    chans, img = _read_exr(path)
    assert chans == ["A", "B", "G", "R"]
    assert np.all(img["A"] == 1)
    for name, c in (("R", 0), ("G", 1), ("B", 2)):
        want = rgb[..., c].astype(np.float16)
        assert np.array_equal(img[name].view(np.uint16), want.view(np.uint16)), name


def test_pfm_layout(built, tmp_path):
    mscgpu, _ = built
    lib = mscgpu.load_library()
    lib.msc_write_image_file.argtypes = [C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_float)]
    rgb = np.arange(2 * 3 * 3, dtype=np.float32).reshape(2, 3, 3)
    path = str(tmp_path / "img.pfm")
    assert lib.msc_write_image_file(path.encode(), 3, 2, rgb.ctypes.data_as(C.POINTER(C.c_float))) == 0
    b = open(path, "rb").read()
    head = b"PF\n3 2\n-1.0\n"
    assert b.startswith(head)
    data = np.frombuffer(b[len(head):], np.float32).reshape(2, 3, 3)
    assert np.array_equal(data[::-1], rgb)  # bottom row first
