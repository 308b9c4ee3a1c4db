"""ctypes binding of the CPU oracle (oracle.h) - TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, as the checker; the product never imports it.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_TINYOBJ = os.path.join(HERE, "_ref", "libreftinyobj.so")

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("the oracle is not built (run oracle/build.py)")
        L = C.CDLL(LIB_PATH)
        P, I, F, D, U32, U64 = (C.c_void_p, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_double),
                                C.POINTER(C.c_uint32), C.POINTER(C.c_uint64))
        I32 = C.POINTER(C.c_int32)
        L.oracle_load.restype = P
        L.oracle_load.argtypes = [C.c_char_p, C.c_char_p, I]
        L.oracle_free.argtypes = [P]
        L.oracle_info.argtypes = [P, C.POINTER(C.c_int)]
        L.oracle_triangles.argtypes = [P, F, I32]
        L.oracle_render_f32.argtypes = [P, I, I, F, F, F, U64]
        L.oracle_render_f64.argtypes = [P, I, I, D, D, D, U64]
        L.oracle_render_range_f32.argtypes = [P, I, I, C.c_uint64, C.c_uint64, U64]
        L.oracle_render_range_rgb_f32.argtypes = [P, I, I, C.c_uint64, C.c_uint64, F, F, U64]
        L.oracle_trace_f32.argtypes = [P, F, F, I, F, F, F, I32, I32]
        L.oracle_occluded_f32.argtypes = [P, F, F, F, I, I32]
        L.oracle_cardinal.argtypes = [F, I, I32]
        L.oracle_ray_keys.argtypes = [F, F, I, U32]
        L.oracle_stable_sort_pairs.argtypes = [U32, U32, I, I]
        L.oracle_median_split_order.argtypes = [F, F, I, U32]
        L.oracle_bin_partition.argtypes = [F, I, I, F, I32]
        L.oracle_ray_bins.argtypes = [F, I, I, I32]
        L.oracle_image_lookup.argtypes = [C.c_char_p, I, F, F, F]
        L.oracle_bin_partition_n.argtypes = [F, I, I, I, F, I32]
        L.oracle_tent_filter.argtypes = [F, F, I, I, I, F]
        L.oracle_obj_load.argtypes = [C.c_char_p, F, F, U32, C.POINTER(C.c_int64)]
        _lib = L
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


class Scene:
    def __init__(self, yaml_path):
        err = C.create_string_buffer(512)
        self._s = lib().oracle_load(os.fsencode(yaml_path), err, 512)
        if not self._s:
            raise RuntimeError("oracle could not load %s: %s" % (yaml_path, err.value.decode()))
        info = (C.c_int * 5)()
        lib().oracle_info(self._s, info)
        self.width, self.height, self.spp, self.triangles, self.lights = list(info)

    def __del__(self):
        if getattr(self, "_s", None):
            lib().oracle_free(self._s)
            self._s = None

    def set_job(self, width=0, height=0, spp=0, min_depth=-1, max_depth=-1, cam_t=None, cam_r=None, focal=0.0,
                seed=0):
        L = lib()
        L.oracle_set_job.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                     C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float, C.c_uint32]
        t = (C.c_float * 3)(*cam_t) if cam_t is not None else None
        r = (C.c_float * 3)(*cam_r) if cam_r is not None else None
        L.oracle_set_job(self._s, width, height, spp, min_depth, max_depth, t, r, focal, seed)
        info = (C.c_int * 5)()
        L.oracle_info(self._s, info)
        self.width, self.height, self.spp, self.triangles, self.lights = list(info)

    def triangles_array(self):
        tv = np.zeros((self.triangles, 9), np.float32)
        tg = np.zeros(self.triangles, np.int32)
        lib().oracle_triangles(self._s, _p(tv, C.c_float), _p(tg, C.c_int32))
        return tv, tg

    @property
    def paths(self):
        return self.width * self.height * self.spp

    def render(self, iteration=0, threads=0, double=False, pixels=None):
        """Returns (pixels (H,W,3), sample_rgb (P,3), sample_xy (P,2), counts)."""
        dt, ct, fn = (np.float64, C.c_double, lib().oracle_render_f64) if double else \
            (np.float32, C.c_float, lib().oracle_render_f32)
        rgb = np.zeros((self.paths, 3), dt)
        xy = np.zeros((self.paths, 2), dt)
        px = np.zeros((self.height, self.width, 3), dt) if pixels is None else pixels.astype(dt).copy()
        counts = np.zeros(2, np.uint64)
        fn(self._s, iteration, threads, _p(rgb, ct), _p(xy, ct), _p(px, ct), _p(counts, C.c_uint64))
        return px, rgb, xy, counts

    def render_range(self, first, n, iteration=0, threads=0):
        counts = np.zeros(2, np.uint64)
        lib().oracle_render_range_f32(self._s, iteration, threads, first, n, _p(counts, C.c_uint64))
        return counts

    def render_range_rgb(self, first, n, iteration=0, threads=0):
        """Radiance (n,3), film positions (n,2) and query counts of paths [first, first+n)."""
        rgb = np.zeros((n, 3), np.float32)
        xy = np.zeros((n, 2), np.float32)
        counts = np.zeros(2, np.uint64)
        lib().oracle_render_range_rgb_f32(self._s, iteration, threads, first, n, _p(rgb, C.c_float), _p(xy, C.c_float),
                                          _p(counts, C.c_uint64))
        return rgb, xy, counts

    def trace(self, org, dirs):
        org = np.ascontiguousarray(org, np.float32)
        dirs = np.ascontiguousarray(dirs, np.float32)
        n = org.shape[0]
        t, u, v = (np.zeros(n, np.float32) for _ in range(3))
        g, p = np.zeros(n, np.int32), np.zeros(n, np.int32)
        lib().oracle_trace_f32(self._s, _p(org, C.c_float), _p(dirs, C.c_float), n, _p(t, C.c_float),
                               _p(u, C.c_float), _p(v, C.c_float), _p(g, C.c_int32), _p(p, C.c_int32))
        return t, u, v, g, p

    def occluded(self, org, dirs, tmax):
        org = np.ascontiguousarray(org, np.float32)
        dirs = np.ascontiguousarray(dirs, np.float32)
        tmax = np.ascontiguousarray(tmax, np.float32)
        occ = np.zeros(org.shape[0], np.int32)
        lib().oracle_occluded_f32(self._s, _p(org, C.c_float), _p(dirs, C.c_float), _p(tmax, C.c_float),
                                  org.shape[0], _p(occ, C.c_int32))
        return occ


def cardinal(dirs):
    dirs = np.ascontiguousarray(dirs, np.float32)
    out = np.zeros(dirs.shape[0], np.int32)
    lib().oracle_cardinal(_p(dirs, C.c_float), dirs.shape[0], _p(out, C.c_int32))
    return out


def ray_keys(org, dirs):
    org = np.ascontiguousarray(org, np.float32)
    dirs = np.ascontiguousarray(dirs, np.float32)
    out = np.zeros(org.shape[0], np.uint32)
    lib().oracle_ray_keys(_p(org, C.c_float), _p(dirs, C.c_float), org.shape[0], _p(out, C.c_uint32))
    return out


def stable_sort_pairs(keys, vals, bits=32):
    k = np.ascontiguousarray(keys, np.uint32).copy()
    v = np.ascontiguousarray(vals, np.uint32).copy()
    lib().oracle_stable_sort_pairs(_p(k, C.c_uint32), _p(v, C.c_uint32), k.shape[0], bits)
    return k, v


def median_split_order(org, dirs):
    """The reference's ray order (RaySort.cpp:7-118): a permutation of the rays."""
    org = np.ascontiguousarray(org, np.float32)
    dirs = np.ascontiguousarray(dirs, np.float32)
    out = np.zeros(org.shape[0], np.uint32)
    lib().oracle_median_split_order(_p(org, C.c_float), _p(dirs, C.c_float), org.shape[0], _p(out, C.c_uint32))
    return out


def image_lookup(path, s, t):
    s = np.ascontiguousarray(s, np.float32)
    t = np.ascontiguousarray(t, np.float32)
    out = np.zeros((s.shape[0], 3), np.float32)
    rc = lib().oracle_image_lookup(os.fsencode(path), s.shape[0], _p(s, C.c_float), _p(t, C.c_float),
                                   _p(out, C.c_float))
    if rc != 0:
        raise ValueError("unreadable image " + path)
    return out


def ray_bins(dirs, nbins):
    dirs = np.ascontiguousarray(dirs, np.float32)
    out = np.zeros(dirs.shape[0], np.int32)
    lib().oracle_ray_bins(_p(dirs, C.c_float), dirs.shape[0], nbins, _p(out, C.c_int32))
    return out


def bin_partition_n(rays, nbins, cap):
    rays = np.ascontiguousarray(rays, np.float32)
    out = np.zeros((nbins * cap, 12), np.float32)
    counts = np.zeros(nbins, np.int32)
    lib().oracle_bin_partition_n(_p(rays, C.c_float), rays.shape[0], nbins, cap, _p(out, C.c_float),
                                 _p(counts, C.c_int32))
    return out, counts


def bin_partition(rays, cap):
    rays = np.ascontiguousarray(rays, np.float32)
    out = np.zeros((6 * cap, 12), np.float32)
    counts = np.zeros(6, np.int32)
    lib().oracle_bin_partition(_p(rays, C.c_float), rays.shape[0], cap, _p(out, C.c_float), _p(counts, C.c_int32))
    return out, counts


def tent_filter(rgb, xy, w, h, spp):
    rgb = np.ascontiguousarray(rgb, np.float32)
    xy = np.ascontiguousarray(xy, np.float32)
    px = np.zeros((h, w, 3), np.float32)
    lib().oracle_tent_filter(_p(rgb, C.c_float), _p(xy, C.c_float), w, h, spp, _p(px, C.c_float))
    return px


def obj_load(path, library=None):
    """(positions (n,3), texcoords (m,2), indices (k,3)) via the oracle or a compatible library."""
    L = library or lib()
    fn = getattr(L, "oracle_obj_load", None) or getattr(L, "ref_obj_load")
    fn.argtypes = [C.c_char_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_uint32),
                   C.POINTER(C.c_int64)]
    sizes = np.zeros(3, np.int64)
    if fn(os.fsencode(path), None, None, None, _p(sizes, C.c_int64)) != 0:
        raise RuntimeError("cannot read " + path)
    pos = np.zeros(int(sizes[0]), np.float32)
    tex = np.zeros(int(sizes[1]), np.float32)
    idx = np.zeros(int(sizes[2]), np.uint32)
    fn(os.fsencode(path), _p(pos, C.c_float), _p(tex, C.c_float), _p(idx, C.c_uint32), _p(sizes, C.c_int64))
    return pos.reshape(-1, 3), tex.reshape(-1, 2), idx.reshape(-1, 3)


def ref_tinyobj():
    """The reference's own tinyobjloader compiled into oracle/_ref, or None."""
    if not os.path.exists(REF_TINYOBJ):
        return None
    return C.CDLL(REF_TINYOBJ)
