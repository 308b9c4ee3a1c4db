"""Python binding of the GB300 path tracer's C ABI (include/msc_gpu.h).

`Pathtracer` mirrors the reference's engine class msc::Pathtracer
(include/core/Pathtracer.h:36-110 of joshbainbridge/msc-project): construct
from a scene YAML, then process() / image() / clear() / active() /
terminate().  The stage helpers call the device stages on numpy arrays.

The CUDA library is required: importing works without it, but every call
raises if libmscgpu.so is missing or no GPU is present.  There is no CPU
fallback.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmscgpu.so")

MSC_OK = 0
STAGES = ["raygen", "bins", "ray_keys", "ray_sort", "gather", "trace", "hit_sort", "shade", "shadow", "filter",
          "other"]


class MscError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("msc error %d: %s" % (code, msg))
        self.code = code


class _Stats(C.Structure):
    _fields_ = [("closest_queries", C.c_uint64), ("shadow_queries", C.c_uint64), ("batches", C.c_uint64),
                ("kernel_launches", C.c_uint64), ("process_ms", C.c_double), ("stage_ms", C.c_double * 12),
                ("stage_launches", C.c_uint64 * 12), ("width", C.c_int), ("height", C.c_int), ("spp", C.c_int),
                ("triangles", C.c_int), ("lights", C.c_int), ("iteration", C.c_int), ("load_ms", C.c_double),
                ("bvh_ms", C.c_double), ("gpu_busy_ms", C.c_double)]


class _JobDesc(C.Structure):
    _fields_ = [("scene", C.c_int), ("width", C.c_int), ("height", C.c_int), ("spp", C.c_int),
                ("min_depth", C.c_int), ("max_depth", C.c_int), ("use_camera", C.c_int),
                ("translation", C.c_float * 3), ("rotation", C.c_float * 3), ("focal_length", C.c_float),
                ("seed", C.c_uint32)]


class _Request(C.Structure):
    _fields_ = [("arrival_s", C.c_double), ("job", _JobDesc)]


class _RequestResult(C.Structure):
    _fields_ = [("job_id", C.c_int), ("status", C.c_int), ("admit_s", C.c_double), ("done_s", C.c_double),
                ("latency_s", C.c_double)]


class _ServeStats(C.Structure):
    _fields_ = [("completed", C.c_int), ("wall_s", C.c_double), ("p50_s", C.c_double), ("p99_s", C.c_double),
                ("p999_s", C.c_double), ("mrays_per_s", C.c_double), ("closest_queries", C.c_uint64),
                ("shadow_queries", C.c_uint64), ("peak_film_samples", C.c_int64), ("gpu_busy_s", C.c_double),
                ("not_admitted", C.c_int)]


_lib = None


def load_library():
    """Loads libmscgpu.so; raises when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise MscError(-3, "libmscgpu.so is not built (run __graft_entry__.build())")
    lib = C.CDLL(LIB_PATH)
    P, I, F, U32 = C.c_void_p, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_uint32)
    sig = {
        "msc_create": (I, [C.c_char_p, C.POINTER(P)]),
        "msc_destroy": (I, [P]),
        "msc_process": (I, [P, C.POINTER(I)]),
        "msc_process_device": (I, [P, C.POINTER(I)]),
        "msc_image": (I, [P, C.POINTER(F), C.POINTER(I), C.POINTER(I)]),
        "msc_clear": (I, [P]),
        "msc_active": (I, [P, C.POINTER(I)]),
        "msc_terminate": (I, [P]),
        "msc_last_error": (C.c_char_p, [P]),
        "msc_get_stats": (I, [P, C.POINTER(_Stats)]),
        "msc_set_profiling": (I, [P, I]),
        "msc_get_samples": (I, [P, F, F]),
        "msc_stage_cardinal": (I, [F, I, C.POINTER(C.c_int32)]),
        "msc_stage_bin_partition": (I, [F, I, I, F, C.POINTER(C.c_int32)]),
        "msc_stage_bin_partition_n": (I, [F, I, I, I, F, C.POINTER(C.c_int32)]),
        "msc_stage_ray_bins": (I, [F, I, I, C.POINTER(C.c_int32)]),
        "msc_stage_ray_keys": (I, [F, F, I, U32]),
        "msc_sort_pairs": (I, [U32, U32, I, I]),
        "msc_sort_pairs_device": (I, [P, P, I, I, P]),
        "msc_sort_pairs_device_noalloc": (I, [P, P, I, I, P]),
        "msc_trace_closest": (I, [P, F, F, I, F, F, F, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
        "msc_trace_occluded": (I, [P, F, F, F, I, C.POINTER(C.c_int32)]),
        "msc_generate_scene": (I, [I, C.c_uint32, C.c_double, C.c_char_p, C.c_char_p, I]),
        "msc_batch_create": (I, [I, C.c_int64, C.POINTER(P)]),
        "msc_batch_destroy": (I, [P]),
        "msc_batch_last_error": (C.c_char_p, [P]),
        "msc_batch_add_scene": (I, [P, C.c_char_p, C.POINTER(I)]),
        "msc_batch_submit": (I, [P, C.POINTER(_JobDesc), C.POINTER(I)]),
        "msc_batch_set_memory_budget": (I, [P, C.c_int64]),
        "msc_batch_memory": (I, [P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
        "msc_batch_run": (I, [P]),
        "msc_batch_job_image": (I, [P, I, C.POINTER(F), C.POINTER(I), C.POINTER(I)]),
        "msc_batch_release_job": (I, [P, I]),
        "msc_batch_get_stats": (I, [P, C.POINTER(_Stats)]),
        "msc_batch_set_profiling": (I, [P, I]),
        "msc_batch_set_max_active": (I, [P, I]),
        "msc_stage_sort_keys64": (I, [C.POINTER(C.c_uint64), I, U32]),
        "msc_write_image_file": (I, [C.c_char_p, I, I, F]),
        "msc_stage_sort_pairs_digits": (I, [U32, U32, I, I, I]),
        "msc_stage_sort_lookback_check": (I, [U32, U32, I, I, I, I]),
        "msc_batch_autotune": (I, [P, I]),
        "msc_get_tuning": (I, [P, C.POINTER(_Tuning)]),
        "msc_set_tuning": (I, [P, C.POINTER(_Tuning)]),
        "msc_batch_get_tuning": (I, [P, C.POINTER(_Tuning)]),
        "msc_batch_set_tuning": (I, [P, C.POINTER(_Tuning)]),
        "msc_batch_tune_log": (I, [P, C.POINTER(_TuneSample), I, C.POINTER(I)]),
        "msc_batch_scene_info": (I, [P, I, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_int64)]),
        "msc_serve": (I, [P, C.POINTER(_Request), I, C.POINTER(_RequestResult), C.POINTER(_ServeStats)]),
        "msc_serve_window": (I, [P, C.POINTER(_Request), I, C.c_double, C.POINTER(_RequestResult),
                                 C.POINTER(_ServeStats)]),
        "msc_obj_load": (I, [C.c_char_p, F, F, U32, C.POINTER(C.c_int64)]),
        "msc_scene_load_host": (I, [C.c_char_p, C.POINTER(C.c_int32), F, C.POINTER(C.c_int32)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    """Names declared in include/msc_gpu.h that the binding resolves."""
    lib = load_library()
    return [n for n in dir(lib) if n.startswith("msc_")]


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def _check(rc, h=None):
    if rc != MSC_OK:
        lib = load_library()
        msg = lib.msc_last_error(h)
        raise MscError(rc, msg.decode() if msg else "")


class Pathtracer:
    """msc::Pathtracer over the C ABI (include/core/Pathtracer.h:36-110)."""

    def __init__(self, yaml_path):
        lib = load_library()
        h = C.c_void_p()
        rc = lib.msc_create(os.fsencode(yaml_path), C.byref(h))
        if rc != MSC_OK:
            msg = lib.msc_last_error(None)
            raise MscError(rc, msg.decode() if msg else "")
        self._h = h
        self._lib = lib

    def close(self):
        if getattr(self, "_h", None):
            self._lib.msc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def process(self):
        it = C.c_int(0)
        _check(self._lib.msc_process(self._h, C.byref(it)), self._h)
        return it.value

    def process_device(self):
        it = C.c_int(0)
        _check(self._lib.msc_process_device(self._h, C.byref(it)), self._h)
        return it.value

    def image(self, copy=True):
        """Accumulated image as an (H, W, 3) float32 array: a copy, or with
        copy=False a view of the handle's host buffer (what msc_image returns;
        valid until the next process / clear / destroy)."""
        p = C.POINTER(C.c_float)()
        w, h = C.c_int(), C.c_int()
        _check(self._lib.msc_image(self._h, C.byref(p), C.byref(w), C.byref(h)), self._h)
        a = np.ctypeslib.as_array(p, shape=(h.value * w.value * 3,)).reshape(h.value, w.value, 3)
        return a.copy() if copy else a

    def clear(self):
        _check(self._lib.msc_clear(self._h), self._h)

    def active(self):
        a = C.c_int(0)
        _check(self._lib.msc_active(self._h, C.byref(a)), self._h)
        return bool(a.value)

    def terminate(self):
        _check(self._lib.msc_terminate(self._h), self._h)

    def set_profiling(self, on):
        _check(self._lib.msc_set_profiling(self._h, 1 if on else 0), self._h)

    def tuning(self):
        t = _Tuning()
        _check(self._lib.msc_get_tuning(self._h, C.byref(t)), self._h)
        return {k: getattr(t, k) for k, _ in _Tuning._fields_}

    def set_tuning(self, batch_exponent=20, trace_block=128, ray_sort=True, hit_sort=True, bins=6, persistent=False,
                   digit_bits=8, ray_key_bits=0):
        t = _Tuning(batch_exponent, trace_block, int(ray_sort), int(hit_sort), bins, int(persistent), digit_bits, 0, 0,
                    ray_key_bits)
        _check(self._lib.msc_set_tuning(self._h, C.byref(t)), self._h)

    def stats(self):
        s = _Stats()
        _check(self._lib.msc_get_stats(self._h, C.byref(s)), self._h)
        d = {k: getattr(s, k) for k, _ in _Stats._fields_ if k not in ("stage_ms", "stage_launches")}
        d["stage_ms"] = {STAGES[i]: s.stage_ms[i] for i in range(len(STAGES))}
        d["stage_launches"] = {STAGES[i]: int(s.stage_launches[i]) for i in range(len(STAGES))}
        return d

    def samples(self):
        st = self.stats()
        n = st["width"] * st["height"] * st["spp"]
        rgb = np.zeros((n, 3), np.float32)
        xy = np.zeros((n, 2), np.float32)
        _check(self._lib.msc_get_samples(self._h, _ptr(rgb, C.c_float), _ptr(xy, C.c_float)), self._h)
        return rgb, xy

    def trace_closest(self, org, dirs):
        org = np.ascontiguousarray(org, np.float32)
        dirs = np.ascontiguousarray(dirs, np.float32)
        n = org.shape[0]
        t, u, v = (np.zeros(n, np.float32) for _ in range(3))
        g, p = np.zeros(n, np.int32), np.zeros(n, np.int32)
        _check(self._lib.msc_trace_closest(self._h, _ptr(org, C.c_float), _ptr(dirs, C.c_float), n,
                                           _ptr(t, C.c_float), _ptr(u, C.c_float), _ptr(v, C.c_float),
                                           _ptr(g, C.c_int32), _ptr(p, C.c_int32)), self._h)
        return t, u, v, g, p

    def trace_occluded(self, org, dirs, tmax):
        org = np.ascontiguousarray(org, np.float32)
        dirs = np.ascontiguousarray(dirs, np.float32)
        tmax = np.ascontiguousarray(tmax, np.float32)
        n = org.shape[0]
        occ = np.zeros(n, np.int32)
        _check(self._lib.msc_trace_occluded(self._h, _ptr(org, C.c_float), _ptr(dirs, C.c_float),
                                            _ptr(tmax, C.c_float), n, _ptr(occ, C.c_int32)), self._h)
        return occ


def cardinal(dirs):
    lib = load_library()
    dirs = np.ascontiguousarray(dirs, np.float32)
    out = np.zeros(dirs.shape[0], np.int32)
    _check(lib.msc_stage_cardinal(_ptr(dirs, C.c_float), dirs.shape[0], _ptr(out, C.c_int32)))
    return out


def bin_partition(rays, cap, nbins=6):
    """rays: (n, 12) float32 records; returns (nbins*cap, 12) bins and nbins counts."""
    lib = load_library()
    rays = np.ascontiguousarray(rays, np.float32)
    out = np.zeros((nbins * cap, 12), np.float32)
    counts = np.zeros(nbins, np.int32)
    _check(lib.msc_stage_bin_partition_n(_ptr(rays, C.c_float), rays.shape[0], nbins, cap, _ptr(out, C.c_float),
                                         _ptr(counts, C.c_int32)))
    return out, counts


def ray_bins(dirs, nbins):
    """Direction bin of each direction among 6, 26 or 98."""
    lib = load_library()
    dirs = np.ascontiguousarray(dirs, np.float32)
    out = np.zeros(dirs.shape[0], np.int32)
    _check(lib.msc_stage_ray_bins(_ptr(dirs, C.c_float), dirs.shape[0], nbins, _ptr(out, C.c_int32)))
    return out


def ray_keys(org, dirs):
    lib = load_library()
    org = np.ascontiguousarray(org, np.float32)
    dirs = np.ascontiguousarray(dirs, np.float32)
    keys = np.zeros(org.shape[0], np.uint32)
    _check(lib.msc_stage_ray_keys(_ptr(org, C.c_float), _ptr(dirs, C.c_float), org.shape[0],
                                  _ptr(keys, C.c_uint32)))
    return keys


def sort_pairs(keys, vals, bits=32):
    lib = load_library()
    k = np.ascontiguousarray(keys, np.uint32).copy()
    v = np.ascontiguousarray(vals, np.uint32).copy()
    _check(lib.msc_sort_pairs(_ptr(k, C.c_uint32), _ptr(v, C.c_uint32), k.shape[0], bits))
    return k, v


def write_image(path, rgb):
    """Writes an (h, w, 3) float image as OpenEXR (RGBA half) or PFM, by the file's extension."""
    lib = load_library()
    rgb = np.ascontiguousarray(rgb, np.float32)
    h, w = rgb.shape[:2]
    _check(lib.msc_write_image_file(os.fsencode(path), w, h, _ptr(rgb, C.c_float)))


def sort_pairs_digits(keys, vals, bits=32, digit_bits=8):
    """Stable radix sort with 4-, 8- or 11-bit digits; returns sorted (keys, vals)."""
    lib = load_library()
    k = np.ascontiguousarray(keys, np.uint32).copy()
    v = np.ascontiguousarray(vals, np.uint32).copy()
    _check(lib.msc_stage_sort_pairs_digits(_ptr(k, C.c_uint32), _ptr(v, C.c_uint32), k.shape[0], bits, digit_bits))
    return k, v


def sort_lookback_check(keys, vals, bits, spin_cap, withhold_first_tile):
    """The sort with a given look-back spin cap (and optionally a first tile
    that never posts): returns (status code, keys, vals); raises nothing."""
    lib = load_library()
    k = np.ascontiguousarray(keys, np.uint32).copy()
    v = np.ascontiguousarray(vals, np.uint32).copy()
    rc = lib.msc_stage_sort_lookback_check(_ptr(k, C.c_uint32), _ptr(v, C.c_uint32), k.shape[0], bits, spin_cap,
                                           1 if withhold_first_tile else 0)
    return rc, k, v


def sort_keys64(keys):
    """Stable order of 64-bit keys as the 64-bit hit sort takes it."""
    lib = load_library()
    k = np.ascontiguousarray(keys, np.uint64)
    perm = np.zeros(k.shape[0], np.uint32)
    _check(lib.msc_stage_sort_keys64(_ptr(k, C.c_uint64), k.shape[0], _ptr(perm, C.c_uint32)))
    return perm


def generate_scene(config, seed, out_dir, scale=1.0):
    lib = load_library()
    os.makedirs(out_dir, exist_ok=True)
    buf = C.create_string_buffer(4096)
    rc = lib.msc_generate_scene(config, seed, scale, os.fsencode(out_dir), buf, 4096)
    if rc != MSC_OK:
        msg = lib.msc_last_error(None)
        raise MscError(rc, msg.decode() if msg else "")
    return buf.value.decode()


def obj_load(path):
    """(positions (n,3), texcoords (m,2), indices (k,3)) read by the product's OBJ reader."""
    lib = load_library()
    sizes = np.zeros(3, np.int64)
    _check(lib.msc_obj_load(os.fsencode(path), None, None, None, _ptr(sizes, C.c_int64)))
    pos = np.zeros(int(sizes[0]), np.float32)
    tex = np.zeros(int(sizes[1]), np.float32)
    idx = np.zeros(int(sizes[2]), np.uint32)
    _check(lib.msc_obj_load(os.fsencode(path), _ptr(pos, C.c_float), _ptr(tex, C.c_float), _ptr(idx, C.c_uint32),
                            _ptr(sizes, C.c_int64)))
    return pos.reshape(-1, 3), tex.reshape(-1, 2), idx.reshape(-1, 3)


def scene_load_host(yaml_path):
    """Host-only scene parse: (info dict, tri_v (T,9), tri_geom (T,))."""
    lib = load_library()
    info = np.zeros(8, np.int32)
    _check(lib.msc_scene_load_host(os.fsencode(yaml_path), _ptr(info, C.c_int32), None, None))
    T = int(info[3])
    tv = np.zeros((T, 9), np.float32)
    tg = np.zeros(T, np.int32)
    _check(lib.msc_scene_load_host(os.fsencode(yaml_path), _ptr(info, C.c_int32), _ptr(tv, C.c_float),
                                   _ptr(tg, C.c_int32)))
    keys = ["width", "height", "spp", "triangles", "lights", "shaders", "geometries", "camera"]
    return dict(zip(keys, [int(x) for x in info])), tv, tg


class _Tuning(C.Structure):
    _fields_ = [("batch_exponent", C.c_int), ("trace_block", C.c_int), ("ray_sort", C.c_int), ("hit_sort", C.c_int),
                ("bins", C.c_int), ("persistent", C.c_int), ("digit_bits", C.c_int), ("tuning", C.c_int),
                ("samples", C.c_int), ("ray_key_bits", C.c_int)]


class _TuneSample(C.Structure):
    _fields_ = [("batch_exponent", C.c_int), ("trace_block", C.c_int), ("ray_sort", C.c_int), ("hit_sort", C.c_int),
                ("bins", C.c_int), ("persistent", C.c_int), ("digit_bits", C.c_int), ("mrays_per_s", C.c_double),
                ("ray_key_bits", C.c_int)]


def _job_desc(scene, width=0, height=0, spp=0, min_depth=-1, max_depth=-1, camera=None, seed=0):
    d = _JobDesc()
    d.scene, d.width, d.height, d.spp = scene, width, height, spp
    d.min_depth, d.max_depth = min_depth, max_depth
    if camera is not None:
        t, r, f = camera
        d.use_camera = 1
        d.translation[:] = list(t)
        d.rotation[:] = list(r)
        d.focal_length = f
    d.seed = seed
    return d


class Batch:
    """Batched and served forms: many resident scenes and jobs in one wavefront."""

    def __init__(self, batch_exponent=20, film_samples=1 << 26):
        self._lib = load_library()
        b = C.c_void_p()
        rc = self._lib.msc_batch_create(batch_exponent, film_samples, C.byref(b))
        if rc != MSC_OK:
            raise MscError(rc, (self._lib.msc_batch_last_error(None) or b"").decode())
        self._b = b

    def _check(self, rc):
        if rc != MSC_OK:
            raise MscError(rc, (self._lib.msc_batch_last_error(self._b) or b"").decode())

    def close(self):
        if getattr(self, "_b", None):
            self._lib.msc_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def add_scene(self, yaml_path):
        sid = C.c_int()
        self._check(self._lib.msc_batch_add_scene(self._b, os.fsencode(yaml_path), C.byref(sid)))
        return sid.value

    def scene_info(self, scene):
        """(lo, hi, triangles) of a resident scene: its triangle box and count."""
        lo, hi, n = (C.c_float * 3)(), (C.c_float * 3)(), C.c_int64()
        self._check(self._lib.msc_batch_scene_info(self._b, scene, lo, hi, C.byref(n)))
        return np.array(lo[:], np.float32), np.array(hi[:], np.float32), n.value

    def set_memory_budget(self, nbytes):
        """Device-memory budget (bytes, 0: none) for scenes, fixed buffers and job images."""
        self._check(self._lib.msc_batch_set_memory_budget(self._b, int(nbytes)))

    def memory(self):
        """(in_use, fixed buffers + scenes, admitted job images) in bytes."""
        a, f, j = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(self._lib.msc_batch_memory(self._b, C.byref(a), C.byref(f), C.byref(j)))
        return a.value, f.value, j.value

    def submit(self, scene, **kw):
        """kw: width, height, spp, min_depth, max_depth, camera=(translation, rotation, focal), seed."""
        jid = C.c_int()
        d = _job_desc(scene, **kw)
        self._check(self._lib.msc_batch_submit(self._b, C.byref(d), C.byref(jid)))
        return jid.value

    def run(self):
        self._check(self._lib.msc_batch_run(self._b))

    def image(self, job):
        p = C.POINTER(C.c_float)()
        w, h = C.c_int(), C.c_int()
        self._check(self._lib.msc_batch_job_image(self._b, job, C.byref(p), C.byref(w), C.byref(h)))
        return np.ctypeslib.as_array(p, shape=(h.value * w.value * 3,)).reshape(h.value, w.value, 3).copy()

    def release(self, job):
        self._check(self._lib.msc_batch_release_job(self._b, job))

    def set_profiling(self, on):
        self._check(self._lib.msc_batch_set_profiling(self._b, 1 if on else 0))

    def autotune(self, windows=0):
        """Start the online autotuner (batch size, traversal block, sorts)."""
        self._check(self._lib.msc_batch_autotune(self._b, windows))

    def tuning(self):
        t = _Tuning()
        self._check(self._lib.msc_batch_get_tuning(self._b, C.byref(t)))
        return {k: getattr(t, k) for k, _ in _Tuning._fields_}

    def set_tuning(self, batch_exponent=20, trace_block=128, ray_sort=True, hit_sort=True, bins=6, persistent=False,
                   digit_bits=8, ray_key_bits=0):
        t = _Tuning(batch_exponent, trace_block, int(ray_sort), int(hit_sort), bins, int(persistent), digit_bits, 0, 0,
                    ray_key_bits)
        self._check(self._lib.msc_batch_set_tuning(self._b, C.byref(t)))

    def tune_log(self):
        n = C.c_int()
        self._check(self._lib.msc_batch_tune_log(self._b, None, 0, C.byref(n)))
        buf = (_TuneSample * max(1, n.value))()
        self._check(self._lib.msc_batch_tune_log(self._b, buf, n.value, C.byref(n)))
        return [{k: getattr(buf[i], k) for k, _ in _TuneSample._fields_} for i in range(n.value)]

    def set_max_active(self, n):
        self._check(self._lib.msc_batch_set_max_active(self._b, n))

    def stats(self):
        s = _Stats()
        self._check(self._lib.msc_batch_get_stats(self._b, C.byref(s)))
        d = {k: getattr(s, k) for k, _ in _Stats._fields_ if k not in ("stage_ms", "stage_launches")}
        d["stage_ms"] = {STAGES[i]: s.stage_ms[i] for i in range(len(STAGES))}
        return d

    def serve(self, requests, window_s=None):
        """requests: list of (arrival_s, job kwargs incl. scene).  Returns (results, stats).
        window_s: admission closes after that many seconds (msc_serve_window)."""
        n = len(requests)
        reqs = (_Request * max(n, 1))()
        for i, (t, kw) in enumerate(requests):
            kw = dict(kw)
            reqs[i].arrival_s = t
            reqs[i].job = _job_desc(kw.pop("scene"), **kw)
        res = (_RequestResult * max(n, 1))()
        st = _ServeStats()
        if window_s is None:
            self._check(self._lib.msc_serve(self._b, reqs, n, res, C.byref(st)))
        else:
            self._check(self._lib.msc_serve_window(self._b, reqs, n, float(window_s), res, C.byref(st)))
        results = [{k: getattr(res[i], k) for k, _ in _RequestResult._fields_} for i in range(n)]
        stats = {k: getattr(st, k) for k, _ in _ServeStats._fields_}
        return results, stats
