"""ctypes binding of libvxr.so (include/vxr.h).

The Python layer only marshals arguments: every render-path operation runs in the
C++/CUDA library. Importing this module never falls back to anything else - when
libvxr.so is missing it raises.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libvxr.so")

VXR_OK = 0
VXR_E_INVALID, VXR_E_CUDA, VXR_E_NOMEM, VXR_E_STATE, VXR_E_DEVICE, VXR_E_NODEVICE, VXR_E_IO = -1, -2, -3, -4, -5, -6, -7
LIGHTS_AREA, LIGHTS_POINT = 0, 1
BLUE_NOISE_WORDS = 327680   # VXR_BLUE_NOISE_WORDS
STAGE_ALBEDO, STAGE_CANDIDATES, STAGE_SPATIAL, STAGE_SHADE, STAGE_ACCUMULATE, STAGE_PATH_TRACE = 1, 2, 3, 4, 5, 6
EMIT_ABOVE_SURFACE, EMIT_AIR, EMIT_BLOBS, EMIT_LAYER = 0, 1, 2, 3


class VxrError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"vxr error {code}: {msg}")
        self.code = code


class Light(C.Structure):
    _fields_ = [("position", C.c_uint32), ("voxel", C.c_uint32), ("size", C.c_uint32)]


class GBufferRec(C.Structure):
    _fields_ = [("voxel", C.c_uint32), ("dist", C.c_float), ("side", C.c_uint32), ("seed", C.c_uint32)]


class ReservoirRec(C.Structure):
    _fields_ = [("sumOfWeights", C.c_float), ("streamLength", C.c_uint32), ("lightIndex", C.c_uint32),
                ("adjustedWeight", C.c_float), ("positionOnVoxel", C.c_float * 3),
                ("invPositionProbability", C.c_float), ("Nlight", C.c_float * 3), ("pHat", C.c_float)]


class FrameConsts(C.Structure):
    _fields_ = [("E", C.c_float * 3), ("p0", C.c_float * 3), ("p1", C.c_float * 3), ("p2", C.c_float * 3),
                ("oneOverRes", C.c_float * 2), ("R0", C.c_uint32), ("frame", C.c_uint32),
                ("framecount", C.c_uint32), ("restirtemporalframe", C.c_uint32),
                ("Nleft", C.c_float * 4), ("Nright", C.c_float * 4), ("Ntop", C.c_float * 4),
                ("Nbottom", C.c_float * 4), ("accumulate", C.c_int32), ("spatial", C.c_int32),
                ("temporal", C.c_int32), ("numberOfLights", C.c_uint32), ("numberOfCandidates", C.c_uint32),
                ("numberOfMaxTemporalImportance", C.c_uint32), ("spatialRadius", C.c_uint32),
                ("spatialTaps", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32)]


class SceneDesc(C.Structure):
    _fields_ = [("extent", C.c_uint32), ("seed", C.c_uint32), ("octaves", C.c_uint32), ("base_freq", C.c_float),
                ("gain", C.c_float), ("height_base", C.c_float), ("height_amp", C.c_float),
                ("albedo_lo", C.c_float), ("albedo_hi", C.c_float), ("cave_threshold", C.c_float),
                ("emitters", C.c_uint32), ("emitter_mode", C.c_uint32), ("radiance_lo", C.c_float),
                ("radiance_hi", C.c_float), ("blob_count", C.c_uint32), ("blob_sigma", C.c_float),
                ("blob_fraction", C.c_float), ("layer_lo", C.c_uint32), ("layer_hi", C.c_uint32),
                ("scatter_fraction", C.c_float)]


class ProposalDesc(C.Structure):
    _fields_ = [("hidden", C.c_uint32), ("table_log2", C.c_uint32), ("res0", C.c_uint32), ("res1", C.c_uint32),
                ("epsilon", C.c_float), ("learning_rate", C.c_float), ("batch", C.c_uint32), ("seed", C.c_uint32),
                ("inference", C.c_uint32), ("training", C.c_uint32), ("pixels_per_eval", C.c_uint32),
                ("share_distance", C.c_float), ("training_lag", C.c_uint32)]


class Tuning(C.Structure):
    _fields_ = [("tile_x", C.c_uint32), ("tile_y", C.c_uint32), ("persistent", C.c_uint32),
                ("shadow_refill", C.c_uint32), ("shadow_burst", C.c_uint32), ("list_blocks_per_sm", C.c_uint32),
                ("occupancy", C.c_uint32), ("shadow_schedule", C.c_uint32), ("shadow_early_out", C.c_uint32),
                ("brick_cache", C.c_uint32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ViewDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("light_model", C.c_uint32),
                ("num_candidates", C.c_uint32), ("spatial_taps", C.c_uint32), ("spatial_radius", C.c_uint32),
                ("temporal_max_importance", C.c_uint32), ("spatial", C.c_int32), ("temporal", C.c_int32),
                ("accumulate", C.c_int32), ("rng_seed", C.c_uint32), ("tile_x", C.c_uint32), ("tile_y", C.c_uint32)]


GBUF_DTYPE = np.dtype([("voxel", "<u4"), ("dist", "<f4"), ("side", "<u4"), ("seed", "<u4")])
RES_DTYPE = np.dtype([("sumOfWeights", "<f4"), ("streamLength", "<u4"), ("lightIndex", "<u4"),
                      ("adjustedWeight", "<f4"), ("positionOnVoxel", "<f4", (3,)),
                      ("invPositionProbability", "<f4"), ("Nlight", "<f4", (3,)), ("pHat", "<f4")])
LIGHT_DTYPE = np.dtype([("position", "<u4"), ("voxel", "<u4"), ("size", "<u4")])
assert GBUF_DTYPE.itemsize == C.sizeof(GBufferRec) and RES_DTYPE.itemsize == C.sizeof(ReservoirRec)

_P = C.c_void_p
_F3 = C.POINTER(C.c_float)
# name -> argtypes (all functions return int status unless listed in _RESTYPES)
_SIGS = {
    "vxr_last_error": [], "vxr_version": [],
    "vxr_world_create": [C.POINTER(_P)], "vxr_world_destroy": [_P], "vxr_world_clear": [_P],
    "vxr_world_set": [_P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32],
    "vxr_world_add_brick": [_P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32],
    "vxr_world_get": [_P, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32)],
    "vxr_world_box": [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint32],
    "vxr_world_track_lights": [_P, C.c_int], "vxr_world_optimize": [_P, C.POINTER(C.c_uint32)],
    "vxr_world_scan_lights": [_P, C.POINTER(C.c_uint32)],
    "vxr_world_set_lights": [_P, C.POINTER(Light), C.c_uint32],
    "vxr_world_arrays": [_P, C.POINTER(C.POINTER(C.c_uint32)), C.POINTER(C.POINTER(C.c_uint32)),
                         C.POINTER(C.c_uint32), C.POINTER(C.POINTER(Light)), C.POINTER(C.c_uint32)],
    "vxr_world_brick_count": [_P, C.POINTER(C.c_uint32)],
    "vxr_world_cluster_lights": [_P, C.c_uint32, C.c_uint32, C.c_uint32],
    "vxr_world_light_clusters": [_P, C.POINTER(C.POINTER(C.c_uint32)), C.POINTER(C.c_uint32)],
    "vxr_scene_preset": [C.c_int, C.POINTER(SceneDesc)], "vxr_scene_generate": [_P, C.POINTER(SceneDesc)],
    "vxr_scene_height": [C.POINTER(SceneDesc), C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32)],
    "vxr_camera_path": [C.POINTER(SceneDesc), C.c_uint32, C.c_uint32, C.c_uint32, _F3, _F3],
    "vxr_world_checksum": [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)],
    "vxr_world_move_light": [_P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32],
    "vxr_world_stamp": [_P, _P, _P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32],
    "vxr_world_upload": [_P], "vxr_world_commit": [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_int)],
    "vxr_world_pending": [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_int), C.POINTER(C.c_int)], "vxr_world_device_bytes": [_P, C.POINTER(C.c_uint64)],
    "vxr_view_default_desc": [C.POINTER(ViewDesc)],
    "vxr_view_create": [_P, C.POINTER(ViewDesc), C.POINTER(_P)], "vxr_view_destroy": [_P],
    "vxr_view_lookat": [_P, _F3, _F3], "vxr_view_set_camera_matrix": [_P, _F3],
    "vxr_view_set_params": [_P, C.POINTER(ViewDesc)],
    "vxr_view_set_sky": [_P, _P, C.c_uint32, C.c_uint32, _P, C.c_float, _P],
    "vxr_sky_lights": [_P, C.c_uint32, C.c_uint32, C.c_uint32, _P],
    "vxr_view_begin_frame": [_P, C.POINTER(FrameConsts)], "vxr_view_set_frame_consts": [_P, C.POINTER(FrameConsts)],
    "vxr_view_stage": [_P, C.c_int], "vxr_view_end_frame": [_P], "vxr_view_render": [_P], "vxr_view_wait": [_P],
    "vxr_view_render_to_host_async": [_P, _F3, _F3, _F3, C.POINTER(C.c_uint64)],
    "vxr_view_proposal_rows": [_P, C.POINTER(C.c_uint32)],
    "vxr_view_image_wait": [_P, C.c_uint64],
    "vxr_view_stage_times": [_P, _F3],
    "vxr_view_read_gbuffer": [_P, C.c_int, _P], "vxr_view_write_gbuffer": [_P, C.c_int, _P],
    "vxr_view_read_reservoirs": [_P, C.c_int, _P], "vxr_view_write_reservoirs": [_P, C.c_int, _P],
    "vxr_view_read_frame": [_P, _F3], "vxr_view_read_accum": [_P, _F3],
    "vxr_view_render_to_host": [_P, _F3, _F3, _F3],
    "vxr_view_timer_begin": [_P], "vxr_view_timer_end": [_P, _F3],
    "vxr_view_stage_stats": [_P, C.POINTER(C.c_double), C.POINTER(C.c_uint32), C.c_int],
    "vxr_camera_create": [C.c_uint32, C.POINTER(_P)], "vxr_camera_destroy": [_P],
    "vxr_camera_lookat": [_P, _F3, _F3], "vxr_camera_set_matrix": [_P, _F3],
    "vxr_camera_begin_frame": [_P, C.c_uint32, C.c_uint32, C.POINTER(FrameConsts)],
    "vxr_camera_end_frame": [_P],
    "vxr_host_alloc": [C.c_size_t, C.POINTER(_P)], "vxr_host_free": [_P],
    "vxr_view_sum64_reset": [_P], "vxr_view_sum64_add": [_P],
    "vxr_view_sum64_mean": [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_double)],
    "vxr_view_error": [_P, C.c_int, _P, C.POINTER(C.c_double), C.POINTER(C.c_double)],
    "vxr_proposal_default_desc": [C.POINTER(ProposalDesc)],
    "vxr_view_proposal_enable": [_P, C.POINTER(ProposalDesc)], "vxr_view_proposal_use": [_P, C.c_int],
    "vxr_view_proposal_train": [_P, C.c_uint32, C.POINTER(C.c_float)],
    "vxr_view_proposal_online": [_P, C.c_uint32],
    "vxr_view_proposal_test_timeout": [_P, C.c_int],
    "vxr_view_proposal_read_candidates": [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)],
    "vxr_view_proposal_param_count": [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)],
    "vxr_view_proposal_get_params": [_P, _F3], "vxr_view_proposal_set_params": [_P, _F3],
    "vxr_view_proposal_grad": [_P, C.c_uint32, _F3, C.POINTER(C.c_uint32), _F3, C.POINTER(C.c_float), _F3],
    "vxr_view_proposal_probs": [_P, C.c_uint32, _F3, _F3],
    "vxr_view_proposal_save": [_P, C.c_char_p], "vxr_view_proposal_load": [_P, C.c_char_p],
    "vxr_batch_create": [C.POINTER(_P), C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(_P)],
    "vxr_batch_destroy": [_P], "vxr_batch_set_tuning": [_P, C.POINTER(Tuning)],
    "vxr_default_tuning": [C.POINTER(Tuning)], "vxr_view_set_tuning": [_P, C.POINTER(Tuning)],
    "vxr_view_get_tuning": [_P, C.POINTER(Tuning)],
    "vxr_view_kernel_timing": [_P, C.c_int],
    "vxr_view_kernel_stats": [_P, C.POINTER(C.c_double), C.POINTER(C.c_uint32), C.c_int],
    "vxr_kernel_name": [C.c_int], "vxr_view_work_counts": [_P, C.POINTER(C.c_uint32)],
    "vxr_device_info": [C.c_char_p, C.c_size_t, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)], "vxr_batch_render": [_P], "vxr_batch_wait": [_P, C.POINTER(C.c_float)],
    "vxr_render_frame_noalloc": [_P, _P, C.c_uint32, _P, C.c_uint32, C.c_uint32, C.POINTER(FrameConsts), _P, _P],
}
_RESTYPES = {"vxr_last_error": C.c_char_p, "vxr_version": C.c_char_p, "vxr_kernel_name": C.c_char_p}

_lib = None


def load(path=None):
    """Load libvxr.so (once). Raises OSError when the library has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError(f"libvxr.so not found at {p}: run __graft_entry__.build() (nvcc, sm_103a) first")
    lib = C.CDLL(p)
    for name, args in _SIGS.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = _RESTYPES.get(name, C.c_int)
    _lib = lib
    return lib


def exported_symbols():
    return sorted(_SIGS)


def check(code):
    if code != VXR_OK:
        raise VxrError(code, load().vxr_last_error().decode())
    return code


def _f3(v):
    return (C.c_float * 3)(*[float(x) for x in v])


class World:
    """Host voxel store (vxr_world)."""

    def __init__(self):
        self._lib = load()
        self.h = _P()
        check(self._lib.vxr_world_create(C.byref(self.h)))

    def close(self):
        if self.h:
            self._lib.vxr_world_destroy(self.h)
            self.h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set(self, x, y, z, v):
        check(self._lib.vxr_world_set(self.h, x, y, z, v))

    def add_brick(self, bx, by, bz, v):
        """World::AddBrick: grid cell (bx, by, bz) becomes solid with voxel value v."""
        check(self._lib.vxr_world_add_brick(self.h, bx, by, bz, v))

    def get(self, x, y, z):
        out = C.c_uint32()
        check(self._lib.vxr_world_get(self.h, x, y, z, C.byref(out)))
        return out.value

    def clear(self):
        """World::Clear (vxr_world_clear): empty map, no bricks, no lights."""
        check(self._lib.vxr_world_clear(self.h))

    def box(self, x1, y1, z1, x2, y2, z2, v):
        check(self._lib.vxr_world_box(self.h, x1, y1, z1, x2, y2, z2, v))

    def track_lights(self, on):
        check(self._lib.vxr_world_track_lights(self.h, 1 if on else 0))

    def optimize(self):
        r = C.c_uint32()
        check(self._lib.vxr_world_optimize(self.h, C.byref(r)))
        return r.value

    def scan_lights(self):
        n = C.c_uint32()
        check(self._lib.vxr_world_scan_lights(self.h, C.byref(n)))
        return n.value

    def set_lights(self, lights):
        arr = np.ascontiguousarray(lights, dtype=LIGHT_DTYPE)
        check(self._lib.vxr_world_set_lights(self.h, arr.ctypes.data_as(C.POINTER(Light)), len(arr)))

    def arrays(self):
        """Copies of (grid uint32[128^3], bricks uint32[n, 512], lights LIGHT_DTYPE[n])."""
        g = C.POINTER(C.c_uint32)()
        b = C.POINTER(C.c_uint32)()
        nb = C.c_uint32()
        l = C.POINTER(Light)()
        nl = C.c_uint32()
        check(self._lib.vxr_world_arrays(self.h, C.byref(g), C.byref(b), C.byref(nb), C.byref(l), C.byref(nl)))
        grid = np.ctypeslib.as_array(g, shape=(128 ** 3,)).copy()
        bricks = (np.ctypeslib.as_array(b, shape=(nb.value * 512,)).copy() if nb.value else
                  np.zeros(512, np.uint32)).reshape(-1, 512)
        if nl.value:
            lights = np.frombuffer(C.string_at(l, nl.value * 12), dtype=LIGHT_DTYPE).copy()
        else:
            lights = np.zeros(0, LIGHT_DTYPE)
        return grid, bricks, lights

    def cluster_lights(self, k, seed=1, iters=8):
        check(self._lib.vxr_world_cluster_lights(self.h, k, seed, iters))

    def light_clusters(self):
        p = C.POINTER(C.c_uint32)()
        k = C.c_uint32()
        check(self._lib.vxr_world_light_clusters(self.h, C.byref(p), C.byref(k)))
        if not k.value:
            return np.zeros(0, np.uint32), 0
        n = self.arrays()[2].shape[0]
        return np.ctypeslib.as_array(p, shape=(n,)).copy(), k.value

    def checksum(self):
        a, b = C.c_uint64(), C.c_uint64()
        check(self._lib.vxr_world_checksum(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def generate(self, desc):
        check(self._lib.vxr_scene_generate(self.h, C.byref(desc)))

    def upload(self):
        """Send the whole world to the device (vxr_world_upload)."""
        check(self._lib.vxr_world_upload(self.h))

    def stamp(self, pos, voxels, origin=(0, 0, 0), or_mask=0):
        """Set voxels[i] | or_mask at origin + unpack(pos[i]) in order (vxr_world_stamp);
        pos packs x | y << 10 | z << 20."""
        p = np.ascontiguousarray(pos, dtype=np.uint32)
        v = np.ascontiguousarray(voxels, dtype=np.uint32)
        if p.shape != v.shape:
            raise ValueError("pos and voxels differ in length")
        check(self._lib.vxr_world_stamp(self.h, p.ctypes.data, v.ctypes.data, len(p), *(int(o) for o in origin),
                                        or_mask))

    def move_light(self, index, x, y, z):
        """Move voxel light `index` of the light list to (x, y, z) (vxr_world_move_light)."""
        check(self._lib.vxr_world_move_light(self.h, index, x, y, z))

    def brick_count(self):
        """Bricks in use (vxr_world_brick_count)."""
        n = C.c_uint32()
        check(self._lib.vxr_world_brick_count(self.h, C.byref(n)))
        return n.value

    def commit(self):
        """Send the edits since the last commit (vxr_world_commit): (bricks sent, everything sent)."""
        n, full = C.c_uint32(), C.c_int()
        check(self._lib.vxr_world_commit(self.h, C.byref(n), C.byref(full)))
        return n.value, bool(full.value)

    def pending(self):
        """What the next commit would send: (changed bricks, grid changed, everything due)."""
        n, g, full = C.c_uint32(), C.c_int(), C.c_int()
        check(self._lib.vxr_world_pending(self.h, C.byref(n), C.byref(g), C.byref(full)))
        return n.value, bool(g.value), bool(full.value)

    def device_bytes(self):
        b = C.c_uint64()
        check(self._lib.vxr_world_device_bytes(self.h, C.byref(b)))
        return b.value


def scene_preset(config, **overrides):
    d = SceneDesc()
    check(load().vxr_scene_preset(config, C.byref(d)))
    for k, v in overrides.items():
        setattr(d, k, v)
    return d


def scene_height(desc, x, z):
    h = C.c_uint32()
    check(load().vxr_scene_height(C.byref(desc), x, z, C.byref(h)))
    return h.value


def camera_path(desc, seed, f, n):
    p, t = (C.c_float * 3)(), (C.c_float * 3)()
    check(load().vxr_camera_path(C.byref(desc), seed, f, n, p, t))
    return list(p), list(t)


def sky_lights(tex, seed=0x12345678):
    """vxr_sky_lights: the six sky-light colours (float32[6, 4]) of a float32[h, w, 4]
    sky texture (World::UpdateSkylights)."""
    t = np.ascontiguousarray(tex, np.float32)
    out = np.zeros((6, 4), np.float32)
    check(load().vxr_sky_lights(t.ctypes.data, t.shape[1], t.shape[0], seed, out.ctypes.data))
    return out


def device_info():
    """(name, SM count, (major, minor)) of the current CUDA device."""
    buf = C.create_string_buffer(256)
    sms, ma, mi = C.c_int(), C.c_int(), C.c_int()
    check(load().vxr_device_info(buf, 256, C.byref(sms), C.byref(ma), C.byref(mi)))
    return buf.value.decode(), sms.value, (ma.value, mi.value)


def tuning(**kw):
    """A vxr_tuning with library defaults, fields overridden by keyword."""
    t = Tuning()
    check(load().vxr_default_tuning(C.byref(t)))
    for k, v in kw.items():
        setattr(t, k, v)
    return t


def view_desc(width, height, light_model=LIGHTS_AREA, **kw):
    d = ViewDesc()
    check(load().vxr_view_default_desc(C.byref(d)))
    d.width, d.height, d.light_model = width, height, light_model
    for k, v in kw.items():
        setattr(d, k, v)
    return d


class View:
    """One camera on one world (vxr_view)."""

    def __init__(self, world, desc):
        self._lib = load()
        self.world = world
        self.desc = desc
        self.h = _P()
        check(self._lib.vxr_view_create(world.h, C.byref(desc), C.byref(self.h)))
        self.n = desc.width * desc.height

    def close(self):
        if self.h:
            self._lib.vxr_view_destroy(self.h)
            self.h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def lookat(self, pos, target):
        check(self._lib.vxr_view_lookat(self.h, _f3(pos), _f3(target)))

    def set_params(self, desc):
        check(self._lib.vxr_view_set_params(self.h, C.byref(desc)))
        self.desc = desc

    def set_sky(self, tex, light=None, scale=0.0, blue_noise=None):
        """Sky dome on (vxr_view_set_sky): tex float32[h, w, 4] texels, light float32[6, 4]
        sky lights (vxr_sky_lights of tex when None), scale = skyLightScale, blue_noise
        uint32[BLUE_NOISE_WORDS]; tex None turns it off."""
        if tex is None:
            check(self._lib.vxr_view_set_sky(self.h, None, 0, 0, None, 0.0, None))
            return
        t = np.ascontiguousarray(tex, np.float32)
        if t.ndim != 3 or t.shape[2] != 4:
            raise ValueError("sky texture must be float32[h, w, 4]")
        l = sky_lights(t) if light is None else np.ascontiguousarray(light, np.float32).reshape(6, 4)
        bn = np.ascontiguousarray(blue_noise, np.uint32)
        if bn.shape != (BLUE_NOISE_WORDS,):
            raise ValueError(f"blue noise must be uint32[{BLUE_NOISE_WORDS}]")
        check(self._lib.vxr_view_set_sky(self.h, t.ctypes.data, t.shape[1], t.shape[0], l.ctypes.data, float(scale),
                                         bn.ctypes.data))

    def begin_frame(self):
        k = FrameConsts()
        check(self._lib.vxr_view_begin_frame(self.h, C.byref(k)))
        return k

    def set_frame_consts(self, k):
        check(self._lib.vxr_view_set_frame_consts(self.h, C.byref(k)))

    def stage(self, s):
        check(self._lib.vxr_view_stage(self.h, s))

    def end_frame(self):
        check(self._lib.vxr_view_end_frame(self.h))

    def render(self):
        check(self._lib.vxr_view_render(self.h))

    def wait(self):
        check(self._lib.vxr_view_wait(self.h))

    def stage_times(self):
        ms = (C.c_float * 5)()
        check(self._lib.vxr_view_stage_times(self.h, ms))
        return list(ms)

    def read_gbuffer(self, which=0):
        out = np.zeros(self.n, GBUF_DTYPE)
        check(self._lib.vxr_view_read_gbuffer(self.h, which, out.ctypes.data))
        return out

    def write_gbuffer(self, which, recs):
        arr = np.ascontiguousarray(recs, dtype=GBUF_DTYPE)
        assert len(arr) == self.n
        check(self._lib.vxr_view_write_gbuffer(self.h, which, arr.ctypes.data))

    def read_reservoirs(self, role):
        out = np.zeros(self.n, RES_DTYPE)
        check(self._lib.vxr_view_read_reservoirs(self.h, role, out.ctypes.data))
        return out

    def write_reservoirs(self, role, recs):
        arr = np.ascontiguousarray(recs, dtype=RES_DTYPE)
        assert len(arr) == self.n
        check(self._lib.vxr_view_write_reservoirs(self.h, role, arr.ctypes.data))

    def read_frame(self):
        out = np.zeros((self.n, 4), np.float32)
        check(self._lib.vxr_view_read_frame(self.h, out.ctypes.data_as(_F3)))
        return out

    def read_accum(self):
        out = np.zeros((self.n, 4), np.float32)
        check(self._lib.vxr_view_read_accum(self.h, out.ctypes.data_as(_F3)))
        return out

    def stage_stats(self, reset=False):
        """(sum_ms[5], count[5]) per stage since the last reset."""
        sm = (C.c_double * 5)()
        cnt = (C.c_uint32 * 5)()
        check(self._lib.vxr_view_stage_stats(self.h, sm, cnt, 1 if reset else 0))
        return list(sm), list(cnt)

    def sum64_reset(self):
        check(self._lib.vxr_view_sum64_reset(self.h))

    def sum64_add(self):
        check(self._lib.vxr_view_sum64_add(self.h))

    def sum64_mean(self):
        n = C.c_uint32()
        out = np.zeros(self.n * 3, np.float64)
        check(self._lib.vxr_view_sum64_mean(self.h, C.byref(n), out.ctypes.data_as(C.POINTER(C.c_double))))
        return n.value, out.reshape(-1, 3)

    def error_vs(self, ref, which=0):
        """(MSE, MAE) of this view's frame (which=0) or accumulator (1) vs ref's FP64 mean."""
        mse, mae = C.c_double(), C.c_double()
        check(self._lib.vxr_view_error(self.h, which, ref.h, C.byref(mse), C.byref(mae)))
        return mse.value, mae.value

    # ---- learned proposal
    def proposal_enable(self, **kw):
        d = ProposalDesc()
        check(self._lib.vxr_proposal_default_desc(C.byref(d)))
        for k, v in kw.items():
            setattr(d, k, v)
        check(self._lib.vxr_view_proposal_enable(self.h, C.byref(d)))
        return d

    def proposal_use(self, on):
        check(self._lib.vxr_view_proposal_use(self.h, 1 if on else 0))

    def proposal_train(self, steps=1):
        loss = C.c_float()
        check(self._lib.vxr_view_proposal_train(self.h, steps, C.byref(loss)))
        return loss.value


    def proposal_candidates(self, k):
        """(hit pixels uint32[n], candidates uint32[k, n, 2] = light, bits(pdf)) drawn by the
        proposal for the current frame (after the candidate stage)."""
        n = C.c_uint32()
        check(self._lib.vxr_view_proposal_read_candidates(self.h, C.byref(n), None, None))
        hits = np.zeros(max(n.value, 1), np.uint32)
        cand = np.zeros((k, max(n.value, 1), 2), np.uint32)
        P = C.POINTER(C.c_uint32)
        check(self._lib.vxr_view_proposal_read_candidates(self.h, C.byref(n), hits.ctypes.data_as(P),
                                                           cand.ctypes.data_as(P)))
        return hits[:n.value], cand[:, :n.value]

    def proposal_rows(self):
        """Network evaluations of the current frame (runs sharing one count once)."""
        n = C.c_uint32()
        check(self._lib.vxr_view_proposal_rows(self.h, C.byref(n)))
        return n.value

    def proposal_test_timeout(self, on):
        """Test hook: the tensor-core inference's waits run out (error flag 16)."""
        check(self._lib.vxr_view_proposal_test_timeout(self.h, 1 if on else 0))

    def proposal_online(self, steps_per_frame=1):
        """Train the proposal inside every rendered frame (0 turns it off)."""
        check(self._lib.vxr_view_proposal_online(self.h, steps_per_frame))
    def proposal_shape(self):
        n, k, h = C.c_uint64(), C.c_uint32(), C.c_uint32()
        check(self._lib.vxr_view_proposal_param_count(self.h, C.byref(n), C.byref(k), C.byref(h)))
        return n.value, k.value, h.value

    def proposal_params(self):
        out = np.zeros(self.proposal_shape()[0], np.float32)
        check(self._lib.vxr_view_proposal_get_params(self.h, out.ctypes.data_as(_F3)))
        return out

    def proposal_set_params(self, p):
        a = np.ascontiguousarray(p, np.float32)
        check(self._lib.vxr_view_proposal_set_params(self.h, a.ctypes.data_as(_F3)))

    def proposal_grad(self, samples, target, weight):
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, 4)
        t = np.ascontiguousarray(target, np.uint32)
        w = np.ascontiguousarray(weight, np.float32)
        g = np.zeros(self.proposal_shape()[0], np.float32)
        loss = C.c_float()
        check(self._lib.vxr_view_proposal_grad(self.h, len(t), s.ctypes.data_as(_F3),
                                               t.ctypes.data_as(C.POINTER(C.c_uint32)), w.ctypes.data_as(_F3),
                                               C.byref(loss), g.ctypes.data_as(_F3)))
        return loss.value, g

    def proposal_probs(self, samples):
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, 4)
        k = self.proposal_shape()[1]
        out = np.zeros((len(s), k), np.float32)
        check(self._lib.vxr_view_proposal_probs(self.h, len(s), s.ctypes.data_as(_F3), out.ctypes.data_as(_F3)))
        return out

    def proposal_save(self, path):
        check(self._lib.vxr_view_proposal_save(self.h, str(path).encode()))

    def proposal_load(self, path):
        check(self._lib.vxr_view_proposal_load(self.h, str(path).encode()))

    def kernel_timing(self, on=True):
        check(self._lib.vxr_view_kernel_timing(self.h, 1 if on else 0))

    def kernel_stats(self, reset=False):
        """{kernel name: (summed ms, launches)} since the last reset."""
        n = KERNEL_COUNT
        sums, counts = (C.c_double * n)(), (C.c_uint32 * n)()
        check(self._lib.vxr_view_kernel_stats(self.h, sums, counts, 1 if reset else 0))
        return {self._lib.vxr_kernel_name(i).decode(): (sums[i], counts[i]) for i in range(n)}

    def work_counts(self):
        """(hit pixels, candidate shadow rays, shading shadow rays) of the last frame."""
        c = (C.c_uint32 * 3)()
        check(self._lib.vxr_view_work_counts(self.h, c))
        return tuple(c)

    def set_tuning(self, t):
        check(self._lib.vxr_view_set_tuning(self.h, C.byref(t)))

    def get_tuning(self):
        t = Tuning()
        check(self._lib.vxr_view_get_tuning(self.h, C.byref(t)))
        return t

    def timer_begin(self):
        check(self._lib.vxr_view_timer_begin(self.h))

    def timer_end(self):
        ms = C.c_float()
        check(self._lib.vxr_view_timer_end(self.h, C.byref(ms)))
        return ms.value

    def render_to_host(self, pos, target, out):
        assert out.dtype == np.float32 and out.size == self.n * 4 and out.flags.c_contiguous
        check(self._lib.vxr_view_render_to_host(self.h, _f3(pos), _f3(target), out.ctypes.data_as(_F3)))

    def render_to_host_async(self, pos, target, out):
        """Enqueue a frame and its image copy into out; returns a ticket for image_wait."""
        assert out.dtype == np.float32 and out.size == self.n * 4 and out.flags.c_contiguous
        t = C.c_uint64()
        check(self._lib.vxr_view_render_to_host_async(self.h, _f3(pos), _f3(target), out.ctypes.data_as(_F3),
                                                      C.byref(t)))
        return t.value

    def image_wait(self, ticket):
        check(self._lib.vxr_view_image_wait(self.h, ticket))


KERNEL_COUNT = 12
BATCH_MAX_VIEWS = 16
BATCH_GRAPH = 1


class Batch:
    """Several views rendered as one frame (vxr_batch): each stage is one launch over all."""

    def __init__(self, views, tile=(0, 0), graph=False, chains=1):
        self._lib = load()
        self.views = list(views)
        arr = (_P * len(self.views))(*[v.h for v in self.views])
        self.h = _P()
        flags = (BATCH_GRAPH if graph else 0) | ((chains & 15) << 8)
        check(self._lib.vxr_batch_create(arr, len(self.views), tile[0], tile[1], flags, C.byref(self.h)))

    def close(self):
        if self.h:
            self._lib.vxr_batch_destroy(self.h)
            self.h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def render(self):
        check(self._lib.vxr_batch_render(self.h))

    def set_tuning(self, t):
        check(self._lib.vxr_batch_set_tuning(self.h, C.byref(t)))

    def wait(self):
        """Wait for the batch; returns the GPU time of the last frame in ms."""
        ms = C.c_float()
        check(self._lib.vxr_batch_wait(self.h, C.byref(ms)))
        return ms.value


class Camera:
    """Host-only camera state (vxr_camera)."""

    def __init__(self, rng_seed=0x12345678):
        self._lib = load()
        self.h = _P()
        check(self._lib.vxr_camera_create(rng_seed, C.byref(self.h)))

    def __del__(self):
        try:
            if self.h:
                self._lib.vxr_camera_destroy(self.h)
        except Exception:
            pass

    def lookat(self, pos, target):
        check(self._lib.vxr_camera_lookat(self.h, _f3(pos), _f3(target)))

    def begin_frame(self, W, H):
        k = FrameConsts()
        check(self._lib.vxr_camera_begin_frame(self.h, W, H, C.byref(k)))
        return k

    def end_frame(self):
        check(self._lib.vxr_camera_end_frame(self.h))


class PinnedBuffer:
    """Page-locked float32 host buffer (vxr_host_alloc) viewed as numpy."""

    def __init__(self, count):
        self._lib = load()
        self.p = _P()
        check(self._lib.vxr_host_alloc(count * 4, C.byref(self.p)))
        self.array = np.ctypeslib.as_array(C.cast(self.p, C.POINTER(C.c_float)), shape=(count,))

    def close(self):
        if self.p:
            self._lib.vxr_host_free(self.p)
            self.p = _P()
            self.array = None
