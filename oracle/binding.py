"""ctypes binding of the CPU oracles (test infrastructure only: imported by tests/,
__graft_entry__.smoke() and bench.py's CPU baseline, never by the product)."""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

GBUF_DTYPE = np.dtype([("voxel", "<u4"), ("dist", "<f4"), ("side", "<u4"), ("seed", "<u4")])
RES_DTYPE = np.dtype([("sumOfWeights", "<f4"), ("streamLength", "<u4"), ("lightIndex", "<u4"),
                      ("adjustedWeight", "<f4"), ("positionOnVoxel", "<f4", (3,)),
                      ("invPositionProbability", "<f4"), ("Nlight", "<f4", (3,)), ("pHat", "<f4")])
LIGHT_DTYPE = np.dtype([("position", "<u4"), ("voxel", "<u4"), ("size", "<u4")])


class FrameConsts(C.Structure):
    _fields_ = [("E", C.c_float * 3), ("p0", C.c_float * 3), ("p1", C.c_float * 3), ("p2", C.c_float * 3),
                ("oneOverRes", C.c_float * 2), ("R0", C.c_uint32), ("frame", C.c_uint32),
                ("framecount", C.c_uint32), ("restirtemporalframe", C.c_uint32),
                ("Nleft", C.c_float * 4), ("Nright", C.c_float * 4), ("Ntop", C.c_float * 4),
                ("Nbottom", C.c_float * 4), ("accumulate", C.c_int32), ("spatial", C.c_int32),
                ("temporal", C.c_int32), ("numberOfLights", C.c_uint32), ("numberOfCandidates", C.c_uint32),
                ("numberOfMaxTemporalImportance", C.c_uint32), ("spatialRadius", C.c_uint32),
                ("spatialTaps", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32)]


class Camera(C.Structure):
    _fields_ = [("M", C.c_float * 16), ("E", C.c_float * 3), ("p0", C.c_float * 3), ("p1", C.c_float * 3),
                ("p2", C.c_float * 3), ("first", C.c_int), ("rng", C.c_uint32), ("frame", C.c_uint32),
                ("framecount", C.c_uint32), ("restirtemporalframe", C.c_uint32)]


def copy_consts(src, dst_cls):
    """Field-wise copy between FrameConsts classes of different modules (same layout)."""
    d = dst_cls()
    C.memmove(C.byref(d), C.byref(src), C.sizeof(d))
    return d


_P = C.c_void_p
_U32P = C.POINTER(C.c_uint32)
_F = C.POINTER(C.c_float)

_port = None
_ref = None


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def load_port():
    global _port
    if _port is not None:
        return _port
    from . import build as B  # noqa: PLC0415
    lib = C.CDLL(B.build_port())
    sig = {
        "orc_build_uber": (None, [_P, _P]),
        "orc_world_get": (C.c_uint32, [_P, _P, C.c_uint32, C.c_uint32, C.c_uint32]),
        "orc_scan_lights": (C.c_uint32, [_P, _P, _P, C.c_uint32]),
        "orc_store_create": (_P, []), "orc_store_destroy": (None, [_P]),
        "orc_store_set": (None, [_P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]),
        "orc_store_get": (C.c_uint32, [_P, C.c_uint32, C.c_uint32, C.c_uint32]),
        "orc_store_optimize": (C.c_uint32, [_P]), "orc_store_lights": (C.c_uint32, [_P, _P, C.c_uint32]),
        "orc_store_grid": (_U32P, [_P]), "orc_store_bricks": (_U32P, [_P]),
        "orc_camera_init": (None, [C.POINTER(Camera), C.c_uint32]),
        "orc_lookat": (None, [C.POINTER(Camera), _F, _F]),
        "orc_begin_frame": (None, [C.POINTER(Camera), C.c_uint32, C.c_uint32, C.POINTER(FrameConsts)]),
        "orc_end_frame": (None, [C.POINTER(Camera)]),
        "orc_create": (_P, [C.c_int, C.c_int, C.c_int]), "orc_destroy": (None, [_P]),
        "orc_set_world": (None, [_P, _P, _P, _P]), "orc_set_lights": (None, [_P, _P, C.c_uint32]),
        "orc_set_candidates": (None, [_P, _P, _P, C.c_size_t]),
        "orc_frame_start": (None, [_P]),
        "orc_stage": (None, [_P, C.POINTER(FrameConsts), C.c_int, C.c_int, C.c_int]),
        "orc_read_gbuffer": (None, [_P, C.c_int, _P]),
        "orc_write_gbuffer": (None, [_P, C.c_int, _P, C.POINTER(FrameConsts)]),
        "orc_read_reservoirs": (None, [_P, C.c_int, _P]), "orc_write_reservoirs": (None, [_P, C.c_int, _P]),
        "orc_read_image": (None, [_P, C.c_int, _P]),
        "orc_trace": (C.c_uint32, [_P, C.c_int, _F, _F, C.c_int, C.c_uint32, C.c_uint32, _F, _U32P]),
        "orc_sincos": (None, [C.c_float, _F, _F]),
    }
    for n, (res, args) in sig.items():
        f = getattr(lib, n)
        f.restype = res
        f.argtypes = args
    _port = lib
    return lib


def load_stb():
    """The reference's stb_image (oracle/stb_ref.c), or None when not available here."""
    from . import build as B  # noqa: PLC0415
    try:
        path = B.build_stb()
    except RuntimeError:
        path = None
    if not path:
        return None
    lib = C.CDLL(path)
    lib.stbref_loadf.restype = C.POINTER(C.c_float)
    lib.stbref_loadf.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.stbref_free.argtypes = [C.c_void_p]
    lib.stbref_write_hdr.restype = C.c_int
    lib.stbref_write_hdr.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, _P]
    return lib


def stb_loadf(path):
    """float32[h, w, comp] through the reference's stbi_loadf, or None if it fails."""
    lib = load_stb()
    w, h, c = C.c_int(), C.c_int(), C.c_int()
    p = lib.stbref_loadf(str(path).encode(), C.byref(w), C.byref(h), C.byref(c))
    if not p:
        return None
    try:
        return np.ctypeslib.as_array(p, (h.value, w.value, c.value)).copy()
    finally:
        lib.stbref_free(p)


def stb_write_hdr(path, rgb):
    """Write float[h, w, 3] with the reference's stbi_write_hdr."""
    a = np.ascontiguousarray(rgb, np.float32)
    if not load_stb().stbref_write_hdr(str(path).encode(), a.shape[1], a.shape[0], a.shape[2], a.ctypes.data):
        raise RuntimeError("stbi_write_hdr failed")


def load_ogt():
    """The reference's ogt_vox reader (oracle/ogt_ref.cpp), or None when not available."""
    from . import build as B  # noqa: PLC0415
    try:
        path = B.build_ogt()
    except RuntimeError:
        path = None
    if not path:
        return None
    lib = C.CDLL(path)
    lib.ogtref_read.restype = C.c_void_p
    lib.ogtref_read.argtypes = [C.c_char_p, C.c_uint32]
    lib.ogtref_free.argtypes = [C.c_void_p]
    lib.ogtref_counts.argtypes = [C.c_void_p, _P]
    lib.ogtref_instance.restype = C.c_uint32
    lib.ogtref_instance.argtypes = [C.c_void_p, C.c_uint32, _P]
    lib.ogtref_model.argtypes = [C.c_void_p, C.c_uint32, _P, _P]
    lib.ogtref_palette.argtypes = [C.c_void_p, _P]
    return lib


def ogt_scene(path):
    """(models, instances, palette) of a .vox file through the reference's
    ogt_vox_read_scene: models uint8[sz, sy, sx], instances (model index, float32[4, 4]
    transform m00 .. m33), palette uint8[256, 4]; None when the reader rejects the file."""
    lib = load_ogt()
    data = open(path, "rb").read()
    s = lib.ogtref_read(data, len(data))
    if not s:
        return None
    try:
        counts = np.zeros(2, np.uint32)
        lib.ogtref_counts(s, counts.ctypes.data)
        models = []
        for m in range(int(counts[1])):
            size = np.zeros(3, np.uint32)
            lib.ogtref_model(s, m, size.ctypes.data, None)
            vox = np.zeros(int(size.prod()), np.uint8)
            lib.ogtref_model(s, m, size.ctypes.data, vox.ctypes.data)
            models.append(vox.reshape(int(size[2]), int(size[1]), int(size[0])))
        instances = []
        for i in range(int(counts[0])):
            t = np.zeros(16, np.float32)
            mid = lib.ogtref_instance(s, i, t.ctypes.data)
            instances.append((int(mid), t.reshape(4, 4)))
        pal = np.zeros(1024, np.uint8)
        lib.ogtref_palette(s, pal.ctypes.data)
        return models, instances, pal.reshape(256, 4)
    finally:
        lib.ogtref_free(s)


def load_ref():
    """The reference oracle, or None when it is not available on this machine."""
    global _ref
    if _ref is not None:
        return _ref or None
    from . import build as B  # noqa: PLC0415
    try:
        path = B.build_ref()
    except RuntimeError:
        path = None
    if not path:
        _ref = False
        return None
    lib = C.CDLL(path)
    for v in ("area", "point"):
        sig = {
            f"vxref_create_{v}": (_P, [C.c_int, C.c_int]), f"vxref_destroy_{v}": (None, [_P]),
            f"vxref_set_world_{v}": (None, [_P, _P, _P, _P]), f"vxref_set_lights_{v}": (None, [_P, _P, C.c_uint32]),
            f"vxref_update_uber_{v}": (None, [_P, _P]), f"vxref_begin_frame_{v}": (None, [_P]),
            f"vxref_stage_{v}": (None, [_P, C.POINTER(FrameConsts), C.c_int]),
            f"vxref_stage_rows_{v}": (None, [_P, C.POINTER(FrameConsts), C.c_int, C.c_int, C.c_int]),
            f"vxref_read_gbuffer_{v}": (None, [_P, C.c_int, _P, _P]),
            f"vxref_read_reservoirs_{v}": (None, [_P, C.c_int, _P]),
            f"vxref_write_reservoirs_{v}": (None, [_P, C.c_int, _P]),
            f"vxref_read_image_{v}": (None, [_P, C.c_int, _P]),
            f"vxref_set_sky_{v}": (None, [_P, _P, C.c_uint32, C.c_uint32, _P, C.c_float, _P]),
            f"vxref_trace_{v}": (C.c_uint32, [_P, C.c_int, _F, _F, C.c_int, C.c_uint32, C.c_uint32, _F, _U32P]),
        }
        for n, (res, args) in sig.items():
            f = getattr(lib, n)
            f.restype = res
            f.argtypes = args
    _ref = lib
    return lib


class SceneDesc(C.Structure):
    """vxr_scene_desc (include/vxr.h)."""
    _fields_ = [("extent", C.c_uint32), ("seed", C.c_uint32), ("octaves", C.c_uint32), ("base_freq", C.c_float),
                ("gain", C.c_float), ("height_base", C.c_float), ("height_amp", C.c_float),
                ("albedo_lo", C.c_float), ("albedo_hi", C.c_float), ("cave_threshold", C.c_float),
                ("emitters", C.c_uint32), ("emitter_mode", C.c_uint32), ("radiance_lo", C.c_float),
                ("radiance_hi", C.c_float), ("blob_count", C.c_uint32), ("blob_sigma", C.c_float),
                ("blob_fraction", C.c_float), ("layer_lo", C.c_uint32), ("layer_hi", C.c_uint32),
                ("scatter_fraction", C.c_float)]


_scene = None


def load_scene_host():
    """oracle/scene_host.cpp + the project's host scene generator (no CUDA library)."""
    global _scene
    if _scene is not None:
        return _scene
    from . import build as B  # noqa: PLC0415
    lib = C.CDLL(B.build_scene_host())
    sig = {"osh_preset": (C.c_int, [C.c_int, C.POINTER(SceneDesc)]),
           "osh_generate": (_P, [C.POINTER(SceneDesc)]),
           "osh_sizes": (None, [_P, _U32P, _U32P]), "osh_copy": (None, [_P, _P, _P, _P]),
           "osh_camera_path": (C.c_int, [C.POINTER(SceneDesc), C.c_uint32, C.c_uint32, C.c_uint32, _F, _F]),
           "osh_free": (None, [_P])}
    for n, (res, args) in sig.items():
        f = getattr(lib, n)
        f.restype = res
        f.argtypes = args
    _scene = lib
    return lib


class HostScene:
    """A benchmark scene (vxr_scene_preset(config)) generated on the host without the CUDA
    library: grid, bricks and lights as numpy arrays, and the seeded camera path."""

    def __init__(self, config):
        lib = load_scene_host()
        self.desc = SceneDesc()
        if lib.osh_preset(config, C.byref(self.desc)) != 0:
            raise ValueError(f"unknown scene configuration {config}")
        h = lib.osh_generate(C.byref(self.desc))
        if not h:
            raise RuntimeError("scene generation failed")
        try:
            nb, nl = C.c_uint32(), C.c_uint32()
            lib.osh_sizes(h, C.byref(nb), C.byref(nl))
            self.grid = np.zeros(128 ** 3, np.uint32)
            self.bricks = np.zeros((max(nb.value, 1), 512), np.uint32)
            self.lights = np.zeros(nl.value, LIGHT_DTYPE)
            lib.osh_copy(h, self.grid.ctypes.data, self.bricks.ctypes.data, self.lights.ctypes.data)
        finally:
            lib.osh_free(h)

    def camera_path(self, seed, f, n):
        p, t = (C.c_float * 3)(), (C.c_float * 3)()
        if load_scene_host().osh_camera_path(C.byref(self.desc), seed, f, n, p, t) != 0:
            raise ValueError("camera_path: bad arguments")
        return list(p), list(t)


class WorldArrays:
    """grid / uber / bricks / lights kept alive as numpy arrays for the oracles."""

    def __init__(self, grid, bricks, lights):
        self.grid = _u32(grid)
        self.bricks = _u32(bricks).reshape(-1)
        if self.bricks.size == 0:
            self.bricks = np.zeros(512, np.uint32)
        self.lights = np.ascontiguousarray(lights, dtype=LIGHT_DTYPE)
        self.uber = np.zeros(32 ** 3, np.uint8)
        load_port().orc_build_uber(self.grid.ctypes.data, self.uber.ctypes.data)


class Renderer:
    """Common frame driver over the port ("port") or the reference oracle ("ref")."""

    def __init__(self, kind, world, W, H, point):
        self.kind, self.W, self.H, self.point, self.world = kind, W, H, point, world
        self.n = W * H
        if kind == "port":
            self.lib = load_port()
            self.h = self.lib.orc_create(W, H, 1 if point else 0)
            self.lib.orc_set_world(self.h, world.grid.ctypes.data, world.uber.ctypes.data, world.bricks.ctypes.data)
            self.lib.orc_set_lights(self.h, world.lights.ctypes.data, len(world.lights))
        else:
            self.lib = load_ref()
            if self.lib is None:
                raise RuntimeError("reference oracle unavailable")
            self.v = "point" if point else "area"
            self.h = self._f("create")(W, H)
            uber = np.zeros(32 ** 3, np.uint8)
            self._f("update_uber")(world.grid.ctypes.data, uber.ctypes.data)
            self.ref_uber = uber
            self._f("set_world")(self.h, world.grid.ctypes.data, uber.ctypes.data, world.bricks.ctypes.data)
            self._f("set_lights")(self.h, world.lights.ctypes.data, len(world.lights))

    def _f(self, name):
        return getattr(self.lib, f"vxref_{name}_{self.v}")

    def close(self):
        if self.h:
            (self.lib.orc_destroy if self.kind == "port" else self._f("destroy"))(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_candidates(self, idx, p):
        """Stage 2 draws its candidates from these [m][pixel] arrays (light index, source pdf)
        instead of uniformly (port only); None restores the uniform draw."""
        if idx is None:
            self._cand = None
            self.lib.orc_set_candidates(self.h, None, None, 0)
            return
        self._cand = (np.ascontiguousarray(idx, np.uint32), np.ascontiguousarray(p, np.float32))
        self.lib.orc_set_candidates(self.h, self._cand[0].ctypes.data, self._cand[1].ctypes.data, self.n)

    def frame_start(self):
        if self.kind == "port":
            self.lib.orc_frame_start(self.h)
        else:
            self._f("begin_frame")(self.h)

    def stage(self, k, s, y0=0, y1=0):
        kk = copy_consts(k, FrameConsts)
        if self.kind == "port":
            self.lib.orc_stage(self.h, C.byref(kk), s, y0, y1)
        elif y0 or y1:
            self._f("stage_rows")(self.h, C.byref(kk), s, y0, y1)
        else:
            self._f("stage")(self.h, C.byref(kk), s)

    def gbuffer(self, which=0):
        out = np.zeros(self.n, GBUF_DTYPE)
        if self.kind == "port":
            self.lib.orc_read_gbuffer(self.h, which, out.ctypes.data)
        else:
            self._f("read_gbuffer")(self.h, which, out.ctypes.data, None)
        return out

    def reservoirs(self, role):
        out = np.zeros(self.n, RES_DTYPE)
        (self.lib.orc_read_reservoirs if self.kind == "port" else self._f("read_reservoirs"))(self.h, role, out.ctypes.data)
        return out

    def write_reservoirs(self, role, recs):
        a = np.ascontiguousarray(recs, dtype=RES_DTYPE)
        (self.lib.orc_write_reservoirs if self.kind == "port" else self._f("write_reservoirs"))(self.h, role, a.ctypes.data)

    def image(self, which):
        out = np.zeros((self.n, 4), np.float32)
        (self.lib.orc_read_image if self.kind == "port" else self._f("read_image"))(self.h, which, out.ctypes.data)
        return out

    def set_sky(self, tex, light, scale, blue_noise):
        """Sky dome on (tex float32[h, w, 4], light float32[6, 4], blue_noise
        uint32[VXR_BLUE_NOISE_WORDS]) or off (tex None); reference oracle only."""
        if self.kind != "ref":
            raise NotImplementedError("the sky dome is checked against the reference oracle")
        if tex is None:
            self._f("set_sky")(self.h, None, 0, 0, None, 0.0, None)
            return
        self._sky = (np.ascontiguousarray(tex, np.float32), np.ascontiguousarray(light, np.float32),
                     np.ascontiguousarray(blue_noise, np.uint32))
        t, l, b = self._sky
        self._f("set_sky")(self.h, t.ctypes.data, t.shape[1], t.shape[0], l.ctypes.data, float(scale), b.ctypes.data)

    def trace(self, mode, O, D, steps=999999, through=0, mask=0):
        o = (C.c_float * 3)(*O)
        d = (C.c_float * 3)(*D)
        dist = C.c_float(0)
        side = C.c_uint32(0)
        if self.kind == "port":
            v = self.lib.orc_trace(self.h, mode, o, d, steps, through, mask, C.byref(dist), C.byref(side))
        else:
            v = self._f("trace")(self.h, mode, o, d, steps, through, mask, C.byref(dist), C.byref(side))
        return v, dist.value, side.value


class CameraPath:
    """The oracle's restatement of the camera / frame-constant host code."""

    def __init__(self, W, H, rng_seed=0x12345678):
        self.lib = load_port()
        self.W, self.H = W, H
        self.cam = Camera()
        self.lib.orc_camera_init(C.byref(self.cam), rng_seed)

    def lookat(self, pos, target):
        self.lib.orc_lookat(C.byref(self.cam), (C.c_float * 3)(*pos), (C.c_float * 3)(*target))

    def begin(self, **params):
        k = FrameConsts()
        self.lib.orc_begin_frame(C.byref(self.cam), self.W, self.H, C.byref(k))
        for n, v in params.items():
            setattr(k, n, v)
        return k

    def end(self):
        self.lib.orc_end_frame(C.byref(self.cam))


def sincos(a):
    s, c = C.c_float(), C.c_float()
    load_port().orc_sincos(a, C.byref(s), C.byref(c))
    return s.value, c.value
