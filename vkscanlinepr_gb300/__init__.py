"""GB300 scanline path renderer — Python host side over the libsr.so C ABI.

Mirrors the reference's public interface for this path
(VkScanlinePR/src/core/rasterizer.h:9-20 and core/vg/vg_container.h:21-87):

    r = ScanlineVGRasterizer()
    r.initialize(None, w, h)        # VGRasterizer::initialize (no window: headless)
    r.loadVG(container)             # VGRasterizer::loadVG
    r.setMVP(m)                     # VGRasterizer::setMVP (rows m0..m3)
    img = r.render()                # VGRasterizer::render -> RGBA8 (h, w, 4)

Every call goes through libsr.so (hand-written sm_103a CUDA).  There is no
CPU fallback: if the library is missing or a CUDA call fails, the call raises.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsr.so")

MODE_REFERENCE = 0
MODE_PIXEL = 1
FLAG_KEEP_STAGES = 0x1
FLAG_PROFILE = 0x2

LINE, QUADRIC, CUBIC = 0x02, 0x03, 0x04
NON_ZERO, EVEN_ODD = 0, 1

STAGES = {
    "transformed_pos": 0, "path_visible": 1, "cutpoints": 2, "curve_count": 3,
    "curve_offset": 4, "intersection": 5, "frag_key": 6, "frag_winding": 7,
    "sorted_key": 8, "sorted_index": 9, "winding_scan": 10, "frag_flag": 11,
    "span_flag": 12, "draw_list": 13, "image": 14, "frag_left": 15,
}

STATUS = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "OVERFLOW_REFIT", 4: "TIMEOUT",
          5: "CUDA", 6: "NO_SCENE", 7: "INTERNAL"}


class SRError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS.get(code, code), msg))
        self.code = code


PAINT_MAX_STOPS = 16
PAINT_LINEAR, PAINT_RADIAL = 1, 2
SPREAD_PAD, SPREAD_REPEAT, SPREAD_REFLECT = 0, 1, 2


class Paint(ctypes.Structure):
    """sr_paint: a linear or radial gradient (see include/sr.h)."""
    _fields_ = [("kind", ctypes.c_int32), ("spread", ctypes.c_int32), ("p0", ctypes.c_float * 2),
                ("p1", ctypes.c_float * 2), ("radius", ctypes.c_float), ("xf", ctypes.c_float * 6),
                ("opacity", ctypes.c_float), ("n_stops", ctypes.c_uint32),
                ("offset", ctypes.c_float * PAINT_MAX_STOPS),
                ("rgba", (ctypes.c_float * 4) * PAINT_MAX_STOPS)]


def fill_paint(i):
    """fill_info of a path painted by gradient paint i."""
    return int(i) + 1


class SceneView(ctypes.Structure):
    _fields_ = [
        ("n_points", ctypes.c_uint32), ("n_curves", ctypes.c_uint32),
        ("n_paths", ctypes.c_uint32),
        ("position", ctypes.c_void_p), ("pos_path_idx", ctypes.c_void_p),
        ("curve_pos_map", ctypes.c_void_p), ("curve_type", ctypes.c_void_p),
        ("curve_path_idx", ctypes.c_void_p), ("fill_rule", ctypes.c_void_p),
        ("fill_info", ctypes.c_void_p),
    ]


class Options(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("mode", ctypes.c_int32),
                ("device", ctypes.c_int32), ("flags", ctypes.c_uint32)]


class Stats(ctypes.Structure):
    _fields_ = [("n_intersections", ctypes.c_uint64), ("n_draw_records", ctypes.c_uint64),
                ("n_merged_fragments", ctypes.c_uint64), ("n_spans", ctypes.c_uint64),
                ("key_bits", ctypes.c_uint32), ("sort_passes", ctypes.c_uint32),
                ("kernel_launches", ctypes.c_uint32), ("reruns", ctypes.c_uint32),
                ("stage_ms", ctypes.c_float * 12)]

STAGE_NAMES = ["transform", "count", "offset_scan", "chains", "merge", "fragment", "sort", "winding_emit",
               "row_sort", "resolve", "wide"]


class BatchRenderOpts(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("use_graph", ctypes.c_uint32),
                ("record_capacity", ctypes.c_int64), ("refit_on_overflow", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("draw_capacity", ctypes.c_int64)]


class Tuning(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("sort_items", ctypes.c_int32), ("resolve_warps", ctypes.c_int32),
                ("wind_items", ctypes.c_int32), ("sort_kind", ctypes.c_int32)]


def _tuning(d):
    return Tuning(ctypes.sizeof(Tuning), int(d["sort_items"]), int(d["resolve_warps"]), int(d["wind_items"]),
                  int(d.get("sort_kind", 0)))


SIZER_FEATURES, SIZER_OUTPUTS, SIZER_PARAMS, SIZER_NORM = 6, 2, 4738, 16


class SizerTrainOpts(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("batch", ctypes.c_uint32), ("epochs", ctypes.c_uint32),
                ("shuffle", ctypes.c_uint32), ("lr", ctypes.c_float), ("beta1", ctypes.c_float),
                ("beta2", ctypes.c_float), ("eps", ctypes.c_float), ("seed", ctypes.c_uint64)]


class SizingMargins(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("path_records", ctypes.c_float), ("path_draws", ctypes.c_float),
                ("frame_records", ctypes.c_float), ("frame_draws", ctypes.c_float)]


class ServerOpts(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("mode", ctypes.c_int32), ("device", ctypes.c_int32),
                ("slots", ctypes.c_uint32), ("max_batch_scenes", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("memory_budget", ctypes.c_uint64), ("margins", SizingMargins)]


class SizingPlan(ctypes.Structure):
    _fields_ = [("records", ctypes.c_int64), ("draws", ctypes.c_int64), ("path_records", ctypes.c_int64),
                ("path_draws", ctypes.c_int64), ("device_bytes", ctypes.c_uint64)]


class RequestInfo(ctypes.Structure):
    _fields_ = [("submit_s", ctypes.c_double), ("admit_s", ctypes.c_double), ("done_s", ctypes.c_double),
                ("predicted_bytes", ctypes.c_uint64), ("batch_scenes", ctypes.c_uint32), ("refit", ctypes.c_uint32),
                ("status", ctypes.c_int32), ("reserved", ctypes.c_uint32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("batches", ctypes.c_uint64),
                ("overflows", ctypes.c_uint64), ("refits", ctypes.c_uint64), ("budget_waits", ctypes.c_uint64),
                ("peak_bytes", ctypes.c_uint64), ("rejected", ctypes.c_uint64)]


class SizingJudge(ctypes.Structure):
    _fields_ = [("paths", ctypes.c_uint32), ("paths_over_records", ctypes.c_uint32),
                ("paths_over_draws", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("records", ctypes.c_int64), ("draws", ctypes.c_int64)]


class SynthParams(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32), ("preset", ctypes.c_int32),
        ("seed", ctypes.c_uint64), ("scene_index", ctypes.c_uint32),
        ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
        ("n_paths", ctypes.c_uint32),
    ]


class BatchStats(ctypes.Structure):
    _fields_ = [("frame", Stats), ("n_scenes", ctypes.c_uint32), ("n_paths", ctypes.c_uint32),
                ("n_curves", ctypes.c_uint32), ("overflows", ctypes.c_uint32), ("refits", ctypes.c_uint32),
                ("graph_captured", ctypes.c_uint32), ("record_capacity", ctypes.c_int64)]


# every symbol include/sr.h declares
EXPORTS = ["sr_create", "sr_load_scene", "sr_set_mvp", "sr_render", "sr_get_stats", "sr_debug_dump",
           "sr_destroy", "sr_last_error", "sr_synth_scene", "sr_rvg_load", "sr_scene_buf_view",
           "sr_scene_buf_free", "sr_exclusive_scan_i32", "sr_render_draw_list",
           "sr_exclusive_scan_i32_noalloc", "sr_batch_create", "sr_batch_add_scene", "sr_batch_add_synth",
           "sr_batch_commit", "sr_batch_set_mvp", "sr_batch_render", "sr_batch_get_image", "sr_batch_info",
           "sr_batch_get_stats", "sr_batch_clear", "sr_batch_destroy", "sr_scene_buf_size", "sr_host_alloc",
           "sr_host_free", "sr_sizer_create", "sr_sizer_destroy", "sr_sizer_set_norm", "sr_sizer_get_state",
           "sr_sizer_set_state", "sr_sizer_loss_grad", "sr_sizer_train", "sr_sizer_predict",
           "sr_batch_path_features", "sr_batch_path_labels", "sr_batch_plan", "sr_batch_judge",
           "sr_batch_frame_bytes", "sr_device_alloc", "sr_device_free", "sr_memcpy", "sr_batch_enqueue",
           "sr_batch_query", "sr_batch_finish", "sr_batch_release", "sr_batch_held_bytes", "sr_batch_path_ranges",
           "sr_server_create", "sr_server_submit", "sr_server_wait", "sr_server_get_stats", "sr_server_destroy",
           "sr_admission_take", "sr_set_tuning", "sr_batch_set_tuning", "sr_batch_get_tuning",
           "sr_batch_tuning_class", "sr_batch_autotune", "sr_scan_status", "sr_set_spin_limit",
           "sr_debug_scan_without_first_tile", "sr_write_image", "sr_rvg_load_full", "sr_set_paints",
           "sr_scene_buf_paints", "sr_render_aa", "sr_debug_sort_tiles", "sr_batch_reserve_like"]

_lib = None


def build(force=False):
    """Compile libsr.so in-tree (nvcc, sm_103a)."""
    from . import builder
    return builder.build(force=force)


def lib():
    """Load libsr.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libsr.so not built: run vkscanlinepr_gb300.build() first")
    L = ctypes.CDLL(LIB_PATH)
    vp = ctypes.c_void_p
    L.sr_create.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(Options), ctypes.POINTER(vp)]
    L.sr_load_scene.argtypes = [vp, ctypes.POINTER(SceneView)]
    L.sr_set_mvp.argtypes = [vp, vp]
    L.sr_render.argtypes = [vp, vp, ctypes.c_int, vp]
    L.sr_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    L.sr_debug_dump.argtypes = [vp, ctypes.c_int, vp, ctypes.POINTER(ctypes.c_size_t)]
    L.sr_destroy.argtypes = [vp]
    L.sr_destroy.restype = None
    L.sr_last_error.restype = ctypes.c_char_p
    L.sr_synth_scene.argtypes = [ctypes.POINTER(SynthParams), ctypes.POINTER(vp)]
    L.sr_rvg_load.argtypes = [ctypes.c_char_p, ctypes.POINTER(vp), vp]
    L.sr_rvg_load_full.argtypes = [ctypes.c_char_p, ctypes.POINTER(vp), vp]
    L.sr_set_paints.argtypes = [vp, vp, ctypes.c_uint32]
    L.sr_render_aa.argtypes = [vp, ctypes.c_uint32, vp, ctypes.c_int, vp]
    L.sr_scene_buf_paints.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_uint32)]
    L.sr_scene_buf_view.argtypes = [vp, ctypes.POINTER(SceneView)]
    L.sr_scene_buf_free.argtypes = [vp]
    L.sr_scan_status.argtypes = [vp]
    L.sr_set_spin_limit.argtypes = [ctypes.c_uint32]
    L.sr_set_spin_limit.restype = None
    L.sr_debug_scan_without_first_tile.argtypes = [vp, vp, ctypes.c_int64, vp]
    L.sr_debug_sort_tiles.argtypes = [vp, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32)]
    L.sr_write_image.argtypes = [ctypes.c_char_p, vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int]
    L.sr_scene_buf_free.restype = None
    L.sr_scene_buf_size.argtypes = [vp, vp]
    L.sr_host_alloc.argtypes = [ctypes.c_size_t]
    L.sr_host_alloc.restype = vp
    L.sr_host_free.argtypes = [vp]
    L.sr_host_free.restype = None
    L.sr_exclusive_scan_i32.argtypes = [vp, vp, ctypes.c_int64, vp]
    L.sr_render_draw_list.argtypes = [vp, vp, ctypes.c_int64, vp, ctypes.c_int, vp]
    L.sr_exclusive_scan_i32_noalloc.argtypes = [vp, vp, ctypes.c_int64, vp]
    L.sr_batch_create.argtypes = [ctypes.POINTER(Options), ctypes.POINTER(vp)]
    L.sr_batch_add_scene.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(SceneView), vp,
                                     ctypes.POINTER(ctypes.c_uint32)]
    L.sr_batch_add_synth.argtypes = [vp, ctypes.POINTER(SynthParams), ctypes.c_uint32,
                                     ctypes.POINTER(ctypes.c_uint32)]
    L.sr_batch_commit.argtypes = [vp]
    L.sr_batch_set_mvp.argtypes = [vp, ctypes.c_uint32, vp]
    L.sr_batch_render.argtypes = [vp, ctypes.POINTER(BatchRenderOpts), vp]
    L.sr_batch_enqueue.argtypes = [vp, ctypes.POINTER(BatchRenderOpts), vp]
    L.sr_batch_query.argtypes = [vp, ctypes.POINTER(ctypes.c_int)]
    L.sr_batch_finish.argtypes = [vp]
    L.sr_batch_get_image.argtypes = [vp, ctypes.c_uint32, vp, ctypes.c_int, vp]
    L.sr_batch_info.argtypes = [vp, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint32),
                                ctypes.POINTER(ctypes.c_uint32)]
    L.sr_batch_get_stats.argtypes = [vp, ctypes.POINTER(BatchStats)]
    L.sr_batch_clear.argtypes = [vp]
    L.sr_batch_destroy.argtypes = [vp]
    L.sr_batch_destroy.restype = None
    fp = ctypes.POINTER(ctypes.c_float)
    L.sr_sizer_create.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(vp)]
    L.sr_sizer_destroy.argtypes = [vp]
    L.sr_sizer_destroy.restype = None
    L.sr_sizer_set_norm.argtypes = [vp, vp]
    L.sr_sizer_get_state.argtypes = [vp, vp, vp, vp, vp, ctypes.POINTER(ctypes.c_int64)]
    L.sr_sizer_set_state.argtypes = [vp, vp, vp, vp, vp, ctypes.c_int64]
    L.sr_sizer_loss_grad.argtypes = [vp, vp, vp, ctypes.c_uint32, vp, fp]
    L.sr_sizer_train.argtypes = [vp, vp, vp, ctypes.c_uint32, ctypes.POINTER(SizerTrainOpts), fp, vp]
    L.sr_sizer_predict.argtypes = [vp, vp, ctypes.c_uint32, vp, vp]
    L.sr_batch_path_features.argtypes = [vp, vp, vp]
    L.sr_batch_path_labels.argtypes = [vp, vp, vp]
    L.sr_batch_plan.argtypes = [vp, vp, ctypes.POINTER(SizingMargins), ctypes.POINTER(SizingPlan), vp, vp]
    L.sr_batch_path_ranges.argtypes = [vp, vp]
    L.sr_server_create.argtypes = [ctypes.POINTER(ServerOpts), vp, ctypes.POINTER(vp)]
    L.sr_server_submit.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(SceneView), vp,
                                   ctypes.POINTER(ctypes.c_uint64)]
    L.sr_server_wait.argtypes = [vp, ctypes.c_uint64, vp, ctypes.c_int, ctypes.POINTER(RequestInfo), ctypes.c_int64]
    L.sr_server_get_stats.argtypes = [vp, ctypes.POINTER(ServerStats)]
    L.sr_server_destroy.argtypes = [vp]
    L.sr_server_destroy.restype = None
    L.sr_admission_take.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                    ctypes.POINTER(ctypes.c_int)]
    L.sr_admission_take.restype = ctypes.c_uint32
    L.sr_set_tuning.argtypes = [vp, ctypes.POINTER(Tuning)]
    L.sr_batch_set_tuning.argtypes = [vp, ctypes.POINTER(Tuning)]
    L.sr_batch_get_tuning.argtypes = [vp, ctypes.POINTER(Tuning)]
    L.sr_batch_tuning_class.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
    L.sr_batch_autotune.argtypes = [vp, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(Tuning), vp]
    L.sr_batch_judge.argtypes = [vp, ctypes.POINTER(SizingJudge), vp]
    L.sr_batch_frame_bytes.argtypes = [vp, ctypes.c_int64, ctypes.c_int64, ctypes.POINTER(ctypes.c_uint64)]
    L.sr_batch_release.argtypes = [vp]
    L.sr_batch_held_bytes.argtypes = [vp, ctypes.POINTER(ctypes.c_uint64)]
    L.sr_batch_reserve_like.argtypes = [vp, vp]
    L.sr_device_alloc.argtypes = [ctypes.c_int, ctypes.c_size_t]
    L.sr_device_alloc.restype = vp
    L.sr_device_free.argtypes = [vp]
    L.sr_device_free.restype = None
    L.sr_memcpy.argtypes = [vp, vp, ctypes.c_size_t]
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise SRError(rc, lib().sr_last_error().decode(errors="replace"))


class VGContainer:
    """Flattened scene, the reference's VGContainer after loadVG's flattening
    (scanline_rasterizer.cpp:67-189): points grouped by curve, curves grouped
    by path, packed RGBA8 fill colours."""

    def __init__(self, width=0, height=0):
        self.width, self.height = int(width), int(height)
        self._pos, self._pos_path = [], []
        self._curve_pos, self._curve_type, self._curve_path = [], [], []
        self._fill_rule, self._fill_info = [], []
        self._arrays = None
        self.paints = None   # gradient paints (ctypes array of Paint), or None

    # builder API, after VGContainer::newPath/newCurve/addCurve (vg_container.h:49-86)
    def new_path(self, fill_rule=NON_ZERO, rgba=(0, 0, 0, 255)):
        r, g, b, a = (int(v) & 0xFF for v in rgba)
        c = r | (g << 8) | (b << 16) | (a << 24)
        self._fill_rule.append(int(fill_rule))
        self._fill_info.append(c if a else 0)
        self._arrays = None
        return len(self._fill_rule) - 1

    def add_curve(self, ctype, points):
        pts = np.asarray(points, np.float32).reshape(-1, 2)
        if pts.shape[0] != (ctype & 7):
            raise ValueError("curve type 0x%x needs %d points" % (ctype, ctype & 7))
        path = len(self._fill_rule) - 1
        if path < 0:
            raise ValueError("new_path() first")
        self._curve_pos.append(len(self._pos_path))
        self._curve_type.append(int(ctype))
        self._curve_path.append(path)
        for x, y in pts:
            self._pos.append((float(x), float(y)))
            self._pos_path.append(path)
        self._arrays = None

    @classmethod
    def from_arrays(cls, width, height, position, pos_path_idx, curve_pos_map, curve_type, curve_path_idx,
                    fill_rule, fill_info):
        c = cls(width, height)
        c.paints = None
        c._arrays = dict(
            position=np.ascontiguousarray(position, np.float32).reshape(-1),
            pos_path_idx=np.ascontiguousarray(pos_path_idx, np.uint32),
            curve_pos_map=np.ascontiguousarray(curve_pos_map, np.uint32),
            curve_type=np.ascontiguousarray(curve_type, np.uint32),
            curve_path_idx=np.ascontiguousarray(curve_path_idx, np.uint32),
            fill_rule=np.ascontiguousarray(fill_rule, np.uint32),
            fill_info=np.ascontiguousarray(fill_info, np.uint32))
        return c

    def arrays(self):
        if self._arrays is None:
            self._arrays = dict(
                position=np.asarray(self._pos, np.float32).reshape(-1),
                pos_path_idx=np.asarray(self._pos_path, np.uint32),
                curve_pos_map=np.asarray(self._curve_pos, np.uint32),
                curve_type=np.asarray(self._curve_type, np.uint32),
                curve_path_idx=np.asarray(self._curve_path, np.uint32),
                fill_rule=np.asarray(self._fill_rule, np.uint32),
                fill_info=np.asarray(self._fill_info, np.uint32))
        return self._arrays

    @property
    def n_points(self):
        return self.arrays()["pos_path_idx"].size

    @property
    def n_curves(self):
        return self.arrays()["curve_type"].size

    @property
    def n_paths(self):
        return self.arrays()["fill_rule"].size

    def view(self):
        a = self.arrays()
        v = SceneView()
        v.n_points = a["pos_path_idx"].size
        v.n_curves = a["curve_type"].size
        v.n_paths = a["fill_rule"].size
        for k in ("position", "pos_path_idx", "curve_pos_map", "curve_type", "curve_path_idx",
                  "fill_rule", "fill_info"):
            setattr(v, k, a[k].ctypes.data if a[k].size else None)
        return v


def _from_buf(h, width=None, height=None):
    L = lib()
    v = SceneView()
    _check(L.sr_scene_buf_view(h, ctypes.byref(v)))
    wh = np.zeros(2, np.uint32)
    L.sr_scene_buf_size(h, wh.ctypes.data)

    def arr(ptr, n, dt):
        if n == 0 or not ptr:
            return np.zeros(0, dt)
        return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(np.ctypeslib.as_ctypes_type(dt))),
                                     shape=(n,)).copy()
    return VGContainer.from_arrays(
        wh[0] if width is None else width, wh[1] if height is None else height,
        arr(v.position, 2 * v.n_points, np.float32), arr(v.pos_path_idx, v.n_points, np.uint32),
        arr(v.curve_pos_map, v.n_curves, np.uint32), arr(v.curve_type, v.n_curves, np.uint32),
        arr(v.curve_path_idx, v.n_curves, np.uint32), arr(v.fill_rule, v.n_paths, np.uint32),
        arr(v.fill_info, v.n_paths, np.uint32))


def synth_scene(preset, seed, scene_index=0, width=0, height=0, n_paths=0):
    """Seeded synthetic scene (preset 0: 1024x1024 star cubics; preset 1:
    4096x4096 mixed curves with backgrounds)."""
    L = lib()
    p = SynthParams(ctypes.sizeof(SynthParams), preset, seed, scene_index, width, height, n_paths)
    h = ctypes.c_void_p()
    _check(L.sr_synth_scene(ctypes.byref(p), ctypes.byref(h)))
    try:
        return _from_buf(h)
    finally:
        L.sr_scene_buf_free(h)


def load_rvg(path, full=False):
    """Read an .rvg file the way the reference's RVG::load does, or with
    full=True also its arcs, quadratics and gradient paints; returns
    (container, viewport[4])."""
    L = lib()
    h = ctypes.c_void_p()
    vp = np.zeros(4, np.float32)
    fn = L.sr_rvg_load_full if full else L.sr_rvg_load
    _check(fn(path.encode(), ctypes.byref(h), vp.ctypes.data))
    try:
        c = _from_buf(h)
        pp, n = ctypes.c_void_p(), ctypes.c_uint32()
        _check(L.sr_scene_buf_paints(h, ctypes.byref(pp), ctypes.byref(n)))
        if n.value:
            c.paints = (Paint * n.value)()
            ctypes.memmove(c.paints, pp.value, ctypes.sizeof(Paint) * n.value)
        return c, vp
    finally:
        L.sr_scene_buf_free(h)


def exclusive_scan_i32(d_in, d_out, n, stream=None):
    """Exclusive scan of n int32 at device address d_in into d_out[0..n]."""
    _check(lib().sr_exclusive_scan_i32(d_in, d_out, int(n), stream))


IMAGE_FORMATS = {"png": 0, "ppm": 1, "pam": 2}


def write_image(path, rgba, fmt=None):
    """Writes an (H, W, 4) uint8 frame to `path` as PNG, PPM or PAM (from the
    file's extension unless `fmt` is given)."""
    img = np.ascontiguousarray(rgba, np.uint8)
    if img.ndim != 3 or img.shape[2] != 4:
        raise ValueError("expected an (H, W, 4) uint8 array")
    if fmt is None:
        fmt = os.path.splitext(str(path))[1].lstrip(".").lower() or "png"
    _check(lib().sr_write_image(str(path).encode(), img.ctypes.data, img.shape[1], img.shape[0],
                                IMAGE_FORMATS[fmt]))


def scan_status(stream=None):
    """Waits for `stream`; raises SrError(SR_ERR_TIMEOUT) if a look-back of a
    standalone scan gave up since the last call (its output is wrong)."""
    _check(lib().sr_scan_status(stream))


def set_spin_limit(polls):
    """Polls every bounded device wait makes before giving up (0: default)."""
    lib().sr_set_spin_limit(int(polls))


NOALLOC_SCAN_MAX_N = 1 << 24


def exclusive_scan_i32_noalloc(d_in, d_out, n, stream=None):
    """The exclusive scan for callers that cannot allocate device memory:
    its scratch is a fixed array inside the library (n <= NOALLOC_SCAN_MAX_N;
    calls that overlap on the GPU race)."""
    _check(lib().sr_exclusive_scan_i32_noalloc(d_in, d_out, int(n), stream))


class PinnedBuffer:
    """Page-locked host buffer (cudaMallocHost) viewed as a numpy array."""

    def __init__(self, nbytes):
        self.nbytes = int(nbytes)
        self.ptr = lib().sr_host_alloc(self.nbytes)
        if not self.ptr:
            raise MemoryError("pinned host allocation of %d bytes failed" % nbytes)
        self.array = np.ctypeslib.as_array(ctypes.cast(self.ptr, ctypes.POINTER(ctypes.c_uint8)),
                                           shape=(self.nbytes,))

    def __del__(self):
        try:
            if self.ptr:
                lib().sr_host_free(self.ptr)
                self.ptr = None
        except Exception:
            pass


class ScanlineVGRasterizer:
    """Headless drop-in for the reference's ScanlineVGRasterizer
    (core/scanline/scanline_rasterizer.h:31-49)."""

    def __init__(self, mode=MODE_PIXEL, device=0, keep_stages=False, profile=False):
        self.mode, self.device = mode, device
        self.flags = (FLAG_KEEP_STAGES if keep_stages else 0) | (FLAG_PROFILE if profile else 0)
        self._ctx = None
        self._scene = None
        self.width = self.height = 0

    def initialize(self, window, w, h):
        L = lib()
        o = Options(ctypes.sizeof(Options), self.mode, self.device, self.flags)
        ctx = ctypes.c_void_p()
        _check(L.sr_create(int(w), int(h), ctypes.byref(o), ctypes.byref(ctx)))
        self._ctx = ctx
        self.width, self.height = int(w), int(h)

    def loadVG(self, container):
        self._scene = container
        v = container.view()
        _check(lib().sr_load_scene(self._ctx, ctypes.byref(v)))
        paints = getattr(container, "paints", None)
        _check(lib().sr_set_paints(self._ctx, ctypes.cast(paints, ctypes.c_void_p) if paints else None,
                                   len(paints) if paints else 0))

    def render_aa(self, samples, out=None, stream=None):
        """Antialiased frame: `samples` (1, 2, 4, 8, 16) samples a pixel on a
        comb (sr_render_aa); returns RGBA8 as (h, w, 4) uint8."""
        if out is None:
            out = np.empty((self.height, self.width, 4), np.uint8)
        _check(lib().sr_render_aa(self._ctx, int(samples), out.ctypes.data, 0, stream))
        return out

    def setMVP(self, m):
        a = np.ascontiguousarray(m, np.float32).reshape(16)
        _check(lib().sr_set_mvp(self._ctx, a.ctypes.data))

    def render(self, out=None, stream=None):
        """Renders one frame; returns RGBA8 as (h, w, 4) uint8.  `out` may be
        a (pinned or pageable) host array of h*w*4 bytes."""
        if out is None:
            out = np.empty((self.height, self.width, 4), np.uint8)
        ptr = out.ctypes.data if isinstance(out, np.ndarray) else out
        _check(lib().sr_render(self._ctx, ptr, 0, stream))
        return out

    def set_tuning(self, sort_items=12, resolve_warps=8, wind_items=8, sort_kind=0):
        t = _tuning({"sort_items": sort_items, "resolve_warps": resolve_warps, "wind_items": wind_items,
                     "sort_kind": sort_kind})
        _check(lib().sr_set_tuning(self._ctx, ctypes.byref(t)))

    def render_draw_list(self, records, out=None, stream=None):
        """Paints an (n, 4) int32 draw list (the reference's MOCK_DATA path)."""
        rec = np.ascontiguousarray(records, np.int32).reshape(-1, 4)
        if out is None:
            out = np.empty((self.height, self.width, 4), np.uint8)
        _check(lib().sr_render_draw_list(self._ctx, rec.ctypes.data if rec.size else None, rec.shape[0],
                                         out.ctypes.data, 0, stream))
        return out

    def render_device(self, dev_ptr=None, stream=None):
        """Renders into device memory (dev_ptr or the context's framebuffer)
        without waiting for the frame."""
        _check(lib().sr_render(self._ctx, dev_ptr, 1, stream))

    def stats(self):
        s = Stats()
        _check(lib().sr_get_stats(self._ctx, ctypes.byref(s)))
        d = {k: getattr(s, k) for k, _ in Stats._fields_ if k != "stage_ms"}
        d["stage_ms"] = dict(zip(STAGE_NAMES, [float(x) for x in s.stage_ms]))
        return d

    def sort_tiles(self):
        """(tiles, tiles sorted with 64-bit items) of the last frame's per-path
        sort; (0, 0) when it took the radix sort."""
        t, w = ctypes.c_uint32(0), ctypes.c_uint32(0)
        _check(lib().sr_debug_sort_tiles(self._ctx, ctypes.byref(t), ctypes.byref(w)))
        return int(t.value), int(w.value)

    def dump(self, stage):
        L = lib()
        sid = STAGES[stage]
        n = ctypes.c_size_t(0)
        _check(L.sr_debug_dump(self._ctx, sid, None, ctypes.byref(n)))
        dt = np.float32 if stage in ("transformed_pos", "cutpoints") else (np.uint8 if stage == "image" else np.int32)
        a = np.zeros(n.value // np.dtype(dt).itemsize, dt)
        if n.value:
            _check(L.sr_debug_dump(self._ctx, sid, a.ctypes.data, ctypes.byref(n)))
        if stage == "image":
            a = a.reshape(self.height, self.width, 4)
        elif stage == "draw_list":
            a = a.reshape(-1, 4)
        elif stage in ("intersection", "transformed_pos"):
            a = a.reshape(-1, 2)
        return a

    def close(self):
        if self._ctx:
            lib().sr_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SceneBatch:
    """Many uneven scenes rendered in the same launches (sr_batch_*).

    Each scene's image is bit-identical to rendering it alone.  render() can
    size the record buffers exactly (one host wait, as the reference does) or
    take a record capacity and enqueue the whole frame without waiting
    (optionally as a replayed CUDA graph); an overflow is detected on the
    device and, with refit=True, the frame reruns with exact sizing."""

    def __init__(self, mode=MODE_PIXEL, device=0, profile=False):
        o = Options(ctypes.sizeof(Options), mode, device, FLAG_PROFILE if profile else 0)
        h = ctypes.c_void_p()
        _check(lib().sr_batch_create(ctypes.byref(o), ctypes.byref(h)))
        self._h = h
        self.mode = mode
        self._keep = []

    def add_scene(self, container, width=None, height=None, mvp=None):
        w = container.width if width is None else width
        h = container.height if height is None else height
        v = container.view()
        m = None if mvp is None else np.ascontiguousarray(mvp, np.float32).reshape(16)
        idx = ctypes.c_uint32()
        _check(lib().sr_batch_add_scene(self._h, int(w), int(h), ctypes.byref(v),
                                        m.ctypes.data if m is not None else None, ctypes.byref(idx)))
        return idx.value

    def add_synth(self, preset, seed, count, scene_index=0, width=0, height=0, n_paths=0):
        p = SynthParams(ctypes.sizeof(SynthParams), preset, seed, scene_index, width, height, n_paths)
        first = ctypes.c_uint32()
        _check(lib().sr_batch_add_synth(self._h, ctypes.byref(p), int(count), ctypes.byref(first)))
        return first.value

    def commit(self):
        _check(lib().sr_batch_commit(self._h))

    def set_mvp(self, index, m):
        a = np.ascontiguousarray(m, np.float32).reshape(16)
        _check(lib().sr_batch_set_mvp(self._h, int(index), a.ctypes.data))

    def render(self, capacity=-1, graph=False, refit=True, stream=None, draw_capacity=-1):
        o = BatchRenderOpts(ctypes.sizeof(BatchRenderOpts), 1 if graph else 0, int(capacity), 1 if refit else 0, 0,
                            int(draw_capacity))
        _check(lib().sr_batch_render(self._h, ctypes.byref(o), stream))

    def enqueue(self, capacity, graph=False, refit=True, stream=None, draw_capacity=-1):
        """Queues a pre-sized frame and returns without waiting (see finish)."""
        o = BatchRenderOpts(ctypes.sizeof(BatchRenderOpts), 1 if graph else 0, int(capacity), 1 if refit else 0, 0,
                            int(draw_capacity))
        _check(lib().sr_batch_enqueue(self._h, ctypes.byref(o), stream))

    def done(self):
        d = ctypes.c_int()
        _check(lib().sr_batch_query(self._h, ctypes.byref(d)))
        return bool(d.value)

    def finish(self):
        _check(lib().sr_batch_finish(self._h))

    def n_paths(self):
        return self.stats()["n_paths"]

    def set_tuning(self, sort_items=12, resolve_warps=8, wind_items=8, sort_kind=0):
        t = _tuning({"sort_items": sort_items, "resolve_warps": resolve_warps, "wind_items": wind_items,
                     "sort_kind": sort_kind})
        _check(lib().sr_batch_set_tuning(self._h, ctypes.byref(t)))

    def tuning(self):
        t = Tuning()
        _check(lib().sr_batch_get_tuning(self._h, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in Tuning._fields_ if k != "struct_size"}

    def tuning_class(self):
        buf = ctypes.create_string_buffer(64)
        _check(lib().sr_batch_tuning_class(self._h, buf, 64))
        return buf.value.decode()

    def autotune(self, cache_path=None, force=False, stream=None):
        """Tuning of this batch's size class, from the JSON cache or by timing."""
        t = Tuning()
        _check(lib().sr_batch_autotune(self._h, cache_path.encode() if cache_path else None, 1 if force else 0,
                                       ctypes.byref(t), stream))
        return {k: getattr(t, k) for k, _ in Tuning._fields_ if k != "struct_size"}

    def features(self, out=None, stream=None):
        """Per-path sizing features under the current transforms: DeviceArray [P, 6]."""
        n = self.n_paths()
        out = out if out is not None else DeviceArray((n, SIZER_FEATURES), np.float32)
        _check(lib().sr_batch_path_features(self._h, out.ptr, stream))
        return out

    def labels(self, out=None, stream=None):
        """Renders once with exact sizing and per-path counters: DeviceArray [P, 2]
        of log(1 + records), log(1 + draw records)."""
        n = self.n_paths()
        out = out if out is not None else DeviceArray((n, SIZER_OUTPUTS), np.float32)
        _check(lib().sr_batch_path_labels(self._h, out.ptr, stream))
        return out

    def plan(self, sizer, margins, per_scene=False, stream=None):
        """Capacities of the next frame from the sizing network.  margins:
        (path_records, path_draws, frame_records, frame_draws) in log units."""
        m = SizingMargins(ctypes.sizeof(SizingMargins), *[float(v) for v in margins])
        p = SizingPlan()
        sc = None
        if per_scene:
            sc = np.zeros((self.stats()["n_scenes"], 2), np.int64)
        _check(lib().sr_batch_plan(self._h, sizer._h, ctypes.byref(m), ctypes.byref(p),
                                   sc.ctypes.data if sc is not None else None, stream))
        d = {k: getattr(p, k) for k, _ in SizingPlan._fields_}
        if per_scene:
            d["scenes"] = sc
        return d

    def path_ranges(self):
        """First path of each scene (n_scenes + 1 entries)."""
        out = np.zeros(self.stats()["n_scenes"] + 1, np.uint32)
        _check(lib().sr_batch_path_ranges(self._h, out.ctypes.data))
        return out

    def judge(self, stream=None):
        """Exact count pass against the last plan's per-path allotments."""
        j = SizingJudge()
        _check(lib().sr_batch_judge(self._h, ctypes.byref(j), stream))
        return {k: getattr(j, k) for k, _ in SizingJudge._fields_ if k != "reserved"}

    def release(self):
        """Frees the record-sized buffers (scenes and images stay)."""
        _check(lib().sr_batch_release(self._h))

    def held_bytes(self):
        b = ctypes.c_uint64()
        _check(lib().sr_batch_held_bytes(self._h, ctypes.byref(b)))
        return b.value

    def reserve_like(self, model):
        """Grows this batch's buffers to at least model's (images and plan
        dropped when a buffer moves; the next frame uploads the scenes)."""
        _check(lib().sr_batch_reserve_like(self._h, model._h))

    def frame_bytes(self, records, draws=-1):
        b = ctypes.c_uint64()
        _check(lib().sr_batch_frame_bytes(self._h, int(records), int(draws), ctypes.byref(b)))
        return b.value

    def size(self, index):
        w, h = ctypes.c_uint32(), ctypes.c_uint32()
        _check(lib().sr_batch_info(self._h, int(index), ctypes.byref(w), ctypes.byref(h)))
        return w.value, h.value

    def image(self, index, out=None, stream=None):
        w, h = self.size(index)
        if out is None:
            out = np.empty((h, w, 4), np.uint8)
        _check(lib().sr_batch_get_image(self._h, int(index), out.ctypes.data, 0, stream))
        return out

    def stats(self):
        s = BatchStats()
        _check(lib().sr_batch_get_stats(self._h, ctypes.byref(s)))
        f = s.frame
        d = {k: getattr(s, k) for k, _ in BatchStats._fields_ if k != "frame"}
        d.update({k: getattr(f, k) for k, _ in Stats._fields_ if k not in ("stage_ms", "reruns")})
        d["stage_ms"] = dict(zip(STAGE_NAMES, [float(x) for x in f.stage_ms]))
        return d

    def clear(self):
        _check(lib().sr_batch_clear(self._h))

    def close(self):
        if self._h:
            lib().sr_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceArray:
    """Device memory owned through sr_device_alloc (no CUDA binding needed)."""

    def __init__(self, shape, dtype, device=0):
        self.shape = tuple(int(x) for x in np.atleast_1d(shape))
        self.dtype = np.dtype(dtype)
        self.nbytes = int(np.prod(self.shape)) * self.dtype.itemsize
        p = lib().sr_device_alloc(int(device), max(self.nbytes, 1))
        if not p:
            raise SRError(2, "sr_device_alloc of %d bytes failed" % self.nbytes)
        self.ptr = ctypes.c_void_p(p)

    @classmethod
    def from_numpy(cls, a, device=0):
        a = np.ascontiguousarray(a)
        d = cls(a.shape, a.dtype, device)
        if a.nbytes:
            _check(lib().sr_memcpy(d.ptr, a.ctypes.data, a.nbytes))
        return d

    def numpy(self):
        a = np.empty(self.shape, self.dtype)
        if self.nbytes:
            _check(lib().sr_memcpy(a.ctypes.data, self.ptr, self.nbytes))
        return a

    def rows(self, start, stop):
        """A view of rows [start, stop) (no copy; valid while self lives)."""
        v = DeviceArray.__new__(DeviceArray)
        row = int(np.prod(self.shape[1:])) * self.dtype.itemsize
        v.shape = (stop - start,) + self.shape[1:]
        v.dtype = self.dtype
        v.nbytes = (stop - start) * row
        v.ptr = ctypes.c_void_p(self.ptr.value + start * row)
        v._base = self
        return v

    def free(self):
        if getattr(self, "_base", None) is None and self.ptr:
            lib().sr_device_free(self.ptr)
        self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def concat_device(arrays):
    """Concatenates device arrays along rows into a new DeviceArray."""
    rows = sum(a.shape[0] for a in arrays)
    out = DeviceArray((rows,) + arrays[0].shape[1:], arrays[0].dtype)
    off = 0
    for a in arrays:
        if a.nbytes:
            _check(lib().sr_memcpy(ctypes.c_void_p(out.ptr.value + off), a.ptr, a.nbytes))
        off += a.nbytes
    return out


def sizer_norm(features, labels):
    """Normaliser (x mean, x inverse std, y mean, y std) of host arrays."""
    f = np.asarray(features, np.float64)
    t = np.asarray(labels, np.float64)
    xs = f.std(0)
    ys = t.std(0)
    xs[xs < 1e-6] = 1.0
    ys[ys < 1e-6] = 1.0
    return np.concatenate([f.mean(0), 1.0 / xs, t.mean(0), ys]).astype(np.float32)


class Sizer:
    """The learned-sizing network (sr_sizer_*): 6 -> 64 -> 64 -> 2 GELU,
    BF16 weights with FP32 accumulation, Adam, all on the GPU."""

    def __init__(self, device=0, seed=0):
        h = ctypes.c_void_p()
        _check(lib().sr_sizer_create(int(device), int(seed), ctypes.byref(h)))
        self._h = h
        self.device = device

    def set_norm(self, norm):
        a = np.ascontiguousarray(norm, np.float32).reshape(SIZER_NORM)
        _check(lib().sr_sizer_set_norm(self._h, a.ctypes.data))

    def state(self):
        p = np.empty(SIZER_PARAMS, np.float32)
        m = np.empty(SIZER_PARAMS, np.float32)
        v = np.empty(SIZER_PARAMS, np.float32)
        nm = np.empty(SIZER_NORM, np.float32)
        step = ctypes.c_int64()
        _check(lib().sr_sizer_get_state(self._h, p.ctypes.data, m.ctypes.data, v.ctypes.data, nm.ctypes.data,
                                        ctypes.byref(step)))
        return {"params": p, "adam_m": m, "adam_v": v, "norm": nm, "step": step.value}

    def load_state(self, st):
        arr = {k: np.ascontiguousarray(st[k], np.float32) for k in ("params", "adam_m", "adam_v", "norm")}
        _check(lib().sr_sizer_set_state(self._h, arr["params"].ctypes.data, arr["adam_m"].ctypes.data,
                                        arr["adam_v"].ctypes.data, arr["norm"].ctypes.data, int(st["step"])))

    def save(self, path):
        np.savez(path, **self.state())

    def load(self, path):
        with np.load(path) as z:
            self.load_state({k: z[k] for k in z.files})

    def loss_grad(self, x, t):
        g = np.empty(SIZER_PARAMS, np.float32)
        loss = ctypes.c_float()
        _check(lib().sr_sizer_loss_grad(self._h, x.ptr, t.ptr, int(x.shape[0]), g.ctypes.data, ctypes.byref(loss)))
        return float(loss.value), g

    def train(self, x, t, epochs=1, batch=4096, lr=1e-3, shuffle=True, seed=0, beta1=0.9, beta2=0.999, eps=1e-8,
              stream=None):
        o = SizerTrainOpts(ctypes.sizeof(SizerTrainOpts), int(batch), int(epochs), 1 if shuffle else 0, lr, beta1,
                           beta2, eps, int(seed))
        loss = ctypes.c_float()
        _check(lib().sr_sizer_train(self._h, x.ptr, t.ptr, int(x.shape[0]), ctypes.byref(o), ctypes.byref(loss),
                                    stream))
        return float(loss.value)

    def predict(self, x, out=None, stream=None):
        n = int(x.shape[0])
        out = out if out is not None else DeviceArray((n, SIZER_OUTPUTS), np.float32, self.device)
        _check(lib().sr_sizer_predict(self._h, x.ptr, n, out.ptr, stream))
        return out

    def close(self):
        if self._h:
            lib().sr_sizer_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def calibrate_margins(pred, labels, path_begin, path_quantile=0.995, frame_slack=0.02):
    """Sizing margins from held-out rows: pred and labels [P, 2] in
    log(1 + count) units, path_begin [S + 1] the scenes' path ranges.

    The path margins are the `path_quantile` quantile of the per-path
    residuals (so about 1 - path_quantile of the paths exceed their
    allotment).  The frame margins are the smallest margins under which the
    summed capacity of every held-out scene covers its exact count, plus
    `frame_slack`."""
    pred = np.asarray(pred, np.float64)
    lab = np.asarray(labels, np.float64)
    exact = np.rint(np.expm1(lab))
    out = []
    for o in range(2):
        out.append(float(np.quantile(lab[:, o] - pred[:, o], path_quantile)))
    for o in range(2):
        need = -np.inf
        for s in range(len(path_begin) - 1):
            a, b = int(path_begin[s]), int(path_begin[s + 1])
            if b <= a:
                continue
            want = exact[a:b, o].sum()
            if want <= 0:
                continue
            lo, hi = -8.0, 8.0
            for _ in range(40):      # smallest m with sum(ceil(expm1(pred + m))) >= want
                mid = 0.5 * (lo + hi)
                got = np.ceil(np.expm1(np.minimum(pred[a:b, o] + mid, 21.0))).clip(0).sum()
                lo, hi = (lo, mid) if got >= want else (mid, hi)
            need = max(need, hi)
        out.append(float((need if np.isfinite(need) else 0.0) + frame_slack))
    return tuple(out)


def admission_take(req_bytes, held_bytes, budget, max_take=None):
    """The server's admission rule: (requests taken in order, rejected)."""
    a = np.ascontiguousarray(req_bytes, np.uint64)
    rej = ctypes.c_int()
    k = lib().sr_admission_take(a.ctypes.data if a.size else None, int(a.size), int(held_bytes), int(budget),
                                int(a.size if max_take is None else max_take), ctypes.byref(rej))
    return int(k), bool(rej.value)


class RenderServer:
    """Continuous-batching render server (sr_server_*): submit() from any
    thread, wait() for each ticket.  With a Sizer the batches are sized by
    the network and kept in flight on several streams; without one every
    batch waits for its exact count."""

    def __init__(self, mode=MODE_PIXEL, device=0, slots=2, max_batch_scenes=64, memory_budget=120e9, sizer=None,
                 margins=(0.5, 1.2, 0.05, 0.25)):
        o = ServerOpts(ctypes.sizeof(ServerOpts), mode, device, slots, max_batch_scenes, 0, int(memory_budget),
                       SizingMargins(ctypes.sizeof(SizingMargins), *[float(v) for v in margins]))
        h = ctypes.c_void_p()
        _check(lib().sr_server_create(ctypes.byref(o), sizer._h if sizer is not None else None, ctypes.byref(h)))
        self._h = h
        self._sizer = sizer
        self._sizes = {}

    def submit(self, container, width=None, height=None, mvp=None):
        w = container.width if width is None else width
        h = container.height if height is None else height
        v = container.view()
        m = None if mvp is None else np.ascontiguousarray(mvp, np.float32).reshape(16)
        t = ctypes.c_uint64()
        _check(lib().sr_server_submit(self._h, int(w), int(h), ctypes.byref(v),
                                      m.ctypes.data if m is not None else None, ctypes.byref(t)))
        self._sizes[t.value] = (int(w), int(h))
        return t.value

    def wait(self, ticket, fetch=True, timeout_ms=-1):
        """(image (h, w, 4) uint8 or None, info dict)."""
        w, h = self._sizes.pop(ticket)
        out = np.empty((h, w, 4), np.uint8) if fetch else None
        info = RequestInfo()
        rc = lib().sr_server_wait(self._h, int(ticket), out.ctypes.data if fetch else None, 0, ctypes.byref(info),
                                  int(timeout_ms))
        d = {k: getattr(info, k) for k, _ in RequestInfo._fields_ if k != "reserved"}
        if rc != 0:
            if rc == 4:
                self._sizes[ticket] = (w, h)
            raise SRError(rc, lib().sr_last_error().decode(errors="replace"))
        return out, d

    def stats(self):
        s = ServerStats()
        _check(lib().sr_server_get_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def close(self):
        if self._h:
            lib().sr_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
