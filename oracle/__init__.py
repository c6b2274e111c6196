"""CPU restatement of the VkScanlinePR scanline pipeline — test infrastructure.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, to check the renderer's output.  The renderer (vkscanlinepr_gb300)
never imports it.

Parity status: unpinned by reference outputs (the reference has no tests and
cannot run here); pinned by hand-computed known-answer scenes and by the
draw-record format of the reference's mock draw lists.  See oracle.cpp.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")

MODE_REFERENCE = 0
MODE_PIXEL = 1

# stage ids, same values as sr_stage in include/sr.h
STAGES = {
    "transformed_pos": 0, "path_visible": 1, "cutpoints": 2, "curve_count": 3,
    "curve_offset": 4, "intersection": 5, "frag_key": 6, "frag_winding": 7,
    "sorted_key": 8, "sorted_index": 9, "winding_scan": 10, "frag_flag": 11,
    "span_flag": 12, "draw_list": 13, "image": 14, "frag_left": 15,
    "path_draws": 100,
}


def build(force=False):
    """Compile oracle.cpp into _build/liboracle.so (g++, -ffp-contract=off)."""
    src = os.path.join(HERE, "oracle.cpp")
    deps = [src, os.path.join(REPO, "include", "sr.h"),
            os.path.join(REPO, "vkscanlinepr_gb300", "csrc", "synth.h")]
    if not force and os.path.exists(LIB) and all(
            os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c++17",
           "-pthread", "-o", tmp, src]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


class SceneView(ctypes.Structure):
    _fields_ = [
        ("n_points", ctypes.c_uint32), ("n_curves", ctypes.c_uint32),
        ("n_paths", ctypes.c_uint32),
        ("position", ctypes.c_void_p), ("pos_path_idx", ctypes.c_void_p),
        ("curve_pos_map", ctypes.c_void_p), ("curve_type", ctypes.c_void_p),
        ("curve_path_idx", ctypes.c_void_p), ("fill_rule", ctypes.c_void_p),
        ("fill_info", ctypes.c_void_p),
    ]


class Paint(ctypes.Structure):
    """sr_paint (include/sr.h): a linear or radial gradient."""
    _fields_ = [("kind", ctypes.c_int32), ("spread", ctypes.c_int32), ("p0", ctypes.c_float * 2),
                ("p1", ctypes.c_float * 2), ("radius", ctypes.c_float), ("xf", ctypes.c_float * 6),
                ("opacity", ctypes.c_float), ("n_stops", ctypes.c_uint32), ("offset", ctypes.c_float * 16),
                ("rgba", (ctypes.c_float * 4) * 16)]


class SynthParams(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32), ("preset", ctypes.c_int32),
        ("seed", ctypes.c_uint64), ("scene_index", ctypes.c_uint32),
        ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
        ("n_paths", ctypes.c_uint32),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.or_render.argtypes = [ctypes.POINTER(SceneView), ctypes.c_uint32, ctypes.c_uint32,
                                ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.POINTER(ctypes.c_void_p)]
        L.or_render_paints.argtypes = [ctypes.POINTER(SceneView), ctypes.c_uint32, ctypes.c_uint32,
                                       ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_void_p)]
        L.or_get.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                             ctypes.POINTER(ctypes.c_size_t)]
        L.or_stats.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.or_free.argtypes = [ctypes.c_void_p]
        L.or_resolve.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_uint32, ctypes.c_uint32,
                                 ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.or_blend.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
        L.or_blend.restype = ctypes.c_uint32
        L.or_synth.argtypes = [ctypes.POINTER(SynthParams), ctypes.POINTER(ctypes.c_void_p)]
        L.or_scene_view.argtypes = [ctypes.c_void_p, ctypes.POINTER(SceneView), ctypes.c_void_p]
        L.or_scene_free.argtypes = [ctypes.c_void_p]
        L.or_hw_threads.restype = ctypes.c_int
        _lib = L
    return _lib


class Scene:
    """A flattened scene held as numpy arrays (the reference's loadVG SoA)."""

    FIELDS = ("position", "pos_path_idx", "curve_pos_map", "curve_type",
              "curve_path_idx", "fill_rule", "fill_info")

    def __init__(self, width, height, position, pos_path_idx, curve_pos_map, curve_type,
                 curve_path_idx, fill_rule, fill_info, paints=None):
        self.paints = paints   # gradient paints: a ctypes array of sr_paint-layout structs, or None
        self.width = int(width)
        self.height = int(height)
        self.position = np.ascontiguousarray(position, dtype=np.float32).reshape(-1)
        self.pos_path_idx = np.ascontiguousarray(pos_path_idx, dtype=np.uint32)
        self.curve_pos_map = np.ascontiguousarray(curve_pos_map, dtype=np.uint32)
        self.curve_type = np.ascontiguousarray(curve_type, dtype=np.uint32)
        self.curve_path_idx = np.ascontiguousarray(curve_path_idx, dtype=np.uint32)
        self.fill_rule = np.ascontiguousarray(fill_rule, dtype=np.uint32)
        self.fill_info = np.ascontiguousarray(fill_info, dtype=np.uint32)

    @property
    def n_points(self):
        return self.pos_path_idx.size

    @property
    def n_curves(self):
        return self.curve_type.size

    @property
    def n_paths(self):
        return self.fill_rule.size

    def view(self):
        v = SceneView()
        v.n_points, v.n_curves, v.n_paths = self.n_points, self.n_curves, self.n_paths
        for f in self.FIELDS:
            setattr(v, f, getattr(self, f).ctypes.data)
        return v


def synth(preset, seed, scene_index=0, width=0, height=0, n_paths=0):
    """Generate a synthetic scene with the shared generator (synth.h)."""
    L = lib()
    p = SynthParams(ctypes.sizeof(SynthParams), preset, seed, scene_index, width, height, n_paths)
    h = ctypes.c_void_p()
    if L.or_synth(ctypes.byref(p), ctypes.byref(h)) != 0:
        raise RuntimeError("or_synth failed")
    try:
        v = SceneView()
        wh = (ctypes.c_uint32 * 2)()
        L.or_scene_view(h, ctypes.byref(v), wh)

        def arr(ptr, n, dt):
            if n == 0:
                return np.zeros(0, dt)
            return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(np.ctypeslib.as_ctypes_type(dt))),
                                         shape=(n,)).copy()
        return Scene(wh[0], wh[1],
                     arr(v.position, 2 * v.n_points, np.float32),
                     arr(v.pos_path_idx, v.n_points, np.uint32),
                     arr(v.curve_pos_map, v.n_curves, np.uint32),
                     arr(v.curve_type, v.n_curves, np.uint32),
                     arr(v.curve_path_idx, v.n_curves, np.uint32),
                     arr(v.fill_rule, v.n_paths, np.uint32),
                     arr(v.fill_info, v.n_paths, np.uint32))
    finally:
        L.or_scene_free(h)


IDENTITY = np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1], np.float32)

_DTYPES = {"transformed_pos": np.float32, "cutpoints": np.float32, "image": np.uint8}


class Frame:
    """One rendered frame of the oracle with every stage kept."""

    def __init__(self, scene, width=None, height=None, mvp=None, mode=MODE_PIXEL, threads=0, fp64=False):
        L = lib()
        self._scene = scene  # keep arrays alive
        w = scene.width if width is None else width
        h = scene.height if height is None else height
        m = IDENTITY if mvp is None else np.ascontiguousarray(mvp, np.float32).reshape(16)
        self._m = m
        self.width, self.height, self.mode, self.fp64 = w, h, mode, fp64
        v = scene.view()
        hd = ctypes.c_void_p()
        paints = getattr(scene, "paints", None)
        rc = L.or_render_paints(ctypes.byref(v), w, h, m.ctypes.data, mode, threads, 1 if fp64 else 0,
                                ctypes.cast(paints, ctypes.c_void_p) if paints else None,
                                len(paints) if paints else 0, ctypes.byref(hd))
        self._h = hd
        if rc != 0:
            raise RuntimeError("oracle render failed (%d)" % rc)
        counts = np.zeros(4, np.int64)
        ms = np.zeros(6, np.float64)
        L.or_stats(hd, counts.ctypes.data, ms.ctypes.data)
        self.n_intersections, self.n_draw, self.n_frag, self.n_span = (int(c) for c in counts)
        self.stage_ms = ms

    def get(self, name):
        L = lib()
        p = ctypes.c_void_p()
        b = ctypes.c_size_t()
        if L.or_get(self._h, STAGES[name], ctypes.byref(p), ctypes.byref(b)) != 0:
            raise KeyError(name)
        dt = _DTYPES.get(name, np.int32)
        n = b.value // np.dtype(dt).itemsize
        if n == 0:
            a = np.zeros(0, dt)
        else:
            a = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(np.ctypeslib.as_ctypes_type(dt))),
                                      shape=(n,)).copy()
        if name == "image":
            a = a.reshape(self.height, self.width, 4)
        elif name == "draw_list":
            a = a.reshape(-1, 4)
        elif name == "intersection":
            a = a.reshape(-1, 2)
        elif name == "transformed_pos":
            a = a.reshape(-1, 2)
        return a

    def __del__(self):
        try:
            if self._h:
                lib().or_free(self._h)
                self._h = None
        except Exception:
            pass


def fp64_flips(scene, mode, mvp=None, threads=0, image=None):
    """Samples (pixels, at 1 sample per pixel) whose colour differs between
    the FP32 frame -- `image` when given (e.g. the GPU's, which is bit-exact
    to the oracle's FP32 frame), else the oracle's own -- and the oracle's
    FP64 instance of the same scene (double arithmetic, 52 bisection steps)."""
    if image is None:
        image = Frame(scene, mvp=mvp, mode=mode, threads=threads).get("image")
    ref = Frame(scene, mvp=mvp, mode=mode, threads=threads, fp64=True).get("image")
    return int(np.any(np.asarray(image) != ref, axis=2).sum())


def aa_offsets(k):
    """Sample positions within a pixel for k-sample antialiasing: sample i
    at (((i * s) mod k + 0.5) / k, (i + 0.5) / k), every sample on a row and
    a column of its own (s = 5 for k = 16, 3 for k = 4 or 8, 1 otherwise).
    float32, in the order the renderer computes them."""
    s = 5 if k == 16 else (3 if k >= 4 else 1)
    f = np.float32
    return [((f((i * s) % k) + f(0.5)) / f(k), (f(i) + f(0.5)) / f(k)) for i in range(k)]


def render_aa(scene, samples, mvp=None, threads=0):
    """The antialiased image (sr_render_aa): each sample is the pixel-mode
    frame with the scene moved by (0.5 - dx, 0.5 - dy) after the matrix (rows
    0 and 1 plus the translation times row 3, in float32), and a pixel is the
    rounded average (sum + k/2) // k of its samples per channel."""
    m = IDENTITY if mvp is None else np.ascontiguousarray(mvp, np.float32).reshape(16)
    acc = None
    f = np.float32
    for ox, oy in aa_offsets(samples):
        tx, ty = f(0.5) - ox, f(0.5) - oy
        mm = m.copy()
        for k in range(4):
            mm[k] = m[k] + tx * m[12 + k]
            mm[4 + k] = m[4 + k] + ty * m[12 + k]
        img = Frame(scene, mvp=mm, mode=MODE_PIXEL, threads=threads).get("image").astype(np.uint32)
        acc = img if acc is None else acc + img
    return ((acc + samples // 2) // samples).astype(np.uint8)


def resolve(draw, width, height, mode, threads=1):
    """Paint an int32x4 draw list with the oracle's resolve step."""
    d = np.ascontiguousarray(draw, np.int32).reshape(-1, 4)
    out = np.zeros((height, width, 4), np.uint8)
    lib().or_resolve(d.ctypes.data, d.shape[0], width, height, mode, threads, out.ctypes.data)
    return out


def blend(dst, src):
    return int(lib().or_blend(dst, src))


def hw_threads():
    return int(lib().or_hw_threads())
