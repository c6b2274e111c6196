/*
 * sr.h — C ABI of the GB300 scanline path renderer.
 *
 * This is the drop-in boundary for the scanline rasterizer of
 * galaxysailing/VkScanlinePR.  The reference exposes an abstract C++ class
 * (VkScanlinePR/src/core/rasterizer.h:9-20):
 *
 *     class VGRasterizer {
 *         virtual void initialize(void* window, uint32_t w, uint32_t h) = 0;
 *         virtual void render() = 0;
 *         virtual void loadVG(std::shared_ptr<VGContainer> vg) = 0;
 *         virtual void setMVP(const glm::mat4& m) = 0;
 *     };
 *
 * implemented by ScanlineVGRasterizer (core/scanline/scanline_rasterizer.h:31-49).
 * Each entry point below names the reference member it replaces.  All calls
 * take plain pointers and sizes; no C++ or torch types cross this boundary and
 * no exception escapes it.  A context is not thread-safe: use one context per
 * host thread or lock externally.  All device work runs on the caller's stream.
 */
#ifndef SR_H_
#define SR_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SR_ABI_VERSION 1

/* Status codes.  The reference reports failures by C++ exceptions
 * (app/vg_app.cpp:181, core/scanline/scanline_rasterizer.cpp:219-225) and by
 * VK_CHECK_RESULT assert/exit (core/vk/vk_util.h:21-29); here every call
 * returns one of these and sr_last_error() gives the message. */
typedef enum sr_status {
    SR_OK = 0,
    SR_ERR_INVALID_ARG = 1,   /* bad pointer, size, curve type or fill rule  */
    SR_ERR_OOM = 2,           /* device or host allocation failed             */
    SR_ERR_OVERFLOW_REFIT = 3,/* a pre-sized buffer overflowed; rerun exact   */
    SR_ERR_TIMEOUT = 4,       /* a bounded device-side wait gave up           */
    SR_ERR_CUDA = 5,          /* a CUDA runtime call failed                   */
    SR_ERR_NO_SCENE = 6,      /* render called before a scene was loaded      */
    SR_ERR_INTERNAL = 7       /* a device-side consistency check failed       */
} sr_status;

/* Curve types, same values as Galaxysailing::CurveType
 * (core/vg/vg_container.h:9-15).  QUADRIC is listed as TODO in every
 * reference shader; this library defines it natively (3 control points,
 * monotonised at the derivative root, evaluated by a 2-level lerp).
 * ARC (a TODO in the reference too) is a rational quadratic, the RVG
 * format's 'A' segment.  It owns 4 point slots: P0, the control point in
 * homogeneous coordinates (w*x, w*y), P2, and (w, w), with w finite and
 * w > -1 (w = 0 is a half ellipse).  It is evaluated by a 2-level lerp of
 * the homogeneous points (x*w, w), then one division, and monotonised at
 * the roots of its derivative's numerator, a quadratic.  Under the matrix,
 * P0 and P2 transform as points; the control point transforms linearly as
 * (w*x, w*y, 0, w), its w becoming the fourth row's result (for an affine
 * matrix, w itself). */
enum { SR_CURVE_LINE = 0x02, SR_CURVE_QUADRIC = 0x03, SR_CURVE_CUBIC = 0x04, SR_CURVE_ARC = 0x13 };

/* Fill rules, same values as Galaxysailing::FillRule (vg_container.h:16-19). */
enum { SR_FILL_NONZERO = 0, SR_FILL_EVENODD = 1 };

/* Gradient paints (the RVG format's linear and radial "dyn_paint", which
 * RVG::load skips, rvg.cpp:234-251).  A path painted by paint i of the
 * context's table (sr_set_paints) has fill_info SR_FILL_PAINT(i): alpha byte
 * 0 and i + 1 in the colour bytes (a solid colour with alpha 0 is stored as
 * 0, so the two never meet).
 *
 * Evaluation, identical in the renderer and the oracle: a pixel's centre
 * (x + 0.5, y + 0.5) -- in reference mode (x + 0.5, cell_y + 1), the centre
 * row of the 2-pixel cell -- is mapped to gradient space by the inverse of
 * (the matrix's affine part) * xf, computed in double and rounded to float
 * once per paint; then in float: linear t = the projection on p0 -> p1
 * (folded into one affine form of the pixel); radial t solves
 * |g - f - t (c - f)| = t r (focus f = p1, centre c = p0; the root the
 * focus-inside case takes; t = 0 where none exists); the spread (pad clamps
 * to [0, 1], repeat takes t - floor t, reflect folds it); the colour is the
 * linear interpolation between the two stops around t (the first or last
 * stop outside them); alpha is multiplied by opacity; each channel is packed
 * as u8(v * 255) truncated, and alpha 0 leaves the pixel alone (pixel mode)
 * or writes 0 (reference mode, whose overwrite writes alpha raw). */
#define SR_PAINT_MAX_STOPS 16
enum { SR_PAINT_LINEAR = 1, SR_PAINT_RADIAL = 2 };
enum { SR_SPREAD_PAD = 0, SR_SPREAD_REPEAT = 1, SR_SPREAD_REFLECT = 2 };
typedef struct sr_paint {
    int32_t  kind;          /* SR_PAINT_LINEAR or SR_PAINT_RADIAL              */
    int32_t  spread;        /* SR_SPREAD_*                                      */
    float    p0[2];         /* linear: start point; radial: centre              */
    float    p1[2];         /* linear: end point; radial: focus                 */
    float    radius;        /* radial                                           */
    float    xf[6];         /* gradient -> scene: (xf0 x + xf1 y + xf2, xf3 x + xf4 y + xf5) */
    float    opacity;       /* multiplies every stop's alpha                     */
    uint32_t n_stops;       /* 1..SR_PAINT_MAX_STOPS, offsets non-decreasing     */
    float    offset[SR_PAINT_MAX_STOPS];
    float    rgba[SR_PAINT_MAX_STOPS][4];   /* each channel in [0, 1]          */
} sr_paint;
#define SR_FILL_PAINT(i) ((uint32_t)(i) + 1u)

/* Render modes.
 * SR_MODE_REFERENCE: the reference's own semantics — 2-px fragment grid
 *   (FRAG_SIZE 2), winding sampled on the line y = cell_y + 1, every boundary
 *   cell painted whole, and the draw list painted with blending off (the last
 *   path wins), as the reference's line pipeline does
 *   (core/scanline/scanline_rasterizer.cpp:881-944, blendEnable FALSE).
 * SR_MODE_PIXEL: 1 sample per pixel at the pixel centre — 1-px grid, winding
 *   sampled on the pixel-centre row, a boundary pixel painted when its centre
 *   passes the fill rule, and integer source-over compositing in path order
 *   over white. */
enum { SR_MODE_REFERENCE = 0, SR_MODE_PIXEL = 1 };

/* The flattened scene, structure-of-arrays, in exactly the layout the
 * reference's loadVG builds (core/scanline/scanline_rasterizer.cpp:67-189):
 * points grouped by curve, curves grouped by path, every curve owning its
 * control points privately (a cubic owns 4, a quadric 3, a line 2).
 * fill_info is the packed colour: bytes R,G,B,A in memory order (little-
 * endian uint32), alpha already multiplied by opacity, zero when alpha is 0
 * (scanline_rasterizer.cpp:107-118). */
typedef struct sr_scene_view {
    uint32_t n_points;
    uint32_t n_curves;
    uint32_t n_paths;
    const float*    position;       /* [2*n_points] x,y pairs               */
    const uint32_t* pos_path_idx;   /* [n_points]  path of each point       */
    const uint32_t* curve_pos_map;  /* [n_curves]  first point of the curve */
    const uint32_t* curve_type;     /* [n_curves]  SR_CURVE_*               */
    const uint32_t* curve_path_idx; /* [n_curves]  path of each curve       */
    const uint32_t* fill_rule;      /* [n_paths]   SR_FILL_*                */
    const uint32_t* fill_info;      /* [n_paths]   packed RGBA8             */
} sr_scene_view;

typedef struct sr_options {
    uint32_t struct_size;   /* sizeof(sr_options)                          */
    int32_t  mode;          /* SR_MODE_REFERENCE or SR_MODE_PIXEL          */
    int32_t  device;        /* CUDA device ordinal                         */
    uint32_t flags;         /* SR_FLAG_*                                   */
} sr_options;

/* Keep every intermediate stage buffer after sr_render so that
 * sr_debug_dump can read it (parity testing; costs extra device writes). */
#define SR_FLAG_KEEP_STAGES 0x1u
/* Record a CUDA event around every stage of sr_render (see sr_stats). */
#define SR_FLAG_PROFILE 0x2u

typedef struct sr_ctx sr_ctx;

/* Replaces VGRasterizer::initialize(window, w, h) (rasterizer.h:11).  There
 * is no window: the canvas is a headless w x h RGBA8 framebuffer. */
sr_status sr_create(uint32_t width, uint32_t height, const sr_options* opt, sr_ctx** out);

/* Replaces VGRasterizer::loadVG (rasterizer.h:15).  Copies the scene into
 * device memory owned by the context; it stays resident until the next load
 * or sr_destroy.  Rejects curve types other than line/quadric/cubic, fill
 * rules other than nonzero/even-odd and out-of-range indices. */
sr_status sr_load_scene(sr_ctx* ctx, const sr_scene_view* scene);

/* Replaces VGRasterizer::setMVP (rasterizer.h:17).  m holds the four rows
 * m0..m3 of the transform, 16 floats: a point (x,y) maps to
 * (dot((x,y,0,1), m0) / dot(.., m3), dot((x,y,0,1), m1) / dot(.., m3)),
 * which is ScanlineVGRasterizer::setMVP (scanline_rasterizer.cpp:191-197)
 * given transpose(camera.mv()) as the application passes it
 * (app/vg_app.cpp:159-160). */
sr_status sr_set_mvp(sr_ctx* ctx, const float m[16]);

/* Antialiased frame (SR_MODE_PIXEL contexts): `samples` (1, 2, 4, 8 or 16)
 * samples a pixel on a comb, every sample on a row and a column of its own:
 * sample i at (x + ((i * s) mod k + 0.5) / k, y + (i + 0.5) / k), s = 5 for
 * k = 16, 3 for k = 4 or 8, 1 otherwise.  Each sample is the pixel-mode test
 * at that point (the pixel-centre sample moved there; composited in path
 * order over white), and the pixel is the rounded average (sum + k/2) / k
 * of its samples per channel.  The samples' frames are rendered by moving
 * the scene by (0.5 - dx, 0.5 - dy) after the matrix (rows 0 and 1 take the
 * translation times row 3), and summed on the device.  This is the
 * reference's antialiasing TODO, the "comb-like multisampling" of
 * README.md:5 and gen_fragment.comp:202.  Waits for the frame. */
sr_status sr_render_aa(sr_ctx* ctx, uint32_t samples, void* rgba_out, int out_is_device, void* stream);

/* Sets the gradient paints the loaded scene's SR_FILL_PAINT(i) fills refer
 * to (copied; they follow later sr_set_mvp calls).  n = 0 clears the table;
 * a fill that names no paint of the table paints nothing. */
sr_status sr_set_paints(sr_ctx* ctx, const sr_paint* paints, uint32_t n);

/* Replaces VGRasterizer::render (rasterizer.h:13).  Renders one frame on
 * `stream` (a cudaStream_t, NULL for the legacy default stream) into
 * rgba_out: width*height*4 bytes, row y of the canvas at byte offset
 * y*width*4 (no vertical flip).  rgba_out may be host memory (copied
 * synchronously at the end) or device memory (out_is_device = 1; the call
 * returns once the frame is enqueued).  rgba_out may be NULL to render
 * into the context's own device framebuffer only. */
sr_status sr_render(sr_ctx* ctx, void* rgba_out, int out_is_device, void* stream);

/* Paints a caller-given draw list: n records of 4 int32 (packed yx, width,
 * RGBA8 colour, fragment index) in host memory, as produced by the emit
 * stage (gen_merged_fragment_and_span.comp:170,195).  This is the
 * reference's MOCK_DATA path (scanline_rasterizer.cpp:251-281, :808-818),
 * which skips the compute passes and draws a draw list read from a CSV.
 * Output as for sr_render; records whose row lies outside the canvas are
 * skipped. */
sr_status sr_render_draw_list(sr_ctx* ctx, const int32_t* records, int64_t n, void* rgba_out, int out_is_device,
                              void* stream);

/* Per-frame counters of the last sr_render. */
typedef struct sr_stats {
    uint64_t n_intersections;  /* N: intersection records (n_fragments)  */
    uint64_t n_draw_records;   /* O: merged fragments + spans            */
    uint64_t n_merged_fragments;
    uint64_t n_spans;
    uint32_t key_bits;         /* bits of the sort key                   */
    uint32_t sort_passes;      /* radix passes run                       */
    uint32_t kernel_launches;  /* kernels this library launched for the frame */
    uint32_t reruns;           /* sr_render: pre-sized frames of this context
                                * that overflowed and were rerun with exact
                                * sizing (cumulative; 0 for batches)        */
    /* with SR_FLAG_PROFILE: device time of each stage (CUDA events):
     * transform, count, offset scan, crossing chains, record merge,
     * fragments (these three on the context's second stream), sort,
     * winding+emit, row sort, resolve; then the wide chains with their
     * curves' merge and fragments, on the render stream beside them */
    float stage_ms[12];
} sr_stats;
sr_status sr_get_stats(const sr_ctx* ctx, sr_stats* out);

/* Stage identifiers for sr_debug_dump; the layouts follow the reference's
 * buffers so that each can be compared with the CPU restatement. */
typedef enum sr_stage {
    SR_STAGE_TRANSFORMED_POS = 0, /* float2[n_points]  (transform_pos.comp:85)             */
    SR_STAGE_PATH_VISIBLE = 1,    /* int32[n_paths]    (transform_pos.comp:71-82)          */
    SR_STAGE_CUTPOINTS = 2,       /* float[5*n_curves] (make_intersection_0.comp:368-372)  */
    SR_STAGE_CURVE_COUNT = 3,     /* int32[n_curves]   (make_intersection_0.comp:410)      */
    SR_STAGE_CURVE_OFFSET = 4,    /* int32[n_curves+1] exclusive scan of the counts        */
    SR_STAGE_INTERSECTION = 5,    /* int32x2[N] (curve, t bits | flags) (make_intersection_1.comp:370-372) */
    SR_STAGE_FRAG_KEY = 6,        /* int32[N] packed yx or 0xFFFEFFFE (gen_fragment.comp:221) */
    SR_STAGE_FRAG_WINDING = 7,    /* int32[N] winding change (gen_fragment.comp:224)       */
    SR_STAGE_SORTED_KEY = 8,      /* int32[N] yx after the per-path sort                   */
    SR_STAGE_SORTED_INDEX = 9,    /* int32[N] record index after the per-path sort         */
    SR_STAGE_WINDING_SCAN = 10,   /* int32[N+1] exclusive scan of sorted winding changes   */
    SR_STAGE_FRAG_FLAG = 11,      /* int32[N] merged-fragment flags                        */
    SR_STAGE_SPAN_FLAG = 12,      /* int32[N] span flags                                   */
    SR_STAGE_DRAW_LIST = 13,      /* int32x4[O] draw records (gen_merged_fragment_and_span.comp:170,195) */
    SR_STAGE_IMAGE = 14,          /* uint8[w*h*4] RGBA8                                    */
    SR_STAGE_FRAG_LEFT = 15       /* int32[N] centre-sample winding part (pixel mode)      */
} sr_stage;

/* Copies one stage of the last sr_render (made with SR_FLAG_KEEP_STAGES) to
 * host memory.  If dst is NULL only *bytes is set to the size needed;
 * otherwise *bytes must hold the capacity of dst on entry. */
sr_status sr_debug_dump(sr_ctx* ctx, int stage, void* dst, size_t* bytes);

/* Replaces the destructor of ScanlineVGRasterizer. */
void sr_destroy(sr_ctx* ctx);

/* Exclusive scan of n int32 values in device memory: d_out[0..n] with
 * d_out[n] = the total (n+1 outputs; d_in and d_out may be the same
 * buffer), wrapping on overflow.  Replaces the reference's standalone scan
 * kernel workdir/shaders/common/naive_scan.comp:27-73 (one workgroup,
 * 1023-element batches) with a single-pass decoupled look-back scan.
 * Asynchronous on `stream`; its look-back scratch comes from
 * cudaMallocAsync/cudaFreeAsync on the same stream.  0 <= n < 2^31.
 * A look-back wait that gives up (SR_ERR_TIMEOUT) leaves a wrong prefix in
 * d_out; it is reported by sr_scan_status, not by this call. */
sr_status sr_exclusive_scan_i32(const int32_t* d_in, int32_t* d_out, int64_t n, void* stream);

/* The same scan for callers that cannot allocate device memory: a host that
 * gives all device memory to its own allocator or runs under a hard memory
 * budget forbids third-party allocations, and a frame loop with a fixed
 * latency budget cannot risk an allocation call that may wait on the device.
 * This entry point calls no cudaMalloc, cudaFree or other allocating routine.
 * It has no counterpart in the reference.
 *
 * Its look-back scratch is a fixed array of SR_NOALLOC_SCAN_SCRATCH_BYTES
 * compiled into the library: every GPU that loads the library holds it until
 * the process exits.  n is limited to SR_NOALLOC_SCAN_MAX_N; larger n is
 * rejected with SR_ERR_INVALID_ARG.  The first call on a device looks up the
 * array's device address (with that device current); make that first call
 * before any stream capture; the address does not survive a cudaDeviceReset.
 * Every call uses the same array and clears the part it needs, so calls that
 * overlap on the GPU (on different streams, or from different threads) race:
 * serialise them on one stream.  Inputs, outputs and results are as for
 * sr_exclusive_scan_i32 (timeouts included, reported by sr_scan_status);
 * asynchronous on `stream`. */
#define SR_NOALLOC_SCAN_MAX_N (1ll << 24)
#define SR_NOALLOC_SCAN_SCRATCH_BYTES (4104u * 8u)
sr_status sr_exclusive_scan_i32_noalloc(const int32_t* d_in, int32_t* d_out, int64_t n, void* stream);

/* Waits for `stream`, then reports whether a look-back wait of a standalone
 * scan (sr_exclusive_scan_i32 or sr_exclusive_scan_i32_noalloc) on the
 * current device gave up since the last call: SR_ERR_TIMEOUT if one did
 * (that scan's output is wrong), else SR_OK.  It clears the report.  Scans
 * still running on other streams are reported by a later call.  The
 * reference's scan has no wait to give up (naive_scan.comp runs in one
 * workgroup), so this has no counterpart there.  Allocates nothing. */
sr_status sr_scan_status(void* stream);

/* Sets how many polls every bounded device-side wait (the look-backs of the
 * scans, of the radix sort and of the winding pass) makes before it gives up
 * and the call reports SR_ERR_TIMEOUT; 0 restores the default of 2^22 polls
 * with back-off (a second or more).  Kernels launched after the call use the
 * new limit, in every context of the process; a captured batch graph keeps
 * the limit it was captured with.  No reference counterpart (its waits are
 * host-side queue idles). */
void sr_set_spin_limit(uint32_t polls);

/* Test hook for the bounded waits: the allocating standalone scan with its
 * tile counter started at 1, so that tile 0 never runs and never publishes
 * its sum.  Tile 1's look-back (and any that reach tile 0) waits until the
 * spin limit and gives up; sr_scan_status then reports SR_ERR_TIMEOUT.
 * d_out[0..4095] is left unwritten and the rest is wrong.  n > 0.  No
 * reference counterpart. */
sr_status sr_debug_scan_without_first_tile(const int32_t* d_in, int32_t* d_out, int64_t n, void* stream);

/* Tiles of the last frame's per-path sort and, of those, the ones sorted
 * with 64-bit items (their packed key fields and payload need more than 32
 * bits); both 0 when the frame took the radix sort.  Waits for the device.
 * No reference counterpart. */
sr_status sr_debug_sort_tiles(sr_ctx* ctx, uint32_t* tiles, uint32_t* wide_tiles);

/* Message of the last failing call on this thread ("" if none). */
const char* sr_last_error(void);

/* ------------------------------------------------------------------ */
/* Batches: many uneven scenes in one frame (no reference counterpart; */
/* the reference renders one scene per VGRasterizer).                  */
/* ------------------------------------------------------------------ */

/* A set of scenes rendered together: their curves go through every stage
 * in the same launches (one scene table gives each kernel its scene's
 * canvas), so small scenes share the GPU instead of each paying the launch
 * and read-back costs of a frame.  Each scene's image is bit-identical to
 * the same scene rendered alone with sr_render. */
typedef struct sr_batch sr_batch;

typedef struct sr_synth_params sr_synth_params;

typedef struct sr_batch_render_opts {
    uint32_t struct_size;
    uint32_t use_graph;          /* capture the frame as a CUDA graph and replay it
                                    (needs record_capacity >= 0) */
    int64_t  record_capacity;    /* < 0: size exactly (one host wait for the
                                    record count, as the reference does);
                                    >= 0: pre-sized, no mid-frame wait */
    uint32_t refit_on_overflow;  /* on overflow, rerun with exact sizing */
    uint32_t reserved;
    int64_t  draw_capacity;      /* draw records (merged fragments + spans) the
                                    frame may emit; <= 0: 2 x record_capacity,
                                    which always suffices.  Callers built
                                    against the 24-byte form of this struct get
                                    the default. */
} sr_batch_render_opts;

typedef struct sr_batch_stats {
    sr_stats frame;              /* counters of the last frame (all scenes) */
    uint32_t n_scenes, n_paths, n_curves;
    uint32_t overflows;          /* pre-sized frames whose records did not fit */
    uint32_t refits;             /* of those, rerun with exact sizing */
    uint32_t graph_captured;
    int64_t  record_capacity;    /* capacity of the last frame */
} sr_batch_stats;

sr_status sr_batch_create(const sr_options* opt, sr_batch** out);
/* Appends a scene (copied; resident on the device after sr_batch_commit).
 * mvp may be NULL (identity). */
sr_status sr_batch_add_scene(sr_batch* b, uint32_t width, uint32_t height, const sr_scene_view* scene,
                             const float* mvp, uint32_t* index);
/* Appends `count` synthetic scenes, scene_index p->scene_index + i. */
sr_status sr_batch_add_synth(sr_batch* b, const sr_synth_params* p, uint32_t count, uint32_t* first_index);
sr_status sr_batch_commit(sr_batch* b);
sr_status sr_batch_set_mvp(sr_batch* b, uint32_t index, const float m[16]);
sr_status sr_batch_render(sr_batch* b, const sr_batch_render_opts* opts, void* stream);
/* sr_batch_render in two halves for hosts that keep several batches in
 * flight: enqueue returns once the frame is queued on `stream` (it needs
 * record_capacity >= 0, so nothing waits mid-frame); query reports whether
 * the frame has finished on the device; finish waits for it, checks for
 * overflow and, with refit_on_overflow, reruns it with exact sizing.  One
 * frame per batch may be in flight. */
sr_status sr_batch_enqueue(sr_batch* b, const sr_batch_render_opts* opts, void* stream);
sr_status sr_batch_query(sr_batch* b, int* done);
sr_status sr_batch_finish(sr_batch* b);
sr_status sr_batch_get_image(sr_batch* b, uint32_t index, void* rgba_out, int out_is_device, void* stream);
sr_status sr_batch_info(const sr_batch* b, uint32_t index, uint32_t* width, uint32_t* height);
sr_status sr_batch_get_stats(const sr_batch* b, sr_batch_stats* out);
sr_status sr_batch_clear(sr_batch* b);
void sr_batch_destroy(sr_batch* b);

/* Launch shapes of the tunable kernels (identical images for every choice). */
typedef struct sr_tuning {
    uint32_t struct_size;
    int32_t  sort_items;      /* keys per thread of a sort tile: 8, 12 (default) or 16 */
    int32_t  resolve_warps;   /* warps per resolve CTA: 8 (default) or 16 */
    int32_t  wind_items;      /* records per thread of a winding tile: 4 or 8 (default) */
    int32_t  sort_kind;       /* 0: per-path segmented sort (default), 1: radix sort of the whole array */
} sr_tuning;

sr_status sr_set_tuning(sr_ctx* c, const sr_tuning* t);
sr_status sr_batch_set_tuning(sr_batch* b, const sr_tuning* t);
sr_status sr_batch_get_tuning(const sr_batch* b, sr_tuning* t);
/* The batch's size class: "m<mode>/s<side>/r<log2 records>", side the
 * largest canvas side rounded up to a power of two (256, 512, 1024, 2048,
 * ...).  Needs a rendered frame (for the record count). */
sr_status sr_batch_tuning_class(sr_batch* b, char* buf, size_t len);
/* Picks the tuning of the batch's size class: from the JSON cache file
 * cache_path (may be NULL) when it holds the class and force is 0,
 * otherwise by timing frames of this batch for every value of each knob in
 * turn (the others held), keeping the fastest, and storing the choice in
 * the cache.  The batch keeps the chosen tuning. */
sr_status sr_batch_autotune(sr_batch* b, const char* cache_path, int force, sr_tuning* chosen, void* stream);

/* ------------------------------------------------------------------ */
/* Learned buffer sizing (replaces the count read-back of              */
/* scanline_rasterizer.cpp:337-358 and pre-sizes the fragment buffers   */
/* of :578-584; no reference counterpart for the network itself).       */
/* ------------------------------------------------------------------ */

/* A 6 -> 64 -> 64 -> 2 GELU network that predicts, per path, log(1 + its
 * intersection records) and log(1 + its draw records) from 6 features of
 * its control points.  Weights are BF16 with an FP32 master copy;
 * arithmetic is FP32.  Training (Adam) and inference run on the GPU.
 * Feature row of a path (all log1p except the last):
 *   segments, clipped bbox width, clipped bbox height (cells),
 *   control-polygon length (cells), sum |turn angle| (turns),
 *   cubic fraction.
 * The normaliser maps features and targets to standard units:
 *   norm = x_mean[6], x_inv_std[6], y_mean[2], y_std[2]. */
#define SR_SIZER_FEATURES 6
#define SR_SIZER_OUTPUTS 2
#define SR_SIZER_PARAMS 4738
#define SR_SIZER_NORM 16
typedef struct sr_sizer sr_sizer;

typedef struct sr_sizer_train_opts {
    uint32_t struct_size;
    uint32_t batch;      /* minibatch size (default 4096) */
    uint32_t epochs;     /* passes over the data (default 1) */
    uint32_t shuffle;    /* reshuffle every epoch (default 1) */
    float    lr;         /* Adam learning rate (default 1e-3) */
    float    beta1, beta2, eps;   /* defaults 0.9, 0.999, 1e-8 */
    uint64_t seed;       /* shuffle seed */
} sr_sizer_train_opts;

/* Weights drawn from a seeded uniform of variance 1/fan_in, zero biases,
 * identity normaliser, zero Adam state. */
sr_status sr_sizer_create(int device, uint64_t seed, sr_sizer** out);
void sr_sizer_destroy(sr_sizer* s);
sr_status sr_sizer_set_norm(sr_sizer* s, const float norm[SR_SIZER_NORM]);
/* Checkpoint: FP32 parameters, Adam moments, normaliser and step count
 * (any pointer may be NULL to skip that part). */
sr_status sr_sizer_get_state(const sr_sizer* s, float* params, float* adam_m, float* adam_v,
                             float norm[SR_SIZER_NORM], int64_t* step);
sr_status sr_sizer_set_state(sr_sizer* s, const float* params, const float* adam_m, const float* adam_v,
                             const float norm[SR_SIZER_NORM], int64_t step);
/* Mean squared error (standard units, over n rows and both outputs) and
 * its gradient with respect to the parameters, at the current weights.
 * d_x[n][6], d_t[n][2] are device arrays; h_grad[SR_SIZER_PARAMS] host. */
sr_status sr_sizer_loss_grad(sr_sizer* s, const float* d_x, const float* d_t, uint32_t n, float* h_grad,
                             float* h_loss);
/* Adam training on device rows (d_x, d_t); h_loss (optional) receives the
 * mean squared error of the last epoch. */
sr_status sr_sizer_train(sr_sizer* s, const float* d_x, const float* d_t, uint32_t n,
                         const sr_sizer_train_opts* opts, float* h_loss, void* stream);
/* d_y[n][2] = predicted log(1 + records), log(1 + draw records). */
sr_status sr_sizer_predict(const sr_sizer* s, const float* d_x, uint32_t n, float* d_y, void* stream);

/* Per-path features of a committed batch under its current transforms:
 * d_feats[n_paths][6] (device). */
sr_status sr_batch_path_features(sr_batch* b, float* d_feats, void* stream);
/* Renders the batch once with exact sizing, counting records and draw
 * records per path: d_labels[n_paths][2] = log(1 + records),
 * log(1 + draw records) (device).  The images are those of a plain render. */
sr_status sr_batch_path_labels(sr_batch* b, float* d_labels, void* stream);

/* Margins in log units.  A path's allotment is ceil(exp(y + path margin) - 1)
 * for its predicted y = log(1 + count); allotments are what the exact count
 * pass judges path by path.  The frame capacities sum the same expression
 * with the frame margins, which can be much smaller: errors of many paths
 * average out. */
typedef struct sr_sizing_margins {
    uint32_t struct_size;
    float path_records, path_draws;
    float frame_records, frame_draws;
} sr_sizing_margins;

typedef struct sr_sizing_plan {
    int64_t  records;        /* record capacity of the frame */
    int64_t  draws;          /* draw-record capacity (at most 2 x records) */
    int64_t  path_records;   /* sums of the per-path allotments */
    int64_t  path_draws;
    uint64_t device_bytes;   /* device memory of the batch with the frame capacities */
} sr_sizing_plan;

/* Sizes the next frame from the network: features, prediction, per-path
 * allotments and frame capacities.  Pass plan.records / plan.draws as the
 * render's capacities.  scene_caps (optional, [n_scenes][2] host) gets each
 * scene's record and draw capacity.  One host wait. */
sr_status sr_batch_plan(sr_batch* b, const sr_sizer* s, const sr_sizing_margins* margins, sr_sizing_plan* plan,
                        int64_t* scene_caps, void* stream);
/* path_begin[n_scenes + 1]: the first path of each scene in the batch's
 * path order (the rows of sr_batch_path_features / _labels). */
sr_status sr_batch_path_ranges(const sr_batch* b, uint32_t* path_begin);

typedef struct sr_sizing_judge {
    uint32_t paths;              /* paths in the batch */
    uint32_t paths_over_records; /* paths whose exact records exceed their allotment */
    uint32_t paths_over_draws;   /* likewise for draw records */
    uint32_t reserved;
    int64_t  records;            /* exact totals */
    int64_t  draws;
} sr_sizing_judge;

/* Runs the exact count pass (a render with exact sizing and per-path
 * counters) and compares every path with the allotment of the last
 * sr_batch_plan. */
sr_status sr_batch_judge(sr_batch* b, sr_sizing_judge* out, void* stream);

/* Device bytes the batch holds when rendered with capacities (records,
 * draws); draws <= 0 means 2 x records. */
sr_status sr_batch_frame_bytes(sr_batch* b, int64_t records, int64_t draws, uint64_t* bytes);
/* Frees the batch's record- and draw-sized buffers (scenes and images stay;
 * the next frame reallocates what it needs) and drops its captured graph. */
sr_status sr_batch_release(sr_batch* b);
/* Device bytes the batch holds now. */
sr_status sr_batch_held_bytes(const sr_batch* b, uint64_t* bytes);
/* Grows b's device buffers to at least the sizes model's hold (no frame of
 * b in flight).  A batch whose frame outgrows its buffers reallocates them
 * before it starts, behind a device-wide wait; a server grows its idle
 * slots like its largest one so that this happens once, not per slot.
 * When a buffer moves, b's images and plan are dropped and its next frame
 * uploads its scenes again. */
sr_status sr_batch_reserve_like(sr_batch* b, const sr_batch* model);

/* ------------------------------------------------------------------ */
/* Continuous-batching render server (no reference counterpart).       */
/* ------------------------------------------------------------------ */

/* Requests (a scene, its canvas and transform) are queued by any thread.
 * One scheduler thread keeps up to `slots` batches in flight, each on its
 * own stream: whenever a slot is free it takes the oldest waiting requests
 * (at most max_batch_scenes), uploads them as one batch, sizes the frame
 * with the sizing network and enqueues it without waiting, so a batch is
 * assembled and uploaded while others render.  Admission keeps the device
 * bytes of the batches in flight plus the finished, not yet collected
 * images under memory_budget, using the predicted sizes; a frame whose
 * records exceed the prediction is rerun with exact sizing, so every
 * image equals the same scene rendered alone.  Without a sizer each batch
 * is rendered with exact sizing (the scheduler waits for its count) and
 * admission counts scenes only. */
typedef struct sr_server sr_server;

typedef struct sr_server_opts {
    uint32_t struct_size;
    int32_t  mode;                /* SR_MODE_* */
    int32_t  device;
    uint32_t slots;               /* batches in flight (default 2) */
    uint32_t max_batch_scenes;    /* scenes per batch (default 64) */
    uint32_t reserved;
    uint64_t memory_budget;       /* bytes (default 120e9) */
    sr_sizing_margins margins;    /* used with a sizer */
} sr_server_opts;

typedef struct sr_request_info {
    double   submit_s;            /* seconds since the server started */
    double   admit_s;             /* the request's batch was enqueued */
    double   done_s;              /* its image is ready */
    uint64_t predicted_bytes;     /* the request's share of its batch */
    uint32_t batch_scenes;        /* scenes in its batch */
    uint32_t refit;               /* its batch overflowed and was rerun exactly */
    int32_t  status;              /* sr_status of its render */
    uint32_t reserved;
} sr_request_info;

typedef struct sr_server_stats {
    uint64_t submitted, completed, batches;
    uint64_t overflows, refits;
    uint64_t budget_waits;        /* admissions deferred by the memory budget */
    uint64_t peak_bytes;          /* largest admitted total */
    uint64_t rejected;            /* requests larger than the whole budget */
} sr_server_stats;

/* sizer may be NULL (exact sizing); it must outlive the server. */
sr_status sr_server_create(const sr_server_opts* opts, const sr_sizer* sizer, sr_server** out);
/* Copies the scene and queues it; thread-safe.  mvp may be NULL (identity). */
sr_status sr_server_submit(sr_server* s, uint32_t width, uint32_t height, const sr_scene_view* scene,
                           const float* mvp, uint64_t* ticket);
/* Waits up to timeout_ms (< 0: forever) for the request, copies its image
 * (width x height RGBA8) to rgba_out (host or device; NULL drops it) and
 * forgets the request.  SR_ERR_TIMEOUT leaves it pending.  Thread-safe. */
sr_status sr_server_wait(sr_server* s, uint64_t ticket, void* rgba_out, int out_is_device, sr_request_info* info,
                         int64_t timeout_ms);
sr_status sr_server_get_stats(sr_server* s, sr_server_stats* out);
/* Stops the scheduler after the queued requests finish. */
void sr_server_destroy(sr_server* s);

/* Admission rule of the server (host logic, exposed for tests): the
 * number of requests, taken in order from req_bytes[0..n), whose bytes fit
 * with held_bytes under budget, at most max_take.  When nothing is held the
 * first request is taken if it fits the budget alone.  *rejected is set
 * when the first request cannot fit even an empty budget. */
uint32_t sr_admission_take(const uint64_t* req_bytes, uint32_t n, uint64_t held_bytes, uint64_t budget,
                           uint32_t max_take, int* rejected);

/* Plain device memory for hosts without a CUDA binding of their own. */
void* sr_device_alloc(int device, size_t bytes);
void sr_device_free(void* p);
/* Synchronous copy between any host and device addresses. */
sr_status sr_memcpy(void* dst, const void* src, size_t bytes);

/* ------------------------------------------------------------------ */
/* Scene sources: synthetic generator and RVG loader (host only).      */
/* ------------------------------------------------------------------ */

/* A scene owned by the library (host memory). */
typedef struct sr_scene_buf sr_scene_buf;

/* Synthetic scene parameters.  preset 0: closed star paths of cubics;
 * preset 1: mixed cubic/quadric/line paths with even-odd paths,
 * figure-eights and full-canvas backgrounds; preset 2: scene `scene_index`
 * of a batch of uneven scenes (square side uniform over 256..2048, path
 * count lognormal with median 200, paths as preset 1).  Fields left 0 take
 * the preset's default. */
struct sr_synth_params {
    uint32_t struct_size;
    int32_t  preset;
    uint64_t seed;
    uint32_t scene_index;   /* independent stream per scene of a batch */
    uint32_t width, height;
    uint32_t n_paths;
};

sr_status sr_synth_scene(const sr_synth_params* p, sr_scene_buf** out);

/* Parses an .rvg file the way RVG::load does (core/vg/rvg.cpp:9-255):
 * M/L/C/Z/fL commands, nzfill/ofill, solid rgb/rgba paint, the last open
 * contour closed by a line; other elements are skipped. */
sr_status sr_rvg_load(const char* path, sr_scene_buf** out, float viewport[4]);

/* The same reader completed where RVG::load stops (rvg.cpp:160-169,
 * :234-251): 'A' segments become SR_CURVE_ARC curves and 'Q' segments
 * quadrics; linear and radial gradient paints are read (see sr_paint). */
sr_status sr_rvg_load_full(const char* path, sr_scene_buf** out, float viewport[4]);

/* The gradient paints a scene read by sr_rvg_load_full refers to (*n = 0
 * for other scenes); valid until sr_scene_buf_free. */
sr_status sr_scene_buf_paints(const sr_scene_buf* buf, const sr_paint** paints, uint32_t* n);

/* Points `view` at the arrays of `buf` (valid until sr_scene_buf_free). */
sr_status sr_scene_buf_view(const sr_scene_buf* buf, sr_scene_view* view);
/* Canvas size the scene was made for: wh[0] = width, wh[1] = height. */
sr_status sr_scene_buf_size(const sr_scene_buf* buf, uint32_t wh[2]);
void sr_scene_buf_free(sr_scene_buf* buf);

/* ------------------------------------------------------------------ */
/* Image output (host only).  The reference presents its frame through */
/* a swapchain (core/scanline/scanline_rasterizer.cpp:610-695); headless */
/* the frame is an RGBA8 host buffer (sr_render to host memory), which  */
/* this writes to a file.                                               */
/* ------------------------------------------------------------------ */
typedef enum sr_image_format {
    SR_IMAGE_PNG = 0,   /* truecolour + alpha, stored (uncompressed) deflate */
    SR_IMAGE_PPM = 1,   /* binary P6, RGB (alpha dropped)                    */
    SR_IMAGE_PAM = 2    /* P7 RGB_ALPHA                                       */
} sr_image_format;

/* Writes width x height RGBA8 pixels (row 0 first, 4 x width bytes a row)
 * to `path`.  Framebuffer row y is scene row y (no vertical flip). */
sr_status sr_write_image(const char* path, const uint8_t* rgba, uint32_t width, uint32_t height, int format);

/* Page-locked host memory (cudaMallocHost) for full-bandwidth copies of
 * scenes and frames; NULL on failure. */
void* sr_host_alloc(size_t bytes);
void sr_host_free(void* p);

#ifdef __cplusplus
}
#endif

#endif /* SR_H_ */
