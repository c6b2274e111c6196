// api.cu — device state, per-frame sequencing and the C ABI of sr.h.
//
// ScanlineVGRasterizer::drawFrame (scanline_rasterizer.cpp:282-696) submits
// eleven compute dispatches with three blocking host read-backs, then draws
// the list through the graphics queue.  Here a frame of a set of scenes is
//   transform -> count -> chain order -> offset scan -> [read N] ->
//   chains -> merge -> fragments -> sort -> winding/mark/emit ->
//   row sort -> resolve
// on the caller's stream.  The read of N is the only mid-frame host wait,
// and only when the record buffers are sized exactly; with a given record
// capacity (learned sizing, or the previous frame's count) the frame
// enqueues without waiting, an overflow is detected on the device, and the
// frame can be captured as a CUDA graph.  A single-scene context is a
// one-scene batch.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sr.h"
#include "kernels.h"
#include "synth.h"

namespace {

thread_local std::string g_err;

sr_status fail(sr_status s, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
sr_status fail(sr_status s, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return s;
}

#define CUDA_TRY(expr)                                                                        \
    do {                                                                                      \
        cudaError_t e_ = (expr);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            sr_status st_ = (e_ == cudaErrorMemoryAllocation) ? SR_ERR_OOM : SR_ERR_CUDA;      \
            return fail(st_, "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                            \
        }                                                                                     \
    } while (0)

#define SR_TRY(expr)                      \
    do {                                  \
        sr_status s_ = (expr);            \
        if (s_ != SR_OK) return s_;       \
    } while (0)

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    template <typename T> T* as() const { return static_cast<T*>(p); }
};

// Grows b to hold `bytes`, with `slack` (a quarter by default) to spare.
cudaError_t ensure(DevBuf& b, size_t bytes, bool slack = true) {
    if (bytes <= b.cap && b.p) return cudaSuccess;
    if (b.p) {
        cudaFree(b.p);
        b.p = nullptr;
        b.cap = 0;
    }
    size_t want = std::max<size_t>(slack ? bytes + bytes / 4 : bytes, 256);
    want = (want + 255) & ~(size_t)255;
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
        b.p = nullptr;
        return e;
    }
    b.cap = want;
    return cudaSuccess;
}

void release(DevBuf& b) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
}

uint32_t bits_for(uint64_t v) {   // bits needed to hold values 0..v
    uint32_t b = 0;
    while (b < 64 && (v >> b) != 0) ++b;
    return b == 0 ? 1 : b;
}

enum Ctl : int {
    CTL_STATUS = 0,
    CTL_SCAN_COUNTER = 1,
    CTL_WIND_COUNTER = 2,
    CTL_NDRAW = 3,     // merged fragments + spans of the frame
    CTL_CHAINS = 4,    // chain counter
    CTL_LONG = 8,      // long-piece counter
    CTL_QUEUE = 9,     // chain work-queue counter
    CTL_WIDE = 10,     // chains solved by a whole warp
    CTL_WIDE_QUEUE = 11,    // their work-queue counter
    CTL_WIDE_CURVES = 12,   // curves with such a chain
    CTL_ROW_SCAN = 13,      // row-start scan's tile counter
    CTL_WORDS = 16,
};

std::atomic<uint64_t> g_launches{0};

}  // namespace

namespace sr {
sr_status report_error(sr_status s, const char* msg) { return fail(s, "%s", msg); }
void count_launches(uint32_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
static std::atomic<uint32_t> g_spin_limit{kSpinLimitDefault};
uint32_t spin_limit() { return g_spin_limit.load(std::memory_order_relaxed); }
uint64_t launches_so_far() { return g_launches.load(std::memory_order_relaxed); }
}  // namespace sr

enum Stage : int {
    ST_TRANSFORM = 0, ST_COUNT, ST_SCAN, ST_CHAINS, ST_MERGE, ST_FRAGMENT, ST_SORT, ST_WINDING, ST_ROWSORT,
    ST_RESOLVE, ST_WIDE, ST_COUNT_ALL
};

static sr_status check_status_word(uint32_t s) {
    if (s == 0) return SR_OK;
    if (s & sr::ERR_LOOKBACK_TIMEOUT) return fail(SR_ERR_TIMEOUT, "device look-back wait timed out (status 0x%x)", s);
    if (s & sr::ERR_COPY_TIMEOUT) return fail(SR_ERR_TIMEOUT, "device bulk-copy wait timed out (status 0x%x)", s);
    if (s & sr::ERR_CAPACITY) return fail(SR_ERR_OVERFLOW_REFIT, "record capacity exceeded (status 0x%x)", s);
    return fail(SR_ERR_INTERNAL, "device consistency check failed (status 0x%x)", s);
}

// Host copy of a set of scenes, concatenated in the flattened layout.
struct HostScenes {
    std::vector<float> pos;
    std::vector<uint32_t> pos_path, curve_pos, curve_type, curve_path, fill_rule, fill_info, path_scene;
    std::vector<sr::SceneInfo> info;

    // keeps the vectors' storage: a batch re-formed for every frame (the
    // server's) reuses host pages that are already mapped
    void clear() {
        pos.clear();
        for (auto* v : {&pos_path, &curve_pos, &curve_type, &curve_path, &fill_rule, &fill_info, &path_scene}) v->clear();
        info.clear();
    }
    uint32_t n_points() const { return (uint32_t)pos_path.size(); }
    uint32_t n_curves() const { return (uint32_t)curve_type.size(); }
    uint32_t n_paths() const { return (uint32_t)fill_rule.size(); }
};

static const float kIdentity[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};

// Validates a caller's scene (the checks of sr_load_scene).
static sr_status validate_scene(const sr_scene_view* s) {
    const uint32_t V = s->n_points, C = s->n_curves, P = s->n_paths;
    if ((V && (!s->position || !s->pos_path_idx)) ||
        (C && (!s->curve_pos_map || !s->curve_type || !s->curve_path_idx)) || (P && (!s->fill_rule || !s->fill_info)))
        return fail(SR_ERR_INVALID_ARG, "scene array missing");
    if (C > (1u << 27) || V > (1u << 29) || P > (1u << 26)) return fail(SR_ERR_INVALID_ARG, "scene too large");
    for (uint32_t i = 0; i < C; ++i) {
        uint32_t t = s->curve_type[i];
        if (t != SR_CURVE_LINE && t != SR_CURVE_QUADRIC && t != SR_CURVE_CUBIC && t != SR_CURVE_ARC)
            return fail(SR_ERR_INVALID_ARG, "curve %u: unsupported type 0x%x", i, t);
        const uint32_t slots = t == SR_CURVE_ARC ? 4u : (t & 7u);
        if ((uint64_t)s->curve_pos_map[i] + slots > V)
            return fail(SR_ERR_INVALID_ARG, "curve %u: control points out of range", i);
        if (t == SR_CURVE_ARC) {
            const float* w = s->position + 2 * ((size_t)s->curve_pos_map[i] + 3);
            if (!(w[0] > -1.0f) || w[0] != w[1])
                return fail(SR_ERR_INVALID_ARG, "curve %u: arc weight must be (w, w) with w > -1", i);
        }
        if (s->curve_path_idx[i] >= P) return fail(SR_ERR_INVALID_ARG, "curve %u: path index out of range", i);
        if (i > 0 && s->curve_path_idx[i] < s->curve_path_idx[i - 1])
            return fail(SR_ERR_INVALID_ARG, "curves must be grouped by path in path order");
    }
    for (uint32_t i = 0; i < V; ++i) {
        if (s->pos_path_idx[i] >= P) return fail(SR_ERR_INVALID_ARG, "point %u: path index out of range", i);
        if (!std::isfinite(s->position[2 * (size_t)i]) || !std::isfinite(s->position[2 * (size_t)i + 1]))
            return fail(SR_ERR_INVALID_ARG, "point %u: coordinate is not finite", i);
    }
    for (uint32_t i = 0; i < P; ++i)
        if (s->fill_rule[i] > 1u) return fail(SR_ERR_INVALID_ARG, "path %u: fill rule %u", i, s->fill_rule[i]);
    return SR_OK;
}

// A gradient paint for the resolve: the map from pixel centres to gradient
// space is the inverse of (the matrix's affine part) * xf, computed in
// double and rounded to float once (the oracle restates this function).
// A paint whose map cannot be inverted, or without stops, paints nothing.
static sr::DevPaint make_dev_paint(const sr_paint& p, const float* m) {
    sr::DevPaint d{};
    d.kind = p.kind == SR_PAINT_RADIAL ? 2 : 1;
    d.spread = p.spread == SR_SPREAD_REPEAT ? 1 : p.spread == SR_SPREAD_REFLECT ? 2 : 0;
    const double A0 = m[0], A1 = m[1], A2 = m[3], A3 = m[4], A4 = m[5], A5 = m[7];
    const double X0 = p.xf[0], X1 = p.xf[1], X2 = p.xf[2], X3 = p.xf[3], X4 = p.xf[4], X5 = p.xf[5];
    // gradient -> pixel
    const double F0 = A0 * X0 + A1 * X3, F1 = A0 * X1 + A1 * X4, F2 = (A0 * X2 + A1 * X5) + A2;
    const double F3 = A3 * X0 + A4 * X3, F4 = A3 * X1 + A4 * X4, F5 = (A3 * X2 + A4 * X5) + A5;
    const double det = F0 * F4 - F1 * F3;
    const uint32_t ns = p.n_stops > (uint32_t)sr::kMaxStops ? (uint32_t)sr::kMaxStops : p.n_stops;
    if (det == 0.0 || !std::isfinite(det)) return d;   // n_stops 0: transparent
    // pixel -> gradient
    const double G0 = F4 / det, G1 = -F1 / det, G3 = -F3 / det, G4 = F0 / det;
    const double G2 = -(G0 * F2 + G1 * F5), G5 = -(G3 * F2 + G4 * F5);
    if (d.kind == 1) {
        const double dx = (double)p.p1[0] - p.p0[0], dy = (double)p.p1[1] - p.p0[1];
        const double l2 = dx * dx + dy * dy;
        if (l2 > 0.0) {
            d.lin[0] = (float)((G0 * dx + G3 * dy) / l2);
            d.lin[1] = (float)((G1 * dx + G4 * dy) / l2);
            d.lin[2] = (float)(((G2 - p.p0[0]) * dx + (G5 - p.p0[1]) * dy) / l2);
        }
    } else {
        const double G[6] = {G0, G1, G2, G3, G4, G5};
        for (int k = 0; k < 6; ++k) d.m[k] = (float)G[k];
        const double dx = (double)p.p0[0] - p.p1[0], dy = (double)p.p0[1] - p.p1[1];
        d.fx = p.p1[0];
        d.fy = p.p1[1];
        d.dx = (float)dx;
        d.dy = (float)dy;
        d.A = (float)(dx * dx + dy * dy - (double)p.radius * p.radius);
    }
    d.opacity = p.opacity;
    d.n_stops = (int32_t)ns;
    for (uint32_t k = 0; k < ns; ++k) {
        d.off[k] = p.offset[k];
        for (int q = 0; q < 4; ++q) d.rgba[k][q] = p.rgba[k][q];
    }
    return d;
}

// Appends one validated scene to a host set.
static void append_scene(HostScenes& h, uint32_t w, uint32_t hgt, const sr_scene_view* s, const float* mvp) {
    const uint32_t pb = h.n_paths(), vb = h.n_points();
    sr::SceneInfo si{};
    si.W = (int32_t)w;
    si.H = (int32_t)hgt;
    si.path_begin = pb;
    si.path_end = pb + s->n_paths;
    std::memcpy(si.mvp, mvp ? mvp : kIdentity, sizeof si.mvp);
    const uint32_t sidx = (uint32_t)h.info.size();
    h.info.push_back(si);
    if (s->n_points) h.pos.insert(h.pos.end(), s->position, s->position + 2 * (size_t)s->n_points);
    for (uint32_t i = 0; i < s->n_points; ++i) h.pos_path.push_back(s->pos_path_idx[i] + pb);
    for (uint32_t i = 0; i < s->n_curves; ++i) {
        h.curve_pos.push_back(s->curve_pos_map[i] + vb);
        h.curve_type.push_back(s->curve_type[i]);
        h.curve_path.push_back(s->curve_path_idx[i] + pb);
    }
    if (s->n_paths) {
        h.fill_rule.insert(h.fill_rule.end(), s->fill_rule, s->fill_rule + s->n_paths);
        h.fill_info.insert(h.fill_info.end(), s->fill_info, s->fill_info + s->n_paths);
        h.path_scene.insert(h.path_scene.end(), s->n_paths, sidx);
    }
}

// --------------------------------------------------------------------------
// The device pipeline of one set of scenes.
struct Pipeline {
    int device = 0, sm_count = 148;
    int32_t mode = SR_MODE_PIXEL, F = 1;
    uint32_t flags = 0;
    bool loaded = false;
    bool arcs = false;   // the scene set has SR_CURVE_ARC curves
    // gradient paints (single-scene contexts): as set, and for the resolve
    std::vector<sr_paint> paints_h;
    DevBuf paints_d;
    DevBuf aa_acc;   // multisampling: per-pixel channel sums (ushort4)
    uint32_t n_paints = 0;
    sr_tuning tune{sizeof(sr_tuning), 12, 8, 8, 0};
    // segmented sort of this frame: merge rounds (-1: radix sort instead) and
    // the largest segment the tables accept without flagging an overflow
    int seg_levels = 0;
    uint32_t seg_check = 0;
    // scenes
    uint32_t S = 0, V = 0, C = 0, P = 0;
    int32_t Wmax = 1, Hmax = 1;
    uint32_t total_rows = 0, res_ctas = 0;
    uint64_t total_pixels = 0;
    std::vector<sr::SceneInfo> info;
    std::vector<uint32_t> cta_base;
    std::vector<uint8_t> cta_narrow;
    bool any_narrow = false;
    DevBuf pos, pos_path, curve_pos, curve_type, curve_path, fill_rule, fill_info, path_scene, scenes_d, cta_base_d;
    DevBuf cta_narrow_d;
    // frame
    DevBuf tpos, path_visible, cut, count, offs, ctl, scan_status, pieces, chain_lists, chain_sort_scratch, long_list;
    DevBuf curve_wide, wide_curves;
    DevBuf cbuf, rec, keys, keys_alt, wnp, skeys, svals, vals_alt, sort_scratch, wind_status, draw, draw_row, totals;
    DevBuf rkeys, rvals, rkeys_alt, rvals_alt, row_sort_scratch, row_start, seg_cut, row_count, row_px, row_scan, image;
    DevBuf d_fkey, d_fwn, d_fleft, d_wscan, d_fflag, d_sflag, d_skey;
    // learned sizing: per-path curve ranges, draw counters, features,
    // predictions, allotments and their sums
    DevBuf path_first, path_draw, feats, preds, allot, plan_tot, judge_out, seg_scratch, seg_tiles;
    bool path_first_valid = false, count_paths = false, planned = false;
    unsigned long long* h_plan_ptr = nullptr;   // pinned plan totals
    size_t h_plan_words = 0;
    // Host-to-device uploads of tables and of small scene sets go through one
    // pinned staging buffer on a stream of their own: one wait instead of a
    // synchronous call per array.
    unsigned char* h_stage = nullptr;
    size_t h_stage_cap = 0, h_stage_used = 0;
    cudaStream_t up_stream = nullptr;
    struct StagedCopy {
        void* dst;
        size_t off, bytes;
    };
    std::vector<StagedCopy> staged;
    // host scalars (pinned): N, status; fragments, spans
    uint32_t* h_u32 = nullptr;
    uint64_t* h_u64 = nullptr;
    // results
    sr_stats stats{};
    int64_t last_N = 0, last_O = 0, last_cap = 0, last_dcap = 0;
    uint32_t last_largest = 0;   // records of the frame's largest sort segment
    bool stages_valid = false;
    bool last_segsort = false;   // the last frame sorted its records per path (segsort.cu)
    // profiling
    cudaEvent_t ev[2 * ST_COUNT_ALL] = {};
    bool ev_pending = false, capturing = false;
    cudaStream_t cur = nullptr;
    // second stream of a frame (lowest priority): the chains other than the
    // wide ones, and their curves' merge and fragments, run on it beside the
    // wide chains on the frame's stream (forked and joined by events)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_merged = nullptr, ev_join = nullptr;

    ~Pipeline() {
        DevBuf* all[] = {&pos, &pos_path, &curve_pos, &curve_type, &curve_path, &fill_rule, &fill_info, &path_scene,
                         &scenes_d, &cta_base_d, &tpos, &path_visible, &cut, &count, &offs, &ctl, &scan_status,
                         &pieces, &chain_lists, &chain_sort_scratch, &long_list, &cbuf, &rec, &keys, &keys_alt,
                         &wnp, &skeys, &svals, &vals_alt, &sort_scratch, &wind_status, &draw, &draw_row, &totals,
                         &rkeys, &rvals, &rkeys_alt, &rvals_alt, &row_sort_scratch, &row_start, &seg_cut, &row_count, &row_px,
                         &row_scan, &image, &d_fkey, &d_fwn, &d_fleft, &d_wscan, &d_fflag, &d_sflag, &d_skey, &path_first, &path_draw,
                         &feats, &preds, &allot, &plan_tot, &judge_out, &seg_scratch, &seg_tiles, &curve_wide,
                         &wide_curves, &cta_narrow_d, &paints_d, &aa_acc};
        for (DevBuf* b : all) release(*b);
        for (cudaEvent_t e : {ev_fork, ev_merged, ev_join})
            if (e) cudaEventDestroy(e);
        if (side) cudaStreamDestroy(side);
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
        if (h_u32) cudaFreeHost(h_u32);
        if (h_u64) cudaFreeHost(h_u64);
        if (h_plan_ptr) cudaFreeHost(h_plan_ptr);
        if (h_stage) cudaFreeHost(h_stage);
        if (up_stream) cudaStreamDestroy(up_stream);
    }

    // Grows the pinned staging buffer to `bytes` (nothing staged).
    sr_status stage_reserve(size_t bytes) {
        if (bytes <= h_stage_cap) return SR_OK;
        if (h_stage) cudaFreeHost(h_stage);
        h_stage = nullptr;
        h_stage_cap = 0;
        const size_t want = std::max<size_t>(bytes + bytes / 2, 1 << 16);
        CUDA_TRY(cudaMallocHost(&h_stage, want));
        h_stage_cap = want;
        return SR_OK;
    }
    // Queues a copy of src into dst through the staging buffer (room was
    // reserved by the caller); stage_flush issues and waits for them.
    void stage(void* dst, const void* src, size_t bytes) {
        if (!bytes) return;
        std::memcpy(h_stage + h_stage_used, src, bytes);
        staged.push_back({dst, h_stage_used, bytes});
        h_stage_used += (bytes + 255) & ~(size_t)255;
    }
    sr_status stage_flush() {
        if (!up_stream) CUDA_TRY(cudaStreamCreateWithFlags(&up_stream, cudaStreamNonBlocking));
        for (const StagedCopy& c : staged)
            CUDA_TRY(cudaMemcpyAsync(c.dst, h_stage + c.off, c.bytes, cudaMemcpyHostToDevice, up_stream));
        staged.clear();
        h_stage_used = 0;
        CUDA_TRY(cudaStreamSynchronize(up_stream));
        return SR_OK;
    }
    static size_t staged_size(size_t bytes) { return (bytes + 255) & ~(size_t)255; }
    static constexpr size_t kStagedUploadMax = 1u << 20;

    sr_status init(int dev, int32_t m, uint32_t fl) {
        device = dev;
        mode = m;
        F = m == SR_MODE_PIXEL ? 1 : 2;
        flags = fl;
        CUDA_TRY(cudaSetDevice(dev));
        cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev);
        if (sm_count <= 0) sm_count = 148;
        CUDA_TRY(cudaMallocHost(&h_u32, sizeof(uint32_t) * 8));
        CUDA_TRY(cudaMallocHost(&h_u64, sizeof(uint64_t) * 4));
        CUDA_TRY(ensure(ctl, sizeof(uint32_t) * CTL_WORDS));
        CUDA_TRY(sr::geom_init());
        // the side stream takes the lowest priority: when both streams'
        // chain kernels become ready at once, the caller's stream, which
        // carries the wide chains (the frame's longest dependency), is
        // placed first
        int lo_prio = 0, hi_prio = 0;
        CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio));
        CUDA_TRY(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, lo_prio));
        for (cudaEvent_t* e : {&ev_fork, &ev_merged, &ev_join})
            CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
        return SR_OK;
    }

    void mark(int stage, bool end, cudaStream_t on = nullptr) {
        if (!(flags & SR_FLAG_PROFILE) || capturing) return;
        cudaEvent_t& e = ev[2 * stage + (end ? 1 : 0)];
        if (!e) cudaEventCreate(&e);
        cudaEventRecord(e, on ? on : cur);
    }

    sr::KeyLayout layout() const {
        sr::KeyLayout L;
        L.F = F;
        L.W = Wmax;
        L.H = Hmax;
        L.Hy = (Hmax + F - 1) / F;
        L.xbits = bits_for((uint64_t)((Wmax & ~1) / F + 2));
        L.rbits = bits_for((uint64_t)L.Hy);
        L.pbits = bits_for(P > 0 ? (uint64_t)(P - 1) : 0);
        return L;
    }

    sr::SceneTable table() const { return sr::SceneTable{scenes_d.as<sr::SceneInfo>(), path_scene.as<uint32_t>(), S}; }

    // Places the scenes' rows and framebuffers and uploads the scene table.
    sr_status upload_table(bool flush = true) {
        total_rows = 0;
        total_pixels = 0;
        res_ctas = 0;
        Wmax = 1;
        Hmax = 1;
        cta_base.assign(S + 1, 0);
        cta_narrow.clear();
        any_narrow = false;
        for (uint32_t s = 0; s < S; ++s) {
            sr::SceneInfo& si = info[s];
            si.rows = (uint32_t)((si.H + F - 1) / F);
            si.row_base = total_rows;
            si.image_off = total_pixels;
            total_rows += si.rows;
            total_pixels += (uint64_t)si.W * (uint64_t)si.H;
            Wmax = std::max(Wmax, si.W);
            Hmax = std::max(Hmax, si.H);
            cta_base[s] = res_ctas;
            uint32_t rpc = sr::resolve_rows_per_cta(si.W, tune.resolve_warps);
            res_ctas += (si.rows + rpc - 1) / rpc;
            cta_narrow.resize(res_ctas, rpc > 1 ? 1 : 0);
            any_narrow = any_narrow || rpc > 1;
        }
        cta_base[S] = res_ctas;
        CUDA_TRY(ensure(scenes_d, sizeof(sr::SceneInfo) * std::max<uint32_t>(S, 1)));
        CUDA_TRY(ensure(cta_base_d, sizeof(uint32_t) * (S + 1)));
        CUDA_TRY(ensure(image, 4 * std::max<uint64_t>(total_pixels, 1)));
        CUDA_TRY(ensure(cta_narrow_d, std::max<size_t>(res_ctas, 1)));
        if (!flush) return SR_OK;   // upload() stages the table with the scenes
        SR_TRY(stage_reserve(table_stage_bytes()));
        stage_table();
        return stage_flush();
    }
    size_t table_stage_bytes() const {
        return staged_size(sizeof(sr::SceneInfo) * S) + staged_size(sizeof(uint32_t) * (S + 1)) + staged_size(res_ctas);
    }
    void stage_table() {
        stage(scenes_d.p, info.data(), sizeof(sr::SceneInfo) * S);
        stage(cta_base_d.p, cta_base.data(), sizeof(uint32_t) * (S + 1));
        stage(cta_narrow_d.p, cta_narrow.data(), res_ctas);
    }

    sr_status upload(const HostScenes& h) {
        CUDA_TRY(cudaSetDevice(device));
        S = (uint32_t)h.info.size();
        V = h.n_points();
        C = h.n_curves();
        P = h.n_paths();
        if (C > (1u << 27) || V > (1u << 29) || P > (1u << 26)) return fail(SR_ERR_INVALID_ARG, "scene set too large");
        info = h.info;
        CUDA_TRY(ensure(pos, sizeof(float) * 2 * (size_t)std::max<uint32_t>(V, 1)));
        CUDA_TRY(ensure(pos_path, sizeof(uint32_t) * std::max<uint32_t>(V, 1)));
        CUDA_TRY(ensure(curve_pos, sizeof(uint32_t) * std::max<uint32_t>(C, 1)));
        CUDA_TRY(ensure(curve_type, sizeof(uint32_t) * std::max<uint32_t>(C, 1)));
        CUDA_TRY(ensure(curve_path, sizeof(uint32_t) * std::max<uint32_t>(C, 1)));
        CUDA_TRY(ensure(fill_rule, sizeof(uint32_t) * std::max<uint32_t>(P, 1)));
        CUDA_TRY(ensure(fill_info, sizeof(uint32_t) * std::max<uint32_t>(P, 1)));
        CUDA_TRY(ensure(path_scene, sizeof(uint32_t) * std::max<uint32_t>(P, 1)));
        arcs = std::find(h.curve_type.begin(), h.curve_type.end(), (uint32_t)SR_CURVE_ARC) != h.curve_type.end();
        SR_TRY(upload_table(false));
        const size_t need = staged_size(sizeof(float) * h.pos.size()) + staged_size(sizeof(uint32_t) * V) +
                            3 * staged_size(sizeof(uint32_t) * C) + 3 * staged_size(sizeof(uint32_t) * P) +
                            table_stage_bytes();
        if (need <= kStagedUploadMax) {
            // a small set (a serving batch): one stream, one wait
            SR_TRY(stage_reserve(need));
            stage(pos.p, h.pos.data(), sizeof(float) * h.pos.size());
            stage(pos_path.p, h.pos_path.data(), sizeof(uint32_t) * V);
            stage(curve_pos.p, h.curve_pos.data(), sizeof(uint32_t) * C);
            stage(curve_type.p, h.curve_type.data(), sizeof(uint32_t) * C);
            stage(curve_path.p, h.curve_path.data(), sizeof(uint32_t) * C);
            stage(fill_rule.p, h.fill_rule.data(), sizeof(uint32_t) * P);
            stage(fill_info.p, h.fill_info.data(), sizeof(uint32_t) * P);
            stage(path_scene.p, h.path_scene.data(), sizeof(uint32_t) * P);
        } else {
            // a large one goes straight from the host vectors: the extra host
            // copy into the staging buffer would cost more than it saves
            auto up = [](DevBuf& d, const void* src, size_t bytes) -> cudaError_t {
                return bytes ? cudaMemcpy(d.p, src, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
            };
            CUDA_TRY(up(pos, h.pos.data(), sizeof(float) * h.pos.size()));
            CUDA_TRY(up(pos_path, h.pos_path.data(), sizeof(uint32_t) * V));
            CUDA_TRY(up(curve_pos, h.curve_pos.data(), sizeof(uint32_t) * C));
            CUDA_TRY(up(curve_type, h.curve_type.data(), sizeof(uint32_t) * C));
            CUDA_TRY(up(curve_path, h.curve_path.data(), sizeof(uint32_t) * C));
            CUDA_TRY(up(fill_rule, h.fill_rule.data(), sizeof(uint32_t) * P));
            CUDA_TRY(up(fill_info, h.fill_info.data(), sizeof(uint32_t) * P));
            CUDA_TRY(up(path_scene, h.path_scene.data(), sizeof(uint32_t) * P));
            SR_TRY(stage_reserve(table_stage_bytes()));
        }
        stage_table();
        SR_TRY(stage_flush());
        loaded = true;
        stages_valid = false;
        path_first_valid = false;
        planned = false;
        return SR_OK;
    }

    // One scene straight from the caller's arrays (no host staging copy;
    // the copies run at pinned-memory speed when the caller's arrays are
    // pinned).
    sr_status upload_single(const sr_scene_view* s, int32_t W, int32_t H, const float* mvp) {
        CUDA_TRY(cudaSetDevice(device));
        S = 1;
        V = s->n_points;
        C = s->n_curves;
        P = s->n_paths;
        info.assign(1, sr::SceneInfo{});
        info[0].W = W;
        info[0].H = H;
        info[0].path_begin = 0;
        info[0].path_end = P;
        std::memcpy(info[0].mvp, mvp, sizeof info[0].mvp);
        CUDA_TRY(ensure(pos, sizeof(float) * 2 * (size_t)std::max<uint32_t>(V, 1)));
        CUDA_TRY(ensure(pos_path, sizeof(uint32_t) * std::max<uint32_t>(V, 1)));
        CUDA_TRY(ensure(curve_pos, sizeof(uint32_t) * std::max<uint32_t>(C, 1)));
        CUDA_TRY(ensure(curve_type, sizeof(uint32_t) * std::max<uint32_t>(C, 1)));
        CUDA_TRY(ensure(curve_path, sizeof(uint32_t) * std::max<uint32_t>(C, 1)));
        CUDA_TRY(ensure(fill_rule, sizeof(uint32_t) * std::max<uint32_t>(P, 1)));
        CUDA_TRY(ensure(fill_info, sizeof(uint32_t) * std::max<uint32_t>(P, 1)));
        CUDA_TRY(ensure(path_scene, sizeof(uint32_t) * std::max<uint32_t>(P, 1)));
        auto up = [](DevBuf& d, const void* src, size_t bytes) -> cudaError_t {
            return bytes ? cudaMemcpy(d.p, src, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
        };
        CUDA_TRY(up(pos, s->position, sizeof(float) * 2 * (size_t)V));
        CUDA_TRY(up(pos_path, s->pos_path_idx, sizeof(uint32_t) * V));
        CUDA_TRY(up(curve_pos, s->curve_pos_map, sizeof(uint32_t) * C));
        CUDA_TRY(up(curve_type, s->curve_type, sizeof(uint32_t) * C));
        CUDA_TRY(up(curve_path, s->curve_path_idx, sizeof(uint32_t) * C));
        CUDA_TRY(up(fill_rule, s->fill_rule, sizeof(uint32_t) * P));
        CUDA_TRY(up(fill_info, s->fill_info, sizeof(uint32_t) * P));
        CUDA_TRY(cudaMemset(path_scene.p, 0, sizeof(uint32_t) * std::max<uint32_t>(P, 1)));
        arcs = s->n_curves && std::find(s->curve_type, s->curve_type + s->n_curves, (uint32_t)SR_CURVE_ARC) !=
                                  s->curve_type + s->n_curves;
        SR_TRY(upload_table());
        loaded = true;
        stages_valid = false;
        path_first_valid = false;
        planned = false;
        return SR_OK;
    }

    sr::GeomArgs geom(int64_t cap) const {
        sr::GeomArgs g;
        g.n_curves = C;
        g.curve_type = curve_type.as<uint32_t>();
        g.curve_pos = curve_pos.as<uint32_t>();
        g.curve_path = curve_path.as<uint32_t>();
        g.tpos = tpos.as<float2>();
        g.path_visible = path_visible.as<int32_t>();
        g.W = Wmax;
        g.H = Hmax;
        g.F = F;
        g.pixel_mode = mode == SR_MODE_PIXEL;
        g.L = layout();
        g.st = table();
        g.rec_cap = cap;
        return g;
    }

    uint32_t list_cap() const { return sr::chain_list_capacity(std::max<uint32_t>(C, 1)); }

    sr::ChainWork chain_work() const {
        sr::ChainWork cw;
        uint32_t* ctlp = ctl.as<uint32_t>();
        uint32_t* cl = chain_lists.as<uint32_t>();
        const uint32_t lc = list_cap();
        cw.pieces = pieces.as<uint4>();
        cw.chain_items = cl;
        cw.chain_keys = cl + lc;
        cw.sorted_items = cl + 2 * (size_t)lc;
        cw.sorted_keys = cl + 3 * (size_t)lc;
        cw.list_cap = lc;
        cw.chain_count = ctlp + CTL_CHAINS;
        cw.chain_queue = ctlp + CTL_QUEUE;
        cw.wide_count = ctlp + CTL_WIDE;
        cw.wide_queue = ctlp + CTL_WIDE_QUEUE;
        cw.curve_wide = curve_wide.as<uint8_t>();
        cw.wide_curves = wide_curves.as<uint32_t>();
        cw.wide_curve_count = ctlp + CTL_WIDE_CURVES;
        cw.long_list = long_list.as<uint32_t>();
        cw.long_count = ctlp + CTL_LONG;
        return cw;
    }

    // Buffers of the stages before the record count is known.
    sr_status prepare_front() {
        CUDA_TRY(ensure(tpos, sizeof(float2) * std::max<uint32_t>(V, 1)));
        CUDA_TRY(ensure(path_visible, sizeof(int32_t) * std::max<uint32_t>(P, 1)));
        CUDA_TRY(ensure(cut, sizeof(float) * 5 * (size_t)std::max<uint32_t>(C, 1)));
        CUDA_TRY(ensure(count, sizeof(int32_t) * ((size_t)C + 1)));
        CUDA_TRY(ensure(offs, sizeof(int32_t) * ((size_t)C + 1)));
        CUDA_TRY(ensure(scan_status, sizeof(uint64_t) * sr::scan_status_words(C)));
        CUDA_TRY(ensure(pieces, sr::piece_table_bytes(std::max<uint32_t>(C, 1))));
        const uint32_t lc = list_cap();
        CUDA_TRY(ensure(chain_lists, sizeof(uint32_t) * 6 * (size_t)lc));
        CUDA_TRY(ensure(long_list, sizeof(uint32_t) * (size_t)lc));
        CUDA_TRY(ensure(curve_wide, std::max<size_t>(C, 1)));
        CUDA_TRY(ensure(wide_curves, sizeof(uint32_t) * std::max<size_t>(C, 1)));
        sr::SortPlan cp = sr::sort_plan(lc, sr::chain_key_bits(), ctl.as<uint32_t>() + CTL_CHAINS);
        CUDA_TRY(ensure(chain_sort_scratch, sr::sort_scratch_bytes(cp)));
        CUDA_TRY(ensure(totals, sizeof(uint64_t) * 4));
        CUDA_TRY(ensure(row_start, sizeof(int32_t) * ((size_t)total_rows + 1)));
        CUDA_TRY(ensure(seg_cut, sizeof(uint32_t) * std::max<size_t>(cut_words(), 1)));
        CUDA_TRY(ensure(row_count, sizeof(uint32_t) * std::max<size_t>(total_rows, 1)));
        CUDA_TRY(ensure(row_px, sizeof(unsigned long long) * std::max<size_t>(total_rows, 1)));
        CUDA_TRY(ensure(row_scan, sizeof(uint64_t) * sr::scan_status_words(total_rows)));
        if (segmented()) CUDA_TRY(ensure(seg_scratch, sr::segsort_scratch_bytes(std::max<uint32_t>(C, 1))));
        return SR_OK;
    }

    // Resolve segments per cell row (the widest scene's) and the words of
    // the per-segment cut table.
    uint32_t cut_segs() const { return (uint32_t)((Wmax + sr::kResolveSeg - 1) / sr::kResolveSeg); }
    size_t cut_words() const { return (size_t)total_rows * cut_segs(); }

    // The production sort is the per-path segmented sort unless the tuning
    // asks for the radix sort or the stages are kept (their sorted-index dump
    // needs the radix sort with record indices).
    bool segmented() const { return tune.sort_kind == 0 && !(flags & SR_FLAG_KEEP_STAGES) && C > 0; }
    static constexpr int kSegLevelsMax = 5;

    // Draw-record capacity: every record gives at most one merged fragment
    // and one span, so 2 x records always suffices.
    static int64_t draw_cap_for(int64_t cap, int64_t dcap) {
        return dcap > 0 ? dcap : 2 * std::max<int64_t>(cap, 1);
    }

    // Bytes each post-count buffer needs for `cap` records and `dcap` draw
    // records; fn(buffer, bytes) is called once per buffer.
    template <typename Fn>
    void post_count_buffers(int64_t cap, int64_t dcap, Fn&& fn) {
        const size_t n1 = (size_t)std::max<int64_t>(cap, 1);
        fn(cbuf, sizeof(int32_t) * n1);
        fn(rec, sizeof(int2) * n1);
        fn(keys, sizeof(uint64_t) * n1);
        fn(keys_alt, sizeof(uint64_t) * n1);
        fn(skeys, sizeof(uint64_t) * n1);
        // record indices and a separate winding-bit array only when the
        // stages are kept (sorted-index dump); otherwise the winding bits
        // ride in the keys
        const bool idx = (flags & SR_FLAG_KEEP_STAGES) != 0;
        fn(wnp, idx ? n1 : 0);
        fn(svals, idx ? sizeof(uint32_t) * n1 : 0);
        fn(vals_alt, idx ? sizeof(uint32_t) * n1 : 0);
        const sr::KeyLayout L = layout();
        fn(sort_scratch,
           sr::sort_scratch_bytes(sr::sort_plan(cap, L.pbits + L.rbits + L.xbits, nullptr, tune.sort_items)));
        fn(wind_status, sizeof(uint64_t) * sr::winding_status_words(cap, tune.wind_items));
        const size_t d1 = (size_t)draw_cap_for(cap, dcap);
        fn(draw, sizeof(int4) * d1);
        fn(draw_row, sizeof(uint32_t) * d1);
        fn(rkeys, sizeof(uint32_t) * d1);
        fn(rvals, sizeof(uint32_t) * d1);
        fn(rkeys_alt, sizeof(uint32_t) * d1);
        fn(rvals_alt, sizeof(uint32_t) * d1);
        fn(row_sort_scratch, sr::sort_scratch_bytes(sr::sort_plan((int64_t)d1, bits_for(total_rows), nullptr)));
        fn(seg_tiles, segmented() ? sr::segsort_tile_bytes(C, std::max<int64_t>(cap, 1)) : 0);
    }

    // Device bytes a frame of this scene set holds with capacities (cap,
    // dcap): scene arrays, per-frame arrays, post-count buffers and images,
    // each rounded as the allocator rounds it.
    uint64_t frame_bytes(int64_t cap, int64_t dcap) {
        uint64_t total = 0;
        auto add = [&](size_t b) {
            if (!b) return;
            size_t want = std::max<size_t>(b + b / 4, 256);
            total += (want + 255) & ~(size_t)255;
        };
        const size_t v1 = std::max<uint32_t>(V, 1), c1 = std::max<uint32_t>(C, 1), p1 = std::max<uint32_t>(P, 1);
        add(8 * v1); add(4 * v1);                                   // pos, pos_path
        add(4 * c1); add(4 * c1); add(4 * c1);                      // curve arrays
        add(4 * p1); add(4 * p1); add(4 * p1);                      // fill rule/info, path scene
        add(sizeof(sr::SceneInfo) * std::max<uint32_t>(S, 1)); add(4 * ((size_t)S + 1));
        add(4 * std::max<uint64_t>(total_pixels, 1));               // images
        add(8 * v1); add(4 * p1); add(20 * c1); add(4 * (c1 + 1)); add(4 * (c1 + 1));
        add(8 * sr::scan_status_words(C)); add(sr::piece_table_bytes((uint32_t)c1));
        const size_t lc = list_cap();
        add(4 * 6 * lc); add(4 * lc);
        add(sr::sort_scratch_bytes(sr::sort_plan((int64_t)lc, sr::chain_key_bits(), nullptr)));
        add(32); add(4 * ((size_t)total_rows + 1));
        post_count_buffers(cap, dcap, [&](DevBuf&, size_t b) { add(b); });
        return total;
    }

    // Frees the buffers sized by the record count (they are reallocated by
    // the next frame).
    void release_post_count() {
        post_count_buffers(0, 0, [](DevBuf& b, size_t) { release(b); });
        DevBuf* dbg[] = {&d_fkey, &d_fwn, &d_fleft, &d_wscan, &d_fflag, &d_sflag, &d_skey};
        for (DevBuf* b : dbg) release(*b);
        stages_valid = false;
    }

    // Grows every device buffer to at least m's capacity for the same
    // buffer (a second batch that will see frames like m's); the pinned
    // plan totals too.  True when a buffer moved.
    sr_status reserve_like(const Pipeline& m, bool* moved) {
        static DevBuf Pipeline::* const bufs[] = {
            &Pipeline::pos, &Pipeline::pos_path, &Pipeline::curve_pos, &Pipeline::curve_type,
            &Pipeline::curve_path, &Pipeline::fill_rule, &Pipeline::fill_info, &Pipeline::path_scene,
            &Pipeline::scenes_d, &Pipeline::cta_base_d, &Pipeline::tpos, &Pipeline::path_visible, &Pipeline::cut,
            &Pipeline::count, &Pipeline::offs, &Pipeline::ctl, &Pipeline::scan_status, &Pipeline::pieces,
            &Pipeline::chain_lists, &Pipeline::chain_sort_scratch, &Pipeline::long_list, &Pipeline::cbuf,
            &Pipeline::rec, &Pipeline::keys, &Pipeline::keys_alt, &Pipeline::wnp, &Pipeline::skeys,
            &Pipeline::svals, &Pipeline::vals_alt, &Pipeline::sort_scratch, &Pipeline::wind_status,
            &Pipeline::draw, &Pipeline::draw_row, &Pipeline::totals, &Pipeline::rkeys, &Pipeline::rvals,
            &Pipeline::rkeys_alt, &Pipeline::rvals_alt, &Pipeline::row_sort_scratch, &Pipeline::row_start,
            &Pipeline::seg_cut, &Pipeline::row_count, &Pipeline::row_px, &Pipeline::row_scan, &Pipeline::image,
            &Pipeline::path_first, &Pipeline::path_draw, &Pipeline::feats, &Pipeline::preds, &Pipeline::allot,
            &Pipeline::plan_tot, &Pipeline::judge_out, &Pipeline::seg_scratch, &Pipeline::seg_tiles,
            &Pipeline::curve_wide, &Pipeline::wide_curves, &Pipeline::cta_narrow_d};
        *moved = false;
        CUDA_TRY(cudaSetDevice(device));
        for (DevBuf Pipeline::* b : bufs) {
            DevBuf& mine = this->*b;
            const size_t want = (m.*b).cap;
            if (want > mine.cap) {
                *moved = true;   // before: a failed ensure has freed the old buffer too
                CUDA_TRY(ensure(mine, want, false));
            }
        }
        SR_TRY(stage_reserve(m.h_stage_cap));
        if (h_plan_words < m.h_plan_words) {
            if (h_plan_ptr) cudaFreeHost(h_plan_ptr);
            h_plan_ptr = nullptr;
            h_plan_words = 0;
            CUDA_TRY(cudaMallocHost(&h_plan_ptr, sizeof(unsigned long long) * m.h_plan_words));
            h_plan_words = m.h_plan_words;
        }
        return SR_OK;
    }

    // Device bytes currently held by this pipeline.
    uint64_t held_bytes() const {
        const DevBuf* all[] = {&pos, &pos_path, &curve_pos, &curve_type, &curve_path, &fill_rule, &fill_info,
                               &path_scene, &scenes_d, &cta_base_d, &tpos, &path_visible, &cut, &count, &offs,
                               &ctl, &scan_status, &pieces, &chain_lists, &chain_sort_scratch, &long_list, &cbuf,
                               &rec, &keys, &keys_alt, &wnp, &skeys, &svals, &vals_alt, &sort_scratch, &wind_status,
                               &draw, &draw_row, &totals, &rkeys, &rvals, &rkeys_alt, &rvals_alt,
                               &row_sort_scratch, &row_start, &seg_cut, &row_count, &row_px, &row_scan, &image, &d_fkey,
                               &d_fwn, &d_fleft,
                               &d_wscan,
                               &d_fflag, &d_sflag, &d_skey, &path_first, &path_draw, &feats, &preds, &allot,
                               &plan_tot, &judge_out, &seg_scratch, &seg_tiles, &curve_wide, &wide_curves,
                               &cta_narrow_d};
        uint64_t t = 0;
        for (const DevBuf* b : all) t += b->cap;
        return t;
    }

    // Buffers of the stages after the count, for `cap` records and `dcap`
    // draw records.
    sr_status reserve(int64_t cap, int64_t dcap) {
        cudaError_t err = cudaSuccess;
        post_count_buffers(cap, dcap, [&](DevBuf& b, size_t bytes) {
            if (err == cudaSuccess && bytes) err = ensure(b, bytes);
        });
        CUDA_TRY(err);
        const size_t n1 = (size_t)std::max<int64_t>(cap, 1);
        if (flags & SR_FLAG_KEEP_STAGES) {
            CUDA_TRY(ensure(d_fkey, sizeof(int32_t) * n1));
            CUDA_TRY(ensure(d_fwn, sizeof(int32_t) * n1));
            CUDA_TRY(ensure(d_fleft, sizeof(int32_t) * n1));
            CUDA_TRY(ensure(d_wscan, sizeof(int32_t) * (n1 + 1)));
            CUDA_TRY(ensure(d_fflag, sizeof(int32_t) * n1));
            CUDA_TRY(ensure(d_sflag, sizeof(int32_t) * n1));
            CUDA_TRY(ensure(d_skey, sizeof(int32_t) * n1));
        }
        return SR_OK;
    }

    // Transform, count, chain order and offset scan (no allocation, no wait).
    sr_status enqueue_front(cudaStream_t st) {
        using namespace sr;
        uint32_t* ctlp = ctl.as<uint32_t>();
        uint32_t* status = ctlp + CTL_STATUS;
        CUDA_TRY(cudaMemsetAsync(ctlp, 0, sizeof(uint32_t) * CTL_WORDS, st));
        CUDA_TRY(cudaMemsetAsync(path_visible.p, 0, sizeof(int32_t) * std::max<uint32_t>(P, 1), st));
        CUDA_TRY(cudaMemsetAsync(scan_status.p, 0, sizeof(uint64_t) * scan_status_words(C), st));
        CUDA_TRY(cudaMemsetAsync(totals.p, 0, sizeof(uint64_t) * 4, st));
        if (count_paths) CUDA_TRY(cudaMemsetAsync(path_draw.p, 0, sizeof(uint32_t) * std::max<uint32_t>(P, 1), st));
        mark(ST_TRANSFORM, false);
        launch_transform(pos.as<float2>(), pos_path.as<uint32_t>(), V, table(), tpos.as<float2>(),
                         path_visible.as<int32_t>(), st);
        if (arcs)
            launch_arc_fixup(curve_type.as<uint32_t>(), curve_pos.as<uint32_t>(), curve_path.as<uint32_t>(), C,
                             pos.as<float2>(), table(), tpos.as<float2>(), path_visible.as<int32_t>(), st);
        mark(ST_TRANSFORM, true);
        const GeomArgs g = geom(0);
        const ChainWork cw = chain_work();
        const uint32_t lc = list_cap();
        SortPlan cp = sort_plan(lc, chain_key_bits(), ctlp + CTL_CHAINS);
        uint32_t* cl = chain_lists.as<uint32_t>();
        mark(ST_COUNT, false);
        launch_count(g, cut.as<float>(), count.as<int32_t>(), cw, status, st);
        launch_sort_u32(cp, cw.chain_keys, cw.chain_items, cw.sorted_keys, cw.sorted_items, cl + 4 * (size_t)lc,
                        cl + 5 * (size_t)lc, chain_sort_scratch.p, status, st);
        mark(ST_COUNT, true);
        mark(ST_SCAN, false);
        launch_exclusive_scan_i32(count.as<int32_t>(), offs.as<int32_t>(), C, scan_status.as<uint64_t>(),
                                  ctlp + CTL_SCAN_COUNTER, status, st);
        if (segmented())
            launch_segsort_tables(curve_path.as<uint32_t>(), offs.as<int32_t>(), C, seg_check, seg_scratch.p, status,
                                  st);
        mark(ST_SCAN, true);
        CUDA_TRY(cudaGetLastError());
        return SR_OK;
    }

    // Everything after the count, sized for `cap` records (no allocation,
    // no wait).  The kernels read the actual count from offs[C].
    sr_status enqueue_back(cudaStream_t st, int64_t cap, int64_t dcap_req) {
        using namespace sr;
        uint32_t* ctlp = ctl.as<uint32_t>();
        uint32_t* status = ctlp + CTL_STATUS;
        const bool keep = (flags & SR_FLAG_KEEP_STAGES) != 0;
        const uint32_t* n_dev = reinterpret_cast<const uint32_t*>(offs.as<int32_t>() + C);
        const GeomArgs g = geom(cap);
        const ChainWork cw = chain_work();
        DebugOut dbg{nullptr, nullptr, nullptr};
        if (keep) {
            dbg.fkey = d_fkey.as<int32_t>();
            dbg.fwn = d_fwn.as<int32_t>();
            dbg.fleft = d_fleft.as<int32_t>();
            CUDA_TRY(cudaMemsetAsync(d_wscan.p, 0, sizeof(int32_t) * ((size_t)std::max<int64_t>(cap, 1) + 1), st));
        }
        // The wide chains -- the frame's longest dependency -- and their
        // curves' merge and fragments stay on st, right behind the count
        // pass, so that they start first; the other chains, merge and
        // fragments run on the side stream beside them.  st's merge waits for
        // the side stream's (which marks the wide curves' records pending and
        // covers the short chains of the wide curves), and st waits for the
        // side stream before the sort.
        CUDA_TRY(cudaEventRecord(ev_fork, st));
        CUDA_TRY(cudaStreamWaitEvent(side, ev_fork, 0));
        mark(ST_WIDE, false, st);
        launch_chains(g, offs.as<int32_t>(), cw, cbuf.as<int32_t>(), sm_count, 0, st);
        mark(ST_CHAINS, false, side);
        launch_chains(g, offs.as<int32_t>(), cw, cbuf.as<int32_t>(), sm_count, 1, side);
        mark(ST_CHAINS, true, side);
        mark(ST_MERGE, false, side);
        launch_merge(g, offs.as<int32_t>(), cw, cbuf.as<int32_t>(), rec.as<int2>(), status, 0, side);
        mark(ST_MERGE, true, side);
        CUDA_TRY(cudaEventRecord(ev_merged, side));
        CUDA_TRY(cudaStreamWaitEvent(st, ev_merged, 0));
        launch_merge(g, offs.as<int32_t>(), cw, cbuf.as<int32_t>(), rec.as<int2>(), status, 1, st);
        mark(ST_FRAGMENT, false, side);
        launch_fragment(g, rec.as<int2>(), offs.as<int32_t>(), cap, n_dev, keys.as<uint64_t>(),
                        keep ? wnp.as<uint8_t>() : nullptr, dbg, cw, 0, side);
        mark(ST_FRAGMENT, true, side);
        launch_fragment(g, rec.as<int2>(), offs.as<int32_t>(), cap, n_dev, keys.as<uint64_t>(),
                        keep ? wnp.as<uint8_t>() : nullptr, dbg, cw, 1, st);
        mark(ST_WIDE, true, st);
        CUDA_TRY(cudaEventRecord(ev_join, side));
        CUDA_TRY(cudaStreamWaitEvent(st, ev_join, 0));
        const KeyLayout L = g.L;
        SortPlan sp = sort_plan(cap, L.pbits + L.rbits + L.xbits, n_dev, tune.sort_items);
        mark(ST_SORT, false);
        last_segsort = segmented() && seg_levels >= 0;
        if (last_segsort)
            launch_segsort(keys.as<uint64_t>(), skeys.as<uint64_t>(), keys_alt.as<uint64_t>(), cap, C, L, seg_levels,
                           seg_scratch.p, seg_tiles.p, sm_count, status, st);
        else
            launch_sort_u64(sp, keys.as<uint64_t>(), nullptr, skeys.as<uint64_t>(),
                            keep ? svals.as<uint32_t>() : nullptr, keys_alt.as<uint64_t>(),
                            keep ? vals_alt.as<uint32_t>() : nullptr, sort_scratch.p, status, st);
        mark(ST_SORT, true);
        CUDA_TRY(cudaMemsetAsync(wind_status.p, 0, sizeof(uint64_t) * winding_status_words(cap, tune.wind_items), st));
        WindArgs wa;
        wa.n = cap;
        wa.n_dev = n_dev;
        wa.skeys = skeys.as<uint64_t>();
        wa.svals = keep ? svals.as<uint32_t>() : nullptr;
        wa.wnp = keep ? wnp.as<uint8_t>() : nullptr;
        wa.fill_rule = fill_rule.as<uint32_t>();
        wa.fill_info = fill_info.as<uint32_t>();
        wa.n_paths = P;
        wa.W = Wmax;
        wa.H = Hmax;
        wa.F = F;
        wa.pixel_mode = g.pixel_mode;
        wa.L = L;
        wa.st = table();
        wa.draw = draw.as<int4>();
        const int64_t dcap = draw_cap_for(cap, dcap_req);
        wa.draw_capacity = dcap;
        wa.draw_row = draw_row.as<uint32_t>();
        wa.totals = totals.as<uint64_t>();
        wa.n_draw = ctlp + CTL_NDRAW;
        wa.path_draw = count_paths ? path_draw.as<uint32_t>() : nullptr;
        wa.dbg_wscan = keep ? d_wscan.as<int32_t>() : nullptr;
        wa.dbg_fflag = keep ? d_fflag.as<int32_t>() : nullptr;
        wa.dbg_sflag = keep ? d_sflag.as<int32_t>() : nullptr;
        wa.dbg_skey = keep ? d_skey.as<int32_t>() : nullptr;
        wa.seg_cut = seg_cut.as<uint32_t>();
        wa.cut_rows = total_rows;
        wa.cut_segs = cut_segs();
        wa.row_count = row_count.as<uint32_t>();
        wa.row_px = row_px.as<unsigned long long>();
        CUDA_TRY(cudaMemsetAsync(seg_cut.p, 0, sizeof(uint32_t) * cut_words(), st));
        CUDA_TRY(cudaMemsetAsync(row_count.p, 0, sizeof(uint32_t) * total_rows, st));
        CUDA_TRY(cudaMemsetAsync(row_px.p, 0, sizeof(unsigned long long) * total_rows, st));
        CUDA_TRY(cudaMemsetAsync(row_scan.p, 0, sizeof(uint64_t) * sr::scan_status_words(total_rows), st));
        mark(ST_WINDING, false);
        launch_winding_emit(wa, tune.wind_items, wind_status.as<uint64_t>(), ctlp + CTL_WIND_COUNTER, status, st);
        mark(ST_WINDING, true);
        SortPlan rp = sort_plan(dcap, bits_for(total_rows), ctlp + CTL_NDRAW);
        mark(ST_ROWSORT, false);
        // the emit counted the records of every row: their exclusive scan is
        // each row's start in the row order, and their digits the sort's
        // histogram
        launch_exclusive_scan_i32(row_count.as<int32_t>(), row_start.as<int32_t>(), total_rows, row_scan.as<uint64_t>(),
                                  ctlp + CTL_ROW_SCAN, status, st);
        sort_hist_from_counts(rp, row_count.as<uint32_t>(), total_rows, row_sort_scratch.p, st);
        launch_sort_u32(rp, draw_row.as<uint32_t>(), nullptr, rkeys.as<uint32_t>(), rvals.as<uint32_t>(),
                        rkeys_alt.as<uint32_t>(), rvals_alt.as<uint32_t>(), row_sort_scratch.p, status, st);
        mark(ST_ROWSORT, true);
        ResolveArgs ra;
        ra.draw = draw.as<int4>();
        ra.row_sorted_idx = rvals.as<uint32_t>();
        ra.row_start = row_start.as<int32_t>();
        ra.cta_base = cta_base_d.as<uint32_t>();
        ra.scenes = scenes_d.as<SceneInfo>();
        ra.n_scenes = S;
        ra.F = F;
        ra.warps = tune.resolve_warps;
        ra.pixel_mode = g.pixel_mode;
        ra.image = image.as<uint32_t>();
        ra.seg_cut = seg_cut.as<uint32_t>();
        ra.cut_segs = cut_segs();
        ra.row_px = row_px.as<unsigned long long>();
        ra.cta_narrow = cta_narrow_d.as<uint8_t>();
        ra.any_narrow = any_narrow ? 1 : 0;
        ra.paints = n_paints ? paints_d.as<DevPaint>() : nullptr;
        ra.n_paints = n_paints;
        mark(ST_RESOLVE, false);
        launch_resolve(ra, res_ctas, st);
        mark(ST_RESOLVE, true);
        CUDA_TRY(cudaGetLastError());
        return SR_OK;
    }

    // Read N back (the reference's count read-back, scanline_rasterizer.cpp:355-356).
    sr_status read_count(cudaStream_t st, int64_t* N) {
        CUDA_TRY(cudaMemcpyAsync(&h_u32[0], offs.as<int32_t>() + C, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(&h_u32[1], ctl.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        h_u32[2] = 0;
        if (segmented())
            CUDA_TRY(cudaMemcpyAsync(&h_u32[2], sr::segsort_largest(seg_scratch.p, C), sizeof(uint32_t),
                                     cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        SR_TRY(check_status_word(h_u32[1]));
        seg_levels = levels_for(h_u32[2]);
        *N = (int64_t)(int32_t)h_u32[0];
        if (*N < 0 || *N >= (1ll << 30))
            return fail(SR_ERR_OVERFLOW_REFIT, "record count %lld out of range", (long long)*N);
        return SR_OK;
    }

    // Merge rounds of the segmented sort for a largest segment of `largest`
    // records; -1 past the limit (the radix sort then).
    static int levels_for(uint32_t largest) {
        int lv = 0;
        const uint32_t T = (uint32_t)sr::segsort_tile();
        const uint32_t chunks = (largest + T - 1) / T;
        while (chunks > (1u << lv)) ++lv;
        return lv > kSegLevelsMax ? -1 : lv;
    }

    // One frame.  cap < 0: size the record buffers exactly (one host wait
    // for N); cap >= 0: use that capacity without waiting, with `levels`
    // merge rounds of the segmented sort (a larger segment flags an
    // overflow).  dcap <= 0 sizes the draw records at 2 x cap.
    sr_status frame(cudaStream_t st, int64_t cap, int64_t dcap = -1, int levels = kSegLevelsMax) {
        CUDA_TRY(cudaSetDevice(device));
        if (!loaded) return fail(SR_ERR_NO_SCENE, "render before a scene was loaded");
        cur = st;
        stages_valid = false;
        const uint64_t launches0 = sr::launches_so_far();
        SR_TRY(prepare_front());
        // exact sizing reads the largest segment back; a pre-sized frame
        // runs the most merge rounds and flags larger segments as overflow
        if (levels < 0 || levels > kSegLevelsMax) levels = kSegLevelsMax;
        seg_check = cap < 0 ? 0u : (uint32_t)sr::segsort_tile() << levels;
        seg_levels = levels;
        SR_TRY(enqueue_front(st));
        if (cap < 0) {
            int64_t N = 0;
            SR_TRY(read_count(st, &N));
            cap = N;
            dcap = -1;
        }
        SR_TRY(reserve(cap, dcap));
        SR_TRY(enqueue_back(st, cap, dcap));
        stats.kernel_launches = (uint32_t)(sr::launches_so_far() - launches0);
        ev_pending = (flags & SR_FLAG_PROFILE) != 0;
        last_cap = cap;
        last_dcap = draw_cap_for(cap, dcap);
        return SR_OK;
    }

    // Waits for the frame and collects its counters and status.
    // Queues the copies of the frame's counters into pinned host memory.
    sr_status enqueue_readback(cudaStream_t st) {
        CUDA_TRY(cudaMemcpyAsync(&h_u32[0], offs.as<int32_t>() + C, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(&h_u32[1], ctl.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(h_u64, totals.p, sizeof(uint64_t) * 2, cudaMemcpyDeviceToHost, st));
        h_u32[2] = 0;
        if (segmented())
            CUDA_TRY(cudaMemcpyAsync(&h_u32[2], sr::segsort_largest(seg_scratch.p, C), sizeof(uint32_t),
                                     cudaMemcpyDeviceToHost, st));
        return SR_OK;
    }

    sr_status finish(cudaStream_t st) {
        SR_TRY(enqueue_readback(st));
        CUDA_TRY(cudaStreamSynchronize(st));
        return collect();
    }

    // The frame's counters and status, once the read-back has landed.
    sr_status collect() {
        last_N = (int64_t)(int32_t)h_u32[0];
        last_O = (int64_t)(h_u64[0] + h_u64[1]);
        last_largest = h_u32[2];
        stats.n_intersections = (uint64_t)last_N;
        stats.n_draw_records = (uint64_t)last_O;
        stats.n_merged_fragments = h_u64[0];
        stats.n_spans = h_u64[1];
        const sr::KeyLayout L = layout();
        stats.key_bits = L.pbits + L.rbits + L.xbits;
        stats.sort_passes = sr::sort_plan(1, stats.key_bits).passes;
        SR_TRY(check_status_word(h_u32[1]));
        if (last_N > last_cap)
            return fail(SR_ERR_OVERFLOW_REFIT, "frame needs %lld records, capacity %lld", (long long)last_N,
                        (long long)last_cap);
        if (last_O > last_dcap)
            return fail(SR_ERR_OVERFLOW_REFIT, "frame needs %lld draw records, capacity %lld", (long long)last_O,
                        (long long)last_dcap);
        stages_valid = (flags & SR_FLAG_KEEP_STAGES) != 0;
        return SR_OK;
    }

    sr_status collect_events() {
        if (!ev_pending) return SR_OK;
        CUDA_TRY(cudaEventSynchronize(ev[2 * ST_RESOLVE + 1]));
        for (int s = 0; s < ST_COUNT_ALL; ++s) {
            float ms = 0.f;
            if (ev[2 * s] && ev[2 * s + 1]) CUDA_TRY(cudaEventElapsedTime(&ms, ev[2 * s], ev[2 * s + 1]));
            stats.stage_ms[s] = ms;
        }
        ev_pending = false;
        return SR_OK;
    }
};

struct sr_ctx {
    Pipeline p;
    int32_t W = 0, H = 0;
    float mvp[16];
    // Counts of the last frame that completed without overflow, and the
    // curve and path counts of its scene: the next frame of a scene with the
    // same counts is pre-sized from them instead of waiting for its count.
    bool hint_valid = false;
    uint32_t hint_C = 0, hint_P = 0;
    int64_t hint_N = 0, hint_O = 0;
    uint32_t hint_largest = 0;
    uint32_t refits = 0;
};

// Batch of scenes (several uneven scenes per frame).
struct sr_batch {
    Pipeline p;
    HostScenes h;
    bool committed = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t graph_cap = -1, graph_dcap = -1;
    uint32_t graph_launches = 0;
    uint32_t overflows = 0, refits = 0;
    cudaStream_t cap_stream = nullptr;   // captures run here: the legacy stream cannot be captured
    // a frame enqueued by sr_batch_enqueue and not yet finished
    bool inflight = false;
    cudaEvent_t done = nullptr;
    sr_batch_render_opts pending{};
    cudaStream_t pending_stream = nullptr;
    ~sr_batch() {
        if (done) cudaEventDestroy(done);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (cap_stream) cudaStreamDestroy(cap_stream);
    }
};

static_assert(SR_SIZER_PARAMS == sr::kMlpParams && SR_SIZER_FEATURES == sr::kMlpIn &&
                  SR_SIZER_OUTPUTS == sr::kMlpOut && SR_SIZER_NORM == sr::kMlpNorm,
              "sizer constants");

// The learned-sizing network: parameters, Adam state and training scratch
// on one device.
struct sr_sizer {
    int device = 0, sm_count = 148;
    DevBuf master, wb, grad, m, v, norm, loss;   // loss: one float
    DevBuf keys, perm, keys_out, alt_k, alt_v, sort_scratch, ctl;
    int64_t step = 0;
    float* h_loss = nullptr;
    ~sr_sizer() {
        DevBuf* all[] = {&master, &wb, &grad, &m, &v, &norm, &loss, &keys, &perm, &keys_out, &alt_k, &alt_v,
                         &sort_scratch, &ctl};
        for (DevBuf* b : all) release(*b);
        if (h_loss) cudaFreeHost(h_loss);
    }
};

// Per-path curve ranges of a batch (curves are grouped by path in order).
static sr_status batch_path_first(sr_batch* b);

extern "C" {

const char* sr_last_error(void) { return g_err.c_str(); }

sr_status sr_create(uint32_t width, uint32_t height, const sr_options* opt, sr_ctx** out) {
    if (!out) return fail(SR_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (width == 0 || height == 0 || width > 16384 || height > 16384)
        return fail(SR_ERR_INVALID_ARG, "canvas %ux%u outside 1..16384", width, height);
    sr_options o{};
    o.struct_size = sizeof(sr_options);
    o.mode = SR_MODE_PIXEL;
    if (opt) {
        if (opt->struct_size < sizeof(sr_options)) return fail(SR_ERR_INVALID_ARG, "sr_options.struct_size too small");
        o = *opt;
    }
    if (o.mode != SR_MODE_REFERENCE && o.mode != SR_MODE_PIXEL) return fail(SR_ERR_INVALID_ARG, "unknown mode %d", o.mode);
    int ndev = 0;
    CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (o.device < 0 || o.device >= ndev) return fail(SR_ERR_INVALID_ARG, "device %d not present", o.device);
    sr_ctx* c = new sr_ctx();
    sr_status s = c->p.init(o.device, o.mode, o.flags);
    if (s != SR_OK) {
        delete c;
        return s;
    }
    c->W = (int32_t)width;
    c->H = (int32_t)height;
    std::memcpy(c->mvp, kIdentity, sizeof c->mvp);
    *out = c;
    return SR_OK;
}

sr_status sr_load_scene(sr_ctx* c, const sr_scene_view* s) {
    if (!c || !s) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    SR_TRY(validate_scene(s));
    return c->p.upload_single(s, c->W, c->H, c->mvp);
}

// The context's paints for matrix m (its own unless given), on the device.
static sr_status upload_paints(sr_ctx* c, const float* m = nullptr) {
    Pipeline& p = c->p;
    p.n_paints = (uint32_t)p.paints_h.size();
    if (!p.n_paints) return SR_OK;
    std::vector<sr::DevPaint> d(p.n_paints);
    for (uint32_t i = 0; i < p.n_paints; ++i) d[i] = make_dev_paint(p.paints_h[i], m ? m : c->mvp);
    CUDA_TRY(cudaSetDevice(p.device));
    CUDA_TRY(ensure(p.paints_d, sizeof(sr::DevPaint) * d.size()));
    CUDA_TRY(cudaMemcpy(p.paints_d.p, d.data(), sizeof(sr::DevPaint) * d.size(), cudaMemcpyHostToDevice));
    return SR_OK;
}

sr_status sr_set_mvp(sr_ctx* c, const float m[16]) {
    if (!c || !m) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    std::memcpy(c->mvp, m, sizeof(float) * 16);
    SR_TRY(upload_paints(c));
    if (c->p.loaded) {
        std::memcpy(c->p.info[0].mvp, m, sizeof(float) * 16);
        CUDA_TRY(cudaSetDevice(c->p.device));
        return c->p.upload_table();
    }
    return SR_OK;
}

sr_status sr_set_paints(sr_ctx* c, const sr_paint* paints, uint32_t n) {
    if (!c || (n && !paints)) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (n > (1u << 24) - 1u) return fail(SR_ERR_INVALID_ARG, "too many paints");
    for (uint32_t i = 0; i < n; ++i) {
        const sr_paint& q = paints[i];
        if ((q.kind != SR_PAINT_LINEAR && q.kind != SR_PAINT_RADIAL) || q.spread < 0 || q.spread > 2 ||
            q.n_stops == 0 || q.n_stops > SR_PAINT_MAX_STOPS)
            return fail(SR_ERR_INVALID_ARG, "paint %u: bad kind, spread or stop count", i);
    }
    c->p.paints_h.assign(paints, paints + n);
    return upload_paints(c);
}

// ScanlineVGRasterizer::render (scanline_rasterizer.cpp:282-696) waits on
// the host twice inside a frame, for the record count (:355-356) and the
// fragment and span counts (:578-580).  A frame here is pre-sized from the
// previous frame of a scene with the same curve and path counts (1/16 more,
// and the merge rounds its largest sort segment needed) and enqueued whole;
// the only host wait is at its end, where the counters are read.  If the
// frame overflowed (a new matrix or scene that needs more), it is rerun with
// exact sizing, which waits for the count as the reference does; so does the
// first frame of a scene.
static sr_status render_core(sr_ctx* c, void* rgba_out, int out_is_device, cudaStream_t st) {
    Pipeline& p = c->p;
    const size_t bytes = (size_t)c->W * c->H * 4;
    const bool presized = c->hint_valid && p.loaded && c->hint_C == p.C && c->hint_P == p.P;
    const uint64_t launches0 = sr::launches_so_far();
    sr_status s = SR_ERR_OVERFLOW_REFIT;
    if (presized) {
        const int64_t cap = c->hint_N + c->hint_N / 16 + 256;
        const int64_t dcap = c->hint_O + c->hint_O / 16 + 256;
        int levels = Pipeline::levels_for(c->hint_largest + c->hint_largest / 16);
        SR_TRY(p.frame(st, cap, dcap, levels < 0 ? Pipeline::kSegLevelsMax : levels));
        if (rgba_out)
            CUDA_TRY(cudaMemcpyAsync(rgba_out, p.image.p, bytes,
                                     out_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
        s = p.finish(st);
        if (s == SR_ERR_OVERFLOW_REFIT) ++c->refits;
    }
    if (s == SR_ERR_OVERFLOW_REFIT) {
        SR_TRY(p.frame(st, -1));
        if (rgba_out)
            CUDA_TRY(cudaMemcpyAsync(rgba_out, p.image.p, bytes,
                                     out_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
        s = p.finish(st);
    }
    p.stats.kernel_launches = (uint32_t)(sr::launches_so_far() - launches0);
    p.stats.reruns = c->refits;
    c->hint_valid = s == SR_OK;
    if (s == SR_OK) {
        c->hint_C = p.C;
        c->hint_P = p.P;
        c->hint_N = p.last_N;
        c->hint_O = p.last_O;
        c->hint_largest = p.last_largest;
    }
    return s;
}

sr_status sr_render(sr_ctx* c, void* rgba_out, int out_is_device, void* stream) {
    if (!c) return fail(SR_ERR_INVALID_ARG, "NULL context");
    return render_core(c, rgba_out, out_is_device, static_cast<cudaStream_t>(stream));
}

// Sample i of k in pixel units: row (i + 0.5) / k, column ((i * s) mod k +
// 0.5) / k with s coprime to k, so that every sample has a row and a column
// of its own (an n-rooks comb).
static void aa_offset(uint32_t k, uint32_t i, float* ox, float* oy) {
    const uint32_t s = k == 16 ? 5u : k >= 4 ? 3u : 1u;
    *ox = ((float)((i * s) % k) + 0.5f) / (float)k;
    *oy = ((float)i + 0.5f) / (float)k;
}

sr_status sr_render_aa(sr_ctx* c, uint32_t samples, void* rgba_out, int out_is_device, void* stream) {
    if (!c) return fail(SR_ERR_INVALID_ARG, "NULL context");
    if (samples != 1 && samples != 2 && samples != 4 && samples != 8 && samples != 16)
        return fail(SR_ERR_INVALID_ARG, "samples must be 1, 2, 4, 8 or 16");
    Pipeline& p = c->p;
    if (p.mode != SR_MODE_PIXEL) return fail(SR_ERR_INVALID_ARG, "multisampling needs SR_MODE_PIXEL");
    if (!p.loaded) return fail(SR_ERR_NO_SCENE, "render before a scene was loaded");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CUDA_TRY(cudaSetDevice(p.device));
    const size_t npx = (size_t)c->W * c->H;
    CUDA_TRY(ensure(p.aa_acc, 8 * std::max<size_t>(npx, 1)));
    const uint64_t launches0 = sr::launches_so_far();
    sr_status s = SR_OK;
    for (uint32_t i = 0; i < samples && s == SR_OK; ++i) {
        // the pipeline samples each pixel at its centre: moving the scene by
        // (0.5 - ox, 0.5 - oy) samples it at (x + ox, y + oy).  Rows 0 and 1
        // of the matrix take that translation times row 3.
        float ox, oy;
        aa_offset(samples, i, &ox, &oy);
        const float tx = 0.5f - ox, ty = 0.5f - oy;
        float* m = p.info[0].mvp;
        for (int k = 0; k < 4; ++k) {
            m[k] = c->mvp[k] + tx * c->mvp[12 + k];
            m[4 + k] = c->mvp[4 + k] + ty * c->mvp[12 + k];
            m[8 + k] = c->mvp[8 + k];
            m[12 + k] = c->mvp[12 + k];
        }
        s = p.upload_table();
        if (s == SR_OK) s = upload_paints(c, m);   // gradients are sampled at the moved centres too
        if (s == SR_OK) s = render_core(c, nullptr, 0, st);
        if (s == SR_OK) {
            sr::launch_aa_accumulate(p.image.as<uint32_t>(), p.aa_acc.p, npx, i == 0, st);
            CUDA_TRY(cudaGetLastError());
        }
    }
    std::memcpy(p.info[0].mvp, c->mvp, sizeof c->mvp);
    sr_status s2 = p.upload_table();
    if (s2 == SR_OK) s2 = upload_paints(c);
    SR_TRY(s);
    SR_TRY(s2);
    sr::launch_aa_resolve(p.aa_acc.p, p.image.as<uint32_t>(), npx, samples, st);
    CUDA_TRY(cudaGetLastError());
    if (rgba_out)
        CUDA_TRY(cudaMemcpyAsync(rgba_out, p.image.p, npx * 4,
                                 out_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    p.stats.kernel_launches = (uint32_t)(sr::launches_so_far() - launches0);
    return SR_OK;
}

sr_status sr_render_draw_list(sr_ctx* c, const int32_t* records, int64_t n, void* rgba_out, int out_is_device,
                              void* stream) {
    if (!c) return fail(SR_ERR_INVALID_ARG, "NULL context");
    if (n < 0 || n >= (1ll << 30) || (n > 0 && !records)) return fail(SR_ERR_INVALID_ARG, "bad draw list");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Pipeline& p = c->p;
    CUDA_TRY(cudaSetDevice(p.device));
    if (!p.loaded || p.S != 1) {
        // a canvas with no scene: the draw list alone decides the pixels
        sr_scene_view empty{};
        SR_TRY(p.upload_single(&empty, c->W, c->H, c->mvp));
    }
    const int32_t rows = (int32_t)p.total_rows;
    const size_t n1 = (size_t)std::max<int64_t>(n, 1);
    std::vector<uint32_t> row((size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        int32_t y = records[4 * i] >> 16;
        row[(size_t)i] = (y < 0 || y >= c->H) ? (uint32_t)rows : (uint32_t)(y / p.F);
    }
    CUDA_TRY(ensure(p.draw, sizeof(int4) * n1));
    CUDA_TRY(ensure(p.draw_row, sizeof(uint32_t) * n1));
    CUDA_TRY(ensure(p.rkeys, sizeof(uint32_t) * n1));
    CUDA_TRY(ensure(p.rvals, sizeof(uint32_t) * n1));
    CUDA_TRY(ensure(p.rkeys_alt, sizeof(uint32_t) * n1));
    CUDA_TRY(ensure(p.rvals_alt, sizeof(uint32_t) * n1));
    CUDA_TRY(ensure(p.row_start, sizeof(int32_t) * ((size_t)rows + 1)));
    CUDA_TRY(cudaMemsetAsync(p.ctl.p, 0, sizeof(uint32_t) * CTL_WORDS, st));
    if (n) {
        CUDA_TRY(cudaMemcpyAsync(p.draw.p, records, sizeof(int4) * (size_t)n, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(p.draw_row.p, row.data(), sizeof(uint32_t) * (size_t)n, cudaMemcpyHostToDevice, st));
    }
    sr::SortPlan rp = sr::sort_plan(n, bits_for((uint64_t)rows));
    CUDA_TRY(ensure(p.row_sort_scratch, sr::sort_scratch_bytes(rp)));
    uint32_t* status = p.ctl.as<uint32_t>() + CTL_STATUS;
    sr::launch_sort_u32(rp, p.draw_row.as<uint32_t>(), nullptr, p.rkeys.as<uint32_t>(), p.rvals.as<uint32_t>(),
                        p.rkeys_alt.as<uint32_t>(), p.rvals_alt.as<uint32_t>(), p.row_sort_scratch.p, status, st);
    sr::launch_row_bounds(p.rkeys.as<uint32_t>(), n, nullptr, rows, p.row_start.as<int32_t>(), st);
    sr::ResolveArgs ra;
    ra.draw = p.draw.as<int4>();
    ra.row_sorted_idx = p.rvals.as<uint32_t>();
    ra.row_start = p.row_start.as<int32_t>();
    ra.cta_base = p.cta_base_d.as<uint32_t>();
    ra.scenes = p.scenes_d.as<sr::SceneInfo>();
    ra.n_scenes = p.S;
    ra.F = p.F;
    ra.warps = p.tune.resolve_warps;
    ra.pixel_mode = p.mode == SR_MODE_PIXEL;
    ra.image = p.image.as<uint32_t>();
    ra.seg_cut = nullptr;
    ra.cut_segs = 0;
    ra.row_px = nullptr;
    ra.cta_narrow = p.cta_narrow_d.as<uint8_t>();
    ra.any_narrow = p.any_narrow ? 1 : 0;
    ra.paints = p.n_paints ? p.paints_d.as<sr::DevPaint>() : nullptr;
    ra.n_paints = p.n_paints;
    sr::launch_resolve(ra, p.res_ctas, st);
    CUDA_TRY(cudaGetLastError());
    p.last_O = n;
    if (rgba_out) {
        CUDA_TRY(cudaMemcpyAsync(rgba_out, p.image.p, (size_t)c->W * c->H * 4,
                                 out_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    }
    CUDA_TRY(cudaMemcpyAsync(&p.h_u32[1], status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return check_status_word(p.h_u32[1]);
}

sr_status sr_get_stats(const sr_ctx* cc, sr_stats* out) {
    if (!cc || !out) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    sr_ctx* c = const_cast<sr_ctx*>(cc);
    SR_TRY(c->p.collect_events());
    *out = c->p.stats;
    return SR_OK;
}

sr_status sr_debug_dump(sr_ctx* c, int stage, void* dst, size_t* bytes) {
    if (!c || !bytes) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    Pipeline& p = c->p;
    const size_t N = (size_t)p.last_N, O = (size_t)p.last_O;
    const void* src = nullptr;
    size_t need = 0;
    bool need_stages = true;
    switch (stage) {
        case SR_STAGE_TRANSFORMED_POS: src = p.tpos.p; need = 8 * (size_t)p.V; need_stages = false; break;
        case SR_STAGE_PATH_VISIBLE: src = p.path_visible.p; need = 4 * (size_t)p.P; need_stages = false; break;
        case SR_STAGE_CUTPOINTS: src = p.cut.p; need = 20 * (size_t)p.C; need_stages = false; break;
        case SR_STAGE_CURVE_COUNT: src = p.count.p; need = 4 * (size_t)p.C; need_stages = false; break;
        case SR_STAGE_CURVE_OFFSET: src = p.offs.p; need = 4 * ((size_t)p.C + 1); need_stages = false; break;
        case SR_STAGE_INTERSECTION: src = p.rec.p; need = 8 * N; need_stages = false; break;
        case SR_STAGE_FRAG_KEY: src = p.d_fkey.p; need = 4 * N; break;
        case SR_STAGE_FRAG_WINDING: src = p.d_fwn.p; need = 4 * N; break;
        case SR_STAGE_FRAG_LEFT: src = p.d_fleft.p; need = 4 * N; break;
        case SR_STAGE_SORTED_KEY: src = p.d_skey.p; need = 4 * N; break;
        case SR_STAGE_SORTED_INDEX: src = p.svals.p; need = 4 * N; break;
        case SR_STAGE_WINDING_SCAN: src = p.d_wscan.p; need = 4 * (N + 1); break;
        case SR_STAGE_FRAG_FLAG: src = p.d_fflag.p; need = 4 * N; break;
        case SR_STAGE_SPAN_FLAG: src = p.d_sflag.p; need = 4 * N; break;
        case SR_STAGE_DRAW_LIST: src = p.draw.p; need = 16 * O; need_stages = false; break;
        case SR_STAGE_IMAGE: src = p.image.p; need = (size_t)c->W * c->H * 4; need_stages = false; break;
        default: return fail(SR_ERR_INVALID_ARG, "unknown stage %d", stage);
    }
    if (need_stages && !p.stages_valid)
        return fail(SR_ERR_INVALID_ARG, "stage %d needs a render with SR_FLAG_KEEP_STAGES", stage);
    if (!dst) {
        *bytes = need;
        return SR_OK;
    }
    if (*bytes < need) return fail(SR_ERR_INVALID_ARG, "buffer of %zu bytes, need %zu", *bytes, need);
    if (need && !src) return fail(SR_ERR_INVALID_ARG, "stage %d not available", stage);
    CUDA_TRY(cudaSetDevice(p.device));
    if (need) CUDA_TRY(cudaMemcpy(dst, src, need, cudaMemcpyDeviceToHost));
    *bytes = need;
    return SR_OK;
}

sr_status sr_debug_sort_tiles(sr_ctx* c, uint32_t* tiles, uint32_t* wide_tiles) {
    if (!c || !tiles || !wide_tiles) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    Pipeline& p = c->p;
    *tiles = *wide_tiles = 0;
    if (!p.last_segsort || !p.seg_tiles.p || p.C == 0 || p.last_cap <= 0) return SR_OK;
    CUDA_TRY(cudaSetDevice(p.device));
    CUDA_TRY(cudaDeviceSynchronize());
    uint32_t v[2] = {0, 0};
    CUDA_TRY(sr::segsort_tile_counts(p.seg_tiles.p, p.C, p.last_cap, v));
    *tiles = v[0];
    *wide_tiles = v[1];
    return SR_OK;
}

// The allocating standalone scan; first_tile > 0 starts the tile counter
// there (tiles before it never run), which only sr_debug_scan_without_first_tile
// asks for.
static sr_status standalone_scan(const int32_t* d_in, int32_t* d_out, int64_t n, uint32_t first_tile,
                                 cudaStream_t st) {
    if (n < 0 || n >= (1ll << 31)) return fail(SR_ERR_INVALID_ARG, "scan length %lld out of range", (long long)n);
    if (!d_out || (n > 0 && !d_in)) return fail(SR_ERR_INVALID_ARG, "NULL device pointer");
    if (n == 0) {
        CUDA_TRY(cudaMemsetAsync(d_out, 0, sizeof(int32_t), st));
        return SR_OK;
    }
    uint32_t* status = nullptr;
    CUDA_TRY(sr::standalone_scan_status(&status));
    // tile words, then the tile counter
    const size_t words = sr::scan_status_words(n) + 1;
    void* scratch = nullptr;
    CUDA_TRY(cudaMallocAsync(&scratch, words * sizeof(uint64_t), st));
    uint64_t* tiles = static_cast<uint64_t*>(scratch);
    uint32_t* counter = reinterpret_cast<uint32_t*>(tiles + words - 1);
    cudaError_t e = cudaMemsetAsync(scratch, 0, words * sizeof(uint64_t), st);
    if (e == cudaSuccess && first_tile) e = cudaMemcpyAsync(counter, &first_tile, sizeof first_tile,
                                                            cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && first_tile) e = cudaStreamSynchronize(st);   // first_tile is on this stack
    if (e == cudaSuccess) {
        sr::launch_exclusive_scan_i32(d_in, d_out, n, tiles, counter, status, st);
        e = cudaGetLastError();
    }
    cudaError_t f = cudaFreeAsync(scratch, st);
    CUDA_TRY(e);
    CUDA_TRY(f);
    return SR_OK;
}

sr_status sr_exclusive_scan_i32(const int32_t* d_in, int32_t* d_out, int64_t n, void* stream) {
    return standalone_scan(d_in, d_out, n, 0, static_cast<cudaStream_t>(stream));
}

sr_status sr_debug_scan_without_first_tile(const int32_t* d_in, int32_t* d_out, int64_t n, void* stream) {
    if (n <= 0) return fail(SR_ERR_INVALID_ARG, "the stalled scan needs n > 0");
    return standalone_scan(d_in, d_out, n, 1, static_cast<cudaStream_t>(stream));
}

sr_status sr_scan_status(void* stream) {
    CUDA_TRY(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
    uint32_t* word = nullptr;
    CUDA_TRY(sr::standalone_scan_status(&word));
    uint32_t h = 0;
    CUDA_TRY(cudaMemcpy(&h, word, sizeof h, cudaMemcpyDeviceToHost));
    if (h) CUDA_TRY(cudaMemset(word, 0, sizeof h));
    return check_status_word(h);
}

void sr_set_spin_limit(uint32_t polls) {
    sr::g_spin_limit.store(polls ? polls : sr::kSpinLimitDefault, std::memory_order_relaxed);
}

void sr_destroy(sr_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->p.device);
    cudaDeviceSynchronize();
    delete c;
}

// ------------------------------------------------------------- batches ---

sr_status sr_batch_create(const sr_options* opt, sr_batch** out) {
    if (!out) return fail(SR_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    sr_options o{};
    o.struct_size = sizeof(sr_options);
    o.mode = SR_MODE_PIXEL;
    if (opt) {
        if (opt->struct_size < sizeof(sr_options)) return fail(SR_ERR_INVALID_ARG, "sr_options.struct_size too small");
        o = *opt;
    }
    if (o.mode != SR_MODE_REFERENCE && o.mode != SR_MODE_PIXEL) return fail(SR_ERR_INVALID_ARG, "unknown mode %d", o.mode);
    int ndev = 0;
    CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (o.device < 0 || o.device >= ndev) return fail(SR_ERR_INVALID_ARG, "device %d not present", o.device);
    sr_batch* b = new sr_batch();
    sr_status s = b->p.init(o.device, o.mode, o.flags & ~SR_FLAG_KEEP_STAGES);
    if (s != SR_OK) {
        delete b;
        return s;
    }
    *out = b;
    return SR_OK;
}

sr_status sr_batch_add_scene(sr_batch* b, uint32_t width, uint32_t height, const sr_scene_view* s, const float* mvp,
                             uint32_t* index) {
    if (!b || !s) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (width == 0 || height == 0 || width > 16384 || height > 16384)
        return fail(SR_ERR_INVALID_ARG, "canvas %ux%u outside 1..16384", width, height);
    SR_TRY(validate_scene(s));
    if ((uint64_t)b->h.n_paths() + s->n_paths > (1u << 26) || (uint64_t)b->h.n_curves() + s->n_curves > (1u << 27))
        return fail(SR_ERR_INVALID_ARG, "batch too large");
    if (index) *index = (uint32_t)b->h.info.size();
    append_scene(b->h, width, height, s, mvp);
    b->committed = false;
    return SR_OK;
}

sr_status sr_batch_add_synth(sr_batch* b, const sr_synth_params* prm, uint32_t count, uint32_t* first_index) {
    if (!b || !prm) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (prm->struct_size < sizeof(sr_synth_params) || prm->preset < 0 || prm->preset > 2)
        return fail(SR_ERR_INVALID_ARG, "bad synth parameters");
    // generate in parallel, append in order
    std::vector<srsynth::Scene> sc(count);
    unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), count));
    std::atomic<uint32_t> next{0};
    auto work = [&]() {
        for (uint32_t i = next.fetch_add(1); i < count; i = next.fetch_add(1)) {
            srsynth::Params q;
            q.preset = prm->preset;
            q.seed = prm->seed;
            q.scene_index = prm->scene_index + i;
            q.width = prm->width;
            q.height = prm->height;
            q.n_paths = prm->n_paths;
            srsynth::generate(q, sc[i]);
        }
    };
    std::vector<std::thread> ts;
    for (unsigned t = 1; t < nt; ++t) ts.emplace_back(work);
    work();
    for (auto& t : ts) t.join();
    if (first_index) *first_index = (uint32_t)b->h.info.size();
    for (uint32_t i = 0; i < count; ++i) {
        const srsynth::Scene& s = sc[i];
        sr_scene_view v{s.n_points(), s.n_curves(), s.n_paths(), s.pos.data(), s.pos_path.data(), s.curve_pos.data(),
                        s.curve_type.data(), s.curve_path.data(), s.fill_rule.data(), s.fill_info.data()};
        append_scene(b->h, s.width, s.height, &v, nullptr);
    }
    b->committed = false;
    return SR_OK;
}

sr_status sr_batch_commit(sr_batch* b) {
    if (!b) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (b->inflight) return fail(SR_ERR_INVALID_ARG, "commit while a frame is in flight");
    SR_TRY(b->p.upload(b->h));
    b->committed = true;
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    b->graph_cap = -1;
    b->graph_dcap = -1;
    return SR_OK;
}

sr_status sr_batch_set_mvp(sr_batch* b, uint32_t index, const float m[16]) {
    if (!b || !m || index >= b->h.info.size()) return fail(SR_ERR_INVALID_ARG, "bad argument");
    std::memcpy(b->h.info[index].mvp, m, sizeof(float) * 16);
    if (b->committed) {
        std::memcpy(b->p.info[index].mvp, m, sizeof(float) * 16);
        CUDA_TRY(cudaSetDevice(b->p.device));
        return b->p.upload_table();
    }
    return SR_OK;
}

static sr_status batch_opts(const sr_batch_render_opts* o, sr_batch_render_opts* d) {
    std::memset(d, 0, sizeof *d);
    d->struct_size = sizeof *d;
    d->record_capacity = -1;
    d->draw_capacity = -1;
    if (o) {
        const size_t base = offsetof(sr_batch_render_opts, draw_capacity);
        if (o->struct_size < base) return fail(SR_ERR_INVALID_ARG, "opts.struct_size too small");
        std::memcpy(d, o, o->struct_size < sizeof *d ? base : sizeof *d);
        d->struct_size = sizeof *d;
    }
    return SR_OK;
}

// Enqueues one frame of the batch (with exact sizing this waits once for
// the record count); the frame's end is recorded in b->done.
static sr_status batch_enqueue(sr_batch* b, const sr_batch_render_opts& d, cudaStream_t st) {
    if (!b->committed) SR_TRY(sr_batch_commit(b));
    Pipeline& p = b->p;
    CUDA_TRY(cudaSetDevice(p.device));
    const int64_t cap = d.record_capacity;
    const int64_t dcap = cap >= 0 ? Pipeline::draw_cap_for(cap, d.draw_capacity) : -1;
    if (cap >= 0 && d.use_graph) {
        if (!b->exec || b->graph_cap != cap || b->graph_dcap != dcap) {
            if (b->exec) cudaGraphExecDestroy(b->exec);
            if (b->graph) cudaGraphDestroy(b->graph);
            b->exec = nullptr;
            b->graph = nullptr;
            // one plain frame first: it allocates every buffer and sets the
            // kernels' attributes, so the capture records launches only
            SR_TRY(p.frame(st, cap, dcap));
            sr_status fs = p.finish(st);
            if (fs != SR_OK && fs != SR_ERR_OVERFLOW_REFIT) return fs;
            if (!b->cap_stream) CUDA_TRY(cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking));
            CUDA_TRY(cudaStreamSynchronize(st));
            const uint64_t l0 = sr::launches_so_far();
            cudaStream_t cs = b->cap_stream;
            p.capturing = true;
            cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
            sr_status s1 = SR_OK, s2 = SR_OK;
            if (e == cudaSuccess) {
                s1 = p.enqueue_front(cs);
                if (s1 == SR_OK) s2 = p.enqueue_back(cs, cap, dcap);
                cudaError_t e2 = cudaStreamEndCapture(cs, &b->graph);   // always end the capture
                if (e2 != cudaSuccess) e = e2;
            }
            p.capturing = false;
            SR_TRY(s1);
            SR_TRY(s2);
            CUDA_TRY(e);
            CUDA_TRY(cudaGraphInstantiate(&b->exec, b->graph, 0));
            b->graph_cap = cap;
            b->graph_dcap = dcap;
            b->graph_launches = (uint32_t)(sr::launches_so_far() - l0);
        }
        CUDA_TRY(cudaGraphLaunch(b->exec, st));
        p.last_cap = cap;
        p.last_dcap = dcap;
        p.stats.kernel_launches = b->graph_launches;
        p.ev_pending = false;
    } else {
        SR_TRY(p.frame(st, cap, dcap));
    }
    SR_TRY(p.enqueue_readback(st));
    if (!b->done) CUDA_TRY(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming));
    CUDA_TRY(cudaEventRecord(b->done, st));
    b->inflight = true;
    return SR_OK;
}

// Waits for the enqueued frame; on overflow reruns it with exact sizing
// when asked to.
static sr_status batch_finish(sr_batch* b, const sr_batch_render_opts& d, cudaStream_t st) {
    Pipeline& p = b->p;
    CUDA_TRY(cudaSetDevice(p.device));
    b->inflight = false;
    // wait for this frame only: later work on the same stream may still run
    CUDA_TRY(cudaEventSynchronize(b->done));
    sr_status s = p.collect();
    if (s == SR_ERR_OVERFLOW_REFIT && d.refit_on_overflow) {
        ++b->overflows;
        ++b->refits;
        SR_TRY(p.frame(st, -1));   // the exact count pass
        s = p.finish(st);
    } else if (s == SR_ERR_OVERFLOW_REFIT) {
        ++b->overflows;
    }
    return s;
}

sr_status sr_batch_render(sr_batch* b, const sr_batch_render_opts* o, void* stream) {
    if (!b) return fail(SR_ERR_INVALID_ARG, "NULL batch");
    sr_batch_render_opts d;
    SR_TRY(batch_opts(o, &d));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    SR_TRY(batch_enqueue(b, d, st));
    return batch_finish(b, d, st);
}

sr_status sr_batch_enqueue(sr_batch* b, const sr_batch_render_opts* o, void* stream) {
    if (!b) return fail(SR_ERR_INVALID_ARG, "NULL batch");
    if (b->inflight) return fail(SR_ERR_INVALID_ARG, "batch already has a frame in flight");
    sr_batch_render_opts d;
    SR_TRY(batch_opts(o, &d));
    if (d.record_capacity < 0) return fail(SR_ERR_INVALID_ARG, "sr_batch_enqueue needs record_capacity >= 0");
    b->pending = d;
    b->pending_stream = static_cast<cudaStream_t>(stream);
    return batch_enqueue(b, d, b->pending_stream);
}

sr_status sr_batch_query(sr_batch* b, int* done) {
    if (!b || !done) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (!b->inflight) {
        *done = 1;
        return SR_OK;
    }
    CUDA_TRY(cudaSetDevice(b->p.device));
    cudaError_t e = cudaEventQuery(b->done);
    if (e == cudaErrorNotReady) {
        *done = 0;
        return SR_OK;
    }
    CUDA_TRY(e);
    *done = 1;
    return SR_OK;
}

sr_status sr_batch_finish(sr_batch* b) {
    if (!b) return fail(SR_ERR_INVALID_ARG, "NULL batch");
    if (!b->inflight) return fail(SR_ERR_INVALID_ARG, "no frame in flight");
    return batch_finish(b, b->pending, b->pending_stream);
}

sr_status sr_batch_get_image(sr_batch* b, uint32_t index, void* rgba_out, int out_is_device, void* stream) {
    if (!b || !rgba_out || index >= b->p.S) return fail(SR_ERR_INVALID_ARG, "bad argument");
    const sr::SceneInfo& si = b->p.info[index];
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CUDA_TRY(cudaSetDevice(b->p.device));
    CUDA_TRY(cudaMemcpyAsync(rgba_out, b->p.image.as<uint32_t>() + si.image_off, (size_t)si.W * si.H * 4,
                             out_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    if (!out_is_device) CUDA_TRY(cudaStreamSynchronize(st));
    return SR_OK;
}

sr_status sr_batch_info(const sr_batch* b, uint32_t index, uint32_t* width, uint32_t* height) {
    if (!b || index >= b->h.info.size()) return fail(SR_ERR_INVALID_ARG, "bad argument");
    if (width) *width = (uint32_t)b->h.info[index].W;
    if (height) *height = (uint32_t)b->h.info[index].H;
    return SR_OK;
}

sr_status sr_batch_get_stats(const sr_batch* cb, sr_batch_stats* out) {
    if (!cb || !out) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    sr_batch* b = const_cast<sr_batch*>(cb);
    SR_TRY(b->p.collect_events());
    std::memset(out, 0, sizeof *out);
    out->frame = b->p.stats;
    out->n_scenes = (uint32_t)b->h.info.size();
    out->n_paths = b->h.n_paths();
    out->n_curves = b->h.n_curves();
    out->record_capacity = b->p.last_cap;
    out->overflows = b->overflows;
    out->refits = b->refits;
    out->graph_captured = b->exec != nullptr;
    return SR_OK;
}

sr_status sr_batch_clear(sr_batch* b) {
    if (!b) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    b->h.clear();
    b->committed = false;
    return SR_OK;
}

void sr_batch_destroy(sr_batch* b) {
    if (!b) return;
    cudaSetDevice(b->p.device);
    cudaDeviceSynchronize();
    delete b;
}

// ------------------------------------------------------- learned sizing ---

sr_status sr_sizer_create(int device, uint64_t seed, sr_sizer** out) {
    if (!out) return fail(SR_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    int ndev = 0;
    CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(SR_ERR_INVALID_ARG, "device %d not present", device);
    CUDA_TRY(cudaSetDevice(device));
    sr_sizer* s = new sr_sizer();
    s->device = device;
    cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, device);
    const size_t pb = sizeof(float) * sr::kMlpParams;
    auto alloc = [&]() -> cudaError_t {
        cudaError_t e;
        if ((e = ensure(s->master, pb)) || (e = ensure(s->wb, 2 * (size_t)sr::kMlpParams)) ||
            (e = ensure(s->grad, pb)) || (e = ensure(s->m, pb)) || (e = ensure(s->v, pb)) ||
            (e = ensure(s->norm, sizeof(float) * sr::kMlpNorm)) || (e = ensure(s->loss, sizeof(float) * 4)) ||
            (e = ensure(s->ctl, sizeof(uint32_t) * 4)) || (e = cudaMallocHost(&s->h_loss, sizeof(float) * 4)))
            return e;
        return cudaSuccess;
    };
    cudaError_t e = alloc();
    if (e != cudaSuccess) {
        delete s;
        CUDA_TRY(e);
    }
    // weights: uniform with variance 1/fan_in from a splitmix64 stream
    std::vector<float> w(sr::kMlpParams, 0.0f);
    uint64_t state = seed;
    auto next = [&]() {
        uint64_t z = (state += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    const int H = sr::kMlpHidden, I = sr::kMlpIn, O = sr::kMlpOut;
    struct Layer { int off, rows, fan_in; } layers[3] = {{0, H, I}, {H * I + H, H, H}, {H * I + H + H * H + H, O, H}};
    for (const Layer& l : layers) {
        const double a = std::sqrt(3.0 / l.fan_in);
        for (int i = 0; i < l.rows * l.fan_in; ++i) w[(size_t)l.off + i] = (float)((2.0 * next() - 1.0) * a);
    }
    float nm[sr::kMlpNorm];
    for (int i = 0; i < sr::kMlpNorm; ++i) nm[i] = 0.0f;
    for (int i = 0; i < I; ++i) nm[I + i] = 1.0f;
    for (int i = 0; i < O; ++i) nm[2 * I + O + i] = 1.0f;
    sr_status st = sr_sizer_set_state(s, w.data(), nullptr, nullptr, nm, 0);
    if (st != SR_OK) {
        delete s;
        return st;
    }
    *out = s;
    return SR_OK;
}

void sr_sizer_destroy(sr_sizer* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    cudaDeviceSynchronize();
    delete s;
}

sr_status sr_sizer_set_norm(sr_sizer* s, const float norm[SR_SIZER_NORM]) {
    if (!s || !norm) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    for (int i = 0; i < sr::kMlpNorm; ++i)
        if (!std::isfinite(norm[i])) return fail(SR_ERR_INVALID_ARG, "normaliser entry %d is not finite", i);
    for (int i = 0; i < sr::kMlpOut; ++i)
        if (!(norm[2 * sr::kMlpIn + sr::kMlpOut + i] > 0.0f)) return fail(SR_ERR_INVALID_ARG, "y_std must be > 0");
    CUDA_TRY(cudaSetDevice(s->device));
    CUDA_TRY(cudaMemcpy(s->norm.p, norm, sizeof(float) * sr::kMlpNorm, cudaMemcpyHostToDevice));
    return SR_OK;
}

sr_status sr_sizer_get_state(const sr_sizer* s, float* params, float* adam_m, float* adam_v, float norm[SR_SIZER_NORM],
                             int64_t* step) {
    if (!s) return fail(SR_ERR_INVALID_ARG, "NULL sizer");
    CUDA_TRY(cudaSetDevice(s->device));
    const size_t pb = sizeof(float) * sr::kMlpParams;
    if (params) CUDA_TRY(cudaMemcpy(params, s->master.p, pb, cudaMemcpyDeviceToHost));
    if (adam_m) CUDA_TRY(cudaMemcpy(adam_m, s->m.p, pb, cudaMemcpyDeviceToHost));
    if (adam_v) CUDA_TRY(cudaMemcpy(adam_v, s->v.p, pb, cudaMemcpyDeviceToHost));
    if (norm) CUDA_TRY(cudaMemcpy(norm, s->norm.p, sizeof(float) * sr::kMlpNorm, cudaMemcpyDeviceToHost));
    if (step) *step = s->step;
    return SR_OK;
}

sr_status sr_sizer_set_state(sr_sizer* s, const float* params, const float* adam_m, const float* adam_v,
                             const float norm[SR_SIZER_NORM], int64_t step) {
    if (!s || step < 0) return fail(SR_ERR_INVALID_ARG, "bad argument");
    CUDA_TRY(cudaSetDevice(s->device));
    const size_t pb = sizeof(float) * sr::kMlpParams;
    if (norm) SR_TRY(sr_sizer_set_norm(s, norm));
    if (params) {
        for (int i = 0; i < sr::kMlpParams; ++i)
            if (!std::isfinite(params[i])) return fail(SR_ERR_INVALID_ARG, "parameter %d is not finite", i);
        CUDA_TRY(cudaMemcpy(s->master.p, params, pb, cudaMemcpyHostToDevice));
        sr::launch_to_bf16(s->master.as<float>(), s->wb.p, nullptr);
        CUDA_TRY(cudaGetLastError());
    }
    if (adam_m) CUDA_TRY(cudaMemcpy(s->m.p, adam_m, pb, cudaMemcpyHostToDevice));
    else CUDA_TRY(cudaMemset(s->m.p, 0, pb));
    if (adam_v) CUDA_TRY(cudaMemcpy(s->v.p, adam_v, pb, cudaMemcpyHostToDevice));
    else CUDA_TRY(cudaMemset(s->v.p, 0, pb));
    CUDA_TRY(cudaMemset(s->grad.p, 0, pb));
    s->step = step;
    CUDA_TRY(cudaDeviceSynchronize());
    return SR_OK;
}

sr_status sr_sizer_loss_grad(sr_sizer* s, const float* d_x, const float* d_t, uint32_t n, float* h_grad,
                             float* h_loss) {
    if (!s || (n && (!d_x || !d_t))) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (n == 0) return fail(SR_ERR_INVALID_ARG, "no rows");
    CUDA_TRY(cudaSetDevice(s->device));
    const size_t pb = sizeof(float) * sr::kMlpParams;
    CUDA_TRY(cudaMemset(s->grad.p, 0, pb));
    CUDA_TRY(cudaMemset(s->loss.p, 0, sizeof(float)));
    CUDA_TRY(sr::launch_mlp_grad(s->wb.p, s->master.as<float>(), s->norm.as<float>(), d_x, d_t, nullptr, n,
                                 s->grad.as<float>(), s->loss.as<float>(), nullptr));
    float loss = 0.0f;
    CUDA_TRY(cudaMemcpy(&loss, s->loss.p, sizeof(float), cudaMemcpyDeviceToHost));
    if (h_grad) CUDA_TRY(cudaMemcpy(h_grad, s->grad.p, pb, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemset(s->grad.p, 0, pb));
    if (h_loss) *h_loss = loss / ((float)n * (float)sr::kMlpOut);
    return SR_OK;
}

sr_status sr_sizer_train(sr_sizer* s, const float* d_x, const float* d_t, uint32_t n, const sr_sizer_train_opts* o,
                         float* h_loss, void* stream) {
    if (!s || (n && (!d_x || !d_t))) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    sr_sizer_train_opts d{};
    d.struct_size = sizeof d;
    d.batch = 4096;
    d.epochs = 1;
    d.shuffle = 1;
    d.lr = 1e-3f;
    d.beta1 = 0.9f;
    d.beta2 = 0.999f;
    d.eps = 1e-8f;
    if (o) {
        if (o->struct_size < sizeof d) return fail(SR_ERR_INVALID_ARG, "opts.struct_size too small");
        d = *o;
    }
    if (n == 0 || d.batch == 0 || d.epochs == 0) return fail(SR_ERR_INVALID_ARG, "empty training run");
    if (!(d.lr > 0.0f) || !(d.beta1 >= 0.0f && d.beta1 < 1.0f) || !(d.beta2 >= 0.0f && d.beta2 < 1.0f) ||
        !(d.eps > 0.0f))
        return fail(SR_ERR_INVALID_ARG, "bad optimiser settings");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CUDA_TRY(cudaSetDevice(s->device));
    uint32_t* idx = nullptr;
    sr::SortPlan sp = sr::sort_plan(n, 32, nullptr);
    if (d.shuffle) {
        CUDA_TRY(ensure(s->keys, sizeof(uint32_t) * n));
        CUDA_TRY(ensure(s->keys_out, sizeof(uint32_t) * n));
        CUDA_TRY(ensure(s->perm, sizeof(uint32_t) * n));
        CUDA_TRY(ensure(s->alt_k, sizeof(uint32_t) * n));
        CUDA_TRY(ensure(s->alt_v, sizeof(uint32_t) * n));
        CUDA_TRY(ensure(s->sort_scratch, sr::sort_scratch_bytes(sp)));
        idx = s->perm.as<uint32_t>();
    }
    CUDA_TRY(cudaMemsetAsync(s->ctl.p, 0, sizeof(uint32_t) * 4, st));
    const double b1 = d.beta1, b2 = d.beta2;
    for (uint32_t ep = 0; ep < d.epochs; ++ep) {
        CUDA_TRY(cudaMemsetAsync(s->loss.p, 0, sizeof(float), st));
        if (d.shuffle) {
            sr::launch_perm_keys(s->keys.as<uint32_t>(), n, d.seed * 0x100000001B3ull + ep, st);
            sr::launch_sort_u32(sp, s->keys.as<uint32_t>(), nullptr, s->keys_out.as<uint32_t>(), idx,
                                s->alt_k.as<uint32_t>(), s->alt_v.as<uint32_t>(), s->sort_scratch.p,
                                s->ctl.as<uint32_t>(), st);
        }
        for (uint32_t b0 = 0; b0 < n; b0 += d.batch) {
            const uint32_t nb = std::min(d.batch, n - b0);
            CUDA_TRY(sr::launch_mlp_grad(s->wb.p, s->master.as<float>(), s->norm.as<float>(), d_x, d_t,
                                         idx ? idx + b0 : nullptr, nb, s->grad.as<float>(), s->loss.as<float>(),
                                         st));
            ++s->step;
            const float bc1 = (float)(1.0 - std::pow(b1, (double)s->step));
            const float bc2 = (float)(1.0 - std::pow(b2, (double)s->step));
            sr::launch_adam(s->master.as<float>(), s->wb.p, s->grad.as<float>(), s->m.as<float>(), s->v.as<float>(),
                            d.lr, d.beta1, d.beta2, d.eps, bc1, bc2, st);
            if (!idx) {   // unshuffled minibatches are consecutive rows
                d_x += (size_t)nb * sr::kMlpIn;
                d_t += (size_t)nb * sr::kMlpOut;
            }
        }
        if (!idx) {
            d_x -= (size_t)n * sr::kMlpIn;
            d_t -= (size_t)n * sr::kMlpOut;
        }
    }
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(s->h_loss, s->loss.p, sizeof(float), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(s->h_loss + 1, s->ctl.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    uint32_t status = 0;
    std::memcpy(&status, s->h_loss + 1, sizeof status);
    SR_TRY(check_status_word(status));
    if (h_loss) *h_loss = s->h_loss[0] / ((float)n * (float)sr::kMlpOut);
    return SR_OK;
}

sr_status sr_sizer_predict(const sr_sizer* s, const float* d_x, uint32_t n, float* d_y, void* stream) {
    if (!s || (n && (!d_x || !d_y))) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    CUDA_TRY(cudaSetDevice(s->device));
    sr::launch_mlp_predict(s->wb.p, s->master.as<float>(), s->norm.as<float>(), d_x, n, d_y, s->sm_count,
                           static_cast<cudaStream_t>(stream));
    CUDA_TRY(cudaGetLastError());
    return SR_OK;
}

sr_status sr_batch_path_features(sr_batch* b, float* d_feats, void* stream) {
    if (!b || !d_feats) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (!b->committed) SR_TRY(sr_batch_commit(b));
    Pipeline& p = b->p;
    CUDA_TRY(cudaSetDevice(p.device));
    SR_TRY(batch_path_first(b));
    SR_TRY(p.prepare_front());
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CUDA_TRY(cudaMemsetAsync(p.path_visible.p, 0, sizeof(int32_t) * std::max<uint32_t>(p.P, 1), st));
    sr::launch_transform(p.pos.as<float2>(), p.pos_path.as<uint32_t>(), p.V, p.table(), p.tpos.as<float2>(),
                         p.path_visible.as<int32_t>(), st);
    if (p.arcs)
        sr::launch_arc_fixup(p.curve_type.as<uint32_t>(), p.curve_pos.as<uint32_t>(), p.curve_path.as<uint32_t>(), p.C,
                             p.pos.as<float2>(), p.table(), p.tpos.as<float2>(), p.path_visible.as<int32_t>(), st);
    sr::launch_path_features(p.geom(0), p.path_first.as<uint32_t>(), p.P, d_feats, st);
    CUDA_TRY(cudaGetLastError());
    return SR_OK;
}

// An exact frame with per-path draw counters (the exact count pass).
static sr_status counted_frame(sr_batch* b, cudaStream_t st) {
    Pipeline& p = b->p;
    SR_TRY(batch_path_first(b));
    CUDA_TRY(ensure(p.path_draw, sizeof(uint32_t) * std::max<uint32_t>(p.P, 1)));
    p.count_paths = true;
    sr_status s = p.frame(st, -1);
    p.count_paths = false;
    SR_TRY(s);
    return p.finish(st);
}

sr_status sr_batch_path_labels(sr_batch* b, float* d_labels, void* stream) {
    if (!b || !d_labels) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (!b->committed) SR_TRY(sr_batch_commit(b));
    Pipeline& p = b->p;
    CUDA_TRY(cudaSetDevice(p.device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    SR_TRY(counted_frame(b, st));
    sr::launch_path_labels(p.path_first.as<uint32_t>(), p.P, p.count.as<int32_t>(), p.path_draw.as<uint32_t>(),
                           d_labels, st);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(st));
    return SR_OK;
}

sr_status sr_batch_plan(sr_batch* b, const sr_sizer* sz, const sr_sizing_margins* mg, sr_sizing_plan* plan,
                        int64_t* scene_caps, void* stream) {
    if (!b || !sz || !mg || !plan) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (mg->struct_size < sizeof(sr_sizing_margins)) return fail(SR_ERR_INVALID_ARG, "margins.struct_size too small");
    const float margins[4] = {mg->path_records, mg->path_draws, mg->frame_records, mg->frame_draws};
    for (float m : margins)
        if (!std::isfinite(m)) return fail(SR_ERR_INVALID_ARG, "margins must be finite");
    if (!b->committed) SR_TRY(sr_batch_commit(b));
    Pipeline& p = b->p;
    if (sz->device != p.device) return fail(SR_ERR_INVALID_ARG, "sizer and batch on different devices");
    CUDA_TRY(cudaSetDevice(p.device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t p1 = std::max<uint32_t>(p.P, 1);
    CUDA_TRY(ensure(p.feats, sizeof(float) * sr::kMlpIn * p1));
    CUDA_TRY(ensure(p.preds, sizeof(float) * sr::kMlpOut * p1));
    CUDA_TRY(ensure(p.allot, sizeof(uint32_t) * 2 * p1));
    const size_t tot_words = 4 + 2 * (size_t)p.S;
    CUDA_TRY(ensure(p.plan_tot, sizeof(unsigned long long) * tot_words));
    SR_TRY(sr_batch_path_features(b, p.feats.as<float>(), stream));
    SR_TRY(sr_sizer_predict(sz, p.feats.as<float>(), p.P, p.preds.as<float>(), stream));
    CUDA_TRY(cudaMemsetAsync(p.plan_tot.p, 0, sizeof(unsigned long long) * tot_words, st));
    unsigned long long* tot = p.plan_tot.as<unsigned long long>();
    sr::launch_allot(p.preds.as<float>(), p.P, p.path_scene.as<uint32_t>(), margins, p.allot.as<uint32_t>(),
                     tot + 4, tot, st);
    CUDA_TRY(cudaGetLastError());
    if (p.h_plan_words < tot_words) {
        if (p.h_plan_ptr) cudaFreeHost(p.h_plan_ptr);
        p.h_plan_ptr = nullptr;
        p.h_plan_words = 0;
        CUDA_TRY(cudaMallocHost(&p.h_plan_ptr, sizeof(unsigned long long) * tot_words));
        p.h_plan_words = tot_words;
    }
    unsigned long long* h = p.h_plan_ptr;
    CUDA_TRY(cudaMemcpyAsync(h, tot, sizeof(unsigned long long) * tot_words, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    plan->records = (int64_t)h[0];
    plan->draws = (int64_t)std::min<unsigned long long>(std::max<unsigned long long>(h[1], 1), 2 * std::max(h[0], 1ull));
    plan->path_records = (int64_t)h[2];
    plan->path_draws = (int64_t)h[3];
    plan->device_bytes = p.frame_bytes(plan->records, plan->draws);
    if (scene_caps)
        for (size_t i = 0; i < 2 * (size_t)p.S; ++i) scene_caps[i] = (int64_t)h[4 + i];
    p.planned = true;
    return SR_OK;
}

sr_status sr_batch_path_ranges(const sr_batch* b, uint32_t* path_begin) {
    if (!b || !path_begin) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    const auto& info = b->h.info;
    for (size_t i = 0; i < info.size(); ++i) path_begin[i] = info[i].path_begin;
    path_begin[info.size()] = b->h.n_paths();
    return SR_OK;
}

sr_status sr_batch_judge(sr_batch* b, sr_sizing_judge* out, void* stream) {
    if (!b || !out) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    Pipeline& p = b->p;
    if (!b->committed || !p.planned) return fail(SR_ERR_INVALID_ARG, "sr_batch_judge needs a plan of this batch");
    CUDA_TRY(cudaSetDevice(p.device));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    SR_TRY(counted_frame(b, st));
    CUDA_TRY(ensure(p.judge_out, sizeof(unsigned long long) * 4));
    CUDA_TRY(cudaMemsetAsync(p.judge_out.p, 0, sizeof(unsigned long long) * 4, st));
    sr::launch_judge(p.path_first.as<uint32_t>(), p.P, p.count.as<int32_t>(), p.path_draw.as<uint32_t>(),
                     p.allot.as<uint32_t>(), p.judge_out.as<unsigned long long>(), st);
    CUDA_TRY(cudaGetLastError());
    unsigned long long h[4];
    CUDA_TRY(cudaMemcpyAsync(h, p.judge_out.p, sizeof h, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    std::memset(out, 0, sizeof *out);
    out->paths = p.P;
    out->paths_over_records = (uint32_t)h[0];
    out->paths_over_draws = (uint32_t)h[1];
    out->records = (int64_t)h[2];
    out->draws = (int64_t)h[3];
    return SR_OK;
}

// ------------------------------------------------------------- tuning ---

static sr_status check_tuning(const sr_tuning* t) {
    if (!t || t->struct_size < sizeof(sr_tuning)) return fail(SR_ERR_INVALID_ARG, "bad sr_tuning");
    if ((t->sort_items != 8 && t->sort_items != 12 && t->sort_items != 16) ||
        (t->resolve_warps != 8 && t->resolve_warps != 16) || (t->wind_items != 4 && t->wind_items != 8) ||
        (t->sort_kind != 0 && t->sort_kind != 1))
        return fail(SR_ERR_INVALID_ARG,
                    "tuning values: sort_items 8/12/16, resolve_warps 8/16, wind_items 4/8, sort_kind 0/1");
    return SR_OK;
}

static sr_status apply_tuning(Pipeline& p, const sr_tuning& t) {
    const bool warps_changed = t.resolve_warps != p.tune.resolve_warps;
    p.tune = t;
    p.tune.struct_size = sizeof(sr_tuning);
    if (warps_changed && p.loaded) {   // resolve CTAs per scene depend on the warps per CTA
        CUDA_TRY(cudaSetDevice(p.device));
        SR_TRY(p.upload_table());
    }
    return SR_OK;
}

static void drop_graph(sr_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->graph_cap = -1;
    b->graph_dcap = -1;
}

sr_status sr_set_tuning(sr_ctx* c, const sr_tuning* t) {
    if (!c) return fail(SR_ERR_INVALID_ARG, "NULL context");
    SR_TRY(check_tuning(t));
    return apply_tuning(c->p, *t);
}

sr_status sr_batch_set_tuning(sr_batch* b, const sr_tuning* t) {
    if (!b) return fail(SR_ERR_INVALID_ARG, "NULL batch");
    if (b->inflight) return fail(SR_ERR_INVALID_ARG, "tuning while a frame is in flight");
    SR_TRY(check_tuning(t));
    drop_graph(b);
    return apply_tuning(b->p, *t);
}

sr_status sr_batch_get_tuning(const sr_batch* b, sr_tuning* t) {
    if (!b || !t) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    *t = b->p.tune;
    return SR_OK;
}

static std::string tuning_class(const Pipeline& p) {
    uint32_t side = 256;
    while (side < (uint32_t)std::max(p.Wmax, p.Hmax) && side < (1u << 15)) side <<= 1;
    uint32_t r = 0;
    while (r < 40 && (1ll << (r + 1)) <= std::max<int64_t>(p.last_N, 1)) ++r;
    char buf[64];
    snprintf(buf, sizeof buf, "m%d/s%u/r%u", p.mode, side, r);
    return buf;
}

sr_status sr_batch_tuning_class(sr_batch* b, char* buf, size_t len) {
    if (!b || !buf || len == 0) return fail(SR_ERR_INVALID_ARG, "bad argument");
    if (!b->committed) SR_TRY(sr_batch_commit(b));
    if (b->p.last_N <= 0) SR_TRY(sr_batch_render(b, nullptr, nullptr));
    snprintf(buf, len, "%s", tuning_class(b->p).c_str());
    return SR_OK;
}

// The tuning cache: a JSON object with one entry per line,
//   "<class>": {"sort_items": 12, "resolve_warps": 16, "wind_items": 8, "frame_ms": 1.234},
// read and rewritten whole; lines it does not recognise are dropped.
struct TuneEntry {
    sr_tuning t;
    double ms;
};

static std::map<std::string, TuneEntry> read_tuning_cache(const char* path) {
    std::map<std::string, TuneEntry> m;
    if (!path) return m;
    std::ifstream in(path);
    std::string line;
    auto field = [](const std::string& l, const char* name, double* v) {
        const std::string key = std::string("\"") + name + "\":";
        size_t at = l.find(key);
        if (at == std::string::npos) return false;
        *v = std::strtod(l.c_str() + at + key.size(), nullptr);
        return true;
    };
    while (std::getline(in, line)) {
        size_t q0 = line.find('"');
        size_t q1 = q0 == std::string::npos ? q0 : line.find('"', q0 + 1);
        if (q1 == std::string::npos || line.find('{', q1) == std::string::npos) continue;
        double si = 0, rw = 0, wi = 0, sk = 0, ms = 0;
        if (!field(line, "sort_items", &si) || !field(line, "resolve_warps", &rw) || !field(line, "wind_items", &wi))
            continue;
        field(line, "sort_kind", &sk);
        field(line, "frame_ms", &ms);
        TuneEntry e{{sizeof(sr_tuning), (int32_t)si, (int32_t)rw, (int32_t)wi, (int32_t)sk}, ms};
        if (check_tuning(&e.t) == SR_OK) m[line.substr(q0 + 1, q1 - q0 - 1)] = e;
    }
    return m;
}

static sr_status write_tuning_cache(const char* path, const std::map<std::string, TuneEntry>& m) {
    const std::string tmp = std::string(path) + ".tmp";
    {
        std::ofstream out(tmp);
        if (!out) return fail(SR_ERR_INVALID_ARG, "cannot write tuning cache %s", path);
        out << "{\n";
        size_t i = 0;
        for (const auto& kv : m) {
            char buf[256];
            snprintf(buf, sizeof buf,
                     "  \"%s\": {\"sort_kind\": %d, \"sort_items\": %d, \"resolve_warps\": %d, "
                     "\"wind_items\": %d, \"frame_ms\": %.4f}%s\n",
                     kv.first.c_str(), kv.second.t.sort_kind, kv.second.t.sort_items, kv.second.t.resolve_warps,
                     kv.second.t.wind_items, kv.second.ms, ++i < m.size() ? "," : "");
            out << buf;
        }
        out << "}\n";
    }
    if (std::rename(tmp.c_str(), path) != 0) return fail(SR_ERR_INVALID_ARG, "cannot replace %s", path);
    return SR_OK;
}

// Device time of the batch's frame with a pre-sized capacity: the best of
// `reps` frames (CUDA events on the stream).
static sr_status time_frames(sr_batch* b, int64_t cap, int reps, cudaStream_t st, float* best) {
    sr_batch_render_opts o{};
    o.struct_size = sizeof o;
    o.record_capacity = cap;
    o.refit_on_overflow = 1;
    o.draw_capacity = -1;
    cudaEvent_t e0, e1;
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    *best = 1e30f;
    sr_status s = sr_batch_render(b, &o, st);   // warm (allocations at this tuning)
    for (int i = 0; i < reps && s == SR_OK; ++i) {
        cudaEventRecord(e0, st);
        s = sr_batch_render(b, &o, st);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        *best = std::min(*best, ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return s;
}

sr_status sr_batch_autotune(sr_batch* b, const char* cache_path, int force, sr_tuning* chosen, void* stream) {
    if (!b) return fail(SR_ERR_INVALID_ARG, "NULL batch");
    if (b->inflight) return fail(SR_ERR_INVALID_ARG, "autotune while a frame is in flight");
    if (!b->committed) SR_TRY(sr_batch_commit(b));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Pipeline& p = b->p;
    SR_TRY(sr_batch_render(b, nullptr, stream));   // exact frame: the record count of the class
    const std::string cls = tuning_class(p);
    std::map<std::string, TuneEntry> cache = read_tuning_cache(cache_path);
    auto it = cache.find(cls);
    if (it != cache.end() && !force) {
        SR_TRY(sr_batch_set_tuning(b, &it->second.t));
        if (chosen) *chosen = p.tune;
        return SR_OK;
    }
    const int64_t cap = p.last_N;
    sr_tuning best = p.tune;
    float best_ms = 0;
    SR_TRY(time_frames(b, cap, 3, st, &best_ms));
    const int kind_opts[] = {0, 1}, sort_opts[] = {8, 12, 16}, warp_opts[] = {8, 16}, wind_opts[] = {4, 8};
    for (int knob = 0; knob < 4; ++knob) {
        // the radix sort's tile only matters when the radix sort is chosen
        if (knob == 1 && best.sort_kind == 0) continue;
        const int* opts = knob == 0 ? kind_opts : knob == 1 ? sort_opts : knob == 2 ? warp_opts : wind_opts;
        const int n = knob == 1 ? 3 : 2;
        for (int i = 0; i < n; ++i) {
            sr_tuning t = best;
            int32_t& v = knob == 0 ? t.sort_kind : knob == 1 ? t.sort_items : knob == 2 ? t.resolve_warps : t.wind_items;
            if (v == opts[i]) continue;
            v = opts[i];
            SR_TRY(sr_batch_set_tuning(b, &t));
            float ms = 0;
            SR_TRY(time_frames(b, cap, 3, st, &ms));
            if (ms < best_ms) {
                best_ms = ms;
                best = t;
            }
        }
    }
    SR_TRY(sr_batch_set_tuning(b, &best));
    if (cache_path) {
        cache[cls] = TuneEntry{best, (double)best_ms};
        SR_TRY(write_tuning_cache(cache_path, cache));
    }
    if (chosen) *chosen = best;
    return SR_OK;
}

sr_status sr_batch_release(sr_batch* b) {
    if (!b) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (b->inflight) return fail(SR_ERR_INVALID_ARG, "release while a frame is in flight");
    CUDA_TRY(cudaSetDevice(b->p.device));
    CUDA_TRY(cudaDeviceSynchronize());
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->graph_cap = -1;
    b->graph_dcap = -1;
    b->p.release_post_count();
    return SR_OK;
}

sr_status sr_batch_held_bytes(const sr_batch* b, uint64_t* bytes) {
    if (!b || !bytes) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    *bytes = b->p.held_bytes();
    return SR_OK;
}

sr_status sr_batch_reserve_like(sr_batch* b, const sr_batch* model) {
    if (!b || !model) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    if (b == model) return SR_OK;
    if (b->inflight) return fail(SR_ERR_INVALID_ARG, "reserve while a frame is in flight");
    if (b->p.device != model->p.device) return fail(SR_ERR_INVALID_ARG, "batches on different devices");
    bool moved = false;
    const sr_status rs = b->p.reserve_like(model->p, &moved);
    if (moved) {
        // the moved buffers' contents are gone: the next frame uploads the
        // scenes again (and plans again); a captured frame holds the old
        // addresses
        b->committed = false;
        b->p.planned = false;
        b->p.path_first_valid = false;
        b->p.stages_valid = false;
        if (b->exec) cudaGraphExecDestroy(b->exec);
        if (b->graph) cudaGraphDestroy(b->graph);
        b->exec = nullptr;
        b->graph = nullptr;
        b->graph_cap = -1;
        b->graph_dcap = -1;
    }
    return rs;
}

sr_status sr_batch_frame_bytes(sr_batch* b, int64_t records, int64_t draws, uint64_t* bytes) {
    if (!b || !bytes || records < 0) return fail(SR_ERR_INVALID_ARG, "bad argument");
    if (!b->committed) SR_TRY(sr_batch_commit(b));
    *bytes = b->p.frame_bytes(records, draws);
    return SR_OK;
}

void* sr_device_alloc(int device, size_t bytes) {
    if (cudaSetDevice(device) != cudaSuccess) return nullptr;
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(bytes, 1)) != cudaSuccess) return nullptr;
    return p;
}

void sr_device_free(void* p) {
    if (p) cudaFree(p);
}

sr_status sr_memcpy(void* dst, const void* src, size_t bytes) {
    if (!bytes) return SR_OK;
    if (!dst || !src) return fail(SR_ERR_INVALID_ARG, "NULL pointer");
    CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyDefault));
    return SR_OK;
}

}  // extern "C"

static sr_status batch_path_first(sr_batch* b) {
    Pipeline& p = b->p;
    if (p.path_first_valid) return SR_OK;
    const std::vector<uint32_t>& cp = b->h.curve_path;
    std::vector<uint32_t> first((size_t)p.P + 1);
    uint32_t c = 0;
    for (uint32_t i = 0; i <= p.P; ++i) {
        while (c < p.C && cp[c] < i) ++c;
        first[i] = c;
    }
    CUDA_TRY(ensure(p.path_first, sizeof(uint32_t) * first.size()));
    CUDA_TRY(cudaMemcpy(p.path_first.p, first.data(), sizeof(uint32_t) * first.size(), cudaMemcpyHostToDevice));
    p.path_first_valid = true;
    return SR_OK;
}
