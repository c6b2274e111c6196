// api.cu — context, device memory and per-frame sequencing behind sr.h.
//
// ScanlineVGRasterizer::drawFrame (scanline_rasterizer.cpp:282-696) submits
// eleven compute dispatches with three blocking host read-backs, then draws
// the list through the graphics queue.  Here one frame is:
//   transform -> count -> offset scan -> [read N] -> intersect+fragment ->
//   onesweep sort -> winding/mark/emit -> [read O] -> row sort -> resolve
// on the caller's stream, with device buffers that only grow.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sr.h"
#include "kernels.h"

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

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    template <typename T> T* as() const { return static_cast<T*>(p); }
};

cudaError_t ensure(DevBuf& b, size_t bytes) {
    if (bytes <= b.cap && b.p) return cudaSuccess;
    if (b.p) {
        cudaFree(b.p);
        b.p = nullptr;
        b.cap = 0;
    }
    size_t want = std::max<size_t>(bytes + bytes / 4, 256);
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
    CTL_BUCKETS = 4,   // 4 chain-bucket counters
    CTL_LONG = 8,      // long-piece counter
    CTL_WORDS = 16,
};

std::atomic<uint64_t> g_launches{0};

}  // namespace

namespace sr {
sr_status report_error(sr_status s, const char* msg) { return fail(s, "%s", msg); }
void count_launches(uint32_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
uint64_t launches_so_far() { return g_launches.load(std::memory_order_relaxed); }
}  // namespace sr

enum Stage : int {
    ST_TRANSFORM = 0, ST_COUNT, ST_SCAN, ST_CHAINS, ST_MERGE, ST_FRAGMENT, ST_SORT, ST_WINDING, ST_ROWSORT,
    ST_RESOLVE, ST_COUNT_ALL
};

struct sr_ctx {
    int device = 0;
    int32_t W = 0, H = 0, mode = 0, F = 2;
    uint32_t flags = 0;
    sr::Mvp mvp;
    bool loaded = false;
    // scene
    uint32_t V = 0, C = 0, P = 0;
    DevBuf pos, pos_path, curve_pos, curve_type, curve_path, fill_rule, fill_info;
    // frame
    DevBuf tpos, path_visible, cut, count, offs, ctl, scan_status, pieces, chain_lists, long_list, cbuf, rec;
    int sm_count = 148;
    DevBuf keys, keys_alt, wnp, skeys, svals, vals_alt, sort_scratch, wind_status;
    DevBuf draw, draw_row, totals;
    DevBuf rkeys, rvals, rkeys_alt, rvals_alt, row_sort_scratch, row_start, image;
    DevBuf d_fkey, d_fwn, d_fleft, d_wscan, d_fflag, d_sflag, d_skey;
    // pinned host scalars
    int32_t* h_n = nullptr;        // [2] N, status
    uint64_t* h_tot = nullptr;     // [3] frags, spans, status
    sr_stats stats{};
    int64_t last_N = 0, last_O = 0;
    bool stages_valid = false;
    // profiling: a start/end event per stage
    cudaEvent_t ev[2 * ST_COUNT_ALL] = {};
    bool ev_pending = false;
    cudaStream_t cur_stream = nullptr;

    void mark(int stage, bool end) {
        if (!(flags & SR_FLAG_PROFILE)) return;
        cudaEvent_t& e = ev[2 * stage + (end ? 1 : 0)];
        if (!e) cudaEventCreate(&e);
        cudaEventRecord(e, cur_stream);
    }

    ~sr_ctx() {
        DevBuf* all[] = {&pos, &pos_path, &curve_pos, &curve_type, &curve_path, &fill_rule, &fill_info,
                         &tpos, &path_visible, &cut, &count, &offs, &ctl, &scan_status, &pieces, &chain_lists,
                         &long_list,
                         &cbuf, &rec, &keys, &keys_alt,
                         &wnp, &skeys, &svals, &vals_alt, &sort_scratch, &wind_status, &draw, &draw_row,
                         &totals, &rkeys, &rvals, &rkeys_alt, &rvals_alt, &row_sort_scratch, &row_start,
                         &image, &d_fkey, &d_fwn, &d_fleft, &d_wscan, &d_fflag, &d_sflag, &d_skey};
        for (DevBuf* b : all) release(*b);
        for (cudaEvent_t e : ev)
            if (e) cudaEventDestroy(e);
        if (h_n) cudaFreeHost(h_n);
        if (h_tot) cudaFreeHost(h_tot);
    }

    sr::KeyLayout layout() const {
        sr::KeyLayout L;
        L.F = F;
        L.W = W;
        L.H = H;
        L.Hy = (H + F - 1) / F;
        L.xbits = bits_for((uint64_t)((W & ~1) / F + 2));
        L.rbits = bits_for((uint64_t)L.Hy);
        L.pbits = bits_for(P > 0 ? (uint64_t)(P - 1) : 0);
        return L;
    }
};

static sr_status check_status_word(uint32_t s) {
    if (s == 0) return SR_OK;
    if (s & sr::ERR_LOOKBACK_TIMEOUT) return fail(SR_ERR_TIMEOUT, "device look-back wait timed out (status 0x%x)", s);
    if (s & sr::ERR_CAPACITY) return fail(SR_ERR_OVERFLOW_REFIT, "device buffer capacity exceeded (status 0x%x)", s);
    return fail(SR_ERR_INTERNAL, "device consistency check failed (status 0x%x)", s);
}

static sr_status render_frame(sr_ctx* c, cudaStream_t st) {
    using namespace sr;
    const bool keep = (c->flags & SR_FLAG_KEEP_STAGES) != 0;
    const uint32_t V = c->V, C = c->C, P = c->P;
    CUDA_TRY(cudaSetDevice(c->device));
    CUDA_TRY(ensure(c->tpos, sizeof(float2) * std::max<uint32_t>(V, 1)));
    CUDA_TRY(ensure(c->path_visible, sizeof(int32_t) * std::max<uint32_t>(P, 1)));
    CUDA_TRY(ensure(c->cut, sizeof(float) * 5 * (size_t)std::max<uint32_t>(C, 1)));
    CUDA_TRY(ensure(c->count, sizeof(int32_t) * ((size_t)C + 1)));
    CUDA_TRY(ensure(c->offs, sizeof(int32_t) * ((size_t)C + 1)));
    CUDA_TRY(ensure(c->ctl, sizeof(uint32_t) * CTL_WORDS));
    CUDA_TRY(ensure(c->scan_status, sizeof(uint64_t) * scan_status_words(C)));
    CUDA_TRY(ensure(c->pieces, piece_table_bytes(std::max<uint32_t>(C, 1))));
    const uint32_t list_cap = chain_list_capacity(std::max<uint32_t>(C, 1));
    CUDA_TRY(ensure(c->chain_lists, sizeof(uint32_t) * 4 * (size_t)list_cap));
    CUDA_TRY(ensure(c->long_list, sizeof(uint32_t) * (size_t)list_cap));
    uint32_t* ctl = c->ctl.as<uint32_t>();
    uint32_t* status = ctl + CTL_STATUS;

    CUDA_TRY(cudaMemsetAsync(ctl, 0, sizeof(uint32_t) * CTL_WORDS, st));
    CUDA_TRY(cudaMemsetAsync(c->path_visible.p, 0, sizeof(int32_t) * std::max<uint32_t>(P, 1), st));
    CUDA_TRY(cudaMemsetAsync(c->scan_status.p, 0, sizeof(uint64_t) * scan_status_words(C), st));

    c->cur_stream = st;
    const uint64_t launches0 = launches_so_far();
    // K1 transform (transform_pos.comp)
    c->mark(ST_TRANSFORM, false);
    launch_transform(c->pos.as<float2>(), c->pos_path.as<uint32_t>(), V, c->mvp, (float)c->W, (float)c->H,
                     c->tpos.as<float2>(), c->path_visible.as<int32_t>(), st);
    c->mark(ST_TRANSFORM, true);
    GeomArgs g;
    g.n_curves = C;
    g.curve_type = c->curve_type.as<uint32_t>();
    g.curve_pos = c->curve_pos.as<uint32_t>();
    g.curve_path = c->curve_path.as<uint32_t>();
    g.tpos = c->tpos.as<float2>();
    g.path_visible = c->path_visible.as<int32_t>();
    g.W = c->W;
    g.H = c->H;
    g.F = c->F;
    g.pixel_mode = c->mode == SR_MODE_PIXEL;
    g.L = c->layout();
    // K2 count pass + K3 offset scan (make_intersection_0.comp, naive_scan.comp)
    ChainWork cw;
    cw.pieces = c->pieces.as<uint4>();
    cw.chain_lists = c->chain_lists.as<uint32_t>();
    cw.list_cap = list_cap;
    cw.bucket_count = ctl + CTL_BUCKETS;
    cw.long_list = c->long_list.as<uint32_t>();
    cw.long_count = ctl + CTL_LONG;
    c->mark(ST_COUNT, false);
    launch_count(g, c->cut.as<float>(), c->count.as<int32_t>(), cw, status, st);
    c->mark(ST_COUNT, true);
    c->mark(ST_SCAN, false);
    launch_exclusive_scan_i32(c->count.as<int32_t>(), c->offs.as<int32_t>(), C, c->scan_status.as<uint64_t>(),
                              ctl + CTL_SCAN_COUNTER, status, st);
    c->mark(ST_SCAN, true);
    CUDA_TRY(cudaGetLastError());
    // read back N, as the reference does (scanline_rasterizer.cpp:355-356)
    CUDA_TRY(cudaMemcpyAsync(&c->h_n[0], c->offs.as<int32_t>() + C, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(&c->h_n[1], status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    {
        sr_status s = check_status_word((uint32_t)c->h_n[1]);
        if (s != SR_OK) return s;
    }
    const int64_t N = c->h_n[0];
    if (N < 0 || N >= (1ll << 30)) return fail(SR_ERR_OVERFLOW_REFIT, "record count %lld out of range", (long long)N);
    c->last_N = N;
    const size_t n1 = (size_t)std::max<int64_t>(N, 1);

    CUDA_TRY(ensure(c->cbuf, sizeof(int32_t) * n1));
    CUDA_TRY(ensure(c->rec, sizeof(int2) * n1));
    CUDA_TRY(ensure(c->keys, sizeof(uint64_t) * n1));
    CUDA_TRY(ensure(c->keys_alt, sizeof(uint64_t) * n1));
    CUDA_TRY(ensure(c->skeys, sizeof(uint64_t) * n1));
    CUDA_TRY(ensure(c->wnp, n1));
    CUDA_TRY(ensure(c->svals, sizeof(uint32_t) * n1));
    CUDA_TRY(ensure(c->vals_alt, sizeof(uint32_t) * n1));
    DebugOut dbg{nullptr, nullptr, nullptr};
    if (keep) {
        CUDA_TRY(ensure(c->d_fkey, sizeof(int32_t) * n1));
        CUDA_TRY(ensure(c->d_fwn, sizeof(int32_t) * n1));
        CUDA_TRY(ensure(c->d_fleft, sizeof(int32_t) * n1));
        CUDA_TRY(ensure(c->d_wscan, sizeof(int32_t) * (n1 + 1)));
        CUDA_TRY(ensure(c->d_fflag, sizeof(int32_t) * n1));
        CUDA_TRY(ensure(c->d_sflag, sizeof(int32_t) * n1));
        CUDA_TRY(ensure(c->d_skey, sizeof(int32_t) * n1));
        dbg.fkey = c->d_fkey.as<int32_t>();
        dbg.fwn = c->d_fwn.as<int32_t>();
        dbg.fleft = c->d_fleft.as<int32_t>();
        CUDA_TRY(cudaMemsetAsync(c->d_wscan.p, 0, sizeof(int32_t) * (n1 + 1), st));
    }
    // K4 intersections: crossing chains, then the per-curve merge
    c->mark(ST_CHAINS, false);
    launch_chains(g, c->offs.as<int32_t>(), cw, c->cbuf.as<int32_t>(), c->sm_count, st);
    c->mark(ST_CHAINS, true);
    c->mark(ST_MERGE, false);
    launch_merge(g, c->offs.as<int32_t>(), cw, c->cbuf.as<int32_t>(), c->rec.as<int2>(), status, st);
    c->mark(ST_MERGE, true);
    // K5 fragments and sort keys
    c->mark(ST_FRAGMENT, false);
    launch_fragment(g, c->rec.as<int2>(), N, c->keys.as<uint64_t>(), c->wnp.as<uint8_t>(), dbg, st);
    c->mark(ST_FRAGMENT, true);
    CUDA_TRY(cudaGetLastError());

    // K6 sort by (path, row rank, x)
    const KeyLayout L = g.L;
    uint32_t key_bits = L.pbits + L.rbits + L.xbits;
    SortPlan sp = sort_plan(N, key_bits);
    CUDA_TRY(ensure(c->sort_scratch, sort_scratch_bytes(sp)));
    c->mark(ST_SORT, false);
    launch_sort_u64(sp, c->keys.as<uint64_t>(), nullptr, c->skeys.as<uint64_t>(), c->svals.as<uint32_t>(),
                    c->keys_alt.as<uint64_t>(), c->vals_alt.as<uint32_t>(), c->sort_scratch.p, status, st);
    c->mark(ST_SORT, true);
    CUDA_TRY(cudaGetLastError());

    // K7..K9 winding scan, flags and draw-list emit
    const int64_t draw_cap = 2 * (int64_t)n1;
    CUDA_TRY(ensure(c->draw, sizeof(int4) * (size_t)draw_cap));
    CUDA_TRY(ensure(c->draw_row, sizeof(uint32_t) * (size_t)draw_cap));
    CUDA_TRY(ensure(c->totals, sizeof(uint64_t) * 4));
    CUDA_TRY(ensure(c->wind_status, sizeof(uint64_t) * winding_status_words(N)));
    CUDA_TRY(cudaMemsetAsync(c->wind_status.p, 0, sizeof(uint64_t) * winding_status_words(N), st));
    CUDA_TRY(cudaMemsetAsync(c->totals.p, 0, sizeof(uint64_t) * 4, st));
    WindArgs wa;
    wa.n = N;
    wa.skeys = c->skeys.as<uint64_t>();
    wa.svals = c->svals.as<uint32_t>();
    wa.wnp = c->wnp.as<uint8_t>();
    wa.fill_rule = c->fill_rule.as<uint32_t>();
    wa.fill_info = c->fill_info.as<uint32_t>();
    wa.n_paths = P;
    wa.W = c->W;
    wa.H = c->H;
    wa.F = c->F;
    wa.pixel_mode = g.pixel_mode;
    wa.L = L;
    wa.draw = c->draw.as<int4>();
    wa.draw_capacity = draw_cap;
    wa.draw_row = c->draw_row.as<uint32_t>();
    wa.row_count = nullptr;
    wa.totals = c->totals.as<uint64_t>();
    wa.dbg_wscan = keep ? c->d_wscan.as<int32_t>() : nullptr;
    wa.dbg_fflag = keep ? c->d_fflag.as<int32_t>() : nullptr;
    wa.dbg_sflag = keep ? c->d_sflag.as<int32_t>() : nullptr;
    wa.dbg_skey = keep ? c->d_skey.as<int32_t>() : nullptr;
    c->mark(ST_WINDING, false);
    launch_winding_emit(wa, c->wind_status.as<uint64_t>(), ctl + CTL_WIND_COUNTER, status, st);
    c->mark(ST_WINDING, true);
    CUDA_TRY(cudaGetLastError());
    // read back the draw-list size (scanline_rasterizer.cpp:578-580)
    CUDA_TRY(cudaMemcpyAsync(c->h_tot, c->totals.p, sizeof(uint64_t) * 2, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(&c->h_n[1], status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    {
        sr_status s = check_status_word((uint32_t)c->h_n[1]);
        if (s != SR_OK) return s;
    }
    const int64_t O = (int64_t)(c->h_tot[0] + c->h_tot[1]);
    c->last_O = O;
    c->stats.n_intersections = (uint64_t)N;
    c->stats.n_draw_records = (uint64_t)O;
    c->stats.n_merged_fragments = c->h_tot[0];
    c->stats.n_spans = c->h_tot[1];
    c->stats.key_bits = key_bits;
    c->stats.sort_passes = sp.passes;

    // K10 resolve: stable sort of draw records by cell row, then paint rows
    const int32_t rows = L.Hy;
    const size_t o1 = (size_t)std::max<int64_t>(O, 1);
    CUDA_TRY(ensure(c->rkeys, sizeof(uint32_t) * o1));
    CUDA_TRY(ensure(c->rvals, sizeof(uint32_t) * o1));
    CUDA_TRY(ensure(c->rkeys_alt, sizeof(uint32_t) * o1));
    CUDA_TRY(ensure(c->rvals_alt, sizeof(uint32_t) * o1));
    CUDA_TRY(ensure(c->row_start, sizeof(int32_t) * ((size_t)rows + 1)));
    SortPlan rp = sort_plan(O, bits_for((uint64_t)rows));
    CUDA_TRY(ensure(c->row_sort_scratch, sort_scratch_bytes(rp)));
    c->mark(ST_ROWSORT, false);
    launch_sort_u32(rp, c->draw_row.as<uint32_t>(), nullptr, c->rkeys.as<uint32_t>(), c->rvals.as<uint32_t>(),
                    c->rkeys_alt.as<uint32_t>(), c->rvals_alt.as<uint32_t>(), c->row_sort_scratch.p, status, st);
    launch_row_bounds(c->rkeys.as<uint32_t>(), O, rows, c->row_start.as<int32_t>(), st);
    c->mark(ST_ROWSORT, true);
    ResolveArgs ra;
    ra.draw = c->draw.as<int4>();
    ra.row_sorted_idx = c->rvals.as<uint32_t>();
    ra.row_start = c->row_start.as<int32_t>();
    ra.W = c->W;
    ra.H = c->H;
    ra.F = c->F;
    ra.pixel_mode = g.pixel_mode;
    ra.image = c->image.as<uint32_t>();
    c->mark(ST_RESOLVE, false);
    launch_resolve(ra, st);
    c->mark(ST_RESOLVE, true);
    CUDA_TRY(cudaGetLastError());
    c->stats.kernel_launches = (uint32_t)(launches_so_far() - launches0);
    c->ev_pending = (c->flags & SR_FLAG_PROFILE) != 0;
    c->stages_valid = keep;
    return SR_OK;
}

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
    CUDA_TRY(cudaSetDevice(o.device));
    sr_ctx* c = new sr_ctx();
    c->device = o.device;
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, o.device);
    if (c->sm_count <= 0) c->sm_count = 148;
    c->W = (int32_t)width;
    c->H = (int32_t)height;
    c->mode = o.mode;
    c->F = o.mode == SR_MODE_PIXEL ? 1 : 2;
    c->flags = o.flags;
    const float id[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    std::memcpy(c->mvp.m, id, sizeof id);
    cudaError_t e = cudaMallocHost(&c->h_n, sizeof(int32_t) * 4);
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_tot, sizeof(uint64_t) * 4);
    if (e == cudaSuccess) e = ensure(c->image, (size_t)width * height * 4);
    if (e != cudaSuccess) {
        delete c;
        return fail(e == cudaErrorMemoryAllocation ? SR_ERR_OOM : SR_ERR_CUDA, "sr_create: %s", cudaGetErrorString(e));
    }
    *out = c;
    return SR_OK;
}

sr_status sr_load_scene(sr_ctx* c, const sr_scene_view* s) {
    if (!c || !s) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    const uint32_t V = s->n_points, C = s->n_curves, P = s->n_paths;
    if ((V && (!s->position || !s->pos_path_idx)) || (C && (!s->curve_pos_map || !s->curve_type || !s->curve_path_idx)) ||
        (P && (!s->fill_rule || !s->fill_info)))
        return fail(SR_ERR_INVALID_ARG, "scene array missing");
    if (C > (1u << 28) || V > (1u << 30) || P > (1u << 26)) return fail(SR_ERR_INVALID_ARG, "scene too large");
    for (uint32_t i = 0; i < C; ++i) {
        uint32_t t = s->curve_type[i];
        if (t != SR_CURVE_LINE && t != SR_CURVE_QUADRIC && t != SR_CURVE_CUBIC)
            return fail(SR_ERR_INVALID_ARG, "curve %u: unsupported type 0x%x", i, t);
        if ((uint64_t)s->curve_pos_map[i] + (t & 7u) > V)
            return fail(SR_ERR_INVALID_ARG, "curve %u: control points out of range", i);
        if (s->curve_path_idx[i] >= P) return fail(SR_ERR_INVALID_ARG, "curve %u: path index out of range", i);
        if (i > 0 && s->curve_path_idx[i] < s->curve_path_idx[i - 1])
            return fail(SR_ERR_INVALID_ARG, "curves must be grouped by path in path order");
    }
    for (uint32_t i = 0; i < V; ++i)
        if (s->pos_path_idx[i] >= P) return fail(SR_ERR_INVALID_ARG, "point %u: path index out of range", i);
    for (uint32_t i = 0; i < P; ++i)
        if (s->fill_rule[i] > 1u) return fail(SR_ERR_INVALID_ARG, "path %u: fill rule %u", i, s->fill_rule[i]);
    CUDA_TRY(cudaSetDevice(c->device));
    CUDA_TRY(ensure(c->pos, sizeof(float) * 2 * (size_t)std::max<uint32_t>(V, 1)));
    CUDA_TRY(ensure(c->pos_path, sizeof(uint32_t) * std::max<uint32_t>(V, 1)));
    CUDA_TRY(ensure(c->curve_pos, sizeof(uint32_t) * std::max<uint32_t>(C, 1)));
    CUDA_TRY(ensure(c->curve_type, sizeof(uint32_t) * std::max<uint32_t>(C, 1)));
    CUDA_TRY(ensure(c->curve_path, sizeof(uint32_t) * std::max<uint32_t>(C, 1)));
    CUDA_TRY(ensure(c->fill_rule, sizeof(uint32_t) * std::max<uint32_t>(P, 1)));
    CUDA_TRY(ensure(c->fill_info, sizeof(uint32_t) * std::max<uint32_t>(P, 1)));
    if (V) {
        CUDA_TRY(cudaMemcpy(c->pos.p, s->position, sizeof(float) * 2 * (size_t)V, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(c->pos_path.p, s->pos_path_idx, sizeof(uint32_t) * V, cudaMemcpyHostToDevice));
    }
    if (C) {
        CUDA_TRY(cudaMemcpy(c->curve_pos.p, s->curve_pos_map, sizeof(uint32_t) * C, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(c->curve_type.p, s->curve_type, sizeof(uint32_t) * C, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(c->curve_path.p, s->curve_path_idx, sizeof(uint32_t) * C, cudaMemcpyHostToDevice));
    }
    if (P) {
        CUDA_TRY(cudaMemcpy(c->fill_rule.p, s->fill_rule, sizeof(uint32_t) * P, cudaMemcpyHostToDevice));
        CUDA_TRY(cudaMemcpy(c->fill_info.p, s->fill_info, sizeof(uint32_t) * P, cudaMemcpyHostToDevice));
    }
    c->V = V;
    c->C = C;
    c->P = P;
    c->loaded = true;
    c->stages_valid = false;
    return SR_OK;
}

sr_status sr_set_mvp(sr_ctx* c, const float m[16]) {
    if (!c || !m) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    std::memcpy(c->mvp.m, m, sizeof(float) * 16);
    return SR_OK;
}

sr_status sr_render(sr_ctx* c, void* rgba_out, int out_is_device, void* stream) {
    if (!c) return fail(SR_ERR_INVALID_ARG, "NULL context");
    if (!c->loaded) return fail(SR_ERR_NO_SCENE, "sr_render before sr_load_scene");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    c->stages_valid = false;
    sr_status s = render_frame(c, st);
    if (s != SR_OK) return s;
    if (rgba_out) {
        size_t bytes = (size_t)c->W * c->H * 4;
        CUDA_TRY(cudaMemcpyAsync(rgba_out, c->image.p, bytes,
                                 out_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    }
    if (!out_is_device || !rgba_out) {
        CUDA_TRY(cudaMemcpyAsync(&c->h_n[1], c->ctl.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        return check_status_word((uint32_t)c->h_n[1]);
    }
    return SR_OK;
}

sr_status sr_render_draw_list(sr_ctx* c, const int32_t* records, int64_t n, void* rgba_out, int out_is_device,
                              void* stream) {
    if (!c) return fail(SR_ERR_INVALID_ARG, "NULL context");
    if (n < 0 || n >= (1ll << 30) || (n > 0 && !records)) return fail(SR_ERR_INVALID_ARG, "bad draw list");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    CUDA_TRY(cudaSetDevice(c->device));
    const int32_t rows = (c->H + c->F - 1) / c->F;
    const size_t n1 = (size_t)std::max<int64_t>(n, 1);
    std::vector<uint32_t> row((size_t)n);
    for (int64_t i = 0; i < n; ++i) {
        int32_t y = records[4 * i] >> 16;
        row[(size_t)i] = (y < 0 || y >= c->H) ? (uint32_t)rows : (uint32_t)(y / c->F);
    }
    CUDA_TRY(ensure(c->draw, sizeof(int4) * n1));
    CUDA_TRY(ensure(c->draw_row, sizeof(uint32_t) * n1));
    CUDA_TRY(ensure(c->ctl, sizeof(uint32_t) * CTL_WORDS));
    CUDA_TRY(ensure(c->rkeys, sizeof(uint32_t) * n1));
    CUDA_TRY(ensure(c->rvals, sizeof(uint32_t) * n1));
    CUDA_TRY(ensure(c->rkeys_alt, sizeof(uint32_t) * n1));
    CUDA_TRY(ensure(c->rvals_alt, sizeof(uint32_t) * n1));
    CUDA_TRY(ensure(c->row_start, sizeof(int32_t) * ((size_t)rows + 1)));
    CUDA_TRY(cudaMemsetAsync(c->ctl.p, 0, sizeof(uint32_t) * CTL_WORDS, st));
    if (n) {
        CUDA_TRY(cudaMemcpyAsync(c->draw.p, records, sizeof(int4) * (size_t)n, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(c->draw_row.p, row.data(), sizeof(uint32_t) * (size_t)n, cudaMemcpyHostToDevice, st));
    }
    sr::SortPlan rp = sr::sort_plan(n, bits_for((uint64_t)rows));
    CUDA_TRY(ensure(c->row_sort_scratch, sr::sort_scratch_bytes(rp)));
    uint32_t* status = c->ctl.as<uint32_t>() + CTL_STATUS;
    sr::launch_sort_u32(rp, c->draw_row.as<uint32_t>(), nullptr, c->rkeys.as<uint32_t>(), c->rvals.as<uint32_t>(),
                        c->rkeys_alt.as<uint32_t>(), c->rvals_alt.as<uint32_t>(), c->row_sort_scratch.p, status, st);
    sr::launch_row_bounds(c->rkeys.as<uint32_t>(), n, rows, c->row_start.as<int32_t>(), st);
    sr::ResolveArgs ra;
    ra.draw = c->draw.as<int4>();
    ra.row_sorted_idx = c->rvals.as<uint32_t>();
    ra.row_start = c->row_start.as<int32_t>();
    ra.W = c->W;
    ra.H = c->H;
    ra.F = c->F;
    ra.pixel_mode = c->mode == SR_MODE_PIXEL;
    ra.image = c->image.as<uint32_t>();
    sr::launch_resolve(ra, st);
    CUDA_TRY(cudaGetLastError());
    c->last_O = n;
    if (rgba_out) {
        CUDA_TRY(cudaMemcpyAsync(rgba_out, c->image.p, (size_t)c->W * c->H * 4,
                                 out_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    }
    if (!out_is_device || !rgba_out) {
        CUDA_TRY(cudaMemcpyAsync(&c->h_n[1], status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        return check_status_word((uint32_t)c->h_n[1]);
    }
    return SR_OK;
}

sr_status sr_get_stats(const sr_ctx* cc, sr_stats* out) {
    if (!cc || !out) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    sr_ctx* c = const_cast<sr_ctx*>(cc);
    if (c->ev_pending) {
        CUDA_TRY(cudaEventSynchronize(c->ev[2 * ST_RESOLVE + 1]));
        for (int s = 0; s < ST_COUNT_ALL; ++s) {
            float ms = 0.f;
            if (c->ev[2 * s] && c->ev[2 * s + 1]) CUDA_TRY(cudaEventElapsedTime(&ms, c->ev[2 * s], c->ev[2 * s + 1]));
            c->stats.stage_ms[s] = ms;
        }
        c->ev_pending = false;
    }
    *out = c->stats;
    return SR_OK;
}

sr_status sr_debug_dump(sr_ctx* c, int stage, void* dst, size_t* bytes) {
    if (!c || !bytes) return fail(SR_ERR_INVALID_ARG, "NULL argument");
    const size_t N = (size_t)c->last_N, O = (size_t)c->last_O;
    const void* src = nullptr;
    size_t need = 0;
    bool need_stages = true;
    switch (stage) {
        case SR_STAGE_TRANSFORMED_POS: src = c->tpos.p; need = 8 * (size_t)c->V; need_stages = false; break;
        case SR_STAGE_PATH_VISIBLE: src = c->path_visible.p; need = 4 * (size_t)c->P; need_stages = false; break;
        case SR_STAGE_CUTPOINTS: src = c->cut.p; need = 20 * (size_t)c->C; need_stages = false; break;
        case SR_STAGE_CURVE_COUNT: src = c->count.p; need = 4 * (size_t)c->C; need_stages = false; break;
        case SR_STAGE_CURVE_OFFSET: src = c->offs.p; need = 4 * ((size_t)c->C + 1); need_stages = false; break;
        case SR_STAGE_INTERSECTION: src = c->rec.p; need = 8 * N; need_stages = false; break;
        case SR_STAGE_FRAG_KEY: src = c->d_fkey.p; need = 4 * N; break;
        case SR_STAGE_FRAG_WINDING: src = c->d_fwn.p; need = 4 * N; break;
        case SR_STAGE_FRAG_LEFT: src = c->d_fleft.p; need = 4 * N; break;
        case SR_STAGE_SORTED_KEY: src = c->d_skey.p; need = 4 * N; break;
        case SR_STAGE_SORTED_INDEX: src = c->svals.p; need = 4 * N; need_stages = false; break;
        case SR_STAGE_WINDING_SCAN: src = c->d_wscan.p; need = 4 * (N + 1); break;
        case SR_STAGE_FRAG_FLAG: src = c->d_fflag.p; need = 4 * N; break;
        case SR_STAGE_SPAN_FLAG: src = c->d_sflag.p; need = 4 * N; break;
        case SR_STAGE_DRAW_LIST: src = c->draw.p; need = 16 * O; need_stages = false; break;
        case SR_STAGE_IMAGE: src = c->image.p; need = (size_t)c->W * c->H * 4; need_stages = false; break;
        default: return fail(SR_ERR_INVALID_ARG, "unknown stage %d", stage);
    }
    if (need_stages && !c->stages_valid)
        return fail(SR_ERR_INVALID_ARG, "stage %d needs a render with SR_FLAG_KEEP_STAGES", stage);
    if (!dst) {
        *bytes = need;
        return SR_OK;
    }
    if (*bytes < need) return fail(SR_ERR_INVALID_ARG, "buffer of %zu bytes, need %zu", *bytes, need);
    if (need && !src) return fail(SR_ERR_INVALID_ARG, "stage %d not available", stage);
    CUDA_TRY(cudaSetDevice(c->device));
    if (need) CUDA_TRY(cudaMemcpy(dst, src, need, cudaMemcpyDeviceToHost));
    *bytes = need;
    return SR_OK;
}

sr_status sr_exclusive_scan_i32(const int32_t* d_in, int32_t* d_out, int64_t n, void* stream) {
    if (n < 0 || n >= (1ll << 31)) return fail(SR_ERR_INVALID_ARG, "scan length %lld out of range", (long long)n);
    if (!d_out || (n > 0 && !d_in)) return fail(SR_ERR_INVALID_ARG, "NULL device pointer");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (n == 0) {
        CUDA_TRY(cudaMemsetAsync(d_out, 0, sizeof(int32_t), st));
        return SR_OK;
    }
    // tile words, then the tile counter and the status word
    const size_t words = sr::scan_status_words(n) + 2;
    void* scratch = nullptr;
    CUDA_TRY(cudaMallocAsync(&scratch, words * sizeof(uint64_t), st));
    uint64_t* tiles = static_cast<uint64_t*>(scratch);
    uint32_t* tail = reinterpret_cast<uint32_t*>(tiles + words - 2);
    cudaError_t e = cudaMemsetAsync(scratch, 0, words * sizeof(uint64_t), st);
    if (e == cudaSuccess) {
        sr::launch_exclusive_scan_i32(d_in, d_out, n, tiles, tail, tail + 1, st);
        e = cudaGetLastError();
    }
    cudaError_t f = cudaFreeAsync(scratch, st);
    CUDA_TRY(e);
    CUDA_TRY(f);
    return SR_OK;
}

void sr_destroy(sr_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    cudaDeviceSynchronize();
    delete c;
}

}  // extern "C"
