// kernels.h — launch interface between the host orchestration and the
// device kernels of the scanline renderer.
#pragma once
#include <atomic>
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace sr {

// Number of kernels this library has launched in this process.
void count_launches(uint32_t n);
// Runs fn (setting a kernel attribute) unless it has already run for
// `flags` on the current device (one bit per device, up to 32 devices).
// The bit is set after fn, so no thread skips it before it has taken
// effect; two threads may both run it, which is harmless.
template <typename Fn> void once_per_device(std::atomic<uint32_t>& flags, Fn&& fn) {
    int dev = 0;
    cudaGetDevice(&dev);
    const uint32_t bit = 1u << (dev & 31);
    if (flags.load(std::memory_order_acquire) & bit) return;
    fn();
    flags.fetch_or(bit, std::memory_order_release);
}
uint64_t launches_so_far();
// Polls a bounded device spin makes before it gives up: kSpinLimitDefault
// unless sr_set_spin_limit chose another.  Read at each launch.
uint32_t spin_limit();
// Device address, on the current device, of the sticky error word of the
// standalone scans (sr_exclusive_scan_i32 and its allocation-free variant),
// which sr_scan_status reads and clears.
cudaError_t standalone_scan_status(uint32_t** out);

struct Mvp {
    float m[16];   // rows m0..m3
};

// One scene of a batch (device layout).  Paths of scene s are
// [path_begin, path_end) in the batch's global path order; its cell rows
// are [row_base, row_base + rows) of the batch's global row order; its
// framebuffer starts at pixel image_off.
struct SceneInfo {
    int32_t W, H;
    uint32_t path_begin, path_end;
    uint32_t row_base, rows;
    uint64_t image_off;
    float mvp[16];
};

struct SceneTable {
    const SceneInfo* scenes;
    const uint32_t* path_scene;   // [n_paths] scene of each path
    uint32_t n_scenes;
};

SR_DEV const SceneInfo& scene_of_path(const SceneTable& t, uint32_t path) { return t.scenes[t.path_scene[path]]; }

// Scene + per-frame arrays the geometry kernels read.  W and H are the
// largest canvas of the batch (key layout); each scene's own canvas comes
// from the scene table.
struct GeomArgs {
    uint32_t n_curves;
    const uint32_t* curve_type;
    const uint32_t* curve_pos;
    const uint32_t* curve_path;
    const float2* tpos;
    const int32_t* path_visible;
    int32_t W, H, F;
    int32_t pixel_mode;
    KeyLayout L;
    SceneTable st;
    int64_t rec_cap;   // capacity of the record buffers; larger counts are an overflow
};

// Optional reference-layout outputs for parity dumps (all NULL in production).
struct DebugOut {
    int32_t* fkey;      // [N] packed yx
    int32_t* fwn;       // [N] winding change
    int32_t* fleft;     // [N] centre-sample part (pixel mode)
};

// Crossing-chain work of the intersection stage.
struct ChainWork {
    uint4* pieces;            // [n_curves][5] per-piece chain set-up
    uint32_t* chain_items;    // [list_cap] (curve << 4 | piece << 1 | side), append order
    uint32_t* chain_keys;     // [list_cap] length-class / type sort key
    uint32_t* sorted_items;   // [list_cap] the same, longest class first
    uint32_t* sorted_keys;
    uint32_t list_cap;
    uint32_t* chain_count;    // [1] zeroed before the count pass
    uint32_t* wide_count;     // [1] chains solved by a whole warp, zeroed before the count pass
    uint32_t* wide_queue;     // [1] their work-queue counter, zeroed likewise
    uint8_t* curve_wide;      // [n_curves] 1 for a curve with a wide chain (written by the count pass)
    uint32_t* wide_curves;    // [n_curves] those curves, in no order
    uint32_t* wide_curve_count;   // [1] zeroed before the count pass
    uint32_t* chain_queue;    // [1] zeroed before the chains
    uint32_t* long_list;      // [list_cap] (curve << 3 | piece) of long pieces
    uint32_t* long_count;     // [1] zeroed before the count pass
};
size_t piece_table_bytes(uint32_t n_curves);
uint32_t chain_key_bits();
uint32_t chain_list_capacity(uint32_t n_curves);

// Arcs' control and weight slots after launch_transform (SR_CURVE_ARC).
void launch_arc_fixup(const uint32_t* curve_type, const uint32_t* curve_pos, const uint32_t* curve_path,
                      uint32_t n_curves, const float2* pos, const SceneTable& t, float2* tpos, int32_t* path_visible,
                      cudaStream_t st);
void launch_transform(const float2* pos, const uint32_t* pos_path, uint32_t n_points, const SceneTable& t,
                      float2* tpos, int32_t* path_visible, cudaStream_t st);
void launch_count(const GeomArgs& g, float* cut_cache, int32_t* count, const ChainWork& w, uint32_t* status,
                  cudaStream_t st);
// Crossing chains (longest first) then the per-curve merge into the
// reference's intersection records rec[N] (curve, t bits | flags).  Each
// runs in two parts: part 0 of the chains solves the wide chains (a warp
// each), part 1 the others; part 0 of the merge and of the fragments covers
// every curve but the wide ones (whose records it marks pending), part 1
// the wide curves.  Part 1 of the merge must follow part 0 of the merge and
// of the chains; the two parts may otherwise run on two streams at once.
// Kernel attributes of the geometry kernels (the long-piece merge's shared
// memory); once per device before the first frame.
cudaError_t geom_init();
void launch_chains(const GeomArgs& g, const int32_t* offs, const ChainWork& w, int32_t* cbuf, int sm_count, int part,
                   cudaStream_t st);
void launch_merge(const GeomArgs& g, const int32_t* offs, const ChainWork& w, int32_t* cbuf, int2* rec,
                  uint32_t* status, int part, cudaStream_t st);
// One fragment per record: sort key + packed winding bits (4 bits: change,
// centre part).  With wnp NULL the bits are stored above the key bits of
// each key instead of in wnp[].
// n_cap launches the grid; the record count is read from n_dev (offs[C]).
void launch_fragment(const GeomArgs& g, const int2* rec, const int32_t* offs, int64_t n_cap, const uint32_t* n_dev,
                     uint64_t* keys, uint8_t* wnp, const DebugOut& dbg, const ChainWork& w, int part,
                     cudaStream_t st);

// ---- scan.cu
// Exclusive scan of n int32 values into out[0..n] (out[n] = total), single
// pass with decoupled look-back.  in and out may alias.  tile_status must
// hold scan_status_words(n) zeroed uint64 words.
size_t scan_status_words(int64_t n);
void launch_exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, uint64_t* tile_status,
                               uint32_t* tile_counter, uint32_t* status, cudaStream_t st);

// ---- sort.cu  (onesweep LSD radix sort, 8-bit digits)
struct SortPlan {
    int64_t n;                 // element count, or the capacity when n_dev is set
    const uint32_t* n_dev;     // optional device-side count (<= n), read by the kernels
    uint32_t key_bits;
    uint32_t passes;
    uint32_t tiles;
    int items;                 // keys per thread of a tile: 8, 12 or 16
    int hist_given = 0;        // 1: the digit counts are already in the scratch (sort_hist_from_counts)
};
SortPlan sort_plan(int64_t n, uint32_t key_bits, const uint32_t* n_dev = nullptr, int items = 12);
// Device scratch needed by a plan (bytes).
size_t sort_scratch_bytes(const SortPlan& p);
// Sorts (keys, values) stably by the low key_bits of the keys; higher bits
// travel with their key.  If vals_in is NULL the values are the identity
// 0..n-1; if vals_out is NULL there are no values (keys only).  Results end
// in (keys_out, vals_out); keys_alt/vals_alt are ping-pong buffers of n items.
void launch_sort_u64(const SortPlan& p, const uint64_t* keys_in, const uint32_t* vals_in, uint64_t* keys_out,
                     uint32_t* vals_out, uint64_t* keys_alt, uint32_t* vals_alt, void* scratch,
                     uint32_t* status, cudaStream_t st);
// For keys that are bin indices 0..n_bins-1 whose counts are known: writes
// each pass's digit counts into the plan's scratch (and sets hist_given on
// the plan), so the sort skips its own histogram pass over the keys.
void sort_hist_from_counts(SortPlan& p, const uint32_t* counts, uint32_t n_bins, void* scratch, cudaStream_t st);
void launch_sort_u32(const SortPlan& p, const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                     uint32_t* vals_out, uint32_t* keys_alt, uint32_t* vals_alt, void* scratch,
                     uint32_t* status, cudaStream_t st);

// ---- segsort.cu  (stable sort of path-ordered keys: per-path segments)
// Tables of the path segments from the curve offsets; max_size > 0 flags a
// segment larger than that as a capacity overflow.
size_t segsort_scratch_bytes(uint32_t n_curves);
// Tile tables of a frame with capacity cap (a second buffer).
size_t segsort_tile_bytes(uint32_t n_curves, int64_t cap);
int segsort_tile();
void launch_segsort_tables(const uint32_t* curve_path, const int32_t* offs, uint32_t n_curves, uint32_t max_size,
                           void* scratch, uint32_t* status, cudaStream_t st);
// Tiles of the last segmented sort with these tables, and of those the
// ones sorted with 64-bit items (synchronous copies).
cudaError_t segsort_tile_counts(const void* tiles, uint32_t n_curves, int64_t cap, uint32_t out[2]);
// Device word holding the largest segment of more than half a tile (0 if none).
const uint32_t* segsort_largest(const void* scratch, uint32_t n_curves);
// Sorts keys_in[0, N) into keys_out by their key bits (layout L; N from the
// tables; cap bounds the tile tables); `levels` merge rounds launched, at
// least ceil(log2(chunks of the largest segment)).  keys_alt is scratch.
// The tile sort and the merge rounds run one wave of persistent CTAs.
// keys_in[0, N) is left unspecified (the tiles that need 64-bit items sort
// through it).
void launch_segsort(uint64_t* keys_in, uint64_t* keys_out, uint64_t* keys_alt, int64_t cap, uint32_t n_curves,
                    const KeyLayout& L, int levels, void* scratch, void* tiles, int sm_count, uint32_t* status,
                    cudaStream_t st);

// ---- winding.cu
struct WindArgs {
    int64_t n;                      // N records: the capacity when n_dev is set
    const uint32_t* n_dev;          // device-side record count (offs[C])
    const uint64_t* skeys;          // sorted keys
    const uint32_t* svals;          // sorted record indices (NULL: winding bits ride in the keys)
    const uint8_t* wnp;             // packed winding bits by record index (NULL likewise)
    const uint32_t* fill_rule;      // [P]
    const uint32_t* fill_info;      // [P]
    uint32_t n_paths;
    int32_t W, H, F;
    int32_t pixel_mode;
    KeyLayout L;
    SceneTable st;
    int4* draw;                     // [capacity] draw records
    int64_t draw_capacity;
    uint32_t* draw_row;             // [capacity] global cell row of each draw record
    uint64_t* totals;               // [2] merged fragments, spans
    uint32_t* n_draw;               // [1] merged fragments + spans
    uint32_t* path_draw;            // [P] draw records per path (NULL unless labelling)
    // [cut_rows][cut_segs]: 1 + the last draw index of a span that covers a
    // resolve segment (kResolveSeg pixels) entirely and leaves nothing of
    // what was under it (opaque in pixel mode, any span in reference mode);
    // zeroed before the emit, NULL to skip
    uint32_t* seg_cut;
    uint32_t cut_rows, cut_segs;
    uint32_t* row_count;            // [cut_rows] draw records per global cell row (zeroed before), or NULL
    unsigned long long* row_px;     // [cut_rows] pixels of a row's records (widths summed; zeroed before), or NULL
    // parity dumps (NULL in production)
    int32_t* dbg_wscan;             // [N+1]
    int32_t* dbg_fflag;             // [N]
    int32_t* dbg_sflag;             // [N]
    int32_t* dbg_skey;              // [N]
};
// items: records per thread of a tile (4 or 8).
size_t winding_status_words(int64_t n, int items = 8);
void launch_winding_emit(const WindArgs& a, int items, uint64_t* tile_status, uint32_t* tile_counter,
                         uint32_t* status, cudaStream_t st);

// ---- resolve.cu
// A gradient paint ready for the resolve (built on the host from an
// sr_paint and the scene's matrix, see sr.h for the definition): linear
// t = (lin0 X + lin1 Y) + lin2 of the pixel-space point (X, Y); radial
// g = (m0 X + m1 Y) + m2, (m3 X + m4 Y) + m5 in gradient space, focus
// (fx, fy), centre - focus (dx, dy), A = dx^2 + dy^2 - r^2.
constexpr int kMaxStops = 16;
struct DevPaint {
    int32_t kind, spread, n_stops, pad;
    float lin[3];
    float m[6];
    float fx, fy, dx, dy, A;
    float opacity;
    float off[kMaxStops];
    float rgba[kMaxStops][4];
};
// The paint a fill_info names: alpha byte 0 and index + 1 in the colour
// bytes; -1 for a solid colour.
__host__ __device__ __forceinline__ int32_t fill_paint(uint32_t info) {
    return (info >> 24) == 0u && (info & 0x00FFFFFFu) != 0u ? (int32_t)(info & 0x00FFFFFFu) - 1 : -1;
}

// Resolve work: each CTA paints rows_per_cta cell rows of one scene;
// cta_base[s] is the first CTA of scene s (host-built, n_scenes+1 entries).
struct ResolveArgs {
    const int4* draw;
    const uint32_t* row_sorted_idx;   // draw indices sorted by global cell row
    const int32_t* row_start;         // [total rows + 1]
    const uint32_t* cta_base;         // [n_scenes + 1]
    const SceneInfo* scenes;
    uint32_t n_scenes;
    int32_t F;
    int32_t pixel_mode;
    int32_t warps;                    // warps per CTA: 8 or 16
    uint32_t* image;                  // all scenes' RGBA8 framebuffers
    const uint32_t* seg_cut;          // [rows][cut_segs] from the emit, or NULL
    const unsigned long long* row_px; // [rows] summed record widths from the emit, or NULL (every row searched)
    uint32_t cut_segs;
    const uint8_t* cta_narrow;        // [CTAs] 1 for a CTA of several rows
    int any_narrow;                   // some CTA is (then pixel mode runs a second kernel for them)
    const DevPaint* paints;           // gradient paints of the scene (single-scene contexts), or NULL
    uint32_t n_paints;
};
// Pixels per warp of a resolve CTA.
constexpr int kResolveSeg = 256;
uint32_t resolve_rows_per_cta(int32_t W, int warps);
void launch_resolve(const ResolveArgs& a, uint32_t n_ctas, cudaStream_t st);
// Multisampling: sum a sample frame into acc (first: start the sums), and
// write the rounded averages of k frames.
void launch_aa_accumulate(const uint32_t* img, void* acc, size_t n, bool first, cudaStream_t st);
void launch_aa_resolve(const void* acc, uint32_t* img, size_t n, uint32_t k, cudaStream_t st);
// n_dev (optional) holds the record count; n is the capacity.
void launch_row_bounds(const uint32_t* srows, int64_t n, const uint32_t* n_dev, int32_t rows, int32_t* row_start,
                       cudaStream_t st);

// ---- mlp.cu  (learned sizing: 6 features -> 64 -> 64 -> 2, GELU)
constexpr int kMlpIn = 6, kMlpHidden = 64, kMlpOut = 2;
constexpr int kMlpParams = kMlpHidden * kMlpIn + kMlpHidden + kMlpHidden * kMlpHidden + kMlpHidden +
                           kMlpOut * kMlpHidden + kMlpOut;
constexpr int kMlpNorm = 2 * kMlpIn + 2 * kMlpOut;
// feats[P][6] of the paths under the current transforms (tpos must be current).
void launch_path_features(const GeomArgs& g, const uint32_t* path_first_curve, uint32_t n_paths, float* feats,
                          cudaStream_t st);
// labels[P][2] = log(1 + records), log(1 + draw records) per path.
void launch_path_labels(const uint32_t* path_first_curve, uint32_t n_paths, const int32_t* count,
                        const uint32_t* path_draw, float* labels, cudaStream_t st);
// y[n][2] in log(1 + count) units.  wb: BF16 weights; master: FP32 copy (biases).
void launch_mlp_predict(const void* wb, const float* master, const float* norm, const float* x, uint32_t n, float* y,
                        int sm_count, cudaStream_t st);
// Adds the minibatch gradient of the mean squared error into grad and the
// sum of squared errors into loss_sum.
cudaError_t launch_mlp_grad(const void* wb, const float* master, const float* norm, const float* x, const float* t,
                            const uint32_t* idx, uint32_t n, float* grad, float* loss_sum, cudaStream_t st);
void launch_adam(float* master, void* wb, float* grad, float* m, float* v, float lr, float b1, float b2, float eps,
                 float bc1, float bc2, cudaStream_t st);
void launch_to_bf16(const float* master, void* wb, cudaStream_t st);
void launch_perm_keys(uint32_t* keys, uint32_t n, uint64_t seed, cudaStream_t st);
// allot[P][2] from predictions with the path margins (margins[0..1]);
// frame capacities with the frame margins (margins[2..3]) accumulate into
// scene_tot[S][2] and tot[0..1], the allotments into tot[2..3] (zero them first).
void launch_allot(const float* y, uint32_t n_paths, const uint32_t* path_scene, const float margins[4],
                  uint32_t* allot, unsigned long long* scene_tot, unsigned long long* tot, cudaStream_t st);
// out[4] (zeroed first): paths over their record allotment, over their draw
// allotment, exact records, exact draw records.
void launch_judge(const uint32_t* path_first_curve, uint32_t n_paths, const int32_t* count, const uint32_t* path_draw,
                  const uint32_t* allot, unsigned long long* out, cudaStream_t st);

}  // namespace sr
