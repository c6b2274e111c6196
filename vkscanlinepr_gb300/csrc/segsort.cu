// segsort.cu — the fragment sort, using the order the records arrive in.
//
// Records are written per curve and curves are grouped by path, so the keys
// (path | row rank | x, see pack_key) arrive sorted by path: only the records
// of each path need ordering.  Each path is a segment of the record array.
//   * Segments of at most kGroup records are packed by where they start: the
//     segments starting in [g*kGroup, (g+1)*kGroup) form one tile of at most
//     kTile records, sorted in shared memory by one CTA.
//   * Larger segments are cut into kTile-record chunks, each sorted the same
//     way, then merged pairwise (merge path), as many rounds as the segment
//     needs.
// Both steps are stable, so the result equals a stable sort of the whole
// array by key: the order the onesweep radix sort produces.  Keys may carry a
// payload above the key bits; it moves with its key and takes no part in the
// order.  Work is handed out through a table of tile descriptors built on
// the device, one per CTA, so no CTA searches for its work.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace sr {

namespace {
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;   // records a CTA sorts or merges
constexpr int kGroup = kTile / 2;          // largest segment packed into a group tile
// 9-bit digits: a tile's compact items need 2.3 passes a record on the
// 4096^2 frame against 2.7 with 8-bit ones, for a histogram of 8 x 512 words
constexpr int kRadixBits = 9;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kDigitsPerThread = kRadix / 256;   // of the pass's digit scan
constexpr uint32_t kChunkBit = 1u << 31;   // descriptor .z: a chunk of a large segment
// Lanes with the same digit: __match_any_sync (tiles hold runs of nearly
// sorted keys, so a warp sees few distinct digits), or one ballot per bit.
constexpr bool kMatchAny = true;

// Front tables (depend on the curves only), in the segment scratch buffer.
struct SegTables {
    int32_t* flag;         // [C + 2] curve starts a path; then exclusive scan -> segment index
    uint32_t* seg_start;   // [C + 2] first record of each segment, then N
    uint64_t* scan_status;
    uint32_t* ctl;         // [0] scan counter, [1] largest segment of more than kGroup records
};

// Back tables (depend on the record capacity), in the tile buffer.
struct TileTables {
    int32_t* ntiles;       // [C + 2] tiles a segment opens; then exclusive scan -> first tile
    uint4* desc;           // [max_tiles] {start, segment size, k | rounds << 16 | chunk bit, -}
    uint32_t* tile_end;    // [max_tiles] end of a group tile (atomic max over its segments)
    uint32_t* chunks;      // [max_tiles] the chunk tiles (of large segments), in no order
    uint32_t* fallback;    // [max_tiles] tiles left to the 64-bit tile sort, in no order
    uint64_t* scan_status;
    // [0] scan counter, [1] chunk tiles, [2] next tile of the tile sort,
    // [3] tiles left to the 64-bit sort, [4] its next, [5 + l] next work
    // item of merge round l
    uint32_t* ctl;
};
constexpr int kCtlChunks = 1, kCtlSortNext = 2, kCtlFallback = 3, kCtlFallbackNext = 4, kCtlMergeNext = 5;

size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }
size_t scan_area(uint32_t C) { return round256(scan_status_words((int64_t)C + 1) * 8); }

SegTables carve_front(void* base, uint32_t C) {
    SegTables t;
    char* b = static_cast<char*>(base);
    const size_t ws = round256(((size_t)C + 2) * 4);
    t.flag = reinterpret_cast<int32_t*>(b);
    b += ws;
    t.seg_start = reinterpret_cast<uint32_t*>(b);
    b += ws;
    t.scan_status = reinterpret_cast<uint64_t*>(b);
    b += scan_area(C);
    t.ctl = reinterpret_cast<uint32_t*>(b);
    return t;
}

// Tiles of a frame: at most one group tile per kGroup records (a head starts
// its own group), plus the chunks of large segments (at most one partial
// chunk per large segment, of which there are fewer than cap / kGroup), and
// never more than the segments plus cap / kTile.
size_t max_tiles(uint32_t C, int64_t cap) {
    const size_t per_tile = (size_t)((cap + kTile - 1) / kTile);
    return std::min<size_t>((size_t)C + 2 + per_tile, 5 * per_tile + 2);
}

TileTables carve_back(void* base, uint32_t C, int64_t cap) {
    TileTables t;
    char* b = static_cast<char*>(base);
    const size_t mt = max_tiles(C, cap);
    t.ntiles = reinterpret_cast<int32_t*>(b);
    b += round256(((size_t)C + 2) * 4);
    t.desc = reinterpret_cast<uint4*>(b);
    b += round256(mt * 16);
    t.tile_end = reinterpret_cast<uint32_t*>(b);
    b += round256(mt * 4);
    t.chunks = reinterpret_cast<uint32_t*>(b);
    b += round256(mt * 4);
    t.fallback = reinterpret_cast<uint32_t*>(b);
    b += round256(mt * 4);
    t.scan_status = reinterpret_cast<uint64_t*>(b);
    b += scan_area(C);
    t.ctl = reinterpret_cast<uint32_t*>(b);
    return t;
}

SR_DEV uint32_t n_segments(const SegTables& t, uint32_t C) { return (uint32_t)t.flag[C]; }

// Merge rounds a large segment of `chunks` sorted chunks needs.
SR_DEV uint32_t rounds_of(uint32_t chunks) {
    uint32_t r = 0;
    while ((1u << r) < chunks) ++r;
    return r;
}
}  // namespace

// ---------------------------------------------------------- segment tables
__global__ void k_seg_flags(const uint32_t* __restrict__ curve_path, uint32_t C, int32_t* __restrict__ flag) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < C) flag[c] = (c == 0 || curve_path[c] != curve_path[c - 1]) ? 1 : 0;
    else if (c == C) flag[c] = 0;
}

// seg_start[s] = record offset of the first curve of segment s; seg_start[S] = N.
__global__ void k_seg_starts(const int32_t* __restrict__ offs, uint32_t C, SegTables t) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    const int32_t s = t.flag[c];
    if (t.flag[c + 1] != s) t.seg_start[s] = (uint32_t)offs[c];   // curve c starts path segment s
    if (c == C - 1) t.seg_start[n_segments(t, C)] = (uint32_t)offs[C];
}

// The largest segment of more than kGroup records.  max_size > 0: a segment
// larger than that is an overflow (the merge rounds of a pre-sized frame
// cannot take it; the frame is redone with exact sizing, which chooses the
// rounds, or the radix sort, from the largest segment).
__global__ void k_seg_largest(uint32_t C, uint32_t max_size, SegTables t, uint32_t* status) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_segments(t, C)) return;
    const uint32_t size = t.seg_start[s + 1] - t.seg_start[s];
    if (size > (uint32_t)kGroup) atomicMax(&t.ctl[1], size);
    if (max_size && size > max_size) set_error(status, ERR_CAPACITY);
}

// Tiles each segment opens: a large one its chunks, a small one that starts
// a group (first small segment starting in its group) one tile.
__global__ void k_seg_ntiles(uint32_t C, SegTables t, TileTables u) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t S = n_segments(t, C);
    int32_t n = 0;
    if (s < S) {
        const uint32_t a = t.seg_start[s], size = t.seg_start[s + 1] - a;
        if (size > (uint32_t)kGroup) {
            n = (int32_t)((size + kTile - 1) / kTile);
        } else {
            bool head = s == 0;
            if (!head) {
                const uint32_t pa = t.seg_start[s - 1];
                head = a - pa > (uint32_t)kGroup || a / (uint32_t)kGroup != pa / (uint32_t)kGroup;
            }
            n = head ? 1 : 0;
        }
    }
    if (s <= C) u.ntiles[s] = n;
}

// Descriptors: a group tile is opened by its head and stretched to the end
// of each small segment of the group; a large segment writes its chunks.
// Tiles past mt exist only in a frame whose records overflowed the capacity
// (it is redone); they are not written.
__global__ void k_seg_desc(uint32_t C, uint32_t mt, SegTables t, TileTables u) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t S = n_segments(t, C);
    if (s >= S) return;
    const uint32_t a = t.seg_start[s], size = t.seg_start[s + 1] - a;
    const int32_t first = u.ntiles[s];
    const int32_t n = u.ntiles[s + 1] - first;
    if (size > (uint32_t)kGroup) {
        const uint32_t rounds = rounds_of((uint32_t)n);
        const int32_t m = (int32_t)min((uint32_t)n, mt - min(mt, (uint32_t)first));   // chunks that fit the table
        const uint32_t at = m > 0 ? atomicAdd(&u.ctl[kCtlChunks], (uint32_t)m) : 0u;
        for (int32_t k = 0; k < m; ++k) {
            u.desc[first + k] = make_uint4(a, size, (uint32_t)k | (rounds << 16) | kChunkBit, 0u);
            u.chunks[at + k] = (uint32_t)(first + k);
        }
        return;
    }
    // a non-head small segment belongs to the tile opened just before it
    const int32_t tile = n == 1 ? first : first - 1;
    if (tile < 0 || (uint32_t)tile >= mt) return;
    if (n == 1) u.desc[tile] = make_uint4(a, 0u, 0u, 0u);
    atomicMax(&u.tile_end[tile], a + size);
}

// ----------------------------------------------------------- local sort ---
// A tile is sorted by one CTA of a persistent kernel (one wave; tiles come
// from a counter, so the grid does not follow the table's bound on them).
//   * The tile reaches shared memory by one bulk copy (TMA) of its 16-byte
//     aligned span; an odd last key comes by a plain load.
//   * Within a tile the order is that of a compact item: the fields
//     (path - pmin, row-rank code, x - xmin) packed in the fewest bits their
//     ranges need (the rank codes of k_tile_sort32 are compacted, see
//     TileRanges).  It usually needs 2-3 digit passes where the whole key
//     needs 4-6, and a digit is one shift of a 32-bit word.
//   * k_tile_sort32 sorts the tiles whose compact fields and payload fit one
//     32-bit word: half the shared memory, so more CTAs per SM.  It hands
//     the others to k_local_sort, whose items are 64-bit (rank - rmin codes,
//     the payload in the high word, or the raw key when the fields need
//     more than 32 bits), sorted through global memory.
//   * A pass ranks the digits per warp (match_any + a per-warp histogram),
//     scans the counts and scatters into the other buffer (stable: digit,
//     then warp, then slot).  Rows of slots past the tile's end are skipped.

// Fields of a key: path, row rank, x (payload bits above the key ignored).
struct KeyFields {
    uint32_t xb, rb, pb;
    uint32_t off_rank;   // rank of the off-canvas records (Hy - 1); row 0 ranks one above
    SR_DEV uint32_t x(uint64_t k) const { return (uint32_t)(k & ((1ull << xb) - 1)); }
    SR_DEV uint32_t r(uint64_t k) const { return (uint32_t)((k >> xb) & ((1ull << rb) - 1)); }
    SR_DEV uint32_t p(uint64_t k) const { return (uint32_t)((k >> (xb + rb)) & ((1ull << pb) - 1)); }
    SR_DEV uint32_t kbits() const { return xb + rb + pb; }
};

SR_DEV uint32_t bits_of(uint32_t v) { return v ? 32u - (uint32_t)__clz((int)v) : 0u; }
SR_DEV uint32_t low_mask(uint32_t b) { return b >= 32 ? 0xFFFFFFFFu : (1u << b) - 1u; }

SR_DEV uint32_t same_digit_lanes(uint32_t d) {
    if (kMatchAny) return __match_any_sync(0xFFFFFFFFu, d);
    uint32_t peers = 0xFFFFFFFFu;
#pragma unroll
    for (int b = 0; b <= kRadixBits; ++b) {   // 9 bits: digit kRadix marks an empty slot
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, (d >> b) & 1u);
        peers &= ((d >> b) & 1u) ? m : ~m;
    }
    return peers;
}

// Shared memory of the pass machinery and the range reduction.
struct PassSmem {
    uint32_t warp_hist[kWarps][kRadix];
    uint32_t digit_start[kRadix];
    uint32_t scan_tmp[kWarps];
    uint32_t red[kWarps][10];
    uint64_t kred[kWarps][3];
    uint64_t bar;
    uint32_t next;
};

// Tile `tile`'s records [a, a + len) and whether its output goes to
// keys_alt (a chunk whose segment's merge rounds end in keys_out); false
// for an empty tile.
SR_DEV bool tile_span(const TileTables& u, uint32_t tile, uint32_t n_cap, uint32_t& a, uint32_t& len, bool& to_alt) {
    const uint4 d = u.desc[tile];
    uint32_t e;
    to_alt = false;
    if (d.z & kChunkBit) {
        const uint32_t k = d.z & 0xFFFFu, rounds = (d.z >> 16) & 0x7FFFu;
        a = d.x + k * (uint32_t)kTile;
        e = min(a + (uint32_t)kTile, d.x + d.y);
        to_alt = (rounds & 1u) != 0;
    } else {
        a = d.x;
        e = u.tile_end[tile];
    }
    // a frame whose records overflowed the buffers is redone: never read past them
    a = min(a, n_cap);
    e = min(max(e, a), n_cap);
    len = e - a;
    return len > 0 && len <= (uint32_t)kTile;
}

// Stages keys [a, a + len) in buf: [a & ~1, e & ~1) by one bulk copy, key
// e - 1 by a load when e is odd.  Returns the slot of key a (0 or 1), or -1
// when the copy wait gave up (uniform over the CTA, which then leaves).
SR_DEV int stage_tile(uint64_t* buf, uint64_t* bar, uint32_t& phase, const uint64_t* __restrict__ keys_in,
                      uint32_t a, uint32_t len, uint32_t* status, uint32_t spin_limit) {
    const uint32_t e = a + len;
    if ((reinterpret_cast<uintptr_t>(keys_in) & 15u) != 0) {
        for (uint32_t j = threadIdx.x; j < len; j += kThreads) buf[j] = keys_in[a + j];
        __syncthreads();
        return 0;
    }
    const uint32_t a0 = a & ~1u, e0 = e & ~1u;
    const uint32_t nb = e0 - a0;   // e > a >= a0, so e0 >= a0
    if (threadIdx.x == 0) {
        if (nb) {
            // the previous tile's reads of the buffer came before (the
            // caller's barrier); order them before the copy's writes
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_expect_tx(bar, nb * 8u);
            bulk_load(buf, keys_in + a0, nb * 8u, bar);
        }
        if (e & 1u) buf[nb] = keys_in[e - 1];
    }
    __syncthreads();
    const bool ok = nb == 0 || mbar_wait_bounded(bar, phase, spin_limit, status);
    if (__syncthreads_or(!ok)) {
        // gave up: let the copy land before the CTA leaves
        if (nb) mbar_wait_bounded(bar, phase, spin_limit, nullptr);
        return -1;
    }
    if (nb) phase ^= 1u;
    return (int)(a - a0);
}

// Field ranges of a tile, reduced over the CTA (every thread gets them).
struct Ranges {
    uint32_t pmin, pmax, rmin, rmax, xmin, xmax;
    uint64_t lo, hi, top;   // key bits' min and max, whole key's max
    SR_DEV void init() {
        pmin = rmin = xmin = ~0u;
        pmax = rmax = xmax = 0;
        lo = ~0ull;
        hi = top = 0;
    }
    SR_DEV void add(const KeyFields& kf, uint64_t k, uint64_t kmask) {
        const uint32_t p = kf.p(k), r = kf.r(k), x = kf.x(k);
        pmin = min(pmin, p); pmax = max(pmax, p);
        rmin = min(rmin, r); rmax = max(rmax, r);
        xmin = min(xmin, x); xmax = max(xmax, x);
        lo = min(lo, k & kmask);
        hi = max(hi, k & kmask);
        top = max(top, k);
    }
    SR_DEV void reduce(PassSmem& S) {
        const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            pmin = min(pmin, __shfl_xor_sync(0xFFFFFFFFu, pmin, o));
            pmax = max(pmax, __shfl_xor_sync(0xFFFFFFFFu, pmax, o));
            rmin = min(rmin, __shfl_xor_sync(0xFFFFFFFFu, rmin, o));
            rmax = max(rmax, __shfl_xor_sync(0xFFFFFFFFu, rmax, o));
            xmin = min(xmin, __shfl_xor_sync(0xFFFFFFFFu, xmin, o));
            xmax = max(xmax, __shfl_xor_sync(0xFFFFFFFFu, xmax, o));
            lo = min(lo, __shfl_xor_sync(0xFFFFFFFFu, lo, o));
            hi = max(hi, __shfl_xor_sync(0xFFFFFFFFu, hi, o));
            top = max(top, __shfl_xor_sync(0xFFFFFFFFu, top, o));
        }
        if (lane == 0) {
            S.red[warp][0] = pmin; S.red[warp][1] = pmax;
            S.red[warp][2] = rmin; S.red[warp][3] = rmax;
            S.red[warp][4] = xmin; S.red[warp][5] = xmax;
            S.kred[warp][0] = lo; S.kred[warp][1] = hi; S.kred[warp][2] = top;
        }
        __syncthreads();
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            pmin = min(pmin, S.red[w][0]); pmax = max(pmax, S.red[w][1]);
            rmin = min(rmin, S.red[w][2]); rmax = max(rmax, S.red[w][3]);
            xmin = min(xmin, S.red[w][4]); xmax = max(xmax, S.red[w][5]);
            lo = min(lo, S.kred[w][0]); hi = max(hi, S.kred[w][1]); top = max(top, S.kred[w][2]);
        }
    }
};

// The minima of the fields and their widths, read back from the
// reduction's shared words (fewer live registers through the passes).
struct Unpack {
    uint32_t pmin, rmin, xmin, rb, xb;
    SR_DEV void load(const PassSmem& S) {
        uint32_t r1 = S.red[0][3], x1 = S.red[0][5];
        pmin = S.red[0][0];
        rmin = S.red[0][2];
        xmin = S.red[0][4];
#pragma unroll
        for (int w = 1; w < kWarps; ++w) {
            pmin = min(pmin, S.red[w][0]);
            rmin = min(rmin, S.red[w][2]); r1 = max(r1, S.red[w][3]);
            xmin = min(xmin, S.red[w][4]); x1 = max(x1, S.red[w][5]);
        }
        rb = bits_of(r1 - rmin);
        xb = bits_of(x1 - xmin);
    }
    // the key of compact fields c
    SR_DEV uint64_t key(const KeyFields& kf, uint32_t c) const {
        const uint32_t x = xmin + (c & low_mask(xb));
        const uint32_t r = rmin + (uint32_t)(((uint64_t)c >> xb) & low_mask(rb));
        const uint32_t p = pmin + (uint32_t)((uint64_t)c >> (rb + xb));
        return ((uint64_t)p << (kf.xb + kf.rb)) | ((uint64_t)r << kf.xb) | (uint64_t)x;
    }
};

// Ranges of a tile for its 32-bit items, with the row ranks compacted: the
// ranks in use below the off-canvas rank (a band), then the off-canvas rank,
// then row 0's rank above it take consecutive codes, so a tile holding off-
// canvas or row-0 records does not need the whole rank range; the x of the
// off-canvas records (all the same when they are packed as keys are) is kept
// aside, so they do not widen the x range either.  The order of the codes
// is the order of the ranks, and equal keys keep equal codes.
struct TileRanges {
    uint32_t pmin, pmax, bmin, bmax, xmin, xmax, xomin, xomax, has_off, has_top;
    uint64_t top;   // the whole key's max (its payload's max)
    SR_DEV void init() {
        pmin = bmin = xmin = xomin = ~0u;
        pmax = bmax = xmax = xomax = 0;
        has_off = has_top = 0;
        top = 0;
    }
    SR_DEV void add(const KeyFields& kf, uint64_t k) {
        const uint32_t p = kf.p(k), r = kf.r(k), x = kf.x(k);
        pmin = min(pmin, p); pmax = max(pmax, p);
        if (r == kf.off_rank) {
            has_off = 1;
            xomin = min(xomin, x); xomax = max(xomax, x);
        } else {
            if (r < kf.off_rank) {
                bmin = min(bmin, r); bmax = max(bmax, r);
            } else {
                has_top = 1;
            }
            xmin = min(xmin, x); xmax = max(xmax, x);
        }
        top = max(top, k);
    }
    SR_DEV void reduce(PassSmem& S) {
        const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            pmin = min(pmin, __shfl_xor_sync(0xFFFFFFFFu, pmin, o));
            pmax = max(pmax, __shfl_xor_sync(0xFFFFFFFFu, pmax, o));
            bmin = min(bmin, __shfl_xor_sync(0xFFFFFFFFu, bmin, o));
            bmax = max(bmax, __shfl_xor_sync(0xFFFFFFFFu, bmax, o));
            xmin = min(xmin, __shfl_xor_sync(0xFFFFFFFFu, xmin, o));
            xmax = max(xmax, __shfl_xor_sync(0xFFFFFFFFu, xmax, o));
            xomin = min(xomin, __shfl_xor_sync(0xFFFFFFFFu, xomin, o));
            xomax = max(xomax, __shfl_xor_sync(0xFFFFFFFFu, xomax, o));
            top = max(top, __shfl_xor_sync(0xFFFFFFFFu, top, o));
        }
        has_off = __any_sync(0xFFFFFFFFu, has_off) ? 1u : 0u;
        has_top = __any_sync(0xFFFFFFFFu, has_top) ? 1u : 0u;
        if (lane == 0) {
            uint32_t* w = S.red[warp];
            w[0] = pmin; w[1] = pmax; w[2] = bmin; w[3] = bmax; w[4] = xmin;
            w[5] = xmax; w[6] = xomin; w[7] = xomax; w[8] = has_off; w[9] = has_top;
            S.kred[warp][2] = top;
        }
        __syncthreads();
        load(S);
        top = S.kred[0][2];
#pragma unroll
        for (int w = 1; w < kWarps; ++w) top = max(top, S.kred[w][2]);
    }
    // the reduced values from the warps' shared words (also used to reload
    // them after the passes, with fewer live registers through them)
    SR_DEV void load(const PassSmem& S) {
        init();
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            const uint32_t* v = S.red[w];
            pmin = min(pmin, v[0]); pmax = max(pmax, v[1]);
            bmin = min(bmin, v[2]); bmax = max(bmax, v[3]);
            xmin = min(xmin, v[4]); xmax = max(xmax, v[5]);
            xomin = min(xomin, v[6]); xomax = max(xomax, v[7]);
            has_off |= v[8]; has_top |= v[9];
        }
        // off-canvas records of different x (not how keys are packed) share
        // the x range like the others
        if (has_off && xomin != xomax) {
            xmin = min(xmin, xomin);
            xmax = max(xmax, xomax);
        }
    }
    SR_DEV bool off_x_apart() const { return has_off && xomin == xomax; }
    SR_DEV uint32_t band() const { return bmin <= bmax ? bmax - bmin + 1u : 0u; }
    SR_DEV uint32_t rank_codes() const { return band() + has_off + has_top; }
    SR_DEV uint32_t bits_p() const { return bits_of(pmax - pmin); }
    SR_DEV uint32_t bits_r() const { return bits_of(rank_codes() - 1u); }
    SR_DEV uint32_t bits_x() const { return xmin <= xmax ? bits_of(xmax - xmin) : 0u; }
    // compact fields of key k (br, bx: bits_r(), bits_x())
    SR_DEV uint32_t code(const KeyFields& kf, uint64_t k, uint32_t br, uint32_t bx) const {
        const uint32_t p = kf.p(k), r = kf.r(k), x = kf.x(k);
        const uint32_t nb = band();
        const bool off = r == kf.off_rank;
        const uint32_t rc = r < kf.off_rank ? r - bmin : (off ? nb : nb + has_off);
        const uint32_t xc = off && off_x_apart() ? 0u : x - xmin;
        const uint32_t pc = bits_p() ? (p - pmin) << (br + bx) : 0u;
        return pc | (br ? rc << bx : 0u) | xc;
    }
    // the key of compact fields c
    SR_DEV uint64_t key(const KeyFields& kf, uint32_t c, uint32_t br, uint32_t bx) const {
        const uint32_t xc = c & low_mask(bx);
        const uint32_t rc = (uint32_t)(((uint64_t)c >> bx) & low_mask(br));
        const uint32_t p = pmin + (uint32_t)((uint64_t)c >> (br + bx));
        const uint32_t nb = band();
        const uint32_t r = rc < nb ? bmin + rc : (has_off && rc == nb ? kf.off_rank : kf.off_rank + 1u);
        const uint32_t x = r == kf.off_rank && off_x_apart() ? xomin : xmin + xc;
        return ((uint64_t)p << (kf.xb + kf.rb)) | ((uint64_t)r << kf.xb) | (uint64_t)x;
    }
};

// `passes` digit passes over items buf[cur][0, len), each into the other
// buffer; returns the buffer holding the result.  digit(item, shift).
template <typename T, typename Digit>
SR_DEV uint32_t radix_passes(PassSmem& S, T* buf0, T* buf1, uint32_t cur, uint32_t len, uint32_t passes,
                             Digit digit) {
    const uint32_t tid = threadIdx.x, lane = lane_id(), warp = tid >> 5;
    const uint32_t wfirst = warp * (32u * kItems);
    const uint32_t rows = wfirst >= len ? 0u : min((uint32_t)kItems, (len - wfirst + 31u) / 32u);
    for (uint32_t pass = 0; pass < passes; ++pass) {
        const uint32_t shift = pass * kRadixBits;
        const T* in = cur ? buf1 : buf0;
        T* out = cur ? buf0 : buf1;
        for (int i = tid; i < kWarps * kRadix; i += kThreads) (&S.warp_hist[0][0])[i] = 0;
        __syncthreads();
        // rank within the warp: warp w holds slots [w*512, w*512 + 512)
        uint32_t rd[kItems];   // rank | digit << 16
#pragma unroll
        for (int it = 0; it < kItems; ++it) {
            if ((uint32_t)it >= rows) break;
            const uint32_t j = wfirst + (uint32_t)it * 32u + lane;
            const bool ok = j < len;
            const uint32_t dg = ok ? digit(in[j], shift) : (uint32_t)kRadix;
            const uint32_t peers = same_digit_lanes(dg);
            const uint32_t leader = (uint32_t)(__ffs(peers) - 1);
            uint32_t before = 0;
            if (ok && lane == leader) {
                before = S.warp_hist[warp][dg];
                S.warp_hist[warp][dg] = before + (uint32_t)__popc(peers);
            }
            before = __shfl_sync(0xFFFFFFFFu, before, leader);
            rd[it] = (before + (uint32_t)__popc(peers & lanemask_lt())) | (dg << 16);
            __syncwarp();
        }
        __syncthreads();
        // per digit: exclusive over warps, then over digits (a thread takes
        // kDigitsPerThread adjacent digits)
        static_assert(kThreads * kDigitsPerThread == kRadix, "digits per thread");
        uint32_t dcnt[kDigitsPerThread];
        uint32_t cnt = 0;
#pragma unroll
        for (int q = 0; q < kDigitsPerThread; ++q) {
            const uint32_t dd = tid * kDigitsPerThread + (uint32_t)q;
            uint32_t sum = 0;
#pragma unroll
            for (int w = 0; w < kWarps; ++w) {
                const uint32_t c = S.warp_hist[w][dd];
                S.warp_hist[w][dd] = sum;
                sum += c;
            }
            dcnt[q] = sum;
            cnt += sum;
        }
        uint32_t x = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
            if ((int)lane >= o) x += y;
        }
        if (lane == 31) S.scan_tmp[warp] = x;
        __syncthreads();
        if (warp == 0) {
            const uint32_t w = lane < kWarps ? S.scan_tmp[lane] : 0u;
            uint32_t wi = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, wi, o);
                if ((int)lane >= o) wi += y;
            }
            if (lane < kWarps) S.scan_tmp[lane] = wi - w;
        }
        __syncthreads();
        uint32_t start = S.scan_tmp[warp] + x - cnt;
#pragma unroll
        for (int q = 0; q < kDigitsPerThread; ++q) {
            S.digit_start[tid * kDigitsPerThread + (uint32_t)q] = start;
            start += dcnt[q];
        }
        __syncthreads();
#pragma unroll
        for (int it = 0; it < kItems; ++it) {
            if ((uint32_t)it >= rows) break;
            const uint32_t j = wfirst + (uint32_t)it * 32u + lane;
            const uint32_t dg = rd[it] >> 16;
            if (j < len) out[S.digit_start[dg] + S.warp_hist[warp][dg] + (rd[it] & 0xFFFFu)] = in[j];
        }
        __syncthreads();
        cur ^= 1u;
    }
    return cur;
}

// ---- 32-bit items
struct Sort32Smem {
    union {
        uint64_t keys[kTile + 2];        // the staged tile
        uint32_t items[2][kTile + 4];    // the passes' buffers, once the keys are read
    };
    PassSmem ps;
};

// Sorts tile `tile` with 32-bit items (payload above the compact fields), or
// hands it to the 64-bit kernel (queued in u.fallback).  False when a copy
// wait gave up.
SR_DEV bool sort_tile32(Sort32Smem& S, uint32_t tile, uint32_t& phase, const uint64_t* __restrict__ keys_in,
                        uint64_t* __restrict__ keys_out, uint64_t* __restrict__ keys_alt, const KeyFields& kf,
                        uint32_t n_cap, const TileTables& u, uint32_t* status, uint32_t spin_limit) {
    const uint32_t tid = threadIdx.x;
    uint32_t a, len;
    bool to_alt;
    if (!tile_span(u, tile, n_cap, a, len, to_alt)) return true;
    uint64_t* dst = to_alt ? keys_alt : keys_out;
    const int off = stage_tile(S.keys, &S.ps.bar, phase, keys_in, a, len, status, spin_limit);
    if (off < 0) return false;

    // the tile's ranges
    const uint32_t kbits = kf.kbits();
    const uint64_t kmask = (1ull << kbits) - 1ull;
    const uint32_t base = (uint32_t)off;
    TileRanges R;
    R.init();
    for (uint32_t j = tid; j < len; j += kThreads) R.add(kf, S.keys[base + j]);
    R.reduce(S.ps);
    const uint32_t br = R.bits_r(), bx = R.bits_x();
    const uint32_t bits = R.bits_p() + br + bx;
    const uint64_t pay_max = R.top >> kbits;
    const uint32_t payb = pay_max > 0xFFFFFFFFull ? 33u : bits_of((uint32_t)pay_max);
    (void)kmask;
    if (bits + payb > 32u) {
        if (tid == 0) u.fallback[atomicAdd(&u.ctl[kCtlFallback], 1u)] = tile;
        return true;
    }
    if (bits == 0) {   // one key: already in order
        for (uint32_t j = tid; j < len; j += kThreads) dst[a + j] = S.keys[base + j];
        return true;
    }
    // the items (payload above the fields; a field shifts only when it is
    // not empty, so no shift reaches 32), through registers: they overwrite
    // the staged keys
    uint32_t iv[kItems];
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        if ((uint32_t)i * kThreads >= len) break;
        const uint32_t j = tid + (uint32_t)i * kThreads;
        if (j < len) {
            const uint64_t k = S.keys[base + j];
            iv[i] = (bits < 32u ? (uint32_t)(k >> kbits) << bits : 0u) | R.code(kf, k, br, bx);
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kItems; ++i) {
        if ((uint32_t)i * kThreads >= len) break;
        const uint32_t j = tid + (uint32_t)i * kThreads;
        if (j < len) S.items[0][j] = iv[i];
    }
    const uint32_t cmask = low_mask(bits);
    const uint32_t passes = (bits + kRadixBits - 1) / kRadixBits;
    const uint32_t cur = radix_passes<uint32_t>(S.ps, S.items[0], S.items[1], 0u, len, passes,
                                                [cmask](uint32_t v, uint32_t shift) -> uint32_t {
                                                    return ((v & cmask) >> shift) & (kRadix - 1);
                                                });
    TileRanges U;
    U.load(S.ps);
    const uint32_t ubr = U.bits_r(), ubx = U.bits_x(), ubits = U.bits_p() + ubr + ubx;
    const uint32_t umask = low_mask(ubits);
    for (uint32_t j = tid; j < len; j += kThreads) {
        const uint32_t v = S.items[cur][j];
        const uint64_t pay = ubits < 32u ? (uint64_t)(v >> ubits) : 0ull;
        dst[a + j] = (pay << kbits) | U.key(kf, v & umask, ubr, ubx);
    }
    return true;
}

__global__ void __launch_bounds__(kThreads, 4) k_tile_sort32(const uint64_t* __restrict__ keys_in,
                                                             uint64_t* __restrict__ keys_out,
                                                             uint64_t* __restrict__ keys_alt, uint32_t C,
                                                             KeyFields kf, uint32_t n_cap, uint32_t mt,
                                                             TileTables u, uint32_t* status, uint32_t spin_limit) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Sort32Smem& S = *reinterpret_cast<Sort32Smem*>(smem_raw);
    // tiles past the table exist only in a frame whose records overflowed (redone)
    const uint32_t n_tiles = min((uint32_t)u.ntiles[C], mt);
    if (threadIdx.x == 0) mbar_init(&S.ps.bar, 1);
    uint32_t phase = 0;
    for (;;) {
        if (threadIdx.x == 0) S.ps.next = atomicAdd(&u.ctl[kCtlSortNext], 1u);
        __syncthreads();   // also: the previous tile is done with the buffers
        const uint32_t tile = S.ps.next;
        __syncthreads();
        if (tile >= n_tiles) break;
        if (!sort_tile32(S, tile, phase, keys_in, keys_out, keys_alt, kf, n_cap, u, status, spin_limit)) return;
    }
}

// ---- 64-bit items (the tiles k_tile_sort32 handed over; rare).  The
// passes run between the tile's range of the input array (scratch by now:
// the 32-bit kernel has staged every tile) and of the output, with the
// histograms in static shared memory (the kernel is launched every frame,
// mostly with nothing handed over, so it holds no large buffers).
SR_DEV void sort_tile64(PassSmem& S, uint32_t tile, uint64_t* keys_in, uint64_t* __restrict__ keys_out,
                        uint64_t* __restrict__ keys_alt, const KeyFields& kf, uint32_t n_cap, const TileTables& u) {
    const uint32_t tid = threadIdx.x;
    uint32_t a, len;
    bool to_alt;
    if (!tile_span(u, tile, n_cap, a, len, to_alt)) return;
    uint64_t* src = keys_in + a;
    uint64_t* dst = (to_alt ? keys_alt : keys_out) + a;
    const uint32_t kbits = kf.kbits();
    const uint64_t kmask = (1ull << kbits) - 1ull;
    Ranges R;
    R.init();
    for (uint32_t j = tid; j < len; j += kThreads) R.add(kf, src[j], kmask);
    R.reduce(S);
    const uint32_t bp = bits_of(R.pmax - R.pmin), br = bits_of(R.rmax - R.rmin), bx = bits_of(R.xmax - R.xmin);
    // compact items when the fields fit 32 bits and the payload the other 32
    const bool compact = bp + br + bx <= 32u && (R.top >> kbits) <= 0xFFFFFFFFull;
    const uint32_t bits =
        compact ? bp + br + bx : (R.lo == R.hi ? 0u : 64u - (uint32_t)__clzll((long long)(R.lo ^ R.hi)));
    const uint32_t passes = (bits + kRadixBits - 1) / kRadixBits;
    if (passes == 0) {
        for (uint32_t j = tid; j < len; j += kThreads) dst[j] = src[j];
        return;
    }
    // the items start where the last pass ends in dst (a thread rewrites only
    // its own slots here; the first pass's barrier publishes them)
    uint64_t* first = (passes & 1u) ? src : dst;
    uint64_t* other = (passes & 1u) ? dst : src;
    for (uint32_t j = tid; j < len; j += kThreads) {
        const uint64_t k = src[j];
        const uint64_t c = ((uint64_t)(kf.p(k) - R.pmin) << (br + bx)) | ((uint64_t)(kf.r(k) - R.rmin) << bx) |
                           (uint64_t)(kf.x(k) - R.xmin);
        first[j] = compact ? ((k >> kbits) << 32) | c : k;
    }
    if (compact) {
        radix_passes<uint64_t>(S, first, other, 0u, len, passes, [](uint64_t v, uint32_t shift) -> uint32_t {
            return ((uint32_t)v >> shift) & (kRadix - 1);
        });
        Unpack U;
        U.load(S);
        for (uint32_t j = tid; j < len; j += kThreads) {
            const uint64_t v = dst[j];
            dst[j] = ((v >> 32) << kbits) | U.key(kf, (uint32_t)v);
        }
    } else {
        radix_passes<uint64_t>(S, first, other, 0u, len, passes, [kmask](uint64_t v, uint32_t shift) -> uint32_t {
            return (uint32_t)((v & kmask) >> shift) & (kRadix - 1);
        });
    }
}

__global__ void __launch_bounds__(kThreads) k_local_sort(uint64_t* keys_in, uint64_t* __restrict__ keys_out,
                                                         uint64_t* __restrict__ keys_alt, KeyFields kf, uint32_t n_cap,
                                                         TileTables u) {
    __shared__ PassSmem S;
    const uint32_t n_tiles = u.ctl[kCtlFallback];
    if (n_tiles == 0) return;   // the usual case: nothing handed over
    for (;;) {
        if (threadIdx.x == 0) S.next = atomicAdd(&u.ctl[kCtlFallbackNext], 1u);
        __syncthreads();   // also: the previous tile is done with the histograms
        const uint32_t i = S.next;
        __syncthreads();
        if (i >= n_tiles) break;
        sort_tile64(S, u.fallback[i], keys_in, keys_out, keys_alt, kf, n_cap, u);
    }
}

// ---------------------------------------------------------------- merge ---
// Round `level` of the merge of large segments: runs of width
// W = kTile << level, pairs merged stably (A before B on equal keys).  The
// CTA of a chunk writes that chunk's output range.  A segment needing r
// rounds has its chunks sorted into keys_out (r even) or keys_alt (r odd),
// and each round flips buffer, so its last round lands in keys_out; rounds
// past r do nothing for it.
constexpr int kMergeParts = 4;                   // work items per chunk
constexpr int kMergeOut = kTile / kMergeParts;   // outputs a merge work item writes
constexpr int kMergeItems = kMergeOut / kThreads;
struct MergeSmem {
    uint64_t in[kMergeOut];    // A part then B part of this item's outputs
    uint64_t out[kMergeOut];
    uint32_t split[4];
};

SR_DEV uint32_t merge_split(const uint64_t* A, uint32_t na, const uint64_t* B, uint32_t nb, uint32_t d, uint64_t kmask) {
    // number of A elements among the first d outputs
    uint32_t lo = d > nb ? d - nb : 0u, hi = min(d, na);
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if ((A[mid] & kmask) <= (B[d - 1 - mid] & kmask)) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// The same split found by a whole warp: 32 probes per step.
SR_DEV uint32_t warp_merge_split(const uint64_t* A, uint32_t na, const uint64_t* B, uint32_t nb, uint32_t d,
                                 uint64_t kmask) {
    const uint32_t lane = lane_id();
    uint32_t lo = d > nb ? d - nb : 0u, hi = min(d, na);
    while (lo < hi) {
        const uint32_t step = (hi - lo + 31) / 32;
        const uint32_t m = lo + lane * step;
        const bool valid = m < hi;
        const bool take_a = valid && (A[m] & kmask) <= (B[d - 1 - m] & kmask);
        const uint32_t ta = (uint32_t)__popc(__ballot_sync(0xFFFFFFFFu, take_a));
        const uint32_t tv = (uint32_t)__popc(__ballot_sync(0xFFFFFFFFu, valid));
        // the predicate holds for the first ta probes and fails from probe ta on
        const uint32_t new_lo = ta == 0 ? lo : lo + (ta - 1) * step + 1;
        const uint32_t new_hi = ta < tv ? lo + ta * step : hi;
        lo = new_lo;
        hi = new_hi;
    }
    return lo;
}

// Work item w is part w % kMergeParts of chunk tile chunks[w / kMergeParts]; the CTAs are
// persistent (one wave) and take items from the round's counter.
SR_DEV void merge_item(MergeSmem& S, uint32_t item, uint64_t* __restrict__ keys_out, uint64_t* __restrict__ keys_alt,
                       uint32_t level, uint32_t key_bits, uint32_t n_cap, const TileTables& u) {
    const uint4 desc = u.desc[u.chunks[item / kMergeParts]];
    const uint32_t k = desc.z & 0xFFFFu, rounds = (desc.z >> 16) & 0x7FFFu;
    if (level >= rounds) return;
    const uint64_t* src = ((rounds - level) & 1u) ? keys_alt : keys_out;
    uint64_t* dst = ((rounds - level) & 1u) ? keys_out : keys_alt;
    const uint32_t s0 = desc.x, size = desc.y;
    if ((uint64_t)s0 + size > n_cap) return;   // overflowed frame: redone
    const uint32_t o0 = k * (uint32_t)kTile + (item % kMergeParts) * (uint32_t)kMergeOut;
    if (o0 >= size) return;
    const uint32_t o1 = min(o0 + (uint32_t)kMergeOut, size);
    const uint32_t W = (uint32_t)kTile << level;
    const uint32_t p0 = (o0 / (2 * W)) * (2 * W);
    const uint32_t na = min(W, size - p0);
    const uint32_t nb = size - p0 > W ? min(W, size - p0 - W) : 0u;
    const uint64_t* A = src + s0 + p0;
    const uint64_t* B = A + na;
    const uint32_t tid = threadIdx.x;
    if (nb == 0) {   // a lone run: already in order
        for (uint32_t j = o0 + tid; j < o1; j += kThreads) dst[s0 + j] = src[s0 + j];
        return;
    }
    const uint64_t kmask = (1ull << key_bits) - 1ull;
    const uint32_t d0 = o0 - p0, d1 = o1 - p0;
    const uint32_t warp = tid >> 5;
    if (warp < 2) {
        const uint32_t sp = warp_merge_split(A, na, B, nb, warp == 0 ? d0 : d1, kmask);
        if (lane_id() == 0) S.split[warp] = sp;
    }
    __syncthreads();
    const uint32_t ia0 = S.split[0], ia1 = S.split[1];
    const uint32_t ib0 = d0 - ia0, ib1 = d1 - ia1;
    const uint32_t nA = ia1 - ia0, nB = ib1 - ib0, n = d1 - d0;
    for (uint32_t j = tid; j < nA; j += kThreads) S.in[j] = A[ia0 + j];
    for (uint32_t j = tid; j < nB; j += kThreads) S.in[nA + j] = B[ib0 + j];
    __syncthreads();
    // each thread merges kItems outputs from its own split
    const uint32_t dt = min(tid * (uint32_t)kMergeItems, n);
    const uint64_t* sA = S.in;
    const uint64_t* sB = S.in + nA;
    uint32_t ia = merge_split(sA, nA, sB, nB, dt, kmask);
    uint32_t ib = dt - ia;
    const uint32_t e = min(dt + (uint32_t)kMergeItems, n);
    for (uint32_t o = dt; o < e; ++o) {
        const bool takeA = ib >= nB || (ia < nA && (sA[ia] & kmask) <= (sB[ib] & kmask));
        S.out[o] = takeA ? sA[ia++] : sB[ib++];
    }
    __syncthreads();
    for (uint32_t j = tid; j < n; j += kThreads) dst[s0 + o0 + j] = S.out[j];
}

__global__ void __launch_bounds__(kThreads) k_merge_level(uint64_t* __restrict__ keys_out,
                                                          uint64_t* __restrict__ keys_alt, uint32_t level,
                                                          uint32_t key_bits, uint32_t n_cap, TileTables u) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    MergeSmem& S = *reinterpret_cast<MergeSmem*>(smem_raw);
    __shared__ uint32_t next;
    const uint32_t n_items = (uint32_t)kMergeParts * u.ctl[kCtlChunks];
    for (;;) {
        if (threadIdx.x == 0) next = atomicAdd(&u.ctl[kCtlMergeNext + level], 1u);
        __syncthreads();   // also: the previous item is done with the buffers
        const uint32_t item = next;
        __syncthreads();
        if (item >= n_items) break;
        merge_item(S, item, keys_out, keys_alt, level, key_bits, n_cap, u);
    }
}

// ------------------------------------------------------------- launches --
size_t segsort_scratch_bytes(uint32_t C) { return 2 * round256(((size_t)C + 2) * 4) + scan_area(C) + 256; }

size_t segsort_tile_bytes(uint32_t C, int64_t cap) {
    const size_t mt = max_tiles(C, cap);
    return round256(((size_t)C + 2) * 4) + round256(mt * 16) + 3 * round256(mt * 4) + scan_area(C) + 256;
}

int segsort_tile() { return kTile; }

void launch_segsort_tables(const uint32_t* curve_path, const int32_t* offs, uint32_t C, uint32_t max_size,
                           void* scratch, uint32_t* status, cudaStream_t st) {
    if (C == 0) return;
    SegTables t = carve_front(scratch, C);
    cudaMemsetAsync(t.scan_status, 0, scan_area(C), st);
    cudaMemsetAsync(t.ctl, 0, 256, st);
    const unsigned g = (C + 1 + 255) / 256;
    count_launches(3);
    k_seg_flags<<<g, 256, 0, st>>>(curve_path, C, t.flag);
    launch_exclusive_scan_i32(t.flag, t.flag, C + 1, t.scan_status, t.ctl + 0, status, st);
    k_seg_starts<<<g, 256, 0, st>>>(offs, C, t);
    k_seg_largest<<<g, 256, 0, st>>>(C, max_size, t, status);
}

cudaError_t segsort_tile_counts(const void* tiles, uint32_t C, int64_t cap, uint32_t out[2]) {
    TileTables u = carve_back(const_cast<void*>(tiles), C, cap);
    cudaError_t e = cudaMemcpy(&out[0], u.ntiles + C, 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&out[1], u.ctl + kCtlFallback, 4, cudaMemcpyDeviceToHost);
    out[0] = std::min<uint32_t>(out[0], (uint32_t)max_tiles(C, cap));
    return e;
}

const uint32_t* segsort_largest(const void* scratch, uint32_t C) {
    return carve_front(const_cast<void*>(scratch), C).ctl + 1;
}

void launch_segsort(uint64_t* keys_in, uint64_t* keys_out, uint64_t* keys_alt, int64_t cap, uint32_t C,
                    const KeyLayout& L, int levels, void* scratch, void* tiles, int sm_count, uint32_t* status,
                    cudaStream_t st) {
    if (cap <= 0 || C == 0) return;
    SegTables t = carve_front(scratch, C);
    TileTables u = carve_back(tiles, C, cap);
    const size_t mt = max_tiles(C, cap);
    cudaMemsetAsync(u.tile_end, 0, mt * 4, st);
    cudaMemsetAsync(u.scan_status, 0, scan_area(C), st);
    cudaMemsetAsync(u.ctl, 0, 256, st);
    const unsigned g = (C + 1 + 255) / 256;
    count_launches(2);
    k_seg_ntiles<<<g, 256, 0, st>>>(C, t, u);
    launch_exclusive_scan_i32(u.ntiles, u.ntiles, C + 1, u.scan_status, u.ctl + 0, status, st);
    k_seg_desc<<<g, 256, 0, st>>>(C, (uint32_t)mt, t, u);
    const uint32_t key_bits = L.pbits + L.rbits + L.xbits;
    const KeyFields kf{L.xbits, L.rbits, L.pbits, (uint32_t)(L.Hy - 1)};
    // resident CTAs per SM of the two persistent kernels (same on every
    // device of the build's architecture)
    static std::atomic<uint32_t> attr{0};
    static std::atomic<int> occ_sort32{0}, occ_merge{0};
    once_per_device(attr, [] {
        cudaFuncSetAttribute(k_tile_sort32, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Sort32Smem));
        cudaFuncSetAttribute(k_merge_level, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MergeSmem));
        int a = 0, c = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_tile_sort32, kThreads, sizeof(Sort32Smem));
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, k_merge_level, kThreads, sizeof(MergeSmem));
        occ_sort32.store(std::max(a, 1));
        occ_merge.store(std::max(c, 1));
    });
    const size_t sms = (size_t)std::max(sm_count, 1);
    const unsigned g_sort32 = (unsigned)std::min<size_t>(mt, sms * (size_t)std::max(occ_sort32.load(), 1));
    // the 64-bit sort takes the few tiles the 32-bit one hands over
    const unsigned g_sort = (unsigned)std::min<size_t>(mt, sms);
    const unsigned g_merge =
        (unsigned)std::min<size_t>(kMergeParts * mt, sms * (size_t)std::max(occ_merge.load(), 1));
    count_launches(2 + (uint32_t)levels);
    const uint32_t n_cap = (uint32_t)cap;
    k_tile_sort32<<<g_sort32, kThreads, sizeof(Sort32Smem), st>>>(keys_in, keys_out, keys_alt, C, kf, n_cap,
                                                                  (uint32_t)mt, u, status, spin_limit());
    k_local_sort<<<g_sort, kThreads, 0, st>>>(keys_in, keys_out, keys_alt, kf, n_cap, u);
    for (int lv = 0; lv < levels; ++lv)
        k_merge_level<<<g_merge, kThreads, sizeof(MergeSmem), st>>>(keys_out, keys_alt, (uint32_t)lv, key_bits, n_cap,
                                                                    u);
}

}  // namespace sr
