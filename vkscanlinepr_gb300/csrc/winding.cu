// winding.cu — one pass over the sorted records that replaces five reference
// dispatches and two host read-backs:
//   shuffle_fragment.comp:17-26            gather of winding changes
//   naive_scan.comp (scanline_rasterizer.cpp:479-506)   winding scan
//   mark_merged_fragment_and_span.comp:22-93            fragment/span flags
//   naive_scan.comp over 2N flags (scanline_rasterizer.cpp:545-580)
//   gen_merged_fragment_and_span.comp:33-103           draw-list emit
//
// Three launches over tiles of 2048 consecutive sorted records (ITEMS 8; 1024
// with ITEMS 4):
//   k_winding_reduce      each tile's (scene head seen, sum since) pair of
//                         winding changes, a fully parallel read of the keys;
//   k_winding_scan_tiles  one CTA scans the tile pairs into each tile's
//                         incoming winding prefix;
//   k_winding_emit        the records' winding scan, fragment and span flags,
//                         output slots (one decoupled look-back over packed
//                         31:31-bit counts of merged fragments and spans) and
//                         the draw records.
// Draw records come out in the reference's order: a record's merged
// fragment, then the span ending at it.
//
// The reference's winding scan is global over its one scene's records
// (scanline_rasterizer.cpp:479-506), so a path whose changes do not sum to
// zero carries into the paths after it.  In a batch of scenes chain A is a
// scan segmented at scene boundaries, so each scene sees exactly the global
// scan it would see alone (with one scene the two are the same).
#include "common.cuh"
#include "kernels.h"

namespace sr {

namespace {
// a winding tile is THREADS x ITEMS records: 256 x 4 or 256 x 8
constexpr uint64_t kFlagA = 1ull << 62;
constexpr uint64_t kFlagP = 2ull << 62;
constexpr uint64_t kValMask = (1ull << 62) - 1;
constexpr uint64_t kHeadBit = 1ull << 61;   // chain A: the tile holds a scene's first record
// chain B value: merged fragments in bits 31..61, spans in bits 0..30
constexpr int kFragShift = 31;
constexpr uint64_t kSpanMask = (1ull << 31) - 1;

SR_DEV bool rule_pass(uint32_t rule, int32_t wn) {
    // mark_merged_fragment_and_span.comp:82
    return (rule == 0u && wn != 0) || (rule == 1u && (wn & 1) != 0);
}

SR_DEV int32_t sx2(uint32_t v) { return (int32_t)(v << 30) >> 30; }   // 2-bit two's complement

template <typename T> SR_DEV T warp_incl(T v) {
    uint32_t lane = lane_id();
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T t = __shfl_up_sync(0xFFFFFFFFu, v, d);
        if ((int)lane >= d) v = v + t;
    }
    return v;
}

// Look-back over 64-bit tile words; `add` combines values (wrapping).
template <bool kSigned32>
SR_DEV uint64_t lookback(uint64_t* tstat, uint32_t tile, uint32_t* status, uint32_t spin_limit) {
    uint32_t lane = lane_id();
    uint64_t excl = 0;
    int64_t look = (int64_t)tile - 1;
    uint32_t spins = 0;
    while (look >= 0) {
        int64_t j = look - (int64_t)lane;
        uint64_t s = j >= 0 ? ld_acquire_u64(&tstat[j]) : kFlagP;
        uint32_t flag = (uint32_t)(s >> 62);
        uint32_t ready = __ballot_sync(0xFFFFFFFFu, flag != 0);
        // a tile that holds a segment head ends the look-back like an
        // inclusive prefix does: its value already starts at that head
        uint32_t pm = __ballot_sync(0xFFFFFFFFu, flag == 2 || (kSigned32 && flag == 1 && (s & kHeadBit)));
        int firstp = pm ? (__ffs(pm) - 1) : 31;
        uint32_t need = firstp == 31 ? 0xFFFFFFFFu : ((2u << firstp) - 1u);
        if ((ready & need) != need) {
            if (++spins > spin_limit) {
                if (lane == 0) set_error(status, ERR_LOOKBACK_TIMEOUT);
                break;
            }
            __nanosleep(64);
            continue;
        }
        uint64_t v = ((int)lane <= firstp) ? (s & (kSigned32 ? 0xFFFFFFFFull : kValMask)) : 0ull;
        if (kSigned32) {
            uint32_t w = (uint32_t)v;
#pragma unroll
            for (int d = 16; d >= 1; d >>= 1) w += __shfl_xor_sync(0xFFFFFFFFu, w, d);
            excl = (uint64_t)(uint32_t)((uint32_t)excl + w);
        } else {
#pragma unroll
            for (int d = 16; d >= 1; d >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, d);
            excl += v;
        }
        if (pm) break;
        look -= 32;
    }
    return excl;
}

// A tile's draw records in output order, as items of shared memory: the
// record's index in the tile (bits 13..), a span bit (12) and, for a merged
// fragment, its index among the tile's fragments (0..11).  A record gives at
// most a fragment and a span, so 2 x kTile items always fit.
constexpr uint32_t kItemSpan = 1u << 12;
constexpr int kItemRecShift = 13;

template <int ITEMS, int THREADS> struct Smem {
    uint32_t tile;
    int32_t warpA[THREADS / 32];
    int32_t warpAf[THREADS / 32];
    uint32_t warpB[THREADS / 32];
    uint64_t prefixB;
    uint32_t count;
    uint32_t lo_prev;                               // low key half of the record before the tile
    // per thread: the key of its first record, the centre parts of its
    // leading run (records with that key) and whether all its records share it
    uint32_t run_p[THREADS], run_l[THREADS];
    int32_t run_sum[THREADS];
    uint32_t run_all[THREADS];
    uint64_t next_key;                              // the record after the tile, ~0 if none
    int32_t next_c;                                 // its centre part
    uint32_t items[2 * THREADS * ITEMS];
    __align__(16) uint32_t lo[THREADS * ITEMS];     // low key half (row rank, x + 1) of each record
    __align__(16) uint32_t paint[THREADS * ITEMS];  // fill_info of each record's path
};

// Key of record i without its payload, and its packed winding bits.
SR_DEV uint64_t wkey(const WindArgs& a, int64_t i, int64_t n, uint32_t& wb, uint32_t* status) {
    const uint64_t kr = a.skeys[i];
    if (a.svals) {
        const uint32_t rec = a.svals[i];
        if (rec < (uint64_t)n) {
            wb = a.wnp[rec];
        } else {
            wb = 0;
            set_error(status, ERR_BAD_INDEX);
        }
        return kr;
    }
    wb = payload_part(a.L, kr);
    return key_part(a.L, kr);
}

// This thread's ITEMS consecutive records from ibase: keys without their
// payload, and the packed winding bits (4 bits a record).  Records at or past
// n read as key 0; a key whose path is out of range reads as 0 and is flagged.
template <int ITEMS>
SR_DEV void load_run(const WindArgs& a, int64_t ibase, int64_t n, uint64_t (&kk)[ITEMS], uint32_t& wbits,
                     uint32_t* status) {
    const uint32_t pshift = a.L.xbits + a.L.rbits;
    wbits = 0;
    if (!a.svals && ibase + ITEMS <= n) {
        const ulonglong2* p = reinterpret_cast<const ulonglong2*>(a.skeys + ibase);
#pragma unroll
        for (int q = 0; q < ITEMS / 2; ++q) {
            const ulonglong2 v = p[q];
            kk[2 * q] = v.x;
            kk[2 * q + 1] = v.y;
        }
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            wbits |= payload_part(a.L, kk[k]) << (4 * k);
            kk[k] = key_part(a.L, kk[k]);
        }
    } else {
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            uint32_t wb = 0;
            kk[k] = ibase + k < n ? wkey(a, ibase + k, n, wb, status) : 0ull;
            wbits |= (wb & 0xFu) << (4 * k);
        }
    }
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        if (ibase + k < n && (kk[k] >> pshift) >= a.n_paths) {
            set_error(status, ERR_BAD_INDEX);
            kk[k] = 0;
        }
    }
}

// The record before this thread's first (a shuffle, or a load at a warp's
// first lane); 0 before record 0.
template <int ITEMS>
SR_DEV uint64_t prev_key(const WindArgs& a, int64_t ibase, int64_t n, const uint64_t (&kk)[ITEMS]) {
    uint64_t kp = __shfl_up_sync(0xFFFFFFFFu, kk[ITEMS - 1], 1);
    if (lane_id() == 0) {
        uint32_t wb;
        kp = ibase > 0 && ibase - 1 < n ? wkey(a, ibase - 1, n, wb, nullptr) : 0ull;
        if ((kp >> (a.L.xbits + a.L.rbits)) >= a.n_paths) kp = 0;
    }
    return kp;
}

// Scene heads among this thread's records (bit k: record ibase + k is the
// first record of a scene) and the thread's (head seen, sum since) pair.
template <int ITEMS>
SR_DEV uint32_t run_heads(const WindArgs& a, int64_t ibase, int64_t n, const uint64_t (&kk)[ITEMS], uint64_t kprev,
                          uint32_t wbits, bool& tf, int32_t& tv) {
    const uint32_t pshift = a.L.xbits + a.L.rbits;
    const bool multi = a.st.n_scenes > 1;
    uint32_t heads = 0;
    tf = false;
    tv = 0;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        const int64_t i = ibase + k;
        if (i >= n) continue;
        bool h = i == 0;
        if (multi && !h) {
            const uint64_t kp = k == 0 ? kprev : kk[k - 1];
            h = a.st.path_scene[(uint32_t)(kk[k] >> pshift)] != a.st.path_scene[(uint32_t)(kp >> pshift)];
        }
        if (h) {
            heads |= 1u << k;
            tf = true;
            tv = 0;
        }
        tv = wadd(tv, sx2(wbits >> (4 * k)));
    }
    return heads;
}

// (fa, va) then (fb, vb), into (fb, vb): a head in the second part restarts
// the sum.
SR_DEV void seg_combine(bool fa, int32_t va, bool& fb, int32_t& vb) {
    vb = fb ? vb : wadd(va, vb);
    fb = fb || fa;
}

// Segmented scan of (head, value) pairs over a CTA of THREADS: this
// thread's exclusive pair and the CTA's aggregate.  wv and wf are
// THREADS / 32 words of shared memory each; ends with a barrier.
template <int THREADS>
SR_DEV void cta_seg_scan(bool tf, int32_t tv, int32_t* wv, int32_t* wf, bool& fe, int32_t& ve, bool& aggf,
                         int32_t& agg) {
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    bool fi = tf;
    int32_t vi = tv;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const bool fp = __shfl_up_sync(0xFFFFFFFFu, (int)fi, d) != 0;
        const int32_t vp = __shfl_up_sync(0xFFFFFFFFu, vi, d);
        if ((int)lane >= d) seg_combine(fp, vp, fi, vi);
    }
    bool xf = __shfl_up_sync(0xFFFFFFFFu, (int)fi, 1) != 0;
    int32_t xv = __shfl_up_sync(0xFFFFFFFFu, vi, 1);
    if (lane == 0) {
        xf = false;
        xv = 0;
    }
    if (lane == 31) {
        wv[warp] = vi;
        wf[warp] = fi ? 1 : 0;
    }
    __syncthreads();
    // the warps before this one, and all of them for the aggregate
    bool pf = false;
    int32_t pv = 0;
    aggf = false;
    agg = 0;
#pragma unroll
    for (int w = 0; w < THREADS / 32; ++w) {
        bool f = wf[w] != 0;
        int32_t v = wv[w];
        if (w < (int)warp) {
            bool f2 = f;
            int32_t v2 = v;
            seg_combine(pf, pv, f2, v2);
            pf = f2;
            pv = v2;
        }
        seg_combine(aggf, agg, f, v);
        aggf = f;
        agg = v;
    }
    seg_combine(pf, pv, xf, xv);
    fe = xf;
    ve = xv;
    __syncthreads();
}
}  // namespace

// Per tile: the (head seen, sum since) pair of its winding changes.
template <int ITEMS, int THREADS>
__global__ void __launch_bounds__(THREADS) k_winding_reduce(const WindArgs a, uint64_t* __restrict__ tagg) {
    constexpr int kTile = THREADS * ITEMS;
    __shared__ int32_t wv[THREADS / 32], wf[THREADS / 32];
    const int64_t n = a.n_dev ? (int64_t)min((uint64_t)*a.n_dev, (uint64_t)a.n) : a.n;
    const int64_t tbase = (int64_t)blockIdx.x * kTile;
    if (tbase >= n) return;
    const int64_t ibase = tbase + (int64_t)threadIdx.x * ITEMS;
    uint64_t kk[ITEMS];
    uint32_t wbits;
    load_run<ITEMS>(a, ibase, n, kk, wbits, nullptr);
    uint64_t kprev = 0;
    if (a.st.n_scenes > 1) kprev = prev_key<ITEMS>(a, ibase, n, kk);
    bool tf, fe, aggf;
    int32_t tv, ve, agg;
    run_heads<ITEMS>(a, ibase, n, kk, kprev, wbits, tf, tv);
    cta_seg_scan<THREADS>(tf, tv, wv, wf, fe, ve, aggf, agg);
    if (threadIdx.x == 0) tagg[blockIdx.x] = (aggf ? kHeadBit : 0ull) | (uint32_t)agg;
}

// The tiles' incoming winding prefixes: an exclusive segmented scan of the
// tile pairs in one CTA, 1,024 tiles a round.  Also writes the scan's total
// (the winding scan's last entry) when the stages are kept.
__global__ void __launch_bounds__(1024) k_winding_scan_tiles(const uint64_t* __restrict__ tagg,
                                                            int32_t* __restrict__ tile_in, const WindArgs a,
                                                            int tile_records) {
    __shared__ int32_t wv[32], wf[32];
    const int64_t n = a.n_dev ? (int64_t)min((uint64_t)*a.n_dev, (uint64_t)a.n) : a.n;
    const int64_t tiles = (n + tile_records - 1) / tile_records;
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    bool cf = false;
    int32_t cv = 0;
    for (int64_t base = 0; base < tiles; base += 1024) {
        const int64_t t = base + threadIdx.x;
        const uint64_t w = t < tiles ? tagg[t] : 0ull;
        bool fi = (w & kHeadBit) != 0;
        int32_t vi = (int32_t)(uint32_t)w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const bool fp = __shfl_up_sync(0xFFFFFFFFu, (int)fi, d) != 0;
            const int32_t vp = __shfl_up_sync(0xFFFFFFFFu, vi, d);
            if ((int)lane >= d) seg_combine(fp, vp, fi, vi);
        }
        if (lane == 31) {
            wv[warp] = vi;
            wf[warp] = fi ? 1 : 0;
        }
        __syncthreads();
        if (warp == 0) {
            bool f2 = wf[lane] != 0;
            int32_t v2 = wv[lane];
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const bool fp = __shfl_up_sync(0xFFFFFFFFu, (int)f2, d) != 0;
                const int32_t vp = __shfl_up_sync(0xFFFFFFFFu, v2, d);
                if ((int)lane >= d) seg_combine(fp, vp, f2, v2);
            }
            wv[lane] = v2;   // inclusive over warps 0..lane
            wf[lane] = f2 ? 1 : 0;
        }
        __syncthreads();
        // the pair before this tile: the carry, the warps before, the lanes before
        bool pf = cf;
        int32_t pv = cv;
        if (warp > 0) {
            bool f2 = wf[warp - 1] != 0;
            int32_t v2 = wv[warp - 1];
            seg_combine(pf, pv, f2, v2);
            pf = f2;
            pv = v2;
        }
        // lanes before: the inclusive pair of lane - 1 within the warp
        bool lf = __shfl_up_sync(0xFFFFFFFFu, (int)fi, 1) != 0;
        int32_t lv = __shfl_up_sync(0xFFFFFFFFu, vi, 1);
        if (lane > 0) seg_combine(pf, pv, lf, lv);
        else {
            lf = pf;
            lv = pv;
        }
        // the value since the last head entering the tile, whatever lf says
        if (t < tiles) tile_in[t] = lv;
        bool nf = wf[31] != 0;
        int32_t nv = wv[31];
        seg_combine(cf, cv, nf, nv);
        __syncthreads();
        cf = nf;
        cv = nv;
    }
    if (threadIdx.x == 0 && a.dbg_wscan) a.dbg_wscan[n] = cv;
}

// Each thread owns ITEMS consecutive sorted records (a blocked layout): its
// keys come in as 16-byte vector loads, the keys on either side of its run
// by warp shuffles (a scalar load at a warp's edges), and the flags stay in
// registers.  The tile's draw records are contiguous in the output, so they
// are listed as items in shared memory and written an item a thread:
// consecutive threads write consecutive records.
template <int ITEMS, int THREADS>
__global__ void __launch_bounds__(THREADS, 5) k_winding_emit(const WindArgs a,
                                                              const int32_t* __restrict__ tile_in,
                                                              uint64_t* __restrict__ tstatB, uint32_t* counter,
                                                              uint32_t* status, uint32_t spin_limit) {
    constexpr int kTile = THREADS * ITEMS;
    static_assert(ITEMS % 2 == 0 && ITEMS <= 8, "records per thread");
    static_assert(kTile <= 4096, "record and fragment index of an item");
    __shared__ Smem<ITEMS, THREADS> S;
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) S.tile = atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t tile = S.tile;
    const int64_t n = a.n_dev ? (int64_t)min((uint64_t)*a.n_dev, (uint64_t)a.n) : a.n;
    const int64_t tbase = (int64_t)tile * kTile;
    const int64_t num_tiles = (n + kTile - 1) / kTile;
    if (tbase >= n) {
        // launched for the capacity: nothing here; an empty frame still
        // reports its (zero) totals
        if (n == 0 && tile == 0 && threadIdx.x == 0) {
            a.totals[0] = 0;
            a.totals[1] = 0;
            *a.n_draw = 0;
            if (a.dbg_wscan) a.dbg_wscan[0] = 0;
        }
        return;
    }
    const int32_t t_in = tile_in[tile];
    const uint32_t xbits = a.L.xbits, pshift = a.L.xbits + a.L.rbits;
    const uint32_t xmask = (1u << xbits) - 1u, rmask = (1u << a.L.rbits) - 1u;
    const uint32_t off_rank = (uint32_t)(a.L.Hy - 1);
    const bool multi = a.st.n_scenes > 1;

    // ---- this thread's records: keys and packed winding bits (4 bits each)
    const int64_t ibase = tbase + (int64_t)threadIdx.x * ITEMS;
    const int nvalid = (int)max((int64_t)0, min((int64_t)ITEMS, n - ibase));
    uint64_t kk[ITEMS];
    uint32_t wbits;
    load_run<ITEMS>(a, ibase, n, kk, wbits, status);
    // the fill rule and paint of the first record's path, fetched early
    uint32_t rule_path = nvalid > 0 ? (uint32_t)(kk[0] >> pshift) : 0xFFFFFFFFu;
    uint32_t rule = nvalid > 0 ? a.fill_rule[rule_path] : 0u;
    uint32_t paint_path = rule_path;
    uint32_t paint0 = nvalid > 0 ? a.fill_info[paint_path] : 0u;
    // the record before this thread's first, and after its last
    const uint64_t kprev = prev_key<ITEMS>(a, ibase, n, kk);
    uint64_t knext = __shfl_down_sync(0xFFFFFFFFu, kk[0], 1);
    uint32_t wnext = 0;
    if (lane == 31) knext = ibase + ITEMS < n ? wkey(a, ibase + ITEMS, n, wnext, nullptr) : ~0ull;
    if (nvalid < ITEMS || ibase + ITEMS == n) knext = ~0ull;   // no record after this thread's last
    if (threadIdx.x == THREADS - 1) {
        S.next_key = knext;
        S.next_c = sx2(wnext >> 2);
    }

    // ---- winding prefix: the tile's from the tile scan, then the CTA's
    // segmented scan (segments start at scene heads)
    bool tf, fe, aggf;
    int32_t tv, ve, agg;
    const uint32_t heads = run_heads<ITEMS>(a, ibase, n, kk, kprev, wbits, tf, tv);
    cta_seg_scan<THREADS>(tf, tv, S.warpA, S.warpAf, fe, ve, aggf, agg);
    int32_t wrun = fe ? ve : wadd(t_in, ve);

    // From here a key is handled as two 32-bit halves: its path, and
    // (row rank, x + 1) below it (at most 29 bits for a 16384-pixel canvas).
    // A key is (path, row rank, x + 1) with the rank of an off-canvas record
    // Hy - 1, so two records share a cell exactly when their keys are equal,
    // and a row of one path when they agree above the x bits.
    const uint32_t lomask = (1u << pshift) - 1u;
    uint32_t kp[ITEMS], kl[ITEMS];
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        kp[k] = (uint32_t)(kk[k] >> pshift);
        kl[k] = (uint32_t)kk[k] & lomask;
    }
    const uint32_t pprev = (uint32_t)(kprev >> pshift), lprev = (uint32_t)kprev & lomask;
    {
        uint4* dst = reinterpret_cast<uint4*>(&S.lo[threadIdx.x * ITEMS]);
#pragma unroll
        for (int q = 0; q < ITEMS / 4; ++q) dst[q] = make_uint4(kl[4 * q], kl[4 * q + 1], kl[4 * q + 2], kl[4 * q + 3]);
        if (threadIdx.x == 0) S.lo_prev = lprev;
    }

    // ---- centre parts of each record's cell from it to the cell's end
    // (pixel mode): a reverse segmented sum over runs of equal keys, with
    // the run that continues past this thread walked in global memory
    int32_t csum[ITEMS];
    if (a.pixel_mode) {
        // within the thread
        const bool cont_last = knext == kk[ITEMS - 1];
        csum[ITEMS - 1] = sx2(wbits >> (4 * (ITEMS - 1) + 2));
#pragma unroll
        for (int k = ITEMS - 2; k >= 0; --k) {
            const bool cont = kp[k + 1] == kp[k] && kl[k + 1] == kl[k];
            csum[k] = wadd(sx2(wbits >> (4 * k + 2)), cont ? csum[k + 1] : 0);
        }
        bool all_same = nvalid == ITEMS;
#pragma unroll
        for (int k = 1; k < ITEMS; ++k) all_same = all_same && kp[k] == kp[0] && kl[k] == kl[0];
        S.run_p[threadIdx.x] = kp[0];
        S.run_l[threadIdx.x] = kl[0];
        S.run_sum[threadIdx.x] = csum[0];
        S.run_all[threadIdx.x] = all_same ? 1u : 0u;
        __syncthreads();
        // the run that continues past this thread: the leading runs of the
        // next threads (a thread whose records all share the key passes it
        // on), then the records after the tile.  Only a merged fragment (an
        // on-canvas cell whose run starts in this thread) needs it;
        // off-canvas records of a path share one key (one per row past its
        // right edge) and make long runs, which are never followed.
        const uint32_t pl = kp[ITEMS - 1], ll = kl[ITEMS - 1];
        bool starts_here = pprev != pl || lprev != ll;
#pragma unroll
        for (int k = 1; k < ITEMS; ++k) starts_here = starts_here || kp[k - 1] != pl || kl[k - 1] != ll;
        const uint32_t rankl = (ll >> xbits) & rmask, xol = ll & xmask;
        const uint32_t xo_maxl = (uint32_t)div_F((multi ? scene_of_path(a.st, pl).W : a.W) + a.F - 1, a.F);
        int32_t tail = 0;
        if (cont_last && starts_here && rankl != off_rank && xol >= 1u && xol <= xo_maxl) {
            uint32_t t = threadIdx.x + 1;
            bool follow = true;
            while (follow && t < THREADS) {
                if (S.run_p[t] != pl || S.run_l[t] != ll) {
                    follow = false;
                    break;
                }
                tail = wadd(tail, S.run_sum[t]);
                follow = S.run_all[t] != 0;
                ++t;
            }
            if (follow && S.next_key == kk[ITEMS - 1]) {
                tail = wadd(tail, S.next_c);
                // a run of two or more records past the tile end (rare)
                for (int64_t j = tbase + kTile + 1; j < n; ++j) {
                    uint32_t wb = 0;
                    if (wkey(a, j, n, wb, nullptr) != kk[ITEMS - 1]) break;
                    tail = wadd(tail, sx2(wb >> 2));
                }
            }
        }
        // the last record's run gets the tail, and so do the records before
        // it in the same run
        bool in_run = true;
#pragma unroll
        for (int k = ITEMS - 1; k >= 0; --k) {
            in_run = in_run && kp[k] == pl && kl[k] == ll;
            if (in_run) csum[k] = wadd(csum[k], tail);
        }
    }

    // ---- flags (mark_merged_fragment_and_span.comp:22-93)
    uint32_t ffm = 0, sfm = 0;
    const int32_t F = a.F;
    // on the canvas: a row of it, and 0 <= x = (xo - 1) F < W, i.e. 1 <= xo <= ceil(W / F)
    const uint32_t xo_max1 = (uint32_t)div_F(a.W + F - 1, F);
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        if ((heads >> k) & 1u) wrun = 0;
        const int32_t wscan = wrun;
        wrun = wadd(wrun, sx2(wbits >> (4 * k)));
        if (k >= nvalid) continue;
        const uint32_t p1 = kp[k], l1 = kl[k];
        const uint32_t p0 = k == 0 ? pprev : kp[k - 1], l0 = k == 0 ? lprev : kl[k - 1];
        const uint32_t xo1 = l1 & xmask, rank1 = l1 >> xbits;
        const uint32_t xo_max = multi ? (uint32_t)div_F(scene_of_path(a.st, p1).W + F - 1, F) : xo_max1;
        const bool on = rank1 != off_rank && xo1 >= 1u && xo1 <= xo_max;
        const bool first = ibase + k == 0;
        bool ff = on && (first || p0 != p1 || l0 != l1);
        bool sf = !first && p0 == p1 && (l0 >> xbits) == rank1 && (l0 & xmask) + 1u < xo1;
        if (sf || (ff && a.pixel_mode)) {
            if (p1 != rule_path) {
                rule = a.fill_rule[p1];
                rule_path = p1;
            }
            if (sf) sf = rule_pass(rule, wscan);
            // centre sample of the merged cell: scan at its first record plus
            // the left-of-centre changes of the cell's pieces
            if (ff && a.pixel_mode) ff = rule_pass(rule, wadd(wscan, csum[k]));
        }
        if (ff || sf) {
            if (p1 != paint_path) {
                paint0 = a.fill_info[p1];
                paint_path = p1;
            }
            S.paint[threadIdx.x * ITEMS + k] = paint0;
        }
        ffm |= (ff ? 1u : 0u) << k;
        sfm |= (sf ? 1u : 0u) << k;
        if (a.dbg_wscan) {
            const int64_t i = ibase + k;
            a.dbg_wscan[i] = wscan;
            a.dbg_fflag[i] = ff ? 1 : 0;
            a.dbg_sflag[i] = sf ? 1 : 0;
            a.dbg_skey[i] = unpack_key(a.L, kk[k]).yx;
        }
    }

    // ---- output slots.  Within the CTA the counts are packed 16:16 (a tile
    // has at most 2 x 2048 outputs); across tiles 31:31 with a look-back.
    const uint32_t bsum = ((uint32_t)__popc(ffm) << 16) | (uint32_t)__popc(sfm);
    const uint32_t inclB = warp_incl<uint32_t>(bsum);
    if (lane == 31) S.warpB[warp] = inclB;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = lane < THREADS / 32 ? S.warpB[lane] : 0u;
        const uint32_t wi = warp_incl<uint32_t>(w);
        if (lane < THREADS / 32) S.warpB[lane] = wi - w;
        const uint32_t agg16 = __shfl_sync(0xFFFFFFFFu, wi, THREADS / 32 - 1);
        const uint64_t aggB = ((uint64_t)(agg16 >> 16) << kFragShift) | (uint64_t)(agg16 & 0xFFFFu);
        if (lane == 0) st_release_u64(&tstatB[tile], (tile == 0 ? kFlagP : kFlagA) | aggB);
        uint64_t excl = 0;
        if (tile > 0) {
            excl = lookback<false>(tstatB, tile, status, spin_limit);
            if (lane == 0) st_release_u64(&tstatB[tile], kFlagP | (excl + aggB));
        }
        if (lane == 0) {
            S.prefixB = excl;
            S.count = (agg16 >> 16) + (agg16 & 0xFFFFu);
            if (tile == num_tiles - 1) {
                const uint64_t tot = excl + aggB;
                a.totals[0] = tot >> kFragShift;
                a.totals[1] = tot & kSpanMask;
                *a.n_draw = (uint32_t)((tot >> kFragShift) + (tot & kSpanMask));
            }
        }
    }
    __syncthreads();
    // this thread's items: in record order, a record's fragment before its span
    {
        const uint32_t l0 = S.warpB[warp] + (inclB - bsum);
        uint32_t lf = l0 >> 16, slot = lf + (l0 & 0xFFFFu);
        if (ffm | sfm) {
#pragma unroll
            for (int k = 0; k < ITEMS; ++k) {
                const uint32_t rec = (threadIdx.x * ITEMS + k) << kItemRecShift;
                if ((ffm >> k) & 1u) S.items[slot++] = rec | lf++;
                if ((sfm >> k) & 1u) S.items[slot++] = rec | kItemSpan;
            }
        }
    }
    __syncthreads();

    // ---- emit draw records (gen_merged_fragment_and_span.comp:33-103), an
    // item a thread, from the key halves and paint staged in shared memory.
    // An emitted record's cell is on the canvas: y = yy F with yy its row
    // (rank Hy is row 0, rank r < Hy - 1 is row r + 1), x = (xo - 1) F.  A
    // span's left end is the cell after the record before it (same path and
    // row: only its x bits are read).  Each record also adds to its row's record count and pixel
    // sum (summed over the lanes of a warp that share the row), and an opaque
    // span to the cuts of the resolve segments it covers whole.
    const uint64_t tprefix = S.prefixB;
    const int64_t tile_first = (int64_t)((tprefix >> kFragShift) + (tprefix & kSpanMask));
    const uint64_t frag0 = tprefix >> kFragShift;
    const uint32_t tile_cnt = S.count;
    const bool need_path = multi || a.path_draw;
    // every lane of a warp runs the same rounds (the row sums are warp-wide)
    const uint32_t rounds_end = (tile_cnt + THREADS - 1) / THREADS * THREADS;
    for (uint32_t j = threadIdx.x; j < rounds_end; j += THREADS) {
        const bool live = j < tile_cnt;
        uint32_t row = 0xFFFFFFFFu, written = 0, px = 0;
        if (live) {
            const uint32_t it = S.items[j];
            const bool span = (it & kItemSpan) != 0;
            const uint32_t r = it >> kItemRecShift;
            const uint32_t l1 = S.lo[r], info = S.paint[r];
            uint32_t path1 = 0;
            if (need_path) {
                path1 = (uint32_t)(key_part(a.L, a.skeys[tbase + r]) >> pshift);
                if (path1 >= a.n_paths) path1 = 0;
            }
            const uint32_t rank1 = (l1 >> xbits) & rmask;
            const int32_t yy = rank1 == (uint32_t)a.L.Hy ? 0 : (int32_t)rank1 + 1;
            row = (multi ? scene_of_path(a.st, path1).row_base : 0u) + (uint32_t)yy;
            const int32_t y = yy * F, x1 = ((int32_t)(l1 & xmask) - 1) * F;
            const int64_t o = tile_first + j;
            int4 d;
            if (!span) {
                d = make_int4((int32_t)((uint32_t)y << 16) | x1, F, (int32_t)info,
                              (int32_t)(frag0 + (it & (kItemSpan - 1u)) + 1u));
                px = (uint32_t)F;
            } else {
                // the span's left cell is the record before it, in the same
                // path and row (a span is never record 0)
                const uint32_t l0 = r > 0 ? S.lo[r - 1] : S.lo_prev;
                const int32_t x0 = imax(0, wadd(((int32_t)(l0 & xmask) - 1) * F, F));
                d = make_int4((int32_t)((uint32_t)y << 16) | x0, x1 - x0, (int32_t)info, 0);
                px = (uint32_t)imax(x1 - x0, 0);
                // a span that hides everything under it ends the resolve's
                // work before it in each segment it covers whole
                if (a.seg_cut && o < a.draw_capacity && row < a.cut_rows && (!a.pixel_mode || (info >> 24) == 255u)) {
                    const int32_t s_hi = imin(x1 / kResolveSeg, (int32_t)a.cut_segs);
                    for (int32_t sg = (x0 + kResolveSeg - 1) / kResolveSeg; sg < s_hi; ++sg)
                        atomicMax(&a.seg_cut[(size_t)row * a.cut_segs + (uint32_t)sg], (uint32_t)o + 1u);
                }
            }
            if (a.path_draw) atomicAdd(&a.path_draw[path1], 1u);
            // only records inside the draw capacity are written and counted,
            // so that the row sort and the resolve stay inside the buffers
            if (o < a.draw_capacity) {
                a.draw[o] = d;
                a.draw_row[o] = row;
                written = 1;
            } else {
                set_error(status, ERR_CAPACITY);
                px = 0;
            }
        }
        if (a.row_count) {
            const bool counted = written != 0 && row < a.cut_rows;
            const uint32_t peers = __match_any_sync(0xFFFFFFFFu, counted ? row : 0xFFFFFFFFu);
            if (counted) {
                const uint32_t cnt = __popc(peers);
                const uint32_t psum = __reduce_add_sync(peers, px);
                if (lane == (uint32_t)(__ffs(peers) - 1)) {
                    atomicAdd(&a.row_count[row], cnt);
                    if (a.row_px) atomicAdd(&a.row_px[row], (unsigned long long)psum);
                }
            }
        }
    }
}

// Tiles of 256 threads with 4 or 8 records each.
static int64_t wind_tile(int items) { return items == 4 ? 1024 : 2048; }

size_t winding_status_words(int64_t n, int items) {
    const int64_t tile = wind_tile(items);
    // look-back words of the output slots, tile pairs, tile prefixes
    return 3 * (size_t)((n + tile - 1) / tile + 1);
}

template <int ITEMS, int THREADS>
static void launch_wind(const WindArgs& a, int64_t tiles, uint64_t* sB, uint64_t* tagg, int32_t* tile_in,
                        uint32_t* tile_counter, uint32_t* status, cudaStream_t st) {
    k_winding_reduce<ITEMS, THREADS><<<(unsigned)tiles, THREADS, 0, st>>>(a, tagg);
    k_winding_scan_tiles<<<1, 1024, 0, st>>>(tagg, tile_in, a, ITEMS * THREADS);
    k_winding_emit<ITEMS, THREADS><<<(unsigned)tiles, THREADS, 0, st>>>(a, tile_in, sB, tile_counter, status,
                                                                        spin_limit());
}

void launch_winding_emit(const WindArgs& a, int items, uint64_t* tile_status, uint32_t* tile_counter,
                         uint32_t* status, cudaStream_t st) {
    if (a.n <= 0) return;
    const int64_t tile = wind_tile(items);
    const int64_t tiles = (a.n + tile - 1) / tile;
    uint64_t* sB = tile_status;
    uint64_t* tagg = tile_status + (tiles + 1);
    int32_t* tile_in = reinterpret_cast<int32_t*>(tile_status + 2 * (tiles + 1));
    count_launches(3);
    if (items == 4) launch_wind<4, 256>(a, tiles, sB, tagg, tile_in, tile_counter, status, st);
    else launch_wind<8, 256>(a, tiles, sB, tagg, tile_in, tile_counter, status, st);
}

}  // namespace sr
