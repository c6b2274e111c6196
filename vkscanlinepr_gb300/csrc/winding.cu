// winding.cu — one pass over the sorted records that replaces five reference
// dispatches and two host read-backs:
//   shuffle_fragment.comp:17-26            gather of winding changes
//   naive_scan.comp (scanline_rasterizer.cpp:479-506)   winding scan
//   mark_merged_fragment_and_span.comp:22-93            fragment/span flags
//   naive_scan.comp over 2N flags (scanline_rasterizer.cpp:545-580)
//   gen_merged_fragment_and_span.comp:33-103           draw-list emit
//
// Each CTA owns 2048 consecutive sorted records.  Chain A (decoupled
// look-back) gives the exclusive winding prefix of each record; the flags of
// each record follow; chain B (a second look-back, packed 31:31-bit counts
// of merged fragments and spans) gives each record's output slot.  Draw
// records come out in the reference's order: a record's merged fragment,
// then the span ending at it.
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
constexpr int kThreads = 256;   // records per tile: kThreads x ITEMS (4 or 8)
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

template <int ITEMS> struct Smem {
    static constexpr int kTile = kThreads * ITEMS;
    uint32_t tile;
    int32_t warpA[kThreads / 32];
    int32_t warpAf[kThreads / 32];
    uint64_t warpB[kThreads / 32];
    int32_t prefixA;
    uint64_t prefixB;
    uint64_t keys[kTile + 1];   // keys[0] = predecessor of the tile
    uint8_t wb[kTile];          // packed winding bits of each record
};
}  // namespace

template <int ITEMS>
__global__ void __launch_bounds__(kThreads) k_winding_emit(const WindArgs a, uint64_t* __restrict__ tstatA,
                                                           uint64_t* __restrict__ tstatB, uint32_t* counter,
                                                           uint32_t* status, uint32_t spin_limit) {
    constexpr int kItems = ITEMS, kTile = kThreads * ITEMS;
    __shared__ Smem<ITEMS> S;
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

    // ---- stage keys (coalesced) and gather winding bits
    for (int j = threadIdx.x; j < kTile; j += kThreads) {
        int64_t i = tbase + j;
        uint64_t k = 0;
        uint8_t w = 0;
        if (i < n) {
            k = a.skeys[i];
            if (a.svals) {
                uint32_t rec = a.svals[i];
                if (rec < (uint64_t)n) w = a.wnp[rec];
                else set_error(status, ERR_BAD_INDEX);
            } else {
                w = (uint8_t)payload_part(a.L, k);
                k = key_part(a.L, k);
            }
            if ((k >> (a.L.xbits + a.L.rbits)) >= a.n_paths) {
                set_error(status, ERR_BAD_INDEX);
                k = 0;
            }
        }
        S.keys[j + 1] = k;
        S.wb[j] = w;
    }
    if (threadIdx.x == 0) {
        uint64_t k0 = tbase > 0 ? key_part(a.L, a.skeys[tbase - 1]) : 0ull;
        if ((k0 >> (a.L.xbits + a.L.rbits)) >= a.n_paths) k0 = 0;
        S.keys[0] = k0;
    }
    __syncthreads();

    const int64_t ibase = tbase + (int64_t)threadIdx.x * kItems;
    int32_t wn[kItems];
    bool hd[kItems];   // first record of a scene
    // thread aggregate of the segmented scan: (head seen, sum since it)
    bool tf = false;
    int32_t tv = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        int64_t i = ibase + k;
        int32_t w = 0;
        bool h = false;
        if (i < n) {
            w = sx2(S.wb[i - tbase]);
            const int jl = (int)(i - tbase);
            const uint32_t p1 = (uint32_t)(S.keys[jl + 1] >> (a.L.xbits + a.L.rbits));
            const uint32_t p0 = (uint32_t)(S.keys[jl] >> (a.L.xbits + a.L.rbits));
            h = (i == 0) || (a.st.n_scenes > 1 && a.st.path_scene[p1] != a.st.path_scene[p0]);
        }
        wn[k] = w;
        hd[k] = h;
        if (h) {
            tf = true;
            tv = 0;
        }
        tv = wadd(tv, w);
    }

    // ---- chain A: segmented winding prefix
    // inclusive warp scan of (f, v) pairs: (fa, va) + (fb, vb) = (fa|fb, fb ? vb : va + vb)
    bool fi = tf;
    int32_t vi = tv;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        bool fp = __shfl_up_sync(0xFFFFFFFFu, (int)fi, d) != 0;
        int32_t vp = __shfl_up_sync(0xFFFFFFFFu, vi, d);
        if ((int)lane >= d) {
            vi = fi ? vi : wadd(vp, vi);
            fi = fi || fp;
        }
    }
    // exclusive value for the lane
    bool fe = __shfl_up_sync(0xFFFFFFFFu, (int)fi, 1) != 0;
    int32_t ve = __shfl_up_sync(0xFFFFFFFFu, vi, 1);
    if (lane == 0) {
        fe = false;
        ve = 0;
    }
    if (lane == 31) {
        S.warpA[warp] = vi;
        S.warpAf[warp] = fi ? 1 : 0;
    }
    __syncthreads();
    if (warp == 0) {
        bool wf = lane < kThreads / 32 ? S.warpAf[lane] != 0 : false;
        int32_t wv = lane < kThreads / 32 ? S.warpA[lane] : 0;
        bool f2 = wf;
        int32_t v2 = wv;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            bool fp = __shfl_up_sync(0xFFFFFFFFu, (int)f2, d) != 0;
            int32_t vp = __shfl_up_sync(0xFFFFFFFFu, v2, d);
            if ((int)lane >= d) {
                v2 = f2 ? v2 : wadd(vp, v2);
                f2 = f2 || fp;
            }
        }
        // exclusive per warp, and the tile aggregate
        bool xf = __shfl_up_sync(0xFFFFFFFFu, (int)f2, 1) != 0;
        int32_t xv = __shfl_up_sync(0xFFFFFFFFu, v2, 1);
        if (lane == 0) {
            xf = false;
            xv = 0;
        }
        const bool aggf = __shfl_sync(0xFFFFFFFFu, (int)f2, kThreads / 32 - 1) != 0;
        const int32_t agg = __shfl_sync(0xFFFFFFFFu, v2, kThreads / 32 - 1);
        if (lane == 0)
            st_release_u64(&tstatA[tile], (tile == 0 ? kFlagP : kFlagA) | (aggf ? kHeadBit : 0ull) | (uint32_t)agg);
        int32_t excl = 0;
        if (tile > 0) {
            excl = (int32_t)(uint32_t)lookback<true>(tstatA, tile, status, spin_limit);
            if (lane == 0) st_release_u64(&tstatA[tile], kFlagP | (uint32_t)(aggf ? agg : wadd(excl, agg)));
        }
        // carry into each warp: the tile prefix combined with the warp's exclusive pair
        if (lane < kThreads / 32) {
            S.warpA[lane] = xf ? xv : wadd(excl, xv);
        }
        if (lane == 0 && tile == num_tiles - 1 && a.dbg_wscan) a.dbg_wscan[n] = aggf ? agg : wadd(excl, agg);
    }
    __syncthreads();
    // carry into this thread, then per record (reset at scene heads)
    int32_t wrun = fe ? ve : wadd(S.warpA[warp], ve);

    // ---- flags
    // From the keys themselves: a key is (path, row rank, x + 1) with the
    // rank of an off-canvas record Hy - 1, so two records share a cell
    // exactly when their keys are equal, and share a row of one path when
    // they agree above the x bits.
    uint32_t ff[kItems], sf[kItems];
    uint64_t bsum = 0;
    const int32_t F = a.F;
    const uint32_t xbits = a.L.xbits, pshift = a.L.xbits + a.L.rbits;
    const uint32_t xmask = (1u << xbits) - 1u, rmask = (1u << a.L.rbits) - 1u;
    const uint32_t off_rank = (uint32_t)(a.L.Hy - 1);
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        int64_t i = ibase + k;
        if (hd[k]) wrun = 0;
        int32_t wscan = wrun;
        wrun = wadd(wrun, wn[k]);
        ff[k] = 0;
        sf[k] = 0;
        if (i >= n) continue;
        int jl = (int)(i - tbase);
        const uint64_t k1 = S.keys[jl + 1], k0 = S.keys[jl];
        const uint32_t path1 = (uint32_t)(k1 >> pshift);
        const uint32_t xo1 = (uint32_t)k1 & xmask, rank1 = (uint32_t)(k1 >> xbits) & rmask;
        const int32_t Wp = a.st.n_scenes > 1 ? scene_of_path(a.st, path1).W : a.W;
        // on the canvas: a row of it, and 0 <= x = (xo - 1) F < W
        const bool on = rank1 != off_rank && xo1 >= 1u && (int32_t)(xo1 - 1u) * F < Wp;
        uint32_t rule = a.fill_rule[path1];
        if (i == 0) {
            ff[k] = on ? 1u : 0u;
        } else {
            if (on && k0 != k1) ff[k] = 1u;
            if (((k0 ^ k1) >> xbits) == 0 && ((uint32_t)k0 & xmask) + 1u < xo1 && rule_pass(rule, wscan)) sf[k] = 1u;
        }
        if (a.pixel_mode && ff[k]) {
            // centre sample of the merged cell: scan at its first record plus
            // the left-of-centre changes of the cell's pieces
            int32_t wc = wscan;
            int64_t j = i;
            for (;;) {
                uint64_t kj;
                int32_t lj;
                int64_t jt = j - tbase;
                if (jt < kTile) {
                    kj = S.keys[jt + 1];
                    lj = sx2((uint32_t)S.wb[jt] >> 2);
                } else if (a.svals) {
                    kj = a.skeys[j];
                    uint32_t rec = a.svals[j];
                    lj = rec < (uint64_t)n ? sx2((uint32_t)a.wnp[rec] >> 2) : 0;
                } else {
                    const uint64_t kr = a.skeys[j];
                    kj = key_part(a.L, kr);
                    lj = sx2(payload_part(a.L, kr) >> 2);
                }
                if (kj != k1) break;
                wc = wadd(wc, lj);
                if (++j >= n) break;
            }
            if (!rule_pass(rule, wc)) ff[k] = 0u;
        }
        if (a.dbg_wscan) {
            a.dbg_wscan[i] = wscan;
            a.dbg_fflag[i] = (int32_t)ff[k];
            a.dbg_sflag[i] = (int32_t)sf[k];
            a.dbg_skey[i] = unpack_key(a.L, k1).yx;
        }
        bsum += ((uint64_t)ff[k] << kFragShift) | (uint64_t)sf[k];
    }

    // ---- chain B: output slots
    uint64_t inclB = warp_incl<uint64_t>(bsum);
    if (lane == 31) S.warpB[warp] = inclB;
    __syncthreads();
    if (warp == 0) {
        uint64_t w = lane < kThreads / 32 ? S.warpB[lane] : 0ull;
        uint64_t wi = warp_incl<uint64_t>(w);
        if (lane < kThreads / 32) S.warpB[lane] = wi - w;
        uint64_t agg = __shfl_sync(0xFFFFFFFFu, wi, kThreads / 32 - 1);
        if (lane == 0) st_release_u64(&tstatB[tile], (tile == 0 ? kFlagP : kFlagA) | agg);
        uint64_t excl = 0;
        if (tile > 0) {
            excl = lookback<false>(tstatB, tile, status, spin_limit);
            if (lane == 0) st_release_u64(&tstatB[tile], kFlagP | (excl + agg));
        }
        if (lane == 0) {
            S.prefixB = excl;
            if (tile == num_tiles - 1) {
                uint64_t tot = excl + agg;
                a.totals[0] = tot >> kFragShift;
                a.totals[1] = tot & kSpanMask;
                *a.n_draw = (uint32_t)((tot >> kFragShift) + (tot & kSpanMask));
            }
        }
    }
    __syncthreads();
    uint64_t brun = S.prefixB + S.warpB[warp] + (inclB - bsum);

    // ---- emit draw records (gen_merged_fragment_and_span.comp:155-196)
    // An emitted record's cell is on the canvas: y = yy F with yy its row
    // (rank Hy is row 0, rank r < Hy - 1 is row r + 1), x = (xo - 1) F.
    // The records written per cell row are counted for the row sort, and
    // their pixels summed for the resolve; a thread's records are
    // consecutive, so it adds a run of one row at once.
    uint32_t run_row = 0, run_cnt = 0, run_px = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) {
        int64_t i = ibase + k;
        uint64_t fb = brun >> kFragShift, sb = brun & kSpanMask;
        brun += ((uint64_t)ff[k] << kFragShift) | (uint64_t)sf[k];
        uint32_t row = 0, written = 0, px = 0;
        if (i < n && (ff[k] | sf[k])) {
            int jl = (int)(i - tbase);
            const uint64_t k1 = S.keys[jl + 1];
            const uint32_t path1 = (uint32_t)(k1 >> pshift);
            const uint32_t rank1 = (uint32_t)(k1 >> xbits) & rmask;
            const int32_t yy = rank1 == (uint32_t)a.L.Hy ? 0 : (int32_t)rank1 + 1;
            const int32_t y = yy * F, x1 = ((int32_t)((uint32_t)k1 & xmask) - 1) * F;
            int32_t info = (int32_t)a.fill_info[path1];
            row = (a.st.n_scenes > 1 ? scene_of_path(a.st, path1).row_base : 0u) + (uint32_t)yy;
            if (a.path_draw) atomicAdd(&a.path_draw[path1], ff[k] + sf[k]);
            int64_t o = (int64_t)(fb + sb);
            if (ff[k]) {
                if (o < a.draw_capacity) {
                    a.draw[o] = make_int4((int32_t)((uint32_t)y << 16) | x1, F, info, (int32_t)(fb + 1));
                    a.draw_row[o] = row;
                    ++written;
                    px += (uint32_t)F;
                } else {
                    set_error(status, ERR_CAPACITY);
                }
                ++o;
            }
            if (sf[k]) {
                // the span's left cell is in the same row: x0 = its x + F
                const int32_t x0 = imax(0, wadd(((int32_t)((uint32_t)S.keys[jl] & xmask) - 1) * F, F));
                if (o < a.draw_capacity) {
                    a.draw[o] = make_int4((int32_t)((uint32_t)y << 16) | x0, x1 - x0, info, 0);
                    a.draw_row[o] = row;
                    ++written;
                    px += (uint32_t)imax(x1 - x0, 0);
                    // a span that hides everything under it ends the resolve's
                    // work before it in each segment it covers whole
                    if (a.seg_cut && (!a.pixel_mode || ((uint32_t)info >> 24) == 255u) && row < a.cut_rows) {
                        const int32_t s_hi = imin(x1 / kResolveSeg, (int32_t)a.cut_segs);
                        for (int32_t sg = (x0 + kResolveSeg - 1) / kResolveSeg; sg < s_hi; ++sg)
                            atomicMax(&a.seg_cut[(size_t)row * a.cut_segs + (uint32_t)sg], (uint32_t)o + 1u);
                    }
                } else {
                    set_error(status, ERR_CAPACITY);
                }
            }
        }
        if (a.row_count && written != 0 && row < a.cut_rows) {
            if (run_cnt != 0 && row != run_row) {
                atomicAdd(&a.row_count[run_row], run_cnt);
                if (a.row_px) atomicAdd(&a.row_px[run_row], (unsigned long long)run_px);
                run_cnt = 0;
                run_px = 0;
            }
            run_row = row;
            run_cnt += written;
            run_px += px;
        }
    }
    if (run_cnt != 0) {
        atomicAdd(&a.row_count[run_row], run_cnt);
        if (a.row_px) atomicAdd(&a.row_px[run_row], (unsigned long long)run_px);
    }
}

size_t winding_status_words(int64_t n, int items) {
    const int64_t tile = (int64_t)kThreads * (items == 4 ? 4 : 8);
    return 2 * (size_t)((n + tile - 1) / tile + 1);
}

void launch_winding_emit(const WindArgs& a, int items, uint64_t* tile_status, uint32_t* tile_counter,
                         uint32_t* status, cudaStream_t st) {
    if (a.n <= 0) return;
    items = items == 4 ? 4 : 8;
    const int64_t tile = (int64_t)kThreads * items;
    int64_t tiles = (a.n + tile - 1) / tile;
    uint64_t* sA = tile_status;
    uint64_t* sB = tile_status + (tiles + 1);
    count_launches(1);
    const uint32_t lim = spin_limit();
    if (items == 4) k_winding_emit<4><<<(unsigned)tiles, kThreads, 0, st>>>(a, sA, sB, tile_counter, status, lim);
    else k_winding_emit<8><<<(unsigned)tiles, kThreads, 0, st>>>(a, sA, sB, tile_counter, status, lim);
}

}  // namespace sr
