// sort.cu — onesweep LSD radix sort (8-bit digits) for 64- and 32-bit keys
// with 32-bit values.
//
// Replaces naive_seg_sort_pairs.comp:26-97, an O(len^2) odd-even
// transposition sort per path segment.  The fragment key already carries the
// path in its high bits (see pack_key), so one stable sort of the whole
// array by key gives the reference's per-path order by (signed yx, index).
//
// Per pass, each CTA (dynamic tile id) loads a 4096-key tile, ranks keys by
// digit with warp __match_any_sync / popc, publishes its per-digit counts,
// and looks back over earlier tiles' per-digit counts to find where its run
// of each digit starts; the thread of a digit reads the words of 8
// preceding tiles per step, all loads in flight together.  Keys are first
// scattered into shared memory in digit order, then written out in runs, so
// global stores stay mostly contiguous.  An upfront kernel histograms every
// pass's digits in one read of the keys.
#include "common.cuh"
#include "kernels.h"

namespace sr {

namespace {
constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
// Keys per thread of a tile: 8, 12 or 16 (chosen per plan; 12 by default).
constexpr uint32_t kFlagA = 1u << 30;
constexpr uint32_t kFlagP = 2u << 30;
constexpr uint32_t kCountMask = (1u << 30) - 1u;
constexpr int kMaxPasses = 8;
constexpr int kHistBlocks = 608;   // 152 SMs x 4
constexpr int kLookWindow = 8;     // look-back words read per step
// Lanes holding the same digit: one __match_any_sync, or one ballot per
// digit bit (9 bits: digit 256 marks an empty slot).  The 64-bit fragment
// keys are ranked by ballots (their low digits vary a lot within a warp);
// the 32-bit keys (draw rows, chain classes) arrive in runs, where one
// match is cheaper.
template <bool kMatchAny> SR_DEV uint32_t same_digit_lanes(uint32_t d) {
    if (kMatchAny) return __match_any_sync(0xFFFFFFFFu, d);
    uint32_t peers = 0xFFFFFFFFu;
#pragma unroll
    for (int b = 0; b <= kRadixBits; ++b) {
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, (d >> b) & 1u);
        peers &= ((d >> b) & 1u) ? m : ~m;
    }
    return peers;
}

// Digit of a pass; bits at or above key_bits do not take part.
template <typename K> SR_DEV uint32_t digit_of(K k, uint32_t shift, uint32_t mask) {
    return (uint32_t)(k >> shift) & mask;
}

__host__ __device__ inline uint32_t digit_mask(uint32_t key_bits, uint32_t shift) {
    const uint32_t left = key_bits > shift ? key_bits - shift : 0u;
    return left >= (uint32_t)kRadixBits ? (uint32_t)(kRadix - 1) : ((1u << left) - 1u);
}

struct Scratch {
    uint32_t* hist;       // [passes][256] digit counts, then exclusive offsets
    uint32_t* lookback;   // [passes][tiles + 1][256]
    uint32_t* counters;   // [passes] tile counters
};

Scratch carve(const SortPlan& p, void* base) {
    Scratch s;
    char* b = static_cast<char*>(base);
    s.hist = reinterpret_cast<uint32_t*>(b);
    b += sizeof(uint32_t) * kMaxPasses * kRadix;
    s.counters = reinterpret_cast<uint32_t*>(b);
    b += sizeof(uint32_t) * 64;
    s.lookback = reinterpret_cast<uint32_t*>(b);
    return s;
}
}  // namespace

SortPlan sort_plan(int64_t n, uint32_t key_bits, const uint32_t* n_dev, int items) {
    SortPlan p;
    p.n = n;
    p.n_dev = n_dev;
    p.key_bits = key_bits;
    p.passes = (key_bits + kRadixBits - 1) / kRadixBits;
    if (p.passes == 0) p.passes = 1;
    p.items = items == 8 || items == 16 ? items : 12;
    p.tiles = (uint32_t)((n + kThreads * p.items - 1) / (kThreads * p.items));
    return p;
}

size_t sort_scratch_bytes(const SortPlan& p) {
    return sizeof(uint32_t) * (kMaxPasses * kRadix + 64) +
           sizeof(uint32_t) * (size_t)p.passes * ((size_t)p.tiles + 1) * kRadix;
}

// Histogram of every pass's digits (grid-stride; warp-aggregated shared
// atomics because neighbouring keys usually share their high digits).
template <typename K>
__global__ void __launch_bounds__(kThreads) k_hist(const K* __restrict__ keys, int64_t n_max,
                                                   const uint32_t* __restrict__ n_dev, uint32_t passes,
                                                   uint32_t key_bits, uint32_t* __restrict__ hist) {
    __shared__ uint32_t sh[kMaxPasses][kRadix];
    const int64_t n = n_dev ? (int64_t)min((uint64_t)*n_dev, (uint64_t)n_max) : n_max;
    for (int i = threadIdx.x; i < kMaxPasses * kRadix; i += kThreads) (&sh[0][0])[i] = 0;
    __syncthreads();
    const uint32_t lane = lane_id();
    int64_t stride = (int64_t)gridDim.x * kThreads;
    for (int64_t i0 = (int64_t)blockIdx.x * kThreads; i0 < n; i0 += stride) {
        int64_t i = i0 + threadIdx.x;
        bool ok = i < n;
        K k = ok ? keys[i] : (K)0;
        uint32_t am = __ballot_sync(0xFFFFFFFFu, ok);
        for (uint32_t p = 0; p < passes; ++p) {
            uint32_t d = digit_of(k, p * kRadixBits, digit_mask(key_bits, p * kRadixBits));
            if (ok) {
                uint32_t peers = __match_any_sync(am, d);
                if (lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&sh[p][d], (uint32_t)__popc(peers));
            }
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < passes * kRadix; i += kThreads) {
        uint32_t v = (&sh[0][0])[i];
        if (v) atomicAdd(&hist[i], v);
    }
}

// Digit counts of every pass for the keys 0..n_bins-1 with the given counts.
__global__ void __launch_bounds__(kThreads) k_hist_from_counts(const uint32_t* __restrict__ counts, uint32_t n_bins,
                                                               uint32_t passes, uint32_t key_bits,
                                                               uint32_t* __restrict__ hist) {
    __shared__ uint32_t sh[kMaxPasses][kRadix];
    for (int i = threadIdx.x; i < kMaxPasses * kRadix; i += kThreads) (&sh[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t b = blockIdx.x * kThreads + threadIdx.x; b < n_bins; b += gridDim.x * kThreads) {
        const uint32_t c = counts[b];
        if (!c) continue;
        for (uint32_t p = 0; p < passes; ++p)
            atomicAdd(&sh[p][digit_of(b, p * kRadixBits, digit_mask(key_bits, p * kRadixBits))], c);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < passes * kRadix; i += kThreads) {
        const uint32_t v = (&sh[0][0])[i];
        if (v) atomicAdd(&hist[i], v);
    }
}

// In-place exclusive scan of each pass's 256 digit counts (one CTA per pass).
__global__ void __launch_bounds__(kRadix) k_hist_scan(uint32_t* hist) {
    __shared__ uint32_t sw[kRadix / 32];
    uint32_t* h = hist + blockIdx.x * kRadix;
    uint32_t v = h[threadIdx.x];
    uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        uint32_t t = __shfl_up_sync(0xFFFFFFFFu, x, d);
        if ((int)lane >= d) x += t;
    }
    if (lane == 31) sw[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kRadix / 32 ? sw[lane] : 0;
        uint32_t wi = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            uint32_t t = __shfl_up_sync(0xFFFFFFFFu, wi, d);
            if ((int)lane >= d) wi += t;
        }
        if (lane < kRadix / 32) sw[lane] = wi - w;
    }
    __syncthreads();
    h[threadIdx.x] = sw[warp] + x - v;
}

template <typename K, bool kVals, int ITEMS> struct OnesweepSmem {
    uint32_t warp_hist[kWarps][kRadix];
    uint32_t digit_start[kRadix];   // tile-local exclusive start of each digit
    uint32_t digit_global[kRadix];  // global base minus digit_start
    uint32_t scan_tmp[kWarps];
    uint32_t tile;
    K keys[kThreads * ITEMS];
    uint32_t vals[kVals ? kThreads * ITEMS : 1];
};

// Resident CTAs per SM the register budget is set for.
constexpr int onesweep_min_blocks(bool vals, int items) {
    return vals ? (items <= 8 ? 4 : items <= 12 ? 3 : 2) : (items <= 8 ? 5 : items <= 12 ? 4 : 3);
}

template <typename K, bool kVals, int ITEMS>
__global__ void __launch_bounds__(kThreads, onesweep_min_blocks(kVals, ITEMS)) k_onesweep(
                                                       const K* __restrict__ keys_in,
                                                       const uint32_t* __restrict__ vals_in,
                                                       K* __restrict__ keys_out, uint32_t* __restrict__ vals_out,
                                                       int64_t n_max, const uint32_t* __restrict__ n_dev,
                                                       uint32_t shift, uint32_t dmask,
                                                       const uint32_t* __restrict__ global_off,
                                                       uint32_t* __restrict__ lookback, uint32_t* counter,
                                                       uint32_t* status, uint32_t spin_limit) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int kItems = ITEMS, kTile = kThreads * ITEMS;
    OnesweepSmem<K, kVals, ITEMS>& S = *reinterpret_cast<OnesweepSmem<K, kVals, ITEMS>*>(smem_raw);
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < kWarps * kRadix; i += kThreads) (&S.warp_hist[0][0])[i] = 0;
    if (threadIdx.x == 0) S.tile = atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t tile = S.tile;
    const int64_t n = n_dev ? (int64_t)min((uint64_t)*n_dev, (uint64_t)n_max) : n_max;
    const int64_t tbase = (int64_t)tile * kTile;
    if (tbase >= n) return;   // launched for a larger capacity than this sort has
    const int64_t wbase = tbase + (int64_t)warp * (32 * kItems);

    // ---- load (warp-striped, coalesced) and rank within the warp
    K k[kItems];
    uint32_t v[kVals ? kItems : 1];
    uint32_t rank[kItems];
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        int64_t idx = wbase + it * 32 + lane;
        bool ok = idx < n;
        k[it] = ok ? keys_in[idx] : (K)0;
        if (kVals) v[it] = ok ? (vals_in ? vals_in[idx] : (uint32_t)idx) : 0u;
    }
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        int64_t idx = wbase + it * 32 + lane;
        bool ok = idx < n;
        uint32_t d = ok ? digit_of(k[it], shift, dmask) : (uint32_t)kRadix;   // kRadix = out of range
        uint32_t peers = same_digit_lanes<sizeof(K) == 4>(d);
        uint32_t leader = (uint32_t)(__ffs(peers) - 1);
        uint32_t before = 0;
        if (ok && lane == leader) {
            before = S.warp_hist[warp][d];
            S.warp_hist[warp][d] = before + (uint32_t)__popc(peers);
        }
        before = __shfl_sync(0xFFFFFFFFu, before, leader);
        rank[it] = before + (uint32_t)__popc(peers & lanemask_lt());
        __syncwarp();
    }
    __syncthreads();

    // ---- per digit: exclusive offsets across warps; tile count; publish
    const uint32_t d = threadIdx.x;   // kThreads == kRadix
    uint32_t cnt = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
        uint32_t t = S.warp_hist[w][d];
        S.warp_hist[w][d] = cnt;
        cnt += t;
    }
    uint32_t* lb_mine = lookback + (size_t)tile * kRadix + d;
    st_relaxed_u32(lb_mine, (tile == 0 ? kFlagP : kFlagA) | cnt);

    // tile-local digit starts: block exclusive scan over the 256 counts
    uint32_t x = cnt;
#pragma unroll
    for (int dd = 1; dd < 32; dd <<= 1) {
        uint32_t t = __shfl_up_sync(0xFFFFFFFFu, x, dd);
        if ((int)lane >= dd) x += t;
    }
    if (lane == 31) S.scan_tmp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kWarps ? S.scan_tmp[lane] : 0;
        uint32_t wi = w;
#pragma unroll
        for (int dd = 1; dd < 32; dd <<= 1) {
            uint32_t t = __shfl_up_sync(0xFFFFFFFFu, wi, dd);
            if ((int)lane >= dd) wi += t;
        }
        if (lane < kWarps) S.scan_tmp[lane] = wi - w;
    }
    __syncthreads();
    const uint32_t dstart = S.scan_tmp[warp] + x - cnt;
    S.digit_start[d] = dstart;

    // ---- look-back for this digit: 8 preceding tiles' words per step, all
    // loads in flight together; stop at the first inclusive prefix, wait
    // (bounded) at the first tile that has published nothing yet
    uint32_t excl = 0;
    if (tile > 0) {
        const uint32_t* base = lookback + d;
        int64_t look = (int64_t)tile - 1;
        uint32_t spins = 0;
        for (;;) {
            uint32_t w[kLookWindow];
#pragma unroll
            for (int q = 0; q < kLookWindow; ++q)
                w[q] = look - q >= 0 ? ld_relaxed_u32(base + (size_t)(look - q) * kRadix) : kFlagP;
            int used = 0;
            bool done = false;
#pragma unroll
            for (int q = 0; q < kLookWindow; ++q) {
                if (done || used < q) continue;   // stopped at an earlier word
                const uint32_t f = w[q] & ~kCountMask;
                if (f == 0) continue;             // not published yet: used stays q
                excl += w[q] & kCountMask;
                used = q + 1;
                done = f == kFlagP;
            }
            if (done) break;
            look -= used;
            if (used == 0) {
                if (++spins > spin_limit) {
                    set_error(status, ERR_LOOKBACK_TIMEOUT);
                    break;
                }
                __nanosleep(32);
            }
        }
        st_relaxed_u32(lb_mine, kFlagP | (excl + cnt));
    }
    S.digit_global[d] = global_off[d] + excl - dstart;
    __syncthreads();

    // ---- scatter into shared memory in digit order
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        int64_t idx = wbase + it * 32 + lane;
        if (idx < n) {
            uint32_t dg = digit_of(k[it], shift, dmask);
            uint32_t pos = S.digit_start[dg] + S.warp_hist[warp][dg] + rank[it];
            S.keys[pos] = k[it];
            if (kVals) S.vals[pos] = v[it];
        }
    }
    __syncthreads();

    // ---- write runs to global memory
    int64_t valid = n - tbase;
    if (valid > kTile) valid = kTile;
    for (int j = threadIdx.x; j < valid; j += kThreads) {
        K kk = S.keys[j];
        uint32_t dg = digit_of(kk, shift, dmask);
        uint32_t o = S.digit_global[dg] + (uint32_t)j;
        if ((int64_t)o < n) {
            keys_out[o] = kk;
            if (kVals) vals_out[o] = S.vals[j];
        } else {
            set_error(status, ERR_BAD_INDEX);
        }
    }
}

template <typename K, bool kVals, int ITEMS>
static void sort_impl(const SortPlan& p, const K* keys_in, const uint32_t* vals_in, K* keys_out, uint32_t* vals_out,
                      K* keys_alt, uint32_t* vals_alt, void* scratch, uint32_t* status, cudaStream_t st) {
    if (p.n <= 0) return;
    Scratch s = carve(p, scratch);
    size_t lb_words = (size_t)p.passes * ((size_t)p.tiles + 1) * kRadix;
    if (p.hist_given) {
        cudaMemsetAsync(s.counters, 0, sizeof(uint32_t) * 64, st);
    } else {
        cudaMemsetAsync(s.hist, 0, sizeof(uint32_t) * (kMaxPasses * kRadix + 64), st);
    }
    cudaMemsetAsync(s.lookback, 0, sizeof(uint32_t) * lb_words, st);
    if (!p.hist_given) {
        int hb = (int)((p.n + kThreads - 1) / kThreads);
        if (hb > kHistBlocks) hb = kHistBlocks;
        count_launches(1);
        k_hist<K><<<hb, kThreads, 0, st>>>(keys_in, p.n, p.n_dev, p.passes, p.key_bits, s.hist);
    }
    count_launches(1);
    k_hist_scan<<<p.passes, kRadix, 0, st>>>(s.hist);
    const size_t smem = sizeof(OnesweepSmem<K, kVals, ITEMS>);
    static std::atomic<uint32_t> attr_set{0};
    once_per_device(attr_set, [&] {
        cudaFuncSetAttribute(k_onesweep<K, kVals, ITEMS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    });
    const K* ksrc = keys_in;
    const uint32_t* vsrc = vals_in;
    for (uint32_t pass = 0; pass < p.passes; ++pass) {
        bool to_out = ((p.passes - 1 - pass) % 2) == 0;
        K* kdst = to_out ? keys_out : keys_alt;
        uint32_t* vdst = to_out ? vals_out : vals_alt;
        count_launches(1);
        k_onesweep<K, kVals, ITEMS><<<p.tiles, kThreads, smem, st>>>(ksrc, vsrc, kdst, vdst, p.n, p.n_dev,
                                                             pass * kRadixBits,
                                                             digit_mask(p.key_bits, pass * kRadixBits),
                                                             s.hist + pass * kRadix,
                                                             s.lookback + (size_t)pass * (p.tiles + 1) * kRadix,
                                                             s.counters + pass, status, spin_limit());
        ksrc = kdst;
        vsrc = vdst;
    }
}

template <typename K>
static void sort_dispatch(const SortPlan& p, const K* keys_in, const uint32_t* vals_in, K* keys_out, uint32_t* vals_out,
                          K* keys_alt, uint32_t* vals_alt, void* scratch, uint32_t* status, cudaStream_t st) {
#define SR_SORT_CASE(ITEMS)                                                                                        \
    if (p.items == ITEMS) {                                                                                        \
        if (vals_out)                                                                                              \
            sort_impl<K, true, ITEMS>(p, keys_in, vals_in, keys_out, vals_out, keys_alt, vals_alt, scratch, status, \
                                      st);                                                                         \
        else                                                                                                       \
            sort_impl<K, false, ITEMS>(p, keys_in, nullptr, keys_out, nullptr, keys_alt, nullptr, scratch, status,  \
                                       st);                                                                        \
        return;                                                                                                    \
    }
    SR_SORT_CASE(8)
    SR_SORT_CASE(16)
    SR_SORT_CASE(12)
#undef SR_SORT_CASE
}

void launch_sort_u64(const SortPlan& p, const uint64_t* keys_in, const uint32_t* vals_in, uint64_t* keys_out,
                     uint32_t* vals_out, uint64_t* keys_alt, uint32_t* vals_alt, void* scratch, uint32_t* status,
                     cudaStream_t st) {
    sort_dispatch<uint64_t>(p, keys_in, vals_in, keys_out, vals_out, keys_alt, vals_alt, scratch, status, st);
}

void sort_hist_from_counts(SortPlan& p, const uint32_t* counts, uint32_t n_bins, void* scratch, cudaStream_t st) {
    Scratch s = carve(p, scratch);
    cudaMemsetAsync(s.hist, 0, sizeof(uint32_t) * kMaxPasses * kRadix, st);
    int blocks = (int)((n_bins + kThreads - 1) / kThreads);
    if (blocks > kHistBlocks) blocks = kHistBlocks;
    if (blocks < 1) blocks = 1;
    count_launches(1);
    k_hist_from_counts<<<blocks, kThreads, 0, st>>>(counts, n_bins, p.passes, p.key_bits, s.hist);
    p.hist_given = 1;
}

void launch_sort_u32(const SortPlan& p, const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                     uint32_t* vals_out, uint32_t* keys_alt, uint32_t* vals_alt, void* scratch, uint32_t* status,
                     cudaStream_t st) {
    sort_dispatch<uint32_t>(p, keys_in, vals_in, keys_out, vals_out, keys_alt, vals_alt, scratch, status, st);
}

}  // namespace sr
