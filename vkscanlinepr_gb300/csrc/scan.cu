// scan.cu — single-pass exclusive scan (decoupled look-back).
//
// Replaces naive_scan.comp:27-73, which runs in ONE workgroup and walks the
// input in dependent batches of 1023.  Here every CTA scans a 4096-element
// tile, publishes its aggregate, and a single warp looks back over the
// predecessors' published values.  Every spin is bounded: after the spin
// limit's polls the tile records ERR_LOOKBACK_TIMEOUT and carries on, so a stalled
// predecessor can never hang the GPU.  Output: out[0..n], out[n] = total
// (exactly n+1 writes).
#include "common.cuh"
#include "kernels.h"

namespace sr {

namespace {
constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;
constexpr uint64_t kFlagA = 1ull << 62;
constexpr uint64_t kFlagP = 2ull << 62;

SR_DEV int32_t warp_incl_scan(int32_t v) {
    uint32_t lane = lane_id();
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        int32_t t = __shfl_up_sync(0xFFFFFFFFu, v, d);
        if ((int)lane >= d) v = wadd(v, t);
    }
    return v;
}

SR_DEV int32_t warp_sum(int32_t v) {
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) v = wadd(v, __shfl_xor_sync(0xFFFFFFFFu, v, d));
    return v;
}
}  // namespace

// Warp-cooperative look-back over 64-bit tile words (flag in bits 62-63,
// value in bits 0-31).  Returns the sum of all predecessors of `tile`.
__device__ int32_t lookback_i32(uint64_t* tstat, uint32_t tile, uint32_t* status, uint32_t spin_limit) {
    uint32_t lane = lane_id();
    int32_t excl = 0;
    int64_t look = (int64_t)tile - 1;
    uint32_t spins = 0;
    while (look >= 0) {
        int64_t j = look - (int64_t)lane;
        uint64_t s = j >= 0 ? ld_acquire_u64(&tstat[j]) : kFlagP;
        uint32_t flag = (uint32_t)(s >> 62);
        uint32_t ready = __ballot_sync(0xFFFFFFFFu, flag != 0);
        uint32_t pm = __ballot_sync(0xFFFFFFFFu, flag == 2);
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
        int32_t v = ((int)lane <= firstp) ? (int32_t)(uint32_t)s : 0;
        excl = wadd(excl, warp_sum(v));
        if (pm) break;
        look -= 32;
    }
    return excl;
}

__global__ void __launch_bounds__(kThreads) k_scan_i32(const int32_t* in, int32_t* out, int64_t n,
                                                       uint64_t* tstat, uint32_t* counter, uint32_t* status,
                                                       uint32_t spin_limit) {
    __shared__ uint32_t s_tile;
    __shared__ int32_t s_warp[kThreads / 32];
    __shared__ int32_t s_prefix;
    if (threadIdx.x == 0) s_tile = atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const int64_t base = (int64_t)tile * kTile + (int64_t)threadIdx.x * kItems;
    int32_t v[kItems];
    if (base + kItems <= n && ((reinterpret_cast<uintptr_t>(in + base) & 15) == 0)) {
        const int4* p = reinterpret_cast<const int4*>(in + base);
#pragma unroll
        for (int k = 0; k < kItems / 4; ++k) {
            int4 q = p[k];
            v[4 * k] = q.x; v[4 * k + 1] = q.y; v[4 * k + 2] = q.z; v[4 * k + 3] = q.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < kItems; ++k) v[k] = (base + k < n) ? in[base + k] : 0;
    }
    int32_t tsum = 0;
#pragma unroll
    for (int k = 0; k < kItems; ++k) tsum = wadd(tsum, v[k]);
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    int32_t incl = warp_incl_scan(tsum);
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int32_t w = lane < kThreads / 32 ? s_warp[lane] : 0;
        int32_t wi = warp_incl_scan(w);
        if (lane < kThreads / 32) s_warp[lane] = wadd(wi, -w);   // exclusive warp offsets
        int32_t agg = __shfl_sync(0xFFFFFFFFu, wi, kThreads / 32 - 1);
        if (lane == 0) st_release_u64(&tstat[tile], (tile == 0 ? kFlagP : kFlagA) | (uint32_t)agg);
        int32_t excl = 0;
        if (tile > 0) {
            excl = lookback_i32(tstat, tile, status, spin_limit);
            if (lane == 0) st_release_u64(&tstat[tile], kFlagP | (uint32_t)wadd(excl, agg));
        }
        if (lane == 0) {
            s_prefix = excl;
            int64_t tile_end = (int64_t)(tile + 1) * kTile;
            if (tile_end >= n) out[n] = wadd(excl, agg);   // total, by the last tile
        }
    }
    __syncthreads();
    int32_t run = wadd(wadd(s_prefix, s_warp[warp]), wadd(incl, -tsum));
    if (base + kItems <= n && ((reinterpret_cast<uintptr_t>(out + base) & 15) == 0)) {
        int4* p = reinterpret_cast<int4*>(out + base);
#pragma unroll
        for (int k = 0; k < kItems / 4; ++k) {
            int4 q;
            q.x = run; run = wadd(run, v[4 * k]);
            q.y = run; run = wadd(run, v[4 * k + 1]);
            q.z = run; run = wadd(run, v[4 * k + 2]);
            q.w = run; run = wadd(run, v[4 * k + 3]);
            p[k] = q;
        }
    } else {
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            if (base + k < n) out[base + k] = run;
            run = wadd(run, v[k]);
        }
    }
}

// Sticky error bits of the standalone scans on each device that loads the
// library (4 bytes, held until exit).
static __device__ uint32_t g_standalone_scan_status;

cudaError_t standalone_scan_status(uint32_t** out) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_standalone_scan_status);
    *out = static_cast<uint32_t*>(p);
    return e;
}

size_t scan_status_words(int64_t n) { return (size_t)((n + kTile - 1) / kTile + 1); }

void launch_exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, uint64_t* tile_status,
                               uint32_t* tile_counter, uint32_t* status, cudaStream_t st) {
    if (n <= 0) {
        cudaMemsetAsync(out, 0, sizeof(int32_t), st);
        return;
    }
    int64_t tiles = (n + kTile - 1) / kTile;
    count_launches(1);
    k_scan_i32<<<(unsigned)tiles, kThreads, 0, st>>>(in, out, n, tile_status, tile_counter, status, spin_limit());
}

}  // namespace sr
