// common.cuh — device helpers shared by the scanline kernels.
//
// Arithmetic that decides a pixel is written with explicit round-to-nearest
// intrinsics (__fadd_rn, __fmul_rn, __fsub_rn, __fdiv_rn) so that no
// multiply-add is ever fused, whatever the compiler flags; the library is
// also built with --fmad=false.  The semantics GLSL leaves open are fixed
// the same way as in the CPU restatement: float->int truncates, saturates and
// maps NaN to 0; int arithmetic wraps; min/max follow GLSL's definition.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define SR_DEV __device__ __forceinline__

namespace sr {

// Error bits written by kernels into the context's device status word.
enum : uint32_t {
    ERR_LOOKBACK_TIMEOUT = 1u << 0,  // a decoupled look-back spin gave up
    ERR_RECORD_RANGE = 1u << 1,      // a curve produced a different record count than counted
    ERR_CAPACITY = 1u << 2,          // a pre-sized buffer was too small
    ERR_BAD_INDEX = 1u << 3,         // an index read from memory was out of range
    ERR_COPY_TIMEOUT = 1u << 4,      // a wait for a bulk copy into shared memory gave up
};

// Polls a bounded spin makes before it gives up (with backoff, ~seconds),
// unless sr_set_spin_limit chose another limit.  Launchers pass the limit to
// each kernel that spins (see spin_limit() in kernels.h).
constexpr uint32_t kSpinLimitDefault = 1u << 22;

SR_DEV float lerp_rn(float a, float b, float t) {
    // LERP(a,b,t) = a + t*(b-a)   (make_intersection_0.comp:10)
    return __fadd_rn(a, __fmul_rn(t, __fsub_rn(b, a)));
}
SR_DEV float gmin(float x, float y) { return (y < x) ? y : x; }
SR_DEV float gmax(float x, float y) { return (x < y) ? y : x; }
SR_DEV int32_t imin(int32_t a, int32_t b) { return b < a ? b : a; }
SR_DEV int32_t imax(int32_t a, int32_t b) { return a < b ? b : a; }
SR_DEV int32_t iclamp(int32_t v, int32_t lo, int32_t hi) { return imin(imax(v, lo), hi); }
SR_DEV int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
SR_DEV int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
SR_DEV int32_t f2i(float x) { return __float2int_rz(x); }  // cvt.rzi.s32.f32: saturates, NaN -> 0
SR_DEV int32_t fbits(float x) { return __float_as_int(x); }
SR_DEV float bitsf(int32_t i) { return __int_as_float(i); }
// float2int_rd (make_intersection_1.comp:76-79)
SR_DEV int32_t float2int_rd(float x) { return x >= 0.0f ? f2i(x) : f2i(__fsub_rn(x, 1.0f)); }

// PATH_VISIBLE (make_intersection_0.comp:14-20)
SR_DEV bool path_visible_mask(int32_t m) {
    bool inv = ((m & 0x11111000) == 0) || ((m & 0x01101011) == 0) || ((m & 0x00011111) == 0) ||
               ((m & 0x11010110) == 0);
    return !inv;
}

// Curve type of a rational quadratic (SR_CURVE_ARC): 4 point slots, the
// last holding its weight.
constexpr uint32_t kArc = 0x13u;
SR_DEV uint32_t curve_slots(uint32_t type) { return type == kArc ? 4u : (type & 7u); }

// Coordinate of a curve at t: line lerp, quadric 2-level, cubic 3-level; an
// arc (p = x0, w*x1, x2, w) a 2-level lerp of the homogeneous points
// (x0, 1), (w*x1, w), (x2, 1), then one division.
SR_DEV float interp(uint32_t type, float t, const float* p) {
    if (type == kArc) {
        const float q0 = lerp_rn(p[0], p[1], t), q1 = lerp_rn(p[1], p[2], t);
        const float r0 = lerp_rn(1.0f, p[3], t), r1 = lerp_rn(p[3], 1.0f, t);
        return __fdiv_rn(lerp_rn(q0, q1, t), lerp_rn(r0, r1, t));
    }
    if (type == 2u) return lerp_rn(p[0], p[1], t);
    if (type == 3u) {
        float q0 = lerp_rn(p[0], p[1], t), q1 = lerp_rn(p[1], p[2], t);
        return lerp_rn(q0, q1, t);
    }
    if (type == 4u) {
        float q0 = lerp_rn(p[0], p[1], t), q1 = lerp_rn(p[1], p[2], t), q2 = lerp_rn(p[2], p[3], t);
        float l0 = lerp_rn(q0, q1, t), l1 = lerp_rn(q1, q2, t);
        return lerp_rn(l0, l1, t);
    }
    return 0.0f;
}

// The fragment size F is 1 (pixel mode) or 2 (reference mode).  v / F for
// v >= 0 or a multiple of F (cell coordinates are), by a shift rather than
// an integer division; and 1 / F, exactly.
SR_DEV int32_t div_F(int32_t v, int32_t F) { return F == 2 ? (v >> 1) : v; }
SR_DEV float inv_F(int32_t F) { return F == 2 ? 0.5f : 1.0f; }

SR_DEV void set_error(uint32_t* status, uint32_t bit) {
    if (status) atomicOr(status, bit);
}

// ------------------------------------------------------------ memory ops --
SR_DEV uint64_t ld_acquire_u64(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
SR_DEV void st_release_u64(uint64_t* p, uint64_t v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
SR_DEV uint32_t ld_acquire_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
SR_DEV void st_release_u32(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Relaxed (no ordering) but coherent at GPU scope: for flag+value words
// whose readers use nothing else the writer published.
SR_DEV uint32_t ld_relaxed_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
SR_DEV void st_relaxed_u32(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

SR_DEV uint32_t lane_id() { return threadIdx.x & 31u; }
SR_DEV uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ------------------------------------------------- bulk copies (TMA) --
// One-dimensional bulk copies from global to shared memory, completed on a
// shared-memory mbarrier (cp.async.bulk with complete_tx).  Addresses and
// the size must be multiples of 16 bytes.
SR_DEV uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

SR_DEV void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    // make the initialised barrier visible to the copy engine
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

SR_DEV void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

SR_DEV void bulk_load(void* dst_smem, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst_smem)),
                 "l"(__cvta_generic_to_global(src)), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

SR_DEV bool mbar_test(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Waits for phase `parity` of the barrier, at most spin_limit polls; false
// (and ERR_COPY_TIMEOUT in the status word) when it gave up.
SR_DEV bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t spin_limit, uint32_t* status) {
    for (uint32_t i = 0; !mbar_test(bar, parity); ++i) {
        if (i >= spin_limit) {
            set_error(status, ERR_COPY_TIMEOUT);
            return false;
        }
        __nanosleep(32);
    }
    return true;
}

// ------------------------------------------------------- scan geometry --
// Key layout of a sorted fragment record (64-bit, unsigned order equal to the
// reference's (path, signed yx) order; see pack_key).
struct KeyLayout {
    int32_t F;        // FRAG_SIZE
    int32_t W, H;     // canvas
    int32_t Hy;       // number of cell rows: ceil(H / F)
    uint32_t xbits, rbits, pbits;
};

// Row rank: cell rows 1..Hy-1 first, then off-canvas/degenerate records,
// then cell row 0 — the order of the signed 16:16 keys the reference sorts
// (gen_fragment.comp:180-187 with 0x7FFF biases).
SR_DEV uint64_t pack_key(const KeyLayout& L, uint32_t path, bool valid, int32_t pos_y, int32_t pos_x) {
    uint32_t rank, xo;
    if (!valid) {
        rank = (uint32_t)(L.Hy - 1);
        xo = 0;
    } else {
        int32_t yy = div_F(pos_y, L.F);
        rank = yy == 0 ? (uint32_t)L.Hy : (uint32_t)(yy - 1);
        xo = (uint32_t)(div_F(pos_x, L.F) + 1);
    }
    return ((uint64_t)path << (L.rbits + L.xbits)) | ((uint64_t)rank << L.xbits) | (uint64_t)xo;
}

struct Decoded {
    uint32_t path;
    bool valid;
    int32_t y, x;   // cell origin in pixels (valid records only)
    int32_t yx;     // the reference's packed key
};

// Bits of the sort key proper.  Above them a key may carry a payload (the
// record's packed winding bits) that the sort moves but does not order by.
__host__ __device__ __forceinline__ uint32_t key_bits(const KeyLayout& L) { return L.pbits + L.rbits + L.xbits; }
SR_DEV uint64_t key_part(const KeyLayout& L, uint64_t k) { return k & ((1ull << key_bits(L)) - 1ull); }
SR_DEV uint32_t payload_part(const KeyLayout& L, uint64_t k) { return (uint32_t)(k >> key_bits(L)) & 0xFu; }

SR_DEV Decoded unpack_key(const KeyLayout& L, uint64_t k) {
    Decoded d;
    k = key_part(L, k);
    uint32_t xo = (uint32_t)(k & ((1ull << L.xbits) - 1));
    uint32_t rank = (uint32_t)((k >> L.xbits) & ((1ull << L.rbits) - 1));
    d.path = (uint32_t)(k >> (L.xbits + L.rbits));
    if (rank == (uint32_t)(L.Hy - 1)) {
        d.valid = false;
        d.y = 0x7FFF;
        d.x = 0x7FFF;
        d.yx = (int32_t)0xFFFEFFFE;
    } else {
        int32_t yy = rank == (uint32_t)L.Hy ? 0 : (int32_t)rank + 1;
        d.valid = true;
        d.y = yy * L.F;
        d.x = ((int32_t)xo - 1) * L.F;
        d.yx = (int32_t)(((uint32_t)(d.y + 0x7FFF) << 16) | ((uint32_t)(d.x + 0x7FFF) & 0xFFFFu));
    }
    return d;
}

}  // namespace sr
