// resolve.cu — paints the draw list into the RGBA8 framebuffer.
//
// Replaces the reference's graphics pass (scanlinepr.vert:18-51,
// scanlinepr.frag:7-14, pipeline at scanline_rasterizer.cpp:881-944 and
// :610-695): each draw record (yx, width, colour, index) covers
// [x, x+width) x [y, y+FRAG_SIZE), the framebuffer is cleared to white, and
// records land in draw order.  Reference mode overwrites (blending is off in
// the reference pipeline); pixel mode composites source-over with integer
// arithmetic.  Draw records are first sorted stably by cell row (onesweep),
// so each CTA owns one cell row, keeps it in shared memory, and applies the
// row's records in path order; a thread owns a fixed set of pixels, so no
// barrier is needed between records.
#include "common.cuh"
#include "kernels.h"

namespace sr {

// First index of every cell row in the row-sorted draw list.
__global__ void k_row_bounds(const uint32_t* __restrict__ srows, int64_t n, int32_t rows,
                             int32_t* __restrict__ row_start) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += stride) {
        int32_t cur = i < n ? (int32_t)srows[i] : rows;
        uint32_t pv = i > 0 ? srows[i - 1] : 0xFFFFFFFFu;
        int32_t prev = pv == 0xFFFFFFFFu ? -1 : (int32_t)(pv > (uint32_t)rows ? (uint32_t)rows : pv);
        if ((uint32_t)cur > (uint32_t)rows) cur = rows;
        for (int32_t r = prev + 1; r <= cur; ++r) row_start[r] = (int32_t)i;
    }
}

// Integer source-over of one RGBA8 pixel, two channels per 32-bit lane:
// c' = (s*a + d*(255-a) + 127) / 255 for R, G, B and, with s = 255, for A.
// x/255 for 0 <= x <= 65152 is (x + 1 + (x >> 8)) >> 8 (checked exhaustively
// by the CPU tests).
struct BlendSrc {
    uint32_t ia;       // 255 - a
    uint32_t pre_rb;   // s_r*a + 127 | (s_b*a + 127) << 16
    uint32_t pre_ga;   // s_g*a + 127 | (255*a + 127) << 16
};

SR_DEV BlendSrc blend_src(uint32_t c) {
    uint32_t a = c >> 24;
    BlendSrc b;
    b.ia = 255u - a;
    b.pre_rb = (c & 0x00FF00FFu) * a + 0x007F007Fu;
    b.pre_ga = (((c >> 8) & 0xFFu) | (255u << 16)) * a + 0x007F007Fu;
    return b;
}

SR_DEV uint32_t blend_px(uint32_t d, const BlendSrc& s) {
    uint32_t rb = (d & 0x00FF00FFu) * s.ia + s.pre_rb;
    uint32_t ga = ((d >> 8) & 0x00FF00FFu) * s.ia + s.pre_ga;
    rb = ((rb + 0x00010001u + ((rb >> 8) & 0x00FF00FFu)) >> 8) & 0x00FF00FFu;
    ga = ((ga + 0x00010001u + ((ga >> 8) & 0x00FF00FFu)) >> 8) & 0x00FF00FFu;
    return rb | (ga << 8);
}

constexpr int kResolveThreads = 256;
constexpr int kChunk = 256;

__global__ void __launch_bounds__(kResolveThreads) k_resolve(const ResolveArgs a) {
    extern __shared__ __align__(16) uint32_t rowbuf[];   // [F][W]
    __shared__ int32_t s_x[kChunk], s_w[kChunk];
    __shared__ uint32_t s_c[kChunk];
    const int32_t r = blockIdx.x;
    const int32_t W = a.W, F = a.F;
    const int32_t y0 = r * F;
    const int32_t nrows = imin(F, a.H - y0);
    const int tid = threadIdx.x;
    for (int32_t p = tid; p < nrows * W; p += kResolveThreads) rowbuf[p] = 0xFFFFFFFFu;
    const int32_t beg = a.row_start[r], end = a.row_start[r + 1];
    __syncthreads();
    for (int32_t c0 = beg; c0 < end; c0 += kChunk) {
        if (c0 + tid < end) {
            int4 d = a.draw[a.row_sorted_idx[c0 + tid]];
            s_x[tid] = d.x & 0xFFFF;
            s_w[tid] = d.y;
            s_c[tid] = (uint32_t)d.z;
        }
        __syncthreads();
        const int32_t cnt = imin(kChunk, end - c0);
        for (int32_t q = 0; q < cnt; ++q) {
            int32_t xa = imax(s_x[q], 0);
            int32_t xb = imin(wadd(s_x[q], s_w[q]), W);
            uint32_t col = s_c[q];
            int32_t p0 = xa + ((tid - xa) & (kResolveThreads - 1));
            if (p0 >= xb) continue;
            if (a.pixel_mode) {
                BlendSrc bs = blend_src(col);
                for (int32_t p = p0; p < xb; p += kResolveThreads) {
                    for (int32_t rr = 0; rr < nrows; ++rr) {
                        uint32_t* px = &rowbuf[rr * W + p];
                        *px = blend_px(*px, bs);
                    }
                }
            } else {
                for (int32_t p = p0; p < xb; p += kResolveThreads)
                    for (int32_t rr = 0; rr < nrows; ++rr) rowbuf[rr * W + p] = col;
            }
        }
        __syncthreads();
    }
    uint32_t* out = a.image + (size_t)y0 * W;
    if ((W & 3) == 0) {
        const uint4* src = reinterpret_cast<const uint4*>(rowbuf);
        uint4* dst = reinterpret_cast<uint4*>(out);
        for (int32_t p = tid; p < nrows * W / 4; p += kResolveThreads) dst[p] = src[p];
    } else {
        for (int32_t p = tid; p < nrows * W; p += kResolveThreads) out[p] = rowbuf[p];
    }
}

void launch_resolve(const ResolveArgs& a, cudaStream_t st) {
    int32_t rows = (a.H + a.F - 1) / a.F;
    if (rows <= 0) return;
    size_t smem = (size_t)a.F * a.W * sizeof(uint32_t);
    static size_t attr = 0;
    if (smem > 48 * 1024 && smem > attr) {
        cudaFuncSetAttribute(k_resolve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        attr = smem;
    }
    count_launches(1);
    k_resolve<<<rows, kResolveThreads, smem, st>>>(a);
}

void launch_row_bounds(const uint32_t* srows, int64_t n, int32_t rows, int32_t* row_start, cudaStream_t st) {
    int64_t work = n + 1;
    int blocks = (int)((work + 255) / 256);
    if (blocks > 1216) blocks = 1216;
    count_launches(1);
    k_row_bounds<<<blocks, 256, 0, st>>>(srows, n, rows, row_start);
}

}  // namespace sr
