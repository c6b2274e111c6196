// resolve.cu — paints the draw list into the RGBA8 framebuffer.
//
// Replaces the reference's graphics pass (scanlinepr.vert:18-51,
// scanlinepr.frag:7-14, pipeline at scanline_rasterizer.cpp:881-944 and
// :610-695): each draw record (yx, width, colour, index) covers
// [x, x+width) x [y, y+FRAG_SIZE), the framebuffer is cleared to white, and
// records land in draw order.  Reference mode overwrites (blending is off in
// the reference pipeline); pixel mode composites source-over with integer
// arithmetic.  Draw records are first sorted stably by cell row (onesweep),
// so a CTA owns one cell row (or several short ones), stages its records in
// shared memory, and applies them in path order; a thread owns a fixed set
// of pixels, so no barrier is needed between records.  In pixel mode a warp
// first finds where its 256-pixel segment's painting may start (the
// collapse cut below) and skips the records before it.
#include "common.cuh"
#include "kernels.h"

namespace sr {

// First index of every cell row in the row-sorted draw list.
__global__ void k_row_bounds(const uint32_t* __restrict__ srows, int64_t n_cap, const uint32_t* __restrict__ n_dev,
                             int32_t rows, int32_t* __restrict__ row_start) {
    const int64_t n = n_dev ? (int64_t)min((uint64_t)*n_dev, (uint64_t)n_cap) : n_cap;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += stride) {
        int32_t cur = i < n ? (int32_t)srows[i] : rows;
        uint32_t pv = i > 0 ? srows[i - 1] : 0xFFFFFFFFu;
        int32_t prev = pv == 0xFFFFFFFFu ? -1 : (int32_t)(pv > (uint32_t)rows ? (uint32_t)rows : pv);
        if ((uint32_t)cur > (uint32_t)rows) cur = rows;
        for (int32_t r = prev + 1; r <= cur; ++r) row_start[r] = (int32_t)i;
    }
}

// ----------------------------------------------------------- pixel mode --
// Source-over in path order over opaque white: for R, G, B
//   c' = floor((s*a + c*(255-a) + 127) / 255) = round((s*a + c*(255-a)) / 255).
// Red and blue share one 32-bit word (r in bits 0-7, b in bits 16-23) and
// blend with integer operations: u = c*ia + s*a + 128 fits each 16-bit
// half (<= 65153), and c' = (u + (u >> 8)) >> 8 per half, the two shifts
// being byte permutes (bytes 1 and 3 to 0 and 2); no half carries into the
// other.  Green blends on the FMA pipe: u = c*ia + s*a is an exact float
// (<= 65025), and fma(u, 1/255, 1.5*2^23) - 1.5*2^23 rounds u/255 to the
// nearest integer.  Both forms equal the formula for every reachable u
// (checked exhaustively by the CPU tests).  Alpha stays 255:
// (255*a + 255*(255-a) + 127) / 255 = 255.
constexpr float kRound = 12582912.0f;   // 1.5 * 2^23
constexpr int kK = kResolveSeg / 32;   // pixels per lane; a warp owns kResolveSeg pixels
constexpr int kChunk = 1024;

struct PixRec {
    int32_t x0, x1;     // [x0, x1) clipped to >= 0
    float ia;           // 255 - a
    float sg;           // s*a of green
    uint32_t iau;       // 255 - a
    uint32_t sab;       // (s*a + 128) of red | of blue << 16
    int32_t row;        // cell row within the CTA
    uint32_t idx1;      // 1 + draw index
};

// q: a record's iau, sab, ia and sg (a PixRec or a RunRec).
template <class Rec> SR_DEV void blend3(uint32_t& rb, float& g, const Rec& q) {
    const uint32_t u = rb * q.iau + q.sab;
    rb = __byte_perm(u + __byte_perm(u, 0u, 0x4341u), 0u, 0x4341u);
    const float ug = __fmaf_rn(g, q.ia, q.sg);
    g = __fsub_rn(__fmaf_rn(ug, 1.0f / 255.0f, kRound), kRound);
}

uint32_t resolve_rows_per_cta(int32_t W, int warps) {
    int32_t segs = (W + kResolveSeg - 1) / kResolveSeg;
    return segs >= warps ? 1u : (uint32_t)(warps / segs);
}

// Which rows and segment a warp paints: a CTA holds rows_per_cta cell rows
// of one scene; small canvases give each row fewer warps than the CTA has.
// A warp skips the records before the last one that covers its whole
// segment and hides what is under it (seg_cut, written by the emit): source-
// over with a = 255 gives floor((255 s + 127) / 255) = s whatever the pixel
// held, and an overwrite leaves nothing of it either.
struct ResolveWork {
    const SceneInfo* si;
    int32_t W, r0, nr, segs, groups, my_row;
    bool active;
};

template <int WARPS> SR_DEV ResolveWork resolve_work(const ResolveArgs& a) {
    constexpr int kResolveWarps = WARPS;
    // scene of this CTA: last s with cta_base[s] <= blockIdx.x
    uint32_t lo = 0, hi = a.n_scenes;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (a.cta_base[mid] <= blockIdx.x) lo = mid;
        else hi = mid;
    }
    ResolveWork w;
    w.si = &a.scenes[lo];
    w.W = w.si->W;
    w.segs = (w.W + kResolveSeg - 1) / kResolveSeg;
    const int32_t R = w.segs >= kResolveWarps ? 1 : kResolveWarps / w.segs;
    w.r0 = (int32_t)(blockIdx.x - a.cta_base[lo]) * R;
    w.nr = imin(R, (int32_t)w.si->rows - w.r0);
    const int warp = threadIdx.x >> 5;
    if (w.segs >= kResolveWarps) {
        w.my_row = 0;
        w.groups = (w.segs + kResolveWarps - 1) / kResolveWarps;
        w.active = true;
    } else {
        w.my_row = warp / w.segs;
        w.groups = 1;
        w.active = w.my_row < w.nr;
    }
    return w;
}

SR_DEV uint32_t resolve_cut(const ResolveArgs& a, const ResolveWork& w, int32_t seg, bool live) {
    if (!a.seg_cut || !live) return 0u;
    return a.seg_cut[(size_t)(w.si->row_base + (uint32_t)(w.r0 + w.my_row)) * a.cut_segs +
                     (uint32_t)(seg / kResolveSeg)];
}

template <int WARPS> SR_DEV int32_t resolve_seg(const ResolveWork& w, int group) {
    constexpr int kResolveWarps = WARPS;
    const int warp = threadIdx.x >> 5;
    return w.segs >= kResolveWarps ? group * kResolveWarps + warp : warp % w.segs;
}

// Colour of gradient paint P at the pixel-space point (x, y), packed RGBA8,
// 0 when transparent (the definition is in sr.h; the oracle restates it).
__device__ __noinline__ uint32_t paint_color(const DevPaint& P, float x, float y) {
    float t;
    if (P.kind == 1) {
        t = __fadd_rn(__fadd_rn(__fmul_rn(P.lin[0], x), __fmul_rn(P.lin[1], y)), P.lin[2]);
    } else {
        const float gx = __fadd_rn(__fadd_rn(__fmul_rn(P.m[0], x), __fmul_rn(P.m[1], y)), P.m[2]);
        const float gy = __fadd_rn(__fadd_rn(__fmul_rn(P.m[3], x), __fmul_rn(P.m[4], y)), P.m[5]);
        const float ex = __fsub_rn(gx, P.fx), ey = __fsub_rn(gy, P.fy);
        const float b = __fadd_rn(__fmul_rn(ex, P.dx), __fmul_rn(ey, P.dy));
        const float c = __fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey));
        if (P.A == 0.0f) {
            t = b != 0.0f ? __fdiv_rn(c, __fmul_rn(2.0f, b)) : 0.0f;
        } else {
            const float disc = __fsub_rn(__fmul_rn(b, b), __fmul_rn(P.A, c));
            if (disc < 0.0f) {
                t = 0.0f;
            } else {
                const float sq = __fsqrt_rn(disc);
                t = __fdiv_rn(P.A < 0.0f ? __fsub_rn(b, sq) : __fadd_rn(b, sq), P.A);
            }
        }
    }
    if (!(t == t)) t = 0.0f;
    if (P.spread == 1) {
        t = __fsub_rn(t, floorf(t));
    } else if (P.spread == 2) {
        const float u = __fsub_rn(t, __fmul_rn(2.0f, floorf(__fmul_rn(t, 0.5f))));
        t = u > 1.0f ? __fsub_rn(2.0f, u) : u;
    } else {
        t = gmin(gmax(t, 0.0f), 1.0f);
    }
    const int n = P.n_stops;
    if (n <= 0) return 0u;
    float ch[4];
    if (!(t > P.off[0])) {
#pragma unroll
        for (int q = 0; q < 4; ++q) ch[q] = P.rgba[0][q];
    } else if (!(t < P.off[n - 1])) {
#pragma unroll
        for (int q = 0; q < 4; ++q) ch[q] = P.rgba[n - 1][q];
    } else {
        int k = 0;
        while (k + 2 < n && !(t < P.off[k + 1])) ++k;
        const float f = __fdiv_rn(__fsub_rn(t, P.off[k]), __fsub_rn(P.off[k + 1], P.off[k]));
#pragma unroll
        for (int q = 0; q < 4; ++q) ch[q] = lerp_rn(P.rgba[k][q], P.rgba[k + 1][q], f);
    }
    ch[3] = __fmul_rn(ch[3], P.opacity);
    uint32_t col = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        float v = __fmul_rn(ch[q], 255.0f);
        if (!(v > 0.0f)) v = 0.0f;
        if (v > 255.0f) v = 255.0f;
        col |= (uint32_t)v << (8 * q);
    }
    return (col >> 24) ? col : 0u;
}

// A gradient record's PixRec carries iau = kGradient and its paint in sab.
constexpr uint32_t kGradient = 0xFFFFFFFFu;

SR_DEV PixRec solid_rec(uint32_t col) {
    PixRec pr;
    const uint32_t al = col >> 24;
    pr.ia = (float)(255u - al);
    pr.sg = (float)(((col >> 8) & 0xFFu) * al);
    pr.iau = 255u - al;
    pr.sab = ((col & 0xFFu) * al + 128u) | ((((col >> 16) & 0xFFu) * al + 128u) << 16);
    return pr;
}

// GRAD: the kernel paints gradients.  Without it a gradient record is a
// solid of alpha 0, which leaves every pixel as it was; the kernels without
// gradients run for scenes without paints and keep their registers.
template <bool GRAD> SR_DEV PixRec pix_rec(const int4 d, uint32_t di) {
    PixRec pr;
    pr.idx1 = di + 1u;
    const int32_t x = d.x & 0xFFFF;
    pr.x0 = x;
    pr.x1 = wadd(x, d.y);
    const uint32_t col = (uint32_t)d.z, al = col >> 24;
    const int32_t paint = GRAD ? fill_paint(col) : -1;
    if (paint >= 0) {
        pr.iau = kGradient;
        pr.sab = (uint32_t)paint;
        pr.ia = 0.0f;
        pr.sg = 0.0f;
        pr.row = 0;
        return pr;
    }
    pr.ia = (float)(255u - al);
    pr.sg = (float)(((col >> 8) & 0xFFu) * al);
    pr.iau = 255u - al;
    pr.sab = ((col & 0xFFu) * al + 128u) | ((((col >> 16) & 0xFFu) * al + 128u) << 16);
    pr.row = 0;
    return pr;
}

// A gradient record: each lane blends its covered pixels with the paint's
// colour at their centres (row centre yc); a paint the table lacks paints
// nothing.
SR_DEV void apply_gradient(const ResolveArgs& a, const PixRec& pr, int32_t seg, int lane, float yc,
                           uint32_t (&rb)[kK], float (&g)[kK]) {
    if (!a.paints || pr.sab >= a.n_paints) return;
    const DevPaint& P = a.paints[pr.sab];
#pragma unroll
    for (int j = 0; j < kK; ++j) {
        const int32_t p = seg + lane + 32 * j;
        if (p >= pr.x0 && p < pr.x1) {
            const uint32_t col = paint_color(P, __fadd_rn((float)p, 0.5f), yc);
            if (col) blend3(rb[j], g[j], solid_rec(col));
        }
    }
}

// A record on this warp's segment: a one-pixel record is a uniform branch on
// its register slot; a record over the whole segment blends every slot;
// otherwise each lane tests its pixels.
template <bool GRAD>
SR_DEV void apply_pix(const ResolveArgs& a, const PixRec& pr, int32_t seg, int lane, float yc, uint32_t (&rb)[kK],
                      float (&g)[kK]) {
    if (GRAD && pr.iau == kGradient) {
        apply_gradient(a, pr, seg, lane, yc, rb, g);
    } else if (pr.x1 - pr.x0 == 1) {
        const int32_t off = pr.x0 - seg;
        const int j = off >> 5;
        if (lane == (off & 31)) {
            switch (j) {
                case 0: blend3(rb[0], g[0], pr); break;
                case 1: blend3(rb[1], g[1], pr); break;
                case 2: blend3(rb[2], g[2], pr); break;
                case 3: blend3(rb[3], g[3], pr); break;
                case 4: blend3(rb[4], g[4], pr); break;
                case 5: blend3(rb[5], g[5], pr); break;
                case 6: blend3(rb[6], g[6], pr); break;
                default: blend3(rb[7], g[7], pr); break;
            }
        }
    } else if (pr.x0 <= seg && pr.x1 >= seg + kResolveSeg) {
#pragma unroll
        for (int j = 0; j < kK; ++j) blend3(rb[j], g[j], pr);
    } else {
#pragma unroll
        for (int j = 0; j < kK; ++j) {
            int32_t p = seg + lane + 32 * j;
            if (p >= pr.x0 && p < pr.x1) blend3(rb[j], g[j], pr);
        }
    }
}

// Where a segment's painting may start.  Every pixel-blend is monotone in
// the pixel's old value (c' = floor((s*a + c*(255-a) + 127) / 255)), and so
// is any composition of them.  If a run of records that each cover the whole
// segment maps 0 and 255 to the same value in R, G and B, it maps every
// value there: the segment holds one colour after the run whatever it held
// before, so painting from white at the run's first record gives the same
// pixels as painting from the row's first record.  With alpha >= 0.4 a run
// of a handful of layers usually does this; an opaque span is a run of one.
// A warp walks the last kChunk records of its row from the end back,
// collects each run of whole-segment records between records that cover
// only part of the segment (the latest 32 of a longer run), and lane t
// tests the run's suffix from its record t: the latest start that collapses
// is the cut.  Without one the segment is painted from the row's start.
// The walk costs about a pass over the records it reads, so it is skipped
// for rows of fewer than kSearchLayers layers a pixel (record widths summed
// by the emit, over the row's width): a cut needs a run of several whole-
// segment layers and saves little there.
constexpr unsigned kSearchLayers = 32;

SR_DEV bool row_searched(const ResolveArgs& a, uint32_t r, int32_t W) {
    return !a.row_px || a.row_px[r] >= (unsigned long long)kSearchLayers * (unsigned long long)W;
}

struct RunRec {
    uint32_t iau, sab;
    float ia, sg;
};

SR_DEV RunRec run_rec(const PixRec& p) {
    RunRec r;
    r.iau = p.iau;
    r.sab = p.sab;
    r.ia = p.ia;
    r.sg = p.sg;
    return r;
}

// A warp's run of whole-segment records, in draw order with the latest at
// [31], and their positions.
struct RunBuf {
    RunRec rec[32];
    int32_t pos[32];
};

// The latest position among the n held records from which the run to [31]
// sends 0 and 255 to one colour, or -1.
SR_DEV int32_t run_collapse(const RunBuf& buf, int n, int lane) {
    uint32_t lo_rb = 0u, hi_rb = 0x00FF00FFu;
    float lo_g = 0.0f, hi_g = 255.0f;
    for (int k = 32 - n; k < 32; ++k) {
        const RunRec r = buf.rec[k];
        if (k >= lane) {
            blend3(lo_rb, lo_g, r);
            blend3(hi_rb, hi_g, r);
        }
    }
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, lane >= 32 - n && lo_rb == hi_rb && lo_g == hi_g);
    return m ? buf.pos[31 - __clz(m)] : -1;
}

// The run bookkeeping of a backward walk: feed() takes 32 records at a time
// (latest lane first), each overlapping the segment or not and covering all
// of it or not.
struct RunWalk {
    int n = 0;          // records of the current run held
    bool full = false;  // the held run filled the buffer and did not collapse
    int32_t cut = -1;

    // Returns true once a cut is found.  Covers above the highest record
    // over part of the segment extend the current run; that record ends it;
    // the covers below it start the next run, and so on.  A run's records
    // enter the buffer together, each lane at its rank from the top.
    SR_DEV bool feed(uint32_t mo, uint32_t mc, const PixRec& mine, int32_t pos, int lane, RunBuf& buf) {
        uint32_t mp = mo & ~mc;
        for (;;) {
            const uint32_t above = mp ? ~((2u << (31 - __clz(mp))) - 1u) : 0xFFFFFFFFu;
            const uint32_t run = mc & above;
            if (run && !full) {
                const int rank = n + __popc(run & ~((2u << lane) - 1u));
                if (((run >> lane) & 1u) && rank < 32) {
                    buf.rec[31 - rank] = run_rec(mine);
                    buf.pos[31 - rank] = pos;
                }
                __syncwarp();
                n += __popc(run);
                if (n >= 32) {
                    n = 32;
                    cut = run_collapse(buf, n, lane);
                    if (cut >= 0) return true;
                    full = true;
                }
            }
            if (!mp) return false;
            if (close(lane, buf)) return true;
            mc &= ~above;
            mp &= ~above & ((1u << (31 - __clz(mp))) - 1u);
            if (!mc) return false;
        }
    }

    SR_DEV bool close(int lane, RunBuf& buf) {
        if (n && !full) {
            cut = run_collapse(buf, n, lane);
            if (cut >= 0) return true;
        }
        n = 0;
        full = false;
        return false;
    }
};

template <bool GRAD> SR_DEV void stage_pix(const ResolveArgs& a, PixRec* sq, int32_t c0, int32_t cnt) {
    for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
        const uint32_t di = a.row_sorted_idx[c0 + q];
        sq[q] = pix_rec<GRAD>(a.draw[di], di);
    }
}

SR_DEV void init_pix(uint32_t (&rb)[kK], float (&g)[kK]) {
#pragma unroll
    for (int j = 0; j < kK; ++j) {
        rb[j] = 0x00FF00FFu;
        g[j] = 255.0f;
    }
}

SR_DEV void store_pix(const ResolveArgs& a, const ResolveWork& w, int32_t seg, int lane, const uint32_t (&rb)[kK],
                      const float (&g)[kK]) {
    uint32_t* out = a.image + w.si->image_off + (size_t)(w.r0 + w.my_row) * w.W;
#pragma unroll
    for (int j = 0; j < kK; ++j) {
        int32_t p = seg + lane + 32 * j;
        if (p < w.W) out[p] = rb[j] | ((uint32_t)__float2int_rn(g[j]) << 8) | 0xFF000000u;
    }
}

// A CTA of several short rows (a canvas narrower than WARPS segments): each
// warp finds its cut and streams its own row's records 32 at a time through
// its own shared-memory slots, without waiting for the other warps.
template <bool GRAD>
SR_DEV void resolve_pixel_rows(const ResolveArgs& a, const ResolveWork& w, int32_t seg, PixRec* slot, RunBuf& buf) {
    const int lane = threadIdx.x & 31;
    const uint32_t r = w.si->row_base + (uint32_t)(w.r0 + w.my_row);
    const int32_t beg = a.row_start[r], end = a.row_start[r + 1];
    const int32_t segend = imin(seg + kResolveSeg, w.W);
    const uint32_t cut = resolve_cut(a, w, seg, true);
    int32_t start = beg;
    if (row_searched(a, r, w.W)) {
        RunWalk rw;
        const int32_t lim = imax(beg, end - kChunk);
        bool found = false;
        for (int32_t c1 = end; c1 > lim && !found; c1 -= 32) {
            const int32_t q = c1 - 32 + lane;
            bool ov = false, cover = false;
            PixRec pr;
            if (q >= lim) {
                const uint32_t di = a.row_sorted_idx[q];
                pr = pix_rec<GRAD>(a.draw[di], di);
                ov = pr.x0 < seg + kResolveSeg && pr.x1 > seg;
                // a gradient's colour varies over the segment: it ends a run
                cover = pr.x0 <= seg && pr.x1 >= segend && pr.iau != kGradient;
            }
            found = rw.feed(__ballot_sync(0xFFFFFFFFu, ov), __ballot_sync(0xFFFFFFFFu, cover), pr, q, lane, buf);
        }
        if (found || rw.close(lane, buf)) start = rw.cut;
    }
    uint32_t rb[kK];
    float g[kK];
    init_pix(rb, g);
    const float yc = __fadd_rn((float)(w.r0 + w.my_row), 0.5f);
    for (int32_t c0 = start; c0 < end; c0 += 32) {
        const int32_t q = c0 + lane;
        bool ov = false;
        if (q < end) {
            const uint32_t di = a.row_sorted_idx[q];
            const PixRec pr = pix_rec<GRAD>(a.draw[di], di);
            ov = pr.x0 < seg + kResolveSeg && pr.x1 > seg && pr.idx1 >= cut;
            if (ov) slot[lane] = pr;
        }
        uint32_t m = __ballot_sync(0xFFFFFFFFu, ov);
        __syncwarp();
        while (m) {
            const PixRec p = slot[__ffs(m) - 1];
            m &= m - 1;
            apply_pix<GRAD>(a, p, seg, lane, yc, rb, g);
        }
        __syncwarp();
    }
    store_pix(a, w, seg, lane, rb, g);
}

// CTAs of several rows (canvases narrower than WARPS segments) run the path
// above in their own kernel, with little shared memory; the kernel below
// skips them.  The two run one after the other over the same grid.
//
// A CTA per cell row (a canvas of at least half as many segments as the CTA
// has warps; warps beyond the row's segments idle): the row's last kChunk
// records are staged once, every warp finds its segment's cut in them, and the CTA
// stages from the earliest cut on (chunks end-aligned, so the last one is
// the chunk already staged); a warp skips the records before its own cut.
template <int WARPS, bool GRAD>
__global__ void __launch_bounds__(32 * WARPS) k_resolve_pixel_rows(const ResolveArgs a) {
    __shared__ PixRec slots[WARPS * 32];
    __shared__ RunBuf bufs[WARPS];
    if (!a.cta_narrow[blockIdx.x]) return;
    const ResolveWork w = resolve_work<WARPS>(a);
    const int warp = threadIdx.x >> 5;
    if (w.active) resolve_pixel_rows<GRAD>(a, w, resolve_seg<WARPS>(w, 0) * kResolveSeg, slots + warp * 32, bufs[warp]);
}

template <int WARPS, bool GRAD>
__global__ void __launch_bounds__(32 * WARPS) k_resolve_pixel(const ResolveArgs a) {
    if (a.any_narrow && a.cta_narrow[blockIdx.x]) return;   // k_resolve_pixel_rows
    __shared__ PixRec sq[kChunk];
    __shared__ RunBuf bufs[WARPS];
    __shared__ int32_t cta_start[2];   // by group parity: a warp may still read the last group's
    const ResolveWork w = resolve_work<WARPS>(a);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int32_t W = w.W;
    const uint32_t r = w.si->row_base + (uint32_t)w.r0;
    const int32_t beg = a.row_start[r], end = a.row_start[r + 1];
    const int32_t tail0 = imax(beg, end - kChunk);
    const bool search = row_searched(a, r, W);
    bool tail_staged = false;   // sq holds [tail0, end)
    if (search) {
        stage_pix<GRAD>(a, sq, tail0, end - tail0);
        tail_staged = true;
    }
    for (int group = 0; group < w.groups; ++group) {
        const int32_t seg = resolve_seg<WARPS>(w, group) * kResolveSeg;
        const bool live = w.active && seg < W;   // a row of fewer segments than warps leaves some idle
        int32_t start = beg, s0 = beg;
        if (search) {
            if (threadIdx.x == 0) cta_start[group & 1] = end;
            __syncthreads();
            if (live) {
                const int32_t segend = imin(seg + kResolveSeg, W);
                RunWalk rw;
                bool found = false;
                for (int32_t c1 = end - tail0; c1 > 0 && !found; c1 -= 32) {
                    const int32_t i = c1 - 32 + lane;
                    bool ov = false, cover = false;
                    if (i >= 0) {
                        const int32_t x0 = sq[i].x0, x1 = sq[i].x1;
                        ov = x0 < seg + kResolveSeg && x1 > seg;
                        cover = x0 <= seg && x1 >= segend && sq[i].iau != kGradient;
                    }
                    found = rw.feed(__ballot_sync(0xFFFFFFFFu, ov), __ballot_sync(0xFFFFFFFFu, cover),
                                    sq[i < 0 ? 0 : i], tail0 + i, lane, bufs[warp]);
                }
                if (found || rw.close(lane, bufs[warp])) start = rw.cut;
                if (lane == 0) atomicMin(&cta_start[group & 1], start);
            }
            __syncthreads();
            s0 = cta_start[group & 1];
        }
        const uint32_t cut = resolve_cut(a, w, seg, live);
        uint32_t rb[kK];
        float g[kK];
        init_pix(rb, g);
        const float yc = __fadd_rn((float)w.r0, 0.5f);
        const int32_t nchunks = (end - s0 + kChunk - 1) / kChunk;
        for (int k = nchunks - 1; k >= 0; --k) {
            const int32_t c0 = imax(s0, end - (k + 1) * kChunk), c1 = end - k * kChunk;
            const int32_t base = k ? c0 : tail0;
            if (k || !tail_staged) {
                __syncthreads();
                stage_pix<GRAD>(a, sq, base, c1 - base);
                __syncthreads();
                tail_staged = k == 0;
            }
            if (!live) continue;
            const int32_t hi = c1 - base;
            for (int32_t g0 = imax(c0, start) - base; g0 < hi; g0 += 32) {
                const int32_t qi = g0 + lane;
                bool ov = false;
                if (qi < hi) ov = sq[qi].x0 < seg + kResolveSeg && sq[qi].x1 > seg && sq[qi].idx1 >= cut;
                uint32_t m = __ballot_sync(0xFFFFFFFFu, ov);
                while (m) {
                    const PixRec pr = sq[g0 + __ffs(m) - 1];
                    m &= m - 1;
                    apply_pix<GRAD>(a, pr, seg, lane, yc, rb, g);
                }
            }
        }
        if (live) store_pix(a, w, seg, lane, rb, g);
    }
}

// ------------------------------------------------------- reference mode --
// Overwrite in draw order (blending off); a cell row is FRAG_SIZE pixel
// rows, painted alike.
struct RefRec {
    int32_t x0, x1;
    uint32_t col;
    int32_t row;
    uint32_t idx1;   // 1 + draw index
};

template <int WARPS, bool GRAD>
__global__ void __launch_bounds__(32 * WARPS) k_resolve_ref(const ResolveArgs a) {
    __shared__ RefRec sq[kChunk];
    const ResolveWork w = resolve_work<WARPS>(a);
    const int tid = threadIdx.x, lane = tid & 31;
    const int32_t W = w.W;
    const uint32_t gr0 = w.si->row_base + (uint32_t)w.r0;
    const int32_t beg = a.row_start[gr0], end = a.row_start[gr0 + (uint32_t)w.nr];
    for (int group = 0; group < w.groups; ++group) {
        const int32_t seg = resolve_seg<WARPS>(w, group) * kResolveSeg;
        const bool live = w.active && seg < W;
        const uint32_t cut = resolve_cut(a, w, seg, live);
        uint32_t px[kK];
#pragma unroll
        for (int j = 0; j < kK; ++j) px[j] = 0xFFFFFFFFu;
        for (int32_t c0 = beg; c0 < end; c0 += kChunk) {
            const int32_t cnt = imin(kChunk, end - c0);
            __syncthreads();
            for (int q = tid; q < cnt; q += blockDim.x) {
                const uint32_t di = a.row_sorted_idx[c0 + q];
                int4 d = a.draw[di];
                RefRec rr;
                rr.idx1 = di + 1u;
                rr.x0 = d.x & 0xFFFF;
                rr.x1 = wadd(rr.x0, d.y);
                rr.col = (uint32_t)d.z;
                rr.row = div_F(d.x >> 16, a.F) - w.r0;
                sq[q] = rr;
            }
            __syncthreads();
            if (!live) continue;
            for (int32_t g0 = 0; g0 < cnt; g0 += 32) {
                const int32_t qi = g0 + lane;
                bool ov = false;
                if (qi < cnt)
                    ov = sq[qi].row == w.my_row && sq[qi].x0 < seg + kResolveSeg && sq[qi].x1 > seg &&
                         sq[qi].idx1 >= cut;
                uint32_t m = __ballot_sync(0xFFFFFFFFu, ov);
                while (m) {
                    const int q = g0 + __ffs(m) - 1;
                    m &= m - 1;
                    const RefRec rr = sq[q];
                    const int32_t paint = GRAD ? fill_paint(rr.col) : -1;
                    if (paint >= 0) {
                        // a gradient, sampled on the cell's centre row; a
                        // paint the table lacks paints nothing
                        if (a.paints && (uint32_t)paint < a.n_paints) {
                            const DevPaint& P = a.paints[paint];
                            const float yc = __fadd_rn((float)((w.r0 + w.my_row) * a.F), 1.0f);
#pragma unroll
                            for (int j = 0; j < kK; ++j) {
                                int32_t p = seg + lane + 32 * j;
                                if (p >= rr.x0 && p < rr.x1) px[j] = paint_color(P, __fadd_rn((float)p, 0.5f), yc);
                            }
                        }
                    } else {
#pragma unroll
                        for (int j = 0; j < kK; ++j) {
                            int32_t p = seg + lane + 32 * j;
                            if (p >= rr.x0 && p < rr.x1) px[j] = rr.col;
                        }
                    }
                }
            }
        }
        if (live) {
            const int32_t y0 = (w.r0 + w.my_row) * a.F;
            const int32_t nrows = imin(a.F, w.si->H - y0);
            for (int32_t yy = 0; yy < nrows; ++yy) {
                uint32_t* out = a.image + w.si->image_off + (size_t)(y0 + yy) * W;
#pragma unroll
                for (int j = 0; j < kK; ++j) {
                    int32_t p = seg + lane + 32 * j;
                    if (p < W) out[p] = px[j];
                }
            }
        }
    }
}

template <int WARPS, bool GRAD> static void launch_resolve_t(const ResolveArgs& a, uint32_t n_ctas, cudaStream_t st) {
    if (a.pixel_mode) {
        k_resolve_pixel<WARPS, GRAD><<<n_ctas, 32 * WARPS, 0, st>>>(a);
        if (a.any_narrow) k_resolve_pixel_rows<WARPS, GRAD><<<n_ctas, 32 * WARPS, 0, st>>>(a);
    } else {
        k_resolve_ref<WARPS, GRAD><<<n_ctas, 32 * WARPS, 0, st>>>(a);
    }
}

void launch_resolve(const ResolveArgs& a, uint32_t n_ctas, cudaStream_t st) {
    if (n_ctas == 0) return;
    count_launches(1);
    if (a.pixel_mode && a.any_narrow) count_launches(1);
    const bool grad = a.paints && a.n_paints;
    if (a.warps == 8) {
        if (grad) launch_resolve_t<8, true>(a, n_ctas, st);
        else launch_resolve_t<8, false>(a, n_ctas, st);
    } else {
        if (grad) launch_resolve_t<16, true>(a, n_ctas, st);
        else launch_resolve_t<16, false>(a, n_ctas, st);
    }
}

// Multisampling: the sample frames summed per channel (ushort4; 16 samples
// of 255 fit), then the rounded average (sum + k/2) / k per channel.
__global__ void k_aa_accumulate(const uint32_t* __restrict__ img, ushort4* __restrict__ acc, size_t n, int first) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t c = img[i];
    ushort4 v = first ? make_ushort4(0, 0, 0, 0) : acc[i];
    v.x = (unsigned short)(v.x + (c & 0xFFu));
    v.y = (unsigned short)(v.y + ((c >> 8) & 0xFFu));
    v.z = (unsigned short)(v.z + ((c >> 16) & 0xFFu));
    v.w = (unsigned short)(v.w + (c >> 24));
    acc[i] = v;
}

__global__ void k_aa_resolve(const ushort4* __restrict__ acc, uint32_t* __restrict__ img, size_t n, uint32_t k) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ushort4 v = acc[i];
    const uint32_t h = k / 2u;
    img[i] = ((v.x + h) / k) | (((v.y + h) / k) << 8) | (((v.z + h) / k) << 16) | (((v.w + h) / k) << 24);
}

void launch_aa_accumulate(const uint32_t* img, void* acc, size_t n, bool first, cudaStream_t st) {
    if (!n) return;
    count_launches(1);
    k_aa_accumulate<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(img, static_cast<ushort4*>(acc), n, first ? 1 : 0);
}

void launch_aa_resolve(const void* acc, uint32_t* img, size_t n, uint32_t k, cudaStream_t st) {
    if (!n) return;
    count_launches(1);
    k_aa_resolve<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(static_cast<const ushort4*>(acc), img, n, k);
}

void launch_row_bounds(const uint32_t* srows, int64_t n, const uint32_t* n_dev, int32_t rows, int32_t* row_start,
                       cudaStream_t st) {
    int64_t work = n + 1;
    int blocks = (int)((work + 255) / 256);
    if (blocks > 1216) blocks = 1216;
    count_launches(1);
    k_row_bounds<<<blocks, 256, 0, st>>>(srows, n, n_dev, rows, row_start);
}

}  // namespace sr
