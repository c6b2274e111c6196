// oracle.cpp — CPU restatement of the VkScanlinePR scanline pipeline.
//
// TEST INFRASTRUCTURE ONLY.  It checks the renderer's output: tests/, the
// smoke check and bench.py's CPU-baseline leg load it; the renderer never does.
//
// Parity status: UNPINNED by the reference's own outputs.  The reference has
// no tests, no golden images and no CPU path, and it cannot be built or run
// here (MSVC/Win32 + Vulkan + GLFW; no graphics stack).  This restatement
// follows its compute shaders operation for operation (file:line cited at
// each step) and is pinned by hand-computed known-answer scenes and by the
// draw-record format of the reference's mock draw lists (workdir/test_data*.csv).
//
// Every floating-point step is one IEEE operation in source order; build with
// -ffp-contract=off so no multiply-add is fused.  Shader semantics that GLSL
// leaves open are fixed here and matched by the CUDA kernels:
//   * float->int conversion truncates, saturates, and maps NaN to 0;
//   * int arithmetic wraps (two's complement);
//   * GLSL min(x,y) = (y < x) ? y : x, max(x,y) = (x < y) ? y : x;
//   * dot((x,y,0,1), m) = ((x*m.x + y*m.y) + 0*m.z) + 1*m.w;
//   * shared-memory slots the shaders read before writing are 0.
//
// Documented extensions (the reference leaves them TODO):
//   * QUADRIC curves (make_intersection_0.comp:273-276, make_intersection_1.comp:
//     386-388, gen_fragment.comp:66-69): 3 control points, one monotonic cut
//     per axis at t = (p0-p1)/((p0-p1)+(p2-p1)), 2-level lerp evaluation, the
//     same 24-step bisection as cubics.
//   * pixel mode (FRAG_SIZE 1): winding sampled on the pixel-centre row
//     y = cell_y + 0.5; a boundary cell is painted iff its centre passes the
//     fill rule, the centre winding being the exclusive scan at the first
//     record of the cell plus the winding changes of the cell's pieces whose
//     chord crosses the centre row left of the centre; integer source-over
//     compositing in path order over white.
//   * reference mode: FRAG_SIZE 2, whole boundary cells, draw records painted
//     over [x, x+width) x [y, y+2) with blending off (last record wins).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

#include "../include/sr.h"
#include "../vkscanlinepr_gb300/csrc/synth.h"

namespace orc {

// Oracle-only stage id: draw records per path (the labels of learned sizing).
constexpr int kStagePathDraws = 100;

// ------------------------------------------------------------- helpers ----
template <class R> struct FT;
template <> struct FT<float> {
    using I = int32_t;
    using U = uint32_t;
    static constexpr int ITER = 24;   // CUBIC_ITERATION_NUMBER (make_intersection_1.comp:7)
};
template <> struct FT<double> {
    using I = int64_t;
    using U = uint64_t;
    static constexpr int ITER = 52;
};

template <class R> static inline typename FT<R>::I bits(R x) {
    typename FT<R>::I i;
    std::memcpy(&i, &x, sizeof x);
    return i;
}
template <class R> static inline R from_bits(typename FT<R>::I i) {
    R x;
    std::memcpy(&x, &i, sizeof x);
    return x;
}
template <class R> static inline int32_t f2i(R x) {
    if (x != x) return 0;
    if (x >= (R)2147483648.0) return INT32_MAX;
    if (x <= (R)-2147483648.0) return INT32_MIN;
    return (int32_t)x;
}
static inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
static inline int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
template <class R> static inline R gmin(R x, R y) { return (y < x) ? y : x; }
template <class R> static inline R gmax(R x, R y) { return (x < y) ? y : x; }
static inline int32_t imin(int32_t a, int32_t b) { return b < a ? b : a; }
static inline int32_t imax(int32_t a, int32_t b) { return a < b ? b : a; }
static inline int32_t iclamp(int32_t v, int32_t lo, int32_t hi) { return imin(imax(v, lo), hi); }
// LERP(a,b,t) = a + t*(b-a)  (make_intersection_0.comp:10)
template <class R> static inline R lerp(R a, R b, R t) { return a + t * (b - a); }
// float2int_rd (make_intersection_1.comp:76-79)
template <class R> static inline int32_t float2int_rd(R x) {
    return x >= (R)0 ? f2i<R>(x) : f2i<R>(x - (R)1);
}
// PATH_INVISIBLE (make_intersection_0.comp:14-20)
static inline bool path_visible_mask(int32_t m) {
    bool inv = ((m & 0x11111000) == 0) || ((m & 0x01101011) == 0) || ((m & 0x00011111) == 0) ||
               ((m & 0x11010110) == 0);
    return !inv;
}

// Curve evaluation of one coordinate: LINE lerp, QUADRIC 2-level, CUBIC
// 3-level de Casteljau (make_intersection_1.comp:117-148).  ARC (an
// extension; p = x0, w*x1, x2, w): a 2-level lerp of the homogeneous points
// (x0, 1), (w*x1, w), (x2, 1), then one division.
template <class R> static inline R interp(uint32_t type, R t, const R* p) {
    switch (type) {
        case SR_CURVE_ARC: {
            R q0 = lerp(p[0], p[1], t), q1 = lerp(p[1], p[2], t);
            R r0 = lerp((R)1, p[3], t), r1 = lerp(p[3], (R)1, t);
            return lerp(q0, q1, t) / lerp(r0, r1, t);
        }
        case SR_CURVE_LINE: return lerp(p[0], p[1], t);
        case SR_CURVE_QUADRIC: {
            R q0 = lerp(p[0], p[1], t), q1 = lerp(p[1], p[2], t);
            return lerp(q0, q1, t);
        }
        case SR_CURVE_CUBIC: {
            R q0 = lerp(p[0], p[1], t), q1 = lerp(p[1], p[2], t), q2 = lerp(p[2], p[3], t);
            R l0 = lerp(q0, q1, t), l1 = lerp(q1, q2, t);
            return lerp(l0, l1, t);
        }
        default: return (R)0;
    }
}

// solveQuadEquation (make_intersection_0.comp:76-129)
template <class R> static inline void solve_quad(R a, R b, R c, R& r0, R& r1) {
    if (a == (R)0) {
        R x = -c / b;
        r0 = x;
        r1 = x;
        return;
    }
    R A = a, B = b * (R)0.5, C = c;
    R Rr = B * B - A * C;
    if (Rr > (R)0) {
        R SR = std::sqrt(Rr);
        if (B > (R)0) {
            R TB = B + SR;
            r0 = -C / TB;
            r1 = -TB / A;
        } else {
            R TB = -B + SR;
            r0 = TB / A;
            r1 = C / TB;
        }
    } else {
        r0 = (R)0;
        r1 = (R)0;
    }
}

// ------------------------------------------------------- thread helper ----
static void parallel_for(int threads, int64_t n, int64_t grain, const std::function<void(int64_t, int64_t)>& fn) {
    if (n <= 0) return;
    if (threads <= 1 || n <= grain) {
        fn(0, n);
        return;
    }
    std::atomic<int64_t> next{0};
    auto worker = [&]() {
        for (;;) {
            int64_t b = next.fetch_add(grain);
            if (b >= n) break;
            fn(b, std::min(n, b + grain));
        }
    };
    std::vector<std::thread> ts;
    for (int i = 1; i < threads; ++i) ts.emplace_back(worker);
    worker();
    for (auto& t : ts) t.join();
}

// exclusive scan, n+1 outputs: out[n] = total (naive_scan.comp:27-73, written
// exactly n+1 entries; the shader's last-batch guard may write past n).
static void excl_scan(int threads, const int32_t* in, int32_t* out, int64_t n) {
    const int64_t chunk = 1 << 20;
    int64_t nch = (n + chunk - 1) / chunk;
    std::vector<int32_t> part(nch + 1, 0);
    parallel_for(threads, nch, 1, [&](int64_t b, int64_t e) {
        for (int64_t c = b; c < e; ++c) {
            int32_t s = 0;
            int64_t lo = c * chunk, hi = std::min(n, lo + chunk);
            for (int64_t i = lo; i < hi; ++i) s = wadd(s, in[i]);
            part[c + 1] = s;
        }
    });
    for (int64_t c = 0; c < nch; ++c) part[c + 1] = wadd(part[c + 1], part[c]);
    // in and out may alias: read each element before writing it
    parallel_for(threads, nch, 1, [&](int64_t b, int64_t e) {
        for (int64_t c = b; c < e; ++c) {
            int32_t s = part[c];
            int64_t lo = c * chunk, hi = std::min(n, lo + chunk);
            for (int64_t i = lo; i < hi; ++i) {
                int32_t v = in[i];
                out[i] = s;
                s = wadd(s, v);
            }
        }
    });
    out[n] = part[nch];
}

// ------------------------------------------------------------ pipeline ----
struct Rec {
    int32_t cidx;
    int64_t tb;   // t bits | flags (float: low 32 bits used)
};

// ---- gradient paints (an extension; sr.h gives the definition) --------
// A paint for the resolve: the pixel -> gradient map in double, rounded to
// float once, then float arithmetic per pixel.
struct OPaint {
    int kind = 1, spread = 0, n = 0;
    float lin[3] = {0, 0, 0}, m[6] = {0, 0, 0, 0, 0, 0};
    float fx = 0, fy = 0, dx = 0, dy = 0, A = 0, opacity = 0;
    float off[SR_PAINT_MAX_STOPS] = {};
    float rgba[SR_PAINT_MAX_STOPS][4] = {};
};

static OPaint make_paint(const sr_paint& p, const float* m) {
    OPaint d;
    d.kind = p.kind == SR_PAINT_RADIAL ? 2 : 1;
    d.spread = p.spread == SR_SPREAD_REPEAT ? 1 : p.spread == SR_SPREAD_REFLECT ? 2 : 0;
    const double A0 = m[0], A1 = m[1], A2 = m[3], A3 = m[4], A4 = m[5], A5 = m[7];
    const double X0 = p.xf[0], X1 = p.xf[1], X2 = p.xf[2], X3 = p.xf[3], X4 = p.xf[4], X5 = p.xf[5];
    const double F0 = A0 * X0 + A1 * X3, F1 = A0 * X1 + A1 * X4, F2 = (A0 * X2 + A1 * X5) + A2;
    const double F3 = A3 * X0 + A4 * X3, F4 = A3 * X1 + A4 * X4, F5 = (A3 * X2 + A4 * X5) + A5;
    const double det = F0 * F4 - F1 * F3;
    const uint32_t ns = p.n_stops > SR_PAINT_MAX_STOPS ? SR_PAINT_MAX_STOPS : p.n_stops;
    if (det == 0.0 || !std::isfinite(det)) return d;
    const double G0 = F4 / det, G1 = -F1 / det, G3 = -F3 / det, G4 = F0 / det;
    const double G2 = -(G0 * F2 + G1 * F5), G5 = -(G3 * F2 + G4 * F5);
    if (d.kind == 1) {
        const double dx = (double)p.p1[0] - p.p0[0], dy = (double)p.p1[1] - p.p0[1];
        const double l2 = dx * dx + dy * dy;
        if (l2 > 0.0) {
            d.lin[0] = (float)((G0 * dx + G3 * dy) / l2);
            d.lin[1] = (float)((G1 * dx + G4 * dy) / l2);
            d.lin[2] = (float)(((G2 - p.p0[0]) * dx + (G5 - p.p0[1]) * dy) / l2);
        }
    } else {
        const double G[6] = {G0, G1, G2, G3, G4, G5};
        for (int k = 0; k < 6; ++k) d.m[k] = (float)G[k];
        const double dx = (double)p.p0[0] - p.p1[0], dy = (double)p.p0[1] - p.p1[1];
        d.fx = p.p1[0];
        d.fy = p.p1[1];
        d.dx = (float)dx;
        d.dy = (float)dy;
        d.A = (float)(dx * dx + dy * dy - (double)p.radius * p.radius);
    }
    d.opacity = p.opacity;
    d.n = (int)ns;
    for (uint32_t k = 0; k < ns; ++k) {
        d.off[k] = p.offset[k];
        for (int q = 0; q < 4; ++q) d.rgba[k][q] = p.rgba[k][q];
    }
    return d;
}

// Colour of paint P at the pixel-space point (x, y), packed RGBA8, 0 when
// transparent; every float operation one IEEE operation in this order.
static uint32_t paint_color(const OPaint& P, float x, float y) {
    float t;
    if (P.kind == 1) {
        t = (P.lin[0] * x + P.lin[1] * y) + P.lin[2];
    } else {
        const float gx = (P.m[0] * x + P.m[1] * y) + P.m[2];
        const float gy = (P.m[3] * x + P.m[4] * y) + P.m[5];
        const float ex = gx - P.fx, ey = gy - P.fy;
        const float b = ex * P.dx + ey * P.dy;
        const float c = ex * ex + ey * ey;
        if (P.A == 0.0f) {
            t = b != 0.0f ? c / (2.0f * b) : 0.0f;
        } else {
            const float disc = b * b - P.A * c;
            if (disc < 0.0f) {
                t = 0.0f;
            } else {
                const float sq = std::sqrt(disc);
                t = (P.A < 0.0f ? b - sq : b + sq) / P.A;
            }
        }
    }
    if (!(t == t)) t = 0.0f;
    if (P.spread == 1) {
        t = t - std::floor(t);
    } else if (P.spread == 2) {
        const float u = t - 2.0f * std::floor(t * 0.5f);
        t = u > 1.0f ? 2.0f - u : u;
    } else {
        t = gmin<float>(gmax<float>(t, 0.0f), 1.0f);
    }
    const int n = P.n;
    if (n <= 0) return 0u;
    float ch[4];
    if (!(t > P.off[0])) {
        for (int q = 0; q < 4; ++q) ch[q] = P.rgba[0][q];
    } else if (!(t < P.off[n - 1])) {
        for (int q = 0; q < 4; ++q) ch[q] = P.rgba[n - 1][q];
    } else {
        int k = 0;
        while (k + 2 < n && !(t < P.off[k + 1])) ++k;
        const float f = (t - P.off[k]) / (P.off[k + 1] - P.off[k]);
        for (int q = 0; q < 4; ++q) ch[q] = lerp(P.rgba[k][q], P.rgba[k + 1][q], f);
    }
    ch[3] = ch[3] * P.opacity;
    uint32_t col = 0;
    for (int q = 0; q < 4; ++q) {
        float v = ch[q] * 255.0f;
        if (!(v > 0.0f)) v = 0.0f;
        if (v > 255.0f) v = 255.0f;
        col |= (uint32_t)v << (8 * q);
    }
    return (col >> 24) ? col : 0u;
}

// The paint a fill names: alpha byte 0 and index + 1 in the colour bytes.
static inline int32_t fill_paint(uint32_t info) {
    return (info >> 24) == 0u && (info & 0x00FFFFFFu) != 0u ? (int32_t)(info & 0x00FFFFFFu) - 1 : -1;
}

template <class R> struct Frame {
    using I = typename FT<R>::I;
    // inputs
    const sr_scene_view* s = nullptr;
    int32_t W = 0, H = 0, F = 2, mode = 0, threads = 1;
    float m[16];
    // outputs
    std::vector<R> tpos;                 // 2V
    std::vector<int32_t> path_visible;   // P
    std::vector<R> cutq;                 // 4C
    std::vector<uint32_t> ncuts;         // C
    std::vector<float> cut_dump;         // 5C (float frame only)
    std::vector<int32_t> count, offs;    // C, C+1
    std::vector<Rec> rec;                // N
    std::vector<int32_t> inter_dump;     // 2N
    std::vector<int32_t> fkey, fpath, fwn, fleft;  // N
    std::vector<int32_t> skey, sval;     // N
    std::vector<int32_t> wscan;          // N+1
    std::vector<int32_t> fflag, sflag;   // N
    std::vector<int32_t> fscan;          // 2N+1
    std::vector<int32_t> draw;           // 4*O
    std::vector<int32_t> path_draws;     // P: draw records per path (sizing labels)
    std::vector<uint32_t> image;         // W*H
    int64_t N = 0, O = 0, n_frag = 0, n_span = 0;
    double ms[8] = {0};
    int error = 0;

    const R* pts(uint32_t c, int axis, R* buf) const {
        uint32_t pi = s->curve_pos_map[c];
        uint32_t np = s->curve_type[c] == SR_CURVE_ARC ? 4u : (s->curve_type[c] & 7u);
        for (uint32_t i = 0; i < 4; ++i) buf[i] = (R)0;
        for (uint32_t i = 0; i < np && i < 4; ++i) buf[i] = tpos[2 * (size_t)(pi + i) + axis];
        return buf;
    }

    // ---- K1 transform_pos (transform_pos.comp:33-86)
    void transform() {
        uint32_t V = s->n_points, P = s->n_paths;
        tpos.assign(2 * (size_t)V, (R)0);
        path_visible.assign(P, 0);   // cleared every frame (the reference never clears it)
        R mm[16];
        for (int i = 0; i < 16; ++i) mm[i] = (R)m[i];
        R fw = (R)(float)W, fh = (R)(float)H;
        parallel_for(threads, V, 65536, [&](int64_t b, int64_t e) {
            for (int64_t p = b; p < e; ++p) {
                R x = (R)s->position[2 * p], y = (R)s->position[2 * p + 1];
                R o[4];
                for (int r = 0; r < 4; ++r) {
                    R acc = x * mm[4 * r + 0];
                    acc = acc + y * mm[4 * r + 1];
                    acc = acc + (R)0 * mm[4 * r + 2];
                    acc = acc + (R)1 * mm[4 * r + 3];
                    o[r] = acc;
                }
                o[0] = o[0] / o[3];
                o[1] = o[1] / o[3];
                tpos[2 * p] = o[0];
                tpos[2 * p + 1] = o[1];
            }
        });
        // region-code OR, sequential (OR semantics of transform_pos.comp:71-82)
        for (uint32_t p = 0; p < V; ++p) {
            R ox = tpos[2 * (size_t)p], oy = tpos[2 * (size_t)p + 1];
            int xf = ox < (R)0 ? 0 : (ox < fw ? 1 : 2);
            int yf = oy < (R)0 ? 0 : (oy < fh ? 1 : 2);
            int32_t v = 0;
            switch ((yf << 4) | xf) {
                case 0x00: v = 0x10000000; break;
                case 0x01: v = 0x01000000; break;
                case 0x02: v = 0x00100000; break;
                case 0x10: v = 0x00010000; break;
                case 0x11: v = 0x10000001; break;
                case 0x12: v = 0x00001000; break;
                case 0x20: v = 0x00000100; break;
                case 0x21: v = 0x00000010; break;
                case 0x22: v = 0x00000001; break;
                default: break;
            }
            path_visible[s->pos_path_idx[p]] |= v;
        }
        // arcs (an extension): the control slot transforms linearly as
        // (w*x, w*y, 0, w) with no division, the weight slot becomes the
        // fourth row's result, and the path is marked visible outright
        for (uint32_t c = 0; c < s->n_curves; ++c) {
            if (s->curve_type[c] != SR_CURVE_ARC) continue;
            const uint32_t f = s->curve_pos_map[c];
            R hx = (R)s->position[2 * (size_t)(f + 1)], hy = (R)s->position[2 * (size_t)(f + 1) + 1];
            R w = (R)s->position[2 * (size_t)(f + 3)];
            R o[4];
            for (int r = 0; r < 4; ++r) {
                R acc = hx * mm[4 * r + 0];
                acc = acc + hy * mm[4 * r + 1];
                acc = acc + (R)0 * mm[4 * r + 2];
                acc = acc + w * mm[4 * r + 3];
                o[r] = acc;
            }
            tpos[2 * (size_t)(f + 1)] = o[0];
            tpos[2 * (size_t)(f + 1) + 1] = o[1];
            tpos[2 * (size_t)(f + 3)] = o[3];
            tpos[2 * (size_t)(f + 3) + 1] = o[3];
            path_visible[s->curve_path_idx[c]] |= 0x11111111;
        }
    }

    // count-pass x/y range (get_xy_begin_end, make_intersection_0.comp:167-183)
    void xy_begin_end_floor(R p0, R p1, int32_t& b, int32_t& e) const {
        R fF = (R)F;
        if (p0 <= p1) {
            b = wadd(f2i<R>(std::floor(p0 / fF) * fF), F);
            e = f2i<R>(std::floor(p1 / fF) * fF);
        } else {
            b = wadd(f2i<R>(std::floor(p1 / fF) * fF), F);
            e = f2i<R>(std::floor(p0 / fF) * fF);
        }
    }
    // intersection-pass x/y range (get_xy_begin_end_delta, make_intersection_1.comp:150-170)
    void xy_begin_end_rd(R p0, R p1, int32_t& b, int32_t& e, R& d) const {
        R fF = (R)F;
        if (p0 <= p1) {
            b = wadd(wmul(float2int_rd<R>(p0 / fF), F), F);
            e = wmul(float2int_rd<R>(p1 / fF), F);
            d = fF;
        } else {
            b = wadd(wmul(float2int_rd<R>(p1 / fF), F), F);
            e = wmul(float2int_rd<R>(p0 / fF), F);
            d = -fF;
        }
    }
    // udpate_cut_range, one axis (make_intersection_0.comp:186-221)
    void cut_range(int32_t size, int32_t& b, int32_t& e, int32_t& n) const {
        int32_t mn = 0, mx = wadd(size & (int32_t)0xFFFFFFFE, F);
        if ((b < mn && e < mn) || (b > mx && e > mx) || (b > e)) {
            n = 0;
        } else {
            b = iclamp(b, mn, mx);
            e = iclamp(e, mn, mx);
            n = imax((e - b) / F + 1, 0);
        }
    }

    // ---- K2 make_intersection_0 (make_intersection_0.comp:226-411)
    void count_pass() {
        uint32_t C = s->n_curves;
        cutq.assign(4 * (size_t)C, (R)0);
        ncuts.assign(C, 0);
        count.assign(C, 0);
        parallel_for(threads, C, 8192, [&](int64_t b, int64_t e) {
            for (int64_t c = b; c < e; ++c) count_curve((uint32_t)c);
        });
        offs.assign((size_t)C + 1, 0);
        excl_scan(threads, count.data(), offs.data(), C);
        if (sizeof(R) == 4) {
            cut_dump.assign(5 * (size_t)C, 0.f);
            for (uint32_t c = 0; c < C; ++c) {
                for (int i = 0; i < 4; ++i) cut_dump[5 * (size_t)c + i] = (float)cutq[4 * (size_t)c + i];
                uint32_t nc = ncuts[c];
                std::memcpy(&cut_dump[5 * (size_t)c + 4], &nc, 4);
            }
        }
    }

    void count_curve(uint32_t c) {
        uint32_t type = s->curve_type[c];
        R px[4], py[4];
        pts(c, 0, px);
        pts(c, 1, py);
        bool vis = path_visible_mask(path_visible[s->curve_path_idx[c]]);
        uint32_t n = 0;
        R q[5] = {(R)0, (R)0, (R)0, (R)0, (R)0};
        if (vis) {
            for (int ax = 0; ax < 2; ++ax) {
                const R* p = ax == 0 ? px : py;
                if (type == SR_CURVE_CUBIC) {
                    R r0 = (R)0, r1 = (R)0;
                    solve_quad<R>((R)3 * (p[1] - p[2]) + (p[3] - p[0]),
                                  (R)2 * ((p[0] - p[1]) + (p[2] - p[1])), p[1] - p[0], r0, r1);
                    if (r0 > (R)0 && r0 < (R)1) q[n++] = r0;
                    if (r1 > (R)0 && r1 < (R)1 && r1 != r0) q[n++] = r1;
                } else if (type == SR_CURVE_QUADRIC) {
                    // extension: derivative root of the quadric
                    R den = (p[0] - p[1]) + (p[2] - p[1]);
                    if (den != (R)0) {
                        R r0 = (p[0] - p[1]) / den;
                        if (r0 > (R)0 && r0 < (R)1) q[n++] = r0;
                    }
                } else if (type == SR_CURVE_ARC) {
                    // extension: roots of the arc's derivative numerator
                    // N'D - ND' (its cubic terms cancel), halved
                    R wm1 = p[3] - (R)1;
                    R r0 = (R)0, r1 = (R)0;
                    solve_quad<R>(wm1 * (p[2] - p[0]), ((p[0] - p[1]) + (p[2] - p[1])) + ((R)2 * p[0]) * wm1,
                                  p[1] - p[3] * p[0], r0, r1);
                    if (r0 > (R)0 && r0 < (R)1) q[n++] = r0;
                    if (r1 > (R)0 && r1 < (R)1 && r1 != r0) q[n++] = r1;
                }
            }
            // insertion network, including the reference's `t2 = q3`
            // (make_intersection_0.comp:315-359), kept verbatim
            R q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3];
            if (n >= 2) {
                R t1 = q1, t0 = q0;
                if (t1 < t0) { q1 = t0; q0 = t1; }
            }
            if (n >= 3) {
                R t2 = q2, t1 = q1;
                if (t2 < t1) {
                    q2 = t1;
                    R t0 = q0;
                    if (t2 < t0) { q1 = t0; q0 = t2; } else { q1 = t2; }
                }
            }
            if (n >= 4) {
                R t3 = q3, t2 = q3;
                if (t3 < t2) {
                    q3 = t2;
                    R t1 = q1;
                    if (t3 < t1) {
                        q2 = t1;
                        R t0 = q0;
                        if (t3 < t0) { q1 = t0; q0 = t3; } else { q1 = t3; }
                    } else {
                        q2 = t3;
                    }
                }
            }
            q[0] = q0; q[1] = q1; q[2] = q2; q[3] = q3;
        }
        for (int i = 0; i < 4; ++i) cutq[4 * (size_t)c + i] = q[i];
        ncuts[c] = n;
        if (vis) q[n++] = (R)1;
        R x0 = px[0], y0 = py[0];
        int32_t pc = 0;
        for (uint32_t i = 0; i < n; ++i) {
            R t1 = q[i];
            R x1 = interp<R>(type, t1, px), y1 = interp<R>(type, t1, py);
            int32_t xb, xe, yb, ye, nx, ny;
            xy_begin_end_floor(x0, x1, xb, xe);
            xy_begin_end_floor(y0, y1, yb, ye);
            cut_range(W, xb, xe, nx);
            cut_range(H, yb, ye, ny);
            pc = wadd(pc, wadd(1, wadd(nx, ny)));
            x0 = x1;
            y0 = y1;
        }
        count[c] = pc;
    }

    // ---- K4 make_intersection_1 (make_intersection_1.comp:217-447)
    void intersect_pass() {
        uint32_t C = s->n_curves;
        N = offs[C];
        if (N < 0) { error = 1; N = 0; }
        rec.assign((size_t)N, Rec{0, 0});
        std::atomic<int> bad{0};
        parallel_for(threads, C, 4096, [&](int64_t b, int64_t e) {
            for (int64_t c = b; c < e; ++c)
                if (!intersect_curve((uint32_t)c)) bad.store(1);
        });
        if (bad.load()) error = 2;
        inter_dump.resize(2 * (size_t)N);
        for (int64_t i = 0; i < N; ++i) {
            inter_dump[2 * i] = rec[i].cidx;
            inter_dump[2 * i + 1] = (int32_t)(uint32_t)(uint64_t)rec[i].tb;
        }
    }

    static I flag_bits(I b, I f) { return (b & ~(I)3) | f; }

    bool intersect_curve(uint32_t c) {
        uint32_t type = s->curve_type[c];
        R P[2][4];
        pts(c, 0, P[0]);
        pts(c, 1, P[1]);
        bool vis = path_visible_mask(path_visible[s->curve_path_idx[c]]);
        R q[5];
        for (int i = 0; i < 4; ++i) q[i] = cutq[4 * (size_t)c + i];
        uint32_t n = ncuts[c];
        if (vis) q[n++] = (R)1;
        R t0_ms = (R)0;
        R x0m = P[0][0], y0m = P[1][0];
        int64_t pc = offs[c], end = offs[c + 1];
        const I minus_one = bits<R>((R)-1);
        for (uint32_t i = 0; i < n; ++i) {
            R t1_ms = q[i];
            R x1m = interp<R>(type, t1_ms, P[0]), y1m = interp<R>(type, t1_ms, P[1]);
            // flag bits of the piece end (make_intersection_1.comp:271-276)
            I tb = bits<R>(t1_ms) & ~(I)3;
            if (std::floor(x1m) == x1m) tb = tb | (I)2;
            else tb = tb | (I)3;
            t1_ms = from_bits<R>(tb);
            int32_t xb, xe, yb, ye, nx, ny;
            R dx, dy;
            xy_begin_end_rd(x0m, x1m, xb, xe, dx);
            xy_begin_end_rd(y0m, y1m, yb, ye, dy);
            cut_range(W, xb, xe, nx);
            cut_range(H, yb, ye, ny);
            int32_t n_loop = nx + ny + 1;
            R x = (R)(dx < (R)0 ? xe : xb);
            R y = (R)(dy < (R)0 ? ye : yb);
            R tnext[2] = {t0_ms, t0_ms};
            I last = minus_one;
            for (int32_t it = -1; it < n_loop; ++it) {
                R t_solve = (R)0, cc = (R)0, t_min;
                int side = 0;
                R ntx = tnext[0], nty = tnext[1];
                if (it == -1) {
                    t_min = ntx;
                    if (nx == 0) { side = 0; t_solve = (R)2; }
                    else if (ny == 0) { side = 1; t_solve = (R)2; }
                    else { side = 0; --nx; cc = x; x = x + dx; }
                } else if (ntx <= nty) {
                    t_min = ntx;
                    side = 0;
                    if (nx > 0) { --nx; cc = x; x = x + dx; }
                    else t_solve = (R)2;
                } else {
                    t_min = nty;
                    side = 1;
                    if (ny > 0) { --ny; cc = y; y = y + dy; }
                    else t_solve = (R)2;
                }
                if (it >= 0) {
                    I out = bits<R>(t_min);
                    if ((out & ~(I)3) == (last & ~(I)3)) {
                        out = out | last;
                        if (pc - 1 < offs[c] || pc - 1 >= end) return false;
                        rec[pc - 1] = Rec{(int32_t)c, (int64_t)out};
                    }
                    if (pc >= end) return false;
                    rec[pc] = Rec{(int32_t)c, (int64_t)out};
                    last = out;
                    ++pc;
                }
                if (t_solve < (R)2) {
                    const R* cv = P[side];
                    if (type == SR_CURVE_LINE) {
                        R a = cv[1] - cv[0];
                        a = (a != (R)0) ? ((R)1 / a) : (R)0;
                        t_solve = gmin<R>(gmax<R>((cc - cv[0]) * a, t_min), t1_ms);
                    } else {
                        R t0 = t_min, t1 = t1_ms;
                        R vt0 = interp<R>(type, t0, cv);
                        t_solve = t0;
                        if (vt0 != cc) {
                            R raw_t0 = t0, last_vtm = (R)0;
                            for (int j = 0; j < FT<R>::ITER; ++j) {
                                R tm = (t0 + t1) * (R)0.5;
                                R vtm = interp<R>(type, tm, cv);
                                t_solve = tm;
                                last_vtm = vtm;
                                if ((bits<R>(vtm - cc) ^ bits<R>(vt0 - cc)) >= 0) { t0 = tm; vt0 = vtm; }
                                else t1 = tm;
                            }
                            if (std::fabs(last_vtm - cc) > (R)1) t_solve = raw_t0;
                        }
                    }
                }
                tnext[side] = from_bits<R>(flag_bits(bits<R>(t_solve), (I)side));
            }
            t0_ms = t1_ms;
            x0m = x1m;
            y0m = y1m;
        }
        return pc == end;
    }

    // ---- K5 gen_fragment (gen_fragment.comp:90-245)
    void fragment_pass() {
        fkey.assign((size_t)N, 0);
        fpath.assign((size_t)N, 0);
        fwn.assign((size_t)N, 0);
        fleft.assign((size_t)N, 0);
        const int32_t invalid = (int32_t)0xFFFEFFFE;
        const R half = (R)0.5;
        parallel_for(threads, N, 65536, [&](int64_t b, int64_t e) {
            for (int64_t i = b; i < e; ++i) {
                Rec r0 = rec[i];
                Rec r1 = (i + 1 != N) ? rec[i + 1] : Rec{-1, (int64_t)bits<R>((R)1)};
                R t0 = from_bits<R>((I)r0.tb & ~(I)3);
                R t1 = from_bits<R>((I)r1.tb & ~(I)3);
                t0 = gmax<R>(t0, (R)0);
                t1 = gmax<R>(t1, (R)0);
                uint32_t c = (uint32_t)r0.cidx;
                uint32_t path = s->curve_path_idx[c];
                int32_t yx = invalid, wn = 0, left = 0;
                if (r0.cidx != r1.cidx) t1 = (R)1;
                if (t0 < t1) {
                    uint32_t type = s->curve_type[c];
                    R px[4], py[4];
                    pts(c, 0, px);
                    pts(c, 1, py);
                    R pfx = interp<R>(type, t0, px), pfy = interp<R>(type, t0, py);
                    R plx = interp<R>(type, t1, px), ply = interp<R>(type, t1, py);
                    R fF = (R)F;
                    int32_t rx = wmul(float2int_rd<R>(((pfx + plx) * half) / fF), F);
                    int32_t ry = wmul(float2int_rd<R>(((pfy + ply) * half) / fF), F);
                    int32_t pos_x = imin(imax(rx, -F), wadd(W & (int32_t)0xFFFFFFFE, F));
                    int32_t pos_y = imin(imax(ry, -F), wadd(H & (int32_t)0xFFFFFFFE, F));
                    int32_t ysh = (int32_t)((uint32_t)wadd(pos_y, 0x7FFF) << 16);
                    int32_t xsh = wadd(pos_x, 0x7FFF) & 0xFFFF;
                    if ((uint32_t)ry < (uint32_t)H) yx = ysh | xsh;
                    // winding sample row: cell_y + FRAG_SIZE/2 (gen_fragment.comp:188)
                    R wn_y = (R)pos_y + (R)0.5 * fF;
                    if (pfy == ply) wn = 0;
                    else if (pfy < wn_y && wn_y <= ply) wn = -1;
                    else if (ply < wn_y && wn_y <= pfy) wn = 1;
                    if (mode == SR_MODE_PIXEL && wn != 0) {
                        R dyv = ply - pfy;
                        R tc = (wn_y - pfy) / dyv;
                        R xc = pfx + tc * (plx - pfx);
                        if (xc < (R)pos_x + half) left = wn;
                    }
                }
                fkey[i] = yx;
                fpath[i] = (int32_t)path;
                fwn[i] = wn;
                fleft[i] = left;
            }
        });
    }

    // ---- K6 naive_seg_sort_pairs: per path, by (signed key, index)
    void sort_pass() {
        skey.assign((size_t)N, 0);
        sval.assign((size_t)N, 0);
        std::vector<int64_t> seg;
        for (int64_t i = 0; i < N; ++i)
            if (i == 0 || fpath[i] != fpath[i - 1]) seg.push_back(i);
        seg.push_back(N);
        int64_t ns = (int64_t)seg.size() - 1;
        parallel_for(threads, ns, 64, [&](int64_t b, int64_t e) {
            std::vector<int64_t> tmp;
            for (int64_t sgi = b; sgi < e; ++sgi) {
                int64_t lo = seg[sgi], hi = seg[sgi + 1];
                tmp.resize(hi - lo);
                for (int64_t i = lo; i < hi; ++i) tmp[i - lo] = ((int64_t)fkey[i] << 32) | (uint32_t)i;
                std::sort(tmp.begin(), tmp.end());
                for (int64_t i = lo; i < hi; ++i) {
                    skey[i] = (int32_t)(tmp[i - lo] >> 32);
                    sval[i] = (int32_t)(uint32_t)tmp[i - lo];
                }
            }
        });
    }

    bool rule_pass(uint32_t rule, int32_t wn) const {
        // mark_merged_fragment_and_span.comp:82
        return (rule == 0 && wn != 0) || (rule == 1 && (wn & 1) != 0);
    }

    // ---- K7 shuffle + K3 winding scan + K8 mark (shuffle_fragment.comp:17-26,
    //      scanline_rasterizer.cpp:479-506, mark_merged_fragment_and_span.comp:22-93)
    void winding_mark_pass() {
        std::vector<int32_t> ws((size_t)N);
        parallel_for(threads, N, 65536, [&](int64_t b, int64_t e) {
            for (int64_t i = b; i < e; ++i) ws[i] = fwn[sval[i]];
        });
        wscan.assign((size_t)N + 1, 0);
        excl_scan(threads, ws.data(), wscan.data(), N);
        fflag.assign((size_t)N, 0);
        sflag.assign((size_t)N, 0);
        parallel_for(threads, N, 65536, [&](int64_t b, int64_t e) {
            for (int64_t i = b; i < e; ++i) {
                int32_t yx1 = skey[i];
                int32_t x1 = (yx1 & 0xFFFF) - 0x7FFF;
                int32_t y1 = ((yx1 >> 16) & 0xFFFF) - 0x7FFF;
                // plane 2 keeps the unsorted path ids; the sort never moves a
                // record across paths, so position i holds the same path
                int32_t p1 = fpath[i] & 0x3FFFFFFF;
                bool on = !(x1 < 0 || y1 < 0 || x1 >= W || y1 >= H);
                int32_t ff = 0, sf = 0;
                uint32_t rule = s->fill_rule[p1];
                if (i == 0) {
                    ff = on ? 1 : 0;
                } else {
                    int32_t p0 = fpath[i - 1] & 0x3FFFFFFF;
                    int32_t yx0 = skey[i - 1];
                    int32_t x0 = (yx0 & 0xFFFF) - 0x7FFF;
                    int32_t y0 = ((yx0 >> 16) & 0xFFFF) - 0x7FFF;
                    if (!on) ff = 0;
                    else if (p0 != p1 || yx0 != yx1) ff = 1;
                    int32_t wn = wscan[i];
                    if (y0 == y1 && wadd(x0, F) < x1 && p0 == p1 && rule_pass(rule, wn)) sf = 1;
                }
                if (mode == SR_MODE_PIXEL && ff) {
                    // centre sample of the merged cell (extension)
                    int32_t wc = wscan[i];
                    for (int64_t j = i; j < N && skey[j] == yx1 && (fpath[j] & 0x3FFFFFFF) == p1; ++j)
                        wc = wadd(wc, fleft[sval[j]]);
                    if (!rule_pass(rule, wc)) ff = 0;
                }
                fflag[i] = ff;
                sflag[i] = sf;
            }
        });
    }

    // ---- K3 flag scan + K9 gen_merged_fragment_and_span
    //      (scanline_rasterizer.cpp:545-608, gen_merged_fragment_and_span.comp:33-103)
    void emit_pass() {
        std::vector<int32_t> flags(2 * (size_t)N);
        for (int64_t i = 0; i < N; ++i) {
            flags[i] = fflag[i];
            flags[N + i] = sflag[i];
        }
        fscan.assign(2 * (size_t)N + 1, 0);
        excl_scan(threads, flags.data(), fscan.data(), 2 * N);
        n_frag = fscan[N];
        n_span = fscan[2 * N] - n_frag;
        O = n_frag + n_span;
        draw.assign(4 * (size_t)O, 0);
        path_draws.assign(s->n_paths, 0);
        for (int64_t i = 0; i < N; ++i)
            if (fflag[i] | sflag[i]) path_draws[fpath[i] & 0x3FFFFFFF] += fflag[i] + sflag[i];
        parallel_for(threads, N, 65536, [&](int64_t b, int64_t e) {
            for (int64_t i = b; i < e; ++i) {
                int32_t ff = fflag[i], sf = sflag[i];
                int32_t frag_index = fscan[i + 1];
                int32_t span_index = fscan[N + i + 1] - (int32_t)n_frag;
                int32_t fb = frag_index - ff, sb = span_index - sf;
                int32_t p = fpath[i] & 0x3FFFFFFF;
                int32_t info = (int32_t)s->fill_info[p];
                if (ff) {
                    int32_t raw = skey[i];
                    int32_t rx = (raw & 0xFFFF) - 0x7FFF;
                    int32_t ry = ((raw >> 16) & 0xFFFF) - 0x7FFF;
                    int64_t o = fb + sb;
                    draw[4 * o + 0] = (int32_t)((uint32_t)ry << 16) | rx;
                    draw[4 * o + 1] = F;
                    draw[4 * o + 2] = info;
                    draw[4 * o + 3] = frag_index;
                }
                if (sf) {
                    int64_t o = fb + sb + ff;
                    int32_t pr0 = skey[i - 1], pr1 = skey[i];
                    int32_t y0 = ((pr0 >> 16) & 0xFFFF) - 0x7FFF;
                    int32_t x0 = (pr0 & 0xFFFF) - 0x7FFF + F;
                    int32_t x1 = (pr1 & 0xFFFF) - 0x7FFF;
                    x0 = imax(0, x0);
                    draw[4 * o + 0] = (int32_t)((uint32_t)y0 << 16) | x0;
                    draw[4 * o + 1] = x1 - x0;
                    draw[4 * o + 2] = info;
                    draw[4 * o + 3] = 0;
                }
            }
        });
    }

    std::vector<OPaint> paints;
    void resolve_pass() { resolve(draw.data(), O, W, H, F, mode, threads, image, &paints); }

    // ---- K10 surface draw (scanlinepr.vert:18-51, scanlinepr.frag:7-14)
    static uint32_t blend(uint32_t dst, uint32_t src) {
        uint32_t a = src >> 24;
        uint32_t out = 0;
        for (int ch = 0; ch < 4; ++ch) {
            uint32_t sc = ch == 3 ? 255u : ((src >> (8 * ch)) & 0xFF);
            uint32_t dc = (dst >> (8 * ch)) & 0xFF;
            uint32_t v = (sc * a + dc * (255u - a) + 127u) / 255u;
            out |= v << (8 * ch);
        }
        return out;
    }

    static void resolve(const int32_t* d, int64_t O, int32_t W, int32_t H, int32_t F, int mode, int threads,
                        std::vector<uint32_t>& img, const std::vector<OPaint>* paints = nullptr) {
        img.assign((size_t)W * H, 0xFFFFFFFFu);  // clear to white (scanline_rasterizer.cpp:622)
        // bin record indices by row, keeping draw order
        std::vector<int64_t> cnt((size_t)H + 1, 0);
        auto rows = [&](int64_t k, int32_t& y0, int32_t& y1) {
            int32_t y = d[4 * k] >> 16;
            y0 = imax(y, 0);
            y1 = imin(wadd(y, F), H);
        };
        for (int64_t k = 0; k < O; ++k) {
            int32_t y0, y1;
            rows(k, y0, y1);
            for (int32_t y = y0; y < y1; ++y) cnt[y + 1]++;
        }
        for (int32_t y = 0; y < H; ++y) cnt[y + 1] += cnt[y];
        std::vector<int64_t> lst((size_t)cnt[H]);
        std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
        for (int64_t k = 0; k < O; ++k) {
            int32_t y0, y1;
            rows(k, y0, y1);
            for (int32_t y = y0; y < y1; ++y) lst[pos[y]++] = k;
        }
        parallel_for(threads, H, 16, [&](int64_t b, int64_t e) {
            for (int64_t y = b; y < e; ++y) {
                uint32_t* row = img.data() + (size_t)y * W;
                for (int64_t q = cnt[y]; q < cnt[y + 1]; ++q) {
                    int64_t k = lst[q];
                    int32_t x = d[4 * k] & 0xFFFF;
                    int32_t w = d[4 * k + 1];
                    uint32_t c = (uint32_t)d[4 * k + 2];
                    int32_t xa = imax(x, 0), xb = imin(wadd(x, w), W);
                    const int32_t pi = fill_paint(c);
                    if (pi >= 0) {
                        // a gradient at each pixel's centre (reference mode:
                        // the centre row of the 2-pixel cell); a paint the
                        // table lacks paints nothing
                        if (!paints || pi >= (int32_t)paints->size()) continue;
                        const OPaint& P = (*paints)[(size_t)pi];
                        const float yc = mode == SR_MODE_PIXEL ? (float)y + 0.5f : (float)(d[4 * k] >> 16) + 1.0f;
                        for (int32_t xx = xa; xx < xb; ++xx) {
                            const uint32_t gc = paint_color(P, (float)xx + 0.5f, yc);
                            if (mode == SR_MODE_PIXEL) row[xx] = blend(row[xx], gc);
                            else row[xx] = gc;
                        }
                        continue;
                    }
                    if (mode == SR_MODE_PIXEL) {
                        for (int32_t xx = xa; xx < xb; ++xx) row[xx] = blend(row[xx], c);
                    } else {
                        for (int32_t xx = xa; xx < xb; ++xx) row[xx] = c;
                    }
                }
            }
        });
    }

    void run() {
        using clk = std::chrono::steady_clock;
        auto t = clk::now();
        auto lap = [&](int k) {
            auto n = clk::now();
            ms[k] = std::chrono::duration<double, std::milli>(n - t).count();
            t = n;
        };
        transform();
        count_pass();
        lap(0);
        intersect_pass();
        if (error) return;
        fragment_pass();
        lap(1);
        sort_pass();
        lap(2);
        winding_mark_pass();
        lap(3);
        emit_pass();
        lap(4);
        resolve_pass();
        lap(5);
    }
};

}  // namespace orc

// ------------------------------------------------------------------ C API --
struct or_frame {
    orc::Frame<float> f;
    orc::Frame<double> d;
    bool is_double = false;
};

struct or_scene {
    srsynth::Scene s;
};

extern "C" {

// mode: SR_MODE_*; fp64: run the double-precision restatement instead.
int or_render_paints(const sr_scene_view* scene, uint32_t w, uint32_t h, const float* mvp, int mode, int threads,
                     int fp64, const sr_paint* paints, uint32_t n_paints, or_frame** out) {
    if (!scene || !mvp || !out || w == 0 || h == 0 || w > 32000 || h > 32000) return 1;
    or_frame* fr = new or_frame();
    fr->is_double = fp64 != 0;
    auto setup = [&](auto& F) {
        for (uint32_t i = 0; i < n_paints; ++i) F.paints.push_back(orc::make_paint(paints[i], mvp));
        F.s = scene;
        F.W = (int32_t)w;
        F.H = (int32_t)h;
        F.F = mode == SR_MODE_PIXEL ? 1 : 2;
        F.mode = mode;
        F.threads = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
        std::memcpy(F.m, mvp, 16 * sizeof(float));
        F.run();
        return F.error;
    };
    int err = fr->is_double ? setup(fr->d) : setup(fr->f);
    *out = fr;
    return err ? 2 : 0;
}

int or_render(const sr_scene_view* scene, uint32_t w, uint32_t h, const float* mvp, int mode, int threads,
              int fp64, or_frame** out) {
    return or_render_paints(scene, w, h, mvp, mode, threads, fp64, nullptr, 0, out);
}

int or_get(const or_frame* fr, int stage, const void** ptr, size_t* bytes) {
    if (!fr || fr->is_double) {
        if (fr && fr->is_double && stage == SR_STAGE_IMAGE) {
            *ptr = fr->d.image.data();
            *bytes = fr->d.image.size() * 4;
            return 0;
        }
        return 1;
    }
    const auto& F = fr->f;
    auto set = [&](const void* p, size_t b) {
        *ptr = p;
        *bytes = b;
        return 0;
    };
    switch (stage) {
        case SR_STAGE_TRANSFORMED_POS: return set(F.tpos.data(), F.tpos.size() * 4);
        case SR_STAGE_PATH_VISIBLE: return set(F.path_visible.data(), F.path_visible.size() * 4);
        case SR_STAGE_CUTPOINTS: return set(F.cut_dump.data(), F.cut_dump.size() * 4);
        case SR_STAGE_CURVE_COUNT: return set(F.count.data(), F.count.size() * 4);
        case SR_STAGE_CURVE_OFFSET: return set(F.offs.data(), F.offs.size() * 4);
        case SR_STAGE_INTERSECTION: return set(F.inter_dump.data(), F.inter_dump.size() * 4);
        case SR_STAGE_FRAG_KEY: return set(F.fkey.data(), F.fkey.size() * 4);
        case SR_STAGE_FRAG_WINDING: return set(F.fwn.data(), F.fwn.size() * 4);
        case SR_STAGE_SORTED_KEY: return set(F.skey.data(), F.skey.size() * 4);
        case SR_STAGE_SORTED_INDEX: return set(F.sval.data(), F.sval.size() * 4);
        case SR_STAGE_WINDING_SCAN: return set(F.wscan.data(), F.wscan.size() * 4);
        case SR_STAGE_FRAG_FLAG: return set(F.fflag.data(), F.fflag.size() * 4);
        case SR_STAGE_SPAN_FLAG: return set(F.sflag.data(), F.sflag.size() * 4);
        case SR_STAGE_DRAW_LIST: return set(F.draw.data(), F.draw.size() * 4);
        case SR_STAGE_IMAGE: return set(F.image.data(), F.image.size() * 4);
        case SR_STAGE_FRAG_LEFT: return set(F.fleft.data(), F.fleft.size() * 4);
        case orc::kStagePathDraws: return set(F.path_draws.data(), F.path_draws.size() * 4);
        default: return 1;
    }
}

// counters: N, O, merged fragments, spans; stage times (ms) in ms_out[6]:
// transform+count, intersect+fragment, sort, winding+mark, emit, resolve.
int or_stats(const or_frame* fr, int64_t* counts4, double* ms_out6) {
    if (!fr) return 1;
    auto put = [&](const auto& F) {
        if (counts4) {
            counts4[0] = F.N;
            counts4[1] = F.O;
            counts4[2] = F.n_frag;
            counts4[3] = F.n_span;
        }
        if (ms_out6)
            for (int i = 0; i < 6; ++i) ms_out6[i] = F.ms[i];
    };
    if (fr->is_double) put(fr->d);
    else put(fr->f);
    return 0;
}

void or_free(or_frame* fr) { delete fr; }

// Paint a draw list (int32x4 records) the way the given mode does.
int or_resolve(const int32_t* draw, int64_t n_records, uint32_t w, uint32_t h, int mode, int threads,
               uint8_t* rgba_out) {
    std::vector<uint32_t> img;
    orc::Frame<float>::resolve(draw, n_records, (int32_t)w, (int32_t)h, mode == SR_MODE_PIXEL ? 1 : 2, mode,
                               threads > 0 ? threads : 1, img);
    std::memcpy(rgba_out, img.data(), img.size() * 4);
    return 0;
}

uint32_t or_blend(uint32_t dst, uint32_t src) { return orc::Frame<float>::blend(dst, src); }

int or_synth(const sr_synth_params* p, or_scene** out) {
    if (!p || !out) return 1;
    srsynth::Params q;
    q.preset = p->preset;
    q.seed = p->seed;
    q.scene_index = p->scene_index;
    q.width = p->width;
    q.height = p->height;
    q.n_paths = p->n_paths;
    or_scene* sc = new or_scene();
    srsynth::generate(q, sc->s);
    *out = sc;
    return 0;
}

int or_scene_view(const or_scene* sc, sr_scene_view* v, uint32_t* wh) {
    if (!sc || !v) return 1;
    const auto& s = sc->s;
    v->n_points = s.n_points();
    v->n_curves = s.n_curves();
    v->n_paths = s.n_paths();
    v->position = s.pos.data();
    v->pos_path_idx = s.pos_path.data();
    v->curve_pos_map = s.curve_pos.data();
    v->curve_type = s.curve_type.data();
    v->curve_path_idx = s.curve_path.data();
    v->fill_rule = s.fill_rule.data();
    v->fill_info = s.fill_info.data();
    if (wh) {
        wh[0] = s.width;
        wh[1] = s.height;
    }
    return 0;
}

void or_scene_free(or_scene* sc) { delete sc; }

int or_hw_threads(void) { return (int)std::thread::hardware_concurrency(); }

}  // extern "C"
