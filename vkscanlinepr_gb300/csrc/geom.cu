// geom.cu — transform, count pass and fused intersect+fragment kernels.
//
// transform_pos.comp          -> k_transform
// make_intersection_0.comp    -> k_count
// make_intersection_1.comp +
// gen_fragment.comp           -> k_intersect_fragment (one pass: each
//                                intersection record's fragment is built as
//                                soon as the next record's t is known)
#include "common.cuh"
#include "kernels.h"

namespace sr {

// ---------------------------------------------------------------- K1 ----
// transform_pos.comp:33-86.  One thread per point; the region-code OR into
// path_visible is aggregated over runs of equal path within a warp (points
// are grouped by path) before one atomicOr per run.
__global__ void __launch_bounds__(256) k_transform(const float2* __restrict__ pos,
                                                   const uint32_t* __restrict__ pos_path, uint32_t n_points,
                                                   const SceneTable t, float2* __restrict__ tpos,
                                                   int32_t* __restrict__ path_visible) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t lane = lane_id();
    uint32_t pidx = 0xFFFFFFFFu;
    int32_t v = 0;
    if (i < n_points) {
        float2 p = pos[i];
        pidx = pos_path[i];
        const SceneInfo& si = scene_of_path(t, pidx);
        const float fw = (float)si.W, fh = (float)si.H;
        float o[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            // dot((x, y, 0, 1), m_r) summed left to right
            float acc = __fmul_rn(p.x, si.mvp[4 * r + 0]);
            acc = __fadd_rn(acc, __fmul_rn(p.y, si.mvp[4 * r + 1]));
            acc = __fadd_rn(acc, __fmul_rn(0.0f, si.mvp[4 * r + 2]));
            acc = __fadd_rn(acc, __fmul_rn(1.0f, si.mvp[4 * r + 3]));
            o[r] = acc;
        }
        float ox = __fdiv_rn(o[0], o[3]);
        float oy = __fdiv_rn(o[1], o[3]);
        tpos[i] = make_float2(ox, oy);
        int xf = ox < 0.0f ? 0 : (ox < fw ? 1 : 2);
        int yf = oy < 0.0f ? 0 : (oy < fh ? 1 : 2);
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
    }
    // segmented OR-scan over runs of equal pidx
#pragma unroll
    for (uint32_t d = 1; d < 32; d <<= 1) {
        int32_t tv = __shfl_up_sync(0xFFFFFFFFu, v, d);
        uint32_t tp = __shfl_up_sync(0xFFFFFFFFu, pidx, d);
        if (lane >= d && tp == pidx) v |= tv;
    }
    uint32_t next = __shfl_down_sync(0xFFFFFFFFu, pidx, 1);
    bool run_end = (lane == 31) || (next != pidx);
    if (i < n_points && run_end && v != 0) atomicOr(&path_visible[pidx], v);
}

// Arcs, after k_transform (which took every slot for a point): the control
// slot (w*x, w*y) transforms linearly as (w*x, w*y, 0, w), the same dot
// products in the same order, with no division; the weight slot becomes the
// fourth row's result.  An arc with w <= 0 can leave the hull of its slots,
// so the region codes cannot cull it: its path is marked visible outright.
__global__ void __launch_bounds__(256) k_arc_fixup(const uint32_t* __restrict__ curve_type,
                                                   const uint32_t* __restrict__ curve_pos,
                                                   const uint32_t* __restrict__ curve_path, uint32_t n_curves,
                                                   const float2* __restrict__ pos, const SceneTable t,
                                                   float2* __restrict__ tpos, int32_t* __restrict__ path_visible) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_curves || curve_type[c] != kArc) return;
    const uint32_t first = curve_pos[c], path = curve_path[c];
    const SceneInfo& si = scene_of_path(t, path);
    const float2 h = pos[first + 1];
    const float w = pos[first + 3].x;
    float o[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        float acc = __fmul_rn(h.x, si.mvp[4 * r + 0]);
        acc = __fadd_rn(acc, __fmul_rn(h.y, si.mvp[4 * r + 1]));
        acc = __fadd_rn(acc, __fmul_rn(0.0f, si.mvp[4 * r + 2]));
        acc = __fadd_rn(acc, __fmul_rn(w, si.mvp[4 * r + 3]));
        o[r] = acc;
    }
    tpos[first + 1] = make_float2(o[0], o[1]);
    tpos[first + 3] = make_float2(o[3], o[3]);
    atomicOr(&path_visible[path], 0x11111111);
}

// ------------------------------------------------- shared curve helpers --
struct CurvePts {
    float x[4], y[4];
};

SR_DEV void load_curve(const float2* __restrict__ tpos, uint32_t first, uint32_t type, CurvePts& c) {
    uint32_t np = curve_slots(type);
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k) {
        float2 p = make_float2(0.0f, 0.0f);
        if (k < np) p = tpos[first + k];
        c.x[k] = p.x;
        c.y[k] = p.y;
    }
}

// solveQuadEquation (make_intersection_0.comp:76-129)
SR_DEV void solve_quad(float a, float b, float c, float& r0, float& r1) {
    if (a == 0.0f) {
        float x = __fdiv_rn(-c, b);
        r0 = x;
        r1 = x;
        return;
    }
    float A = a, B = __fmul_rn(b, 0.5f), C = c;
    float R = __fsub_rn(__fmul_rn(B, B), __fmul_rn(A, C));
    if (R > 0.0f) {
        float SR = __fsqrt_rn(R);
        if (B > 0.0f) {
            float TB = __fadd_rn(B, SR);
            r0 = __fdiv_rn(-C, TB);
            r1 = __fdiv_rn(-TB, A);
        } else {
            float TB = __fadd_rn(-B, SR);
            r0 = __fdiv_rn(TB, A);
            r1 = __fdiv_rn(C, TB);
        }
    } else {
        r0 = 0.0f;
        r1 = 0.0f;
    }
}

// udpate_cut_range for one axis (make_intersection_0.comp:186-221)
SR_DEV int32_t cut_range(int32_t size, int32_t F, int32_t& b, int32_t& e) {
    int32_t mn = 0, mx = wadd(size & (int32_t)0xFFFFFFFE, F);
    if ((b < mn && e < mn) || (b > mx && e > mx) || (b > e)) return 0;
    b = iclamp(b, mn, mx);
    e = iclamp(e, mn, mx);
    return imax((e - b) / F + 1, 0);
}


// Pieces of a curve: at most 4 monotonic cuts + the end at t = 1.
constexpr int kMaxPieces = 5;
// Pieces with at least this many records are merged by a whole CTA.
constexpr int32_t kLongPiece = 64;

// Piece record layout in the output: [t0][x crossings][y crossings], the
// crossing values of each side solved by one chain (k_chains), then merged
// in t order (k_merge).  PieceInfo packs what the chains and the merge need.
SR_DEV uint32_t pack_n(int32_t nx, bool xneg, int32_t ny, bool yneg) {
    return (uint32_t)nx | (xneg ? 0x8000u : 0u) | ((uint32_t)ny << 16) | (yneg ? 0x80000000u : 0u);
}
SR_DEV int32_t piece_nx(uint32_t n) { return (int32_t)(n & 0x7FFFu); }
SR_DEV int32_t piece_ny(uint32_t n) { return (int32_t)((n >> 16) & 0x7FFFu); }

// Sort key of a chain: longest length class first (so the longest dependency
// chains start in the first wave of k_chains), then cubic, quadric, line, so
// that a warp runs one curve type with lengths within a factor of 2.  A line
// root is a closed form, far cheaper than a 24-step bisection, so a line
// chain is classed 7 length classes lower (at most class 7, below every
// wide chain).
SR_DEV uint32_t chain_key(int32_t len, uint32_t type) {
    uint32_t lg = 31u - (uint32_t)__clz(len);
    if (lg > 14u) lg = 14u;
    if (type == 2u) lg = lg > 7u ? lg - 7u : 0u;
    uint32_t cls = type == 4u ? 0u : (type == 3u ? 1u : (type == kArc ? 3u : 2u));
    return ((14u - lg) << 2) | cls;
}
// Cubic, quadric and arc chains of >= 512 bisected roots (class >= 9) are solved
// by a whole warp each (run_chain_warp); they sort before every other chain.
SR_DEV bool chain_key_wide(uint32_t key) { return (key >> 2) <= 14u - 9u && (key & 3u) != 2u; }
constexpr uint32_t kChainKeyBits = 6;

// get_xy_begin_end_delta + udpate_cut_range for one axis
// (make_intersection_1.comp:150-213): number of grid crossings, first
// grid line and step.
SR_DEV int32_t axis_range_rd(float a0, float a1, int32_t size, int32_t F, float& start, bool& neg) {
    const float invF = inv_F(F);   // x / F == x * (1/F) exactly for F in {1, 2}
    int32_t b, e;
    if (a0 <= a1) {
        b = wadd(wmul(float2int_rd(__fmul_rn(a0, invF)), F), F);
        e = wmul(float2int_rd(__fmul_rn(a1, invF)), F);
        neg = false;
    } else {
        b = wadd(wmul(float2int_rd(__fmul_rn(a1, invF)), F), F);
        e = wmul(float2int_rd(__fmul_rn(a0, invF)), F);
        neg = true;
    }
    int32_t n = cut_range(size, F, b, e);
    start = (float)(neg ? e : b);
    return n;
}

// ---------------------------------------------------------------- K2 ----
// make_intersection_0.comp:226-411.  One thread per curve: path cull,
// monotonic cut points (cached, 5 floats per curve), the number of records
// the curve emits (the reference's count), and the set-up of each piece's
// x and y crossing chains, which are appended with their sort keys.
__global__ void __launch_bounds__(256) k_count(const GeomArgs g, float* __restrict__ cut_cache,
                                               int32_t* __restrict__ count, uint4* __restrict__ pieces,
                                               uint32_t* __restrict__ chain_items, uint32_t* __restrict__ chain_keys,
                                               uint32_t list_cap, uint32_t* __restrict__ chain_count,
                                               uint32_t* __restrict__ wide_count,
                                               uint8_t* __restrict__ curve_wide, uint32_t* __restrict__ wide_curves,
                                               uint32_t* __restrict__ wide_curve_count,
                                               uint32_t* __restrict__ long_list, uint32_t* __restrict__ long_count,
                                               uint32_t* __restrict__ status) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = c < g.n_curves;
    uint32_t my_chains[2 * kMaxPieces];
    uint32_t my_key[2 * kMaxPieces];
    int n_chains = 0;
    uint32_t long_mask = 0;   // pieces merged by k_merge_long
    if (active) {
        uint32_t type = g.curve_type[c];
        CurvePts P;
        load_curve(g.tpos, g.curve_pos[c], type, P);
        const uint32_t path = g.curve_path[c];
        bool vis = path_visible_mask(g.path_visible[path]);
        const SceneInfo& si = scene_of_path(g.st, path);
        const int32_t W = si.W, H = si.H;
        const int32_t F = g.F;
        uint32_t n = 0;
        float q[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        if (vis) {
#pragma unroll
            for (int ax = 0; ax < 2; ++ax) {
                const float* p = ax == 0 ? P.x : P.y;
                if (type == 4u) {
                    float r0 = 0.0f, r1 = 0.0f;
                    float a = __fadd_rn(__fmul_rn(3.0f, __fsub_rn(p[1], p[2])), __fsub_rn(p[3], p[0]));
                    float b = __fmul_rn(2.0f, __fadd_rn(__fsub_rn(p[0], p[1]), __fsub_rn(p[2], p[1])));
                    solve_quad(a, b, __fsub_rn(p[1], p[0]), r0, r1);
                    if (r0 > 0.0f && r0 < 1.0f) q[n++] = r0;
                    if (r1 > 0.0f && r1 < 1.0f && r1 != r0) q[n++] = r1;
                } else if (type == 3u) {
                    float den = __fadd_rn(__fsub_rn(p[0], p[1]), __fsub_rn(p[2], p[1]));
                    if (den != 0.0f) {
                        float r0 = __fdiv_rn(__fsub_rn(p[0], p[1]), den);
                        if (r0 > 0.0f && r0 < 1.0f) q[n++] = r0;
                    }
                } else if (type == kArc) {
                    // roots of the derivative's numerator N'D - ND' (a
                    // quadratic; its cubic terms cancel), halved:
                    // (w-1)(x2-x0) t^2 + ((x0-x1) + (x2-x1) + 2 x0 (w-1)) t + (x1 - w x0)
                    const float wm1 = __fsub_rn(p[3], 1.0f);
                    float r0 = 0.0f, r1 = 0.0f;
                    solve_quad(__fmul_rn(wm1, __fsub_rn(p[2], p[0])),
                               __fadd_rn(__fadd_rn(__fsub_rn(p[0], p[1]), __fsub_rn(p[2], p[1])),
                                         __fmul_rn(__fmul_rn(2.0f, p[0]), wm1)),
                               __fsub_rn(p[1], __fmul_rn(p[3], p[0])), r0, r1);
                    if (r0 > 0.0f && r0 < 1.0f) q[n++] = r0;
                    if (r1 > 0.0f && r1 < 1.0f && r1 != r0) q[n++] = r1;
                }
            }
            // insertion network of make_intersection_0.comp:315-359, including
            // its `t2 = q3` (the 4th cut is never moved)
            float q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3];
            if (n >= 2) {
                float t1 = q1, t0 = q0;
                if (t1 < t0) { q1 = t0; q0 = t1; }
            }
            if (n >= 3) {
                float t2 = q2, t1 = q1;
                if (t2 < t1) {
                    q2 = t1;
                    float t0 = q0;
                    if (t2 < t0) { q1 = t0; q0 = t2; } else { q1 = t2; }
                }
            }
            if (n >= 4) {
                float t3 = q3, t2 = q3;
                if (t3 < t2) {
                    q3 = t2;
                    float t1 = q1;
                    if (t3 < t1) {
                        q2 = t1;
                        float t0 = q0;
                        if (t3 < t0) { q1 = t0; q0 = t3; } else { q1 = t3; }
                    } else {
                        q2 = t3;
                    }
                }
            }
            q[0] = q0; q[1] = q1; q[2] = q2; q[3] = q3;
        }
        float* cc = cut_cache + 5 * (size_t)c;
        cc[0] = q[0];
        cc[1] = q[1];
        cc[2] = q[2];
        cc[3] = q[3];
        cc[4] = __uint_as_float(n);
        if (vis) q[n++] = 1.0f;
        float x0 = P.x[0], y0 = P.y[0];
        const float fF = (float)F;
        int32_t pc = 0, walk = 0;
        uint4* pt = pieces + (size_t)c * kMaxPieces;
#pragma unroll
        for (uint32_t i = 0; i < (uint32_t)kMaxPieces; ++i) {
            if (i >= n) break;
            float t1 = q[i];
            float x1 = interp(type, t1, P.x), y1 = interp(type, t1, P.y);
            // count: get_xy_begin_end (make_intersection_0.comp:167-183)
            int32_t xb, xe, yb, ye;
            if (x0 <= x1) {
                xb = wadd(f2i(__fmul_rn(floorf(__fdiv_rn(x0, fF)), fF)), F);
                xe = f2i(__fmul_rn(floorf(__fdiv_rn(x1, fF)), fF));
            } else {
                xb = wadd(f2i(__fmul_rn(floorf(__fdiv_rn(x1, fF)), fF)), F);
                xe = f2i(__fmul_rn(floorf(__fdiv_rn(x0, fF)), fF));
            }
            if (y0 <= y1) {
                yb = wadd(f2i(__fmul_rn(floorf(__fdiv_rn(y0, fF)), fF)), F);
                ye = f2i(__fmul_rn(floorf(__fdiv_rn(y1, fF)), fF));
            } else {
                yb = wadd(f2i(__fmul_rn(floorf(__fdiv_rn(y1, fF)), fF)), F);
                ye = f2i(__fmul_rn(floorf(__fdiv_rn(y0, fF)), fF));
            }
            int32_t nxc = cut_range(W, F, xb, xe);
            int32_t nyc = cut_range(H, F, yb, ye);
            pc = wadd(pc, wadd(1, wadd(nxc, nyc)));
            // chain set-up: the intersection pass's own range formulas
            float sx, sy;
            bool xneg, yneg;
            int32_t nx = axis_range_rd(x0, x1, W, F, sx, xneg);
            int32_t ny = axis_range_rd(y0, y1, H, F, sy, yneg);
            int32_t tb = fbits(t1) & ~3;
            tb |= (floorf(x1) == x1) ? 2 : 3;   // make_intersection_1.comp:271-276
            pt[i] = make_uint4(pack_n(nx, xneg, ny, yneg), (uint32_t)tb, __float_as_uint(sx), __float_as_uint(sy));
            if (nx > 0) {
                my_chains[n_chains] = (c << 4) | (i << 1) | 0u;
                my_key[n_chains++] = chain_key(nx, type);
            }
            if (ny > 0) {
                my_chains[n_chains] = (c << 4) | (i << 1) | 1u;
                my_key[n_chains++] = chain_key(ny, type);
            }
            walk += 1 + nx + ny;
            if (1 + nx + ny >= kLongPiece) long_mask |= 1u << i;
            x0 = x1;
            y0 = y1;
        }
        count[c] = pc;
        if (walk != pc) set_error(status, ERR_RECORD_RANGE);
        bool wide = false;
        for (int k = 0; k < n_chains; ++k) wide |= chain_key_wide(my_key[k]);
        curve_wide[c] = wide ? 1 : 0;
        if (wide) wide_curves[atomicAdd(wide_curve_count, 1u)] = c;
    }
    // append long pieces (warp-aggregated)
    const uint32_t lane = lane_id();
    for (int i = 0; i < kMaxPieces; ++i) {
        bool has = (long_mask >> i) & 1u;
        uint32_t m = __ballot_sync(0xFFFFFFFFu, has);
        if (!m) continue;
        uint32_t leader = (uint32_t)(__ffs(m) - 1);
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(long_count, (uint32_t)__popc(m));
        base = __shfl_sync(0xFFFFFFFFu, base, leader);
        if (has) {
            uint32_t slot = base + (uint32_t)__popc(m & lanemask_lt());
            if (slot < list_cap) long_list[slot] = (c << 3) | (uint32_t)i;
            else set_error(status, ERR_CAPACITY);
        }
    }
    // append the chains with their sort keys (warp-aggregated)
    for (int k = 0; k < 2 * kMaxPieces; ++k) {
        bool has = k < n_chains;
        uint32_t m = __ballot_sync(0xFFFFFFFFu, has);
        if (!m) break;
        uint32_t leader = (uint32_t)(__ffs(m) - 1);
        uint32_t base = 0;
        const uint32_t wm = __ballot_sync(0xFFFFFFFFu, has && chain_key_wide(my_key[k]));
        if (lane == leader) {
            base = atomicAdd(chain_count, (uint32_t)__popc(m));
            if (wm) atomicAdd(wide_count, (uint32_t)__popc(wm));
        }
        base = __shfl_sync(0xFFFFFFFFu, base, leader);
        if (has) {
            uint32_t slot = base + (uint32_t)__popc(m & lanemask_lt());
            if (slot < list_cap) {
                chain_items[slot] = my_chains[k];
                chain_keys[slot] = my_key[k];
            } else {
                set_error(status, ERR_CAPACITY);
            }
        }
    }
}

// ------------------------------------------------------------ chains -----
// One crossing chain: the successive roots of one coordinate of one piece
// at the grid lines start, start+d, ... (make_intersection_1.comp:377-440).
// Each solve starts from the previous root of the same side (flag bits
// included), so a chain is sequential but chains are independent.
struct AxisPoly {
    float p0, p1, p2, p3;
    float d01, d12, d23;
};

template <int kType> SR_DEV float eval_axis(const AxisPoly& a, float t) {
    if (kType == 2) return __fadd_rn(a.p0, __fmul_rn(t, a.d01));
    if (kType == (int)kArc) {
        // as interp(): the homogeneous lerps, then the division (p3 = w)
        float q0 = __fadd_rn(a.p0, __fmul_rn(t, a.d01));
        float q1 = __fadd_rn(a.p1, __fmul_rn(t, a.d12));
        float r0 = __fadd_rn(1.0f, __fmul_rn(t, __fsub_rn(a.p3, 1.0f)));
        float r1 = __fadd_rn(a.p3, __fmul_rn(t, __fsub_rn(1.0f, a.p3)));
        return __fdiv_rn(__fadd_rn(q0, __fmul_rn(t, __fsub_rn(q1, q0))),
                         __fadd_rn(r0, __fmul_rn(t, __fsub_rn(r1, r0))));
    }
    float q0 = __fadd_rn(a.p0, __fmul_rn(t, a.d01));
    float q1 = __fadd_rn(a.p1, __fmul_rn(t, a.d12));
    if (kType == 3) return __fadd_rn(q0, __fmul_rn(t, __fsub_rn(q1, q0)));
    float q2 = __fadd_rn(a.p2, __fmul_rn(t, a.d23));
    float l0 = __fadd_rn(q0, __fmul_rn(t, __fsub_rn(q1, q0)));
    float l1 = __fadd_rn(q1, __fmul_rn(t, __fsub_rn(q2, q1)));
    return __fadd_rn(l0, __fmul_rn(t, __fsub_rn(l1, l0)));
}

SR_DEV float mid_rn(float lo, float hi) { return __fmul_rn(__fadd_rn(lo, hi), 0.5f); }

// The step test of make_intersection_1.comp:421 is
// (bits(v - c) ^ bits(v_lo - c)) >= 0, v_lo the value at the interval's low
// end; for finite values v - c is negative exactly when v < c (x - x is +0).
// The low end moves only to a midpoint that passes the test, i.e. one on the
// same side of c, so the side s0 = (value at t_min < c) holds for the whole
// solve: a step goes right exactly when (v < c) == s0, whatever the other
// steps did.  Both solvers below rest on that.

// 24-step bisection of the reference (make_intersection_1.comp:402-434), a
// thread per chain.  (Evaluating both possible next midpoints with each one
// halves the dependent depth, but the chains left to this solver are
// throughput-bound, and the extra evaluations made the frame slower.)
template <int kType>
SR_DEV float bisect(const AxisPoly& a, float c, float t_min, float t_max) {
    const float v0 = eval_axis<kType>(a, t_min);
    const bool s0 = v0 < c;
    float ta = t_min, tb = t_max;
    float t_solve = t_min, last = 0.0f;
#pragma unroll 4
    for (int j = 0; j < 24; ++j) {
        const float tm = mid_rn(ta, tb);
        const float v = eval_axis<kType>(a, tm);
        t_solve = tm;
        last = v;
        if ((v < c) == s0) ta = tm;
        else tb = tm;
    }
    // vt0 == c returns t_min at once; a solve that ends more than one unit
    // away from c falls back to t_min too
    if (v0 == c || fabsf(__fsub_rn(last, c)) > 1.0f) t_solve = t_min;
    return t_solve;
}

template <int kType>
SR_DEV void run_chain(const AxisPoly& a, int32_t len, float x, float dx, float t_lo, float t_hi, int side,
                      int32_t* __restrict__ out) {
    float lo = t_lo;
    float inv = 0.0f;
    if (kType == 2) {
        float d = __fsub_rn(a.p1, a.p0);
        inv = (d != 0.0f) ? __fdiv_rn(1.0f, d) : 0.0f;
    }
    for (int32_t k = 0; k < len; ++k) {
        float c = x;
        x = __fadd_rn(x, dx);
        float t;
        if (kType == 2) t = gmin(gmax(__fmul_rn(__fsub_rn(c, a.p0), inv), lo), t_hi);
        else t = bisect<kType>(a, c, lo, t_hi);
        int32_t ob = (fbits(t) & ~3) | side;
        out[k] = ob;
        lo = bitsf(ob);
    }
}

// Warp-cooperative solve of one long chain.  By the invariant above, the 31
// midpoints of the next five bisection steps can be evaluated at once: lane
// l holds node l+1 of the complete binary tree of those steps in heap order
// (node n's children are 2n and 2n+1, the right child taken when the step
// goes right), and one ballot of the (v < c) bits gives every node's turn.
// The leaf whose ancestors all turn toward it is on the path; it hands the
// new interval to the warp through a max-reduction over the lanes (every
// other lane offers 0; t >= 0, so the bit patterns order like the values).  Lane 31 evaluates the root's t_min in the first
// round, which gives s0 in the same ballot.  24 steps = four 5-level rounds
// and a last 4-level round, whose leaf midpoint is the 24th midpoint.
struct TreeLane {
    int32_t depth;            // node depth (lane 31: -1)
    bool d1, d2, d3, d4;      // turn at level j toward this lane's node (right = true)
    uint32_t anc5, want5, anc4, want4;   // path masks of the leaves of a 5- and a 4-level round
};

SR_DEV TreeLane tree_lane(uint32_t lane) {
    TreeLane tl;
    const uint32_t n = lane + 1u;
    const int32_t d = lane == 31u ? -1 : 31 - __clz((int32_t)n);
    tl.depth = d;
    tl.d1 = d >= 1 && ((n >> (d - 1)) & 1u);
    tl.d2 = d >= 2 && ((n >> (d - 2)) & 1u);
    tl.d3 = d >= 3 && ((n >> (d - 3)) & 1u);
    tl.d4 = d >= 4 && (n & 1u);
    tl.anc5 = tl.want5 = tl.anc4 = tl.want4 = 0;
    for (int32_t i = 0; i < d; ++i) {   // ancestor at depth i and the turn it takes toward n
        const uint32_t anc = n >> (d - i), dir = (n >> (d - i - 1)) & 1u;
        const uint32_t bit = 1u << (anc - 1u);
        if (d == 4) { tl.anc5 |= bit; tl.want5 |= dir ? bit : 0u; }
        if (d == 3) { tl.anc4 |= bit; tl.want4 |= dir ? bit : 0u; }
    }
    return tl;
}

// This lane's node of a kLevels-level tree from [ta, tb]: its midpoint,
// and its interval in lb/rb.  m_j = (m_{j-1} + the interval's other end) *
// 0.5, the other end being older than m_{j-1}, so a level costs one add and
// one multiply on the dependency path.
template <int kLevels>
SR_DEV float tree_node(float ta, float tb, const TreeLane& tl, float& lb, float& rb) {
    lb = ta;
    rb = tb;
    float m = mid_rn(ta, tb);
#pragma unroll
    for (int j = 1; j < kLevels; ++j) {
        if (j <= tl.depth) {
            const bool dir = j == 1 ? tl.d1 : (j == 2 ? tl.d2 : (j == 3 ? tl.d3 : tl.d4));
            const float other = dir ? rb : lb;
            if (dir) lb = m;
            else rb = m;
            m = __fmul_rn(__fadd_rn(m, other), 0.5f);
        }
    }
    return m;
}

template <int kType>
SR_DEV float bisect_warp(const AxisPoly& a, float c, float t_min, float t_max, const TreeLane& tl) {
    float lb, rb;
    // first round; lane 31's interval is [t_min, t_min], whose midpoint is
    // t_min itself (2t and 2t * 0.5 are exact), so its bit of the ballot is s0
    float m = tree_node<5>(t_min, tl.depth < 0 ? t_min : t_max, tl, lb, rb);
    float v = eval_axis<kType>(a, m);
    uint32_t B = __ballot_sync(0xFFFFFFFFu, v < c);
    const bool s0 = (B >> 31) & 1u;
    const bool eq0 = (__ballot_sync(0xFFFFFFFFu, v == c) >> 31) != 0u;
    // node l+1 goes right when bit l of B equals s0: the leaf on the path is
    // the one with ((B ^ key) & anc) == 0, key = want ^ (s0 ? 0 : ~0)
    const uint32_t flip = s0 ? 0u : 0xFFFFFFFFu;
    const uint32_t key5 = tl.want5 ^ flip, key4 = tl.want4 ^ flip;
    float ta, tb;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        if (r > 0) {
            m = tree_node<5>(ta, tb, tl, lb, rb);
            v = eval_axis<kType>(a, m);
            B = __ballot_sync(0xFFFFFFFFu, v < c);
        }
        const bool on = tl.depth == 4 && ((B ^ key5) & tl.anc5) == 0u;
        const bool right = (v < c) == s0;
        const uint32_t nta = on ? __float_as_uint(right ? m : lb) : 0u;
        const uint32_t ntb = on ? __float_as_uint(right ? rb : m) : 0u;
        ta = __uint_as_float(__reduce_max_sync(0xFFFFFFFFu, nta));
        tb = __uint_as_float(__reduce_max_sync(0xFFFFFFFFu, ntb));
    }
    // steps 21-24: the chosen depth-3 node's midpoint is the 24th midpoint
    m = tree_node<4>(ta, tb, tl, lb, rb);
    v = eval_axis<kType>(a, m);
    B = __ballot_sync(0xFFFFFFFFu, v < c);
    const bool on = tl.depth == 3 && ((B ^ key4) & tl.anc4) == 0u;
    const float fin = fabsf(__fsub_rn(v, c)) > 1.0f ? t_min : m;
    const float t = __uint_as_float(__reduce_max_sync(0xFFFFFFFFu, on ? __float_as_uint(fin) : 0u));
    return eq0 ? t_min : t;
}

// A chain solved by the whole warp; lane k%32 keeps root k until 32 roots
// are stored at once.
template <int kType>
SR_DEV void run_chain_warp(const AxisPoly& a, int32_t len, float x, float dx, float t_lo, float t_hi, int side,
                           int32_t* __restrict__ out, const TreeLane& tl) {
    const uint32_t lane = lane_id();
    float lo = t_lo;
    int32_t keep = 0;
    for (int32_t k = 0; k < len; ++k) {
        const float c = x;
        x = __fadd_rn(x, dx);
        const float t = bisect_warp<kType>(a, c, lo, t_hi, tl);
        const int32_t ob = (fbits(t) & ~3) | side;
        if ((uint32_t)(k & 31) == lane) keep = ob;
        if ((k & 31) == 31 || k + 1 == len) {
            const int32_t k0 = k & ~31;
            if ((int32_t)lane <= (k - k0)) out[k0 + (int32_t)lane] = keep;
        }
        lo = bitsf(ob);
    }
}

struct ChainSetup {
    AxisPoly a;
    uint32_t type;
    int32_t len;
    float x, dx, t_lo, t_hi;
    int side;
    int64_t base;
};

// Chain item (curve << 4 | piece << 1 | side): its polynomial, first grid
// line and step, t range and output slot.
SR_DEV ChainSetup chain_setup(const GeomArgs& g, const int32_t* __restrict__ offs, const uint4* __restrict__ pieces,
                              uint32_t item) {
    ChainSetup s;
    const uint32_t c = item >> 4, piece = (item >> 1) & 7u;
    s.side = (int)(item & 1u);
    s.type = g.curve_type[c];
    const uint4* pt = pieces + (size_t)c * kMaxPieces;
    int64_t base = offs[c];
    for (uint32_t j = 0; j < piece; ++j) base += 1 + piece_nx(pt[j].x) + piece_ny(pt[j].x);
    const uint4 me = pt[piece];
    const int32_t nx = piece_nx(me.x), ny = piece_ny(me.x);
    s.base = base + 1 + (s.side ? nx : 0);
    s.len = s.side ? ny : nx;
    const bool neg = s.side ? (me.x & 0x80000000u) != 0 : (me.x & 0x8000u) != 0;
    s.x = __uint_as_float(s.side ? me.w : me.z);
    s.dx = neg ? -(float)g.F : (float)g.F;
    s.t_lo = piece == 0 ? 0.0f : __uint_as_float(pt[piece - 1].y);
    s.t_hi = __uint_as_float(me.y);
    const float2* cp = g.tpos + g.curve_pos[c];
    const uint32_t np = curve_slots(s.type);
    float p[4];
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k) {
        float2 v = k < np ? cp[k] : make_float2(0.0f, 0.0f);
        p[k] = s.side ? v.y : v.x;
    }
    s.a.p0 = p[0]; s.a.p1 = p[1]; s.a.p2 = p[2]; s.a.p3 = p[3];
    s.a.d01 = __fsub_rn(p[1], p[0]);
    s.a.d12 = __fsub_rn(p[2], p[1]);
    s.a.d23 = __fsub_rn(p[3], p[2]);
    return s;
}

// Part 0 solves the wide chains (first in the list), one per warp; part 1
// the others in groups of 32 in list order, so the longest groups go to the
// first warp of every SM rather than to one block.  The two parts run on two
// streams at once.
__global__ void __launch_bounds__(128) k_chains(const GeomArgs g, const int32_t* __restrict__ offs,
                                                const uint4* __restrict__ pieces,
                                                const uint32_t* __restrict__ items, const uint32_t* __restrict__ keys,
                                                uint32_t list_cap, const uint32_t* __restrict__ chain_count,
                                                const uint32_t* __restrict__ wide_count,
                                                uint32_t* __restrict__ queue, int32_t* __restrict__ cbuf, int part) {
    const uint32_t total = imin((int32_t)*chain_count, (int32_t)list_cap);
    const uint32_t n_wide = imin((int32_t)*wide_count, (int32_t)total);
    const uint32_t lane = lane_id();
    if (part == 0) {
        const TreeLane tl = tree_lane(lane);
        for (;;) {
            uint32_t ticket = 0;
            if (lane == 0) ticket = atomicAdd(queue, 1u);
            ticket = __shfl_sync(0xFFFFFFFFu, ticket, 0);
            if (ticket >= n_wide) break;
            const ChainSetup s = chain_setup(g, offs, pieces, items[ticket]);
            if (s.base + s.len > g.rec_cap) continue;   // overflow: k_merge reports it
            int32_t* out = cbuf + s.base;
            if (s.type == 4u) run_chain_warp<4>(s.a, s.len, s.x, s.dx, s.t_lo, s.t_hi, s.side, out, tl);
            else if (s.type == 3u) run_chain_warp<3>(s.a, s.len, s.x, s.dx, s.t_lo, s.t_hi, s.side, out, tl);
            else if (s.type == kArc)
                run_chain_warp<(int)kArc>(s.a, s.len, s.x, s.dx, s.t_lo, s.t_hi, s.side, out, tl);
        }
        return;
    }
    for (;;) {
        uint32_t ticket = 0;
        if (lane == 0) ticket = atomicAdd(queue, 1u);
        ticket = __shfl_sync(0xFFFFFFFFu, ticket, 0);
        const uint32_t first = n_wide + ticket * 32u;
        if (first >= total) break;
        const uint32_t it = first + lane;
        if (it >= total) continue;
        const ChainSetup s = chain_setup(g, offs, pieces, items[it]);
        if (s.base + s.len > g.rec_cap) continue;   // overflow: k_merge reports it
        int32_t* out = cbuf + s.base;
        if (s.type == 2u) run_chain<2>(s.a, s.len, s.x, s.dx, s.t_lo, s.t_hi, s.side, out);
        else if (s.type == 3u) run_chain<3>(s.a, s.len, s.x, s.dx, s.t_lo, s.t_hi, s.side, out);
        else if (s.type == kArc) run_chain<(int)kArc>(s.a, s.len, s.x, s.dx, s.t_lo, s.t_hi, s.side, out);
        else run_chain<4>(s.a, s.len, s.x, s.dx, s.t_lo, s.t_hi, s.side, out);
    }
}

// ------------------------------------------------------------- merge -----
// The record order of make_intersection_1.comp:310-441: per piece, the
// start t0 and the two chains merged by `next_tx <= next_ty`, an exhausted
// side counting as 2.0 (with its side bit); a record whose t (flag bits
// masked) equals the previous one ORs the flags into both
// (make_intersection_1.comp:361-375).
// Records of a wide curve hold this until its merge, which runs on the other
// stream, writes them; the record-parallel fragment pass skips them.
constexpr int32_t kPendingCurve = -1;

// Piece j of curve c, a thread each (pieces are merged independently: each
// starts from its own t0 and flag state).  The piece-0 thread also checks
// that the pieces cover the curve's records exactly.
SR_DEV void merge_piece(const GeomArgs& g, const int32_t* __restrict__ offs, const uint4* __restrict__ pieces,
                        const int32_t* __restrict__ cbuf, int2* __restrict__ rec, uint32_t* __restrict__ status,
                        uint32_t c, int j, bool pending_only) {
    const int64_t start = offs[c], end = offs[c + 1];
    if (start >= end) return;
    if (end > g.rec_cap) {
        if (j == 0) set_error(status, ERR_CAPACITY);
        return;
    }
    const uint4* pt = pieces + (size_t)c * kMaxPieces;
    if (j == 0) {
        int64_t tot = start;
        for (int i = 0; i < kMaxPieces && tot < end; ++i) tot += 1 + piece_nx(pt[i].x) + piece_ny(pt[i].x);
        if (tot != end) set_error(status, ERR_RECORD_RANGE);
    }
    int64_t pc = start;
    for (int i = 0; i < j; ++i) pc += 1 + piece_nx(pt[i].x) + piece_ny(pt[i].x);
    if (pc >= end) return;   // the curve has fewer pieces
    const uint4 me = pt[j];
    const int32_t nx = piece_nx(me.x), ny = piece_ny(me.x);
    const int32_t n_loop = nx + ny + 1;
    if (pc + n_loop > end) return;   // reported by the piece-0 thread
    if (n_loop >= kLongPiece) return;   // k_merge_long
    if (pending_only) {
        for (int32_t k = 0; k < n_loop; ++k) rec[pc + k] = make_int2(kPendingCurve, 0);
        return;
    }
    const int32_t t0 = j == 0 ? 0 : (int32_t)pt[j - 1].y;   // bits of 0.0f for the first piece
    const int32_t minus_one = fbits(-1.0f);
    const int32_t ex_x = fbits(2.0f), ex_y = fbits(2.0f) | 1;
    const int32_t* X = cbuf + pc + 1;
    const int32_t* Y = X + nx;
    // heads: A = x side, B = y side (make_intersection_1.comp:321-359)
    int32_t ia = 0, ib = 0;
    // both sides cross: A = x chain, B = [t0, y chain]; no x crossing:
    // A empty, B = [t0, y chain]; no y crossing: A = [t0, x chain], B empty
    const bool a_has_t0 = (nx > 0 && ny == 0);
    const int32_t lenA = nx + (a_has_t0 ? 1 : 0);
    const int32_t lenB = a_has_t0 ? 0 : ny + 1;
    int32_t last = minus_one;
    for (int32_t k = 0; k < n_loop; ++k) {
        int32_t av = ex_x, bv = ex_y;
        if (ia < lenA) av = a_has_t0 ? (ia == 0 ? t0 : X[ia - 1]) : X[ia];
        if (ib < lenB) bv = ib == 0 ? t0 : Y[ib - 1];
        int32_t out;
        if (bitsf(av) <= bitsf(bv)) {
            out = av;
            ++ia;
        } else {
            out = bv;
            ++ib;
        }
        if ((out & ~3) == (last & ~3)) {
            out |= last;
            rec[pc - 1] = make_int2((int32_t)c, out);
        }
        rec[pc] = make_int2((int32_t)c, out);
        last = out;
        ++pc;
    }
}

// Part 0 merges every curve but the wide ones, whose records it marks
// pending; part 1 merges the wide curves once their chains are done.  A
// thread per (curve, piece).
__global__ void __launch_bounds__(128) k_merge(const GeomArgs g, const int32_t* __restrict__ offs,
                                               const uint4* __restrict__ pieces, const int32_t* __restrict__ cbuf,
                                               int2* __restrict__ rec, uint32_t* __restrict__ status,
                                               const uint8_t* __restrict__ curve_wide,
                                               const uint32_t* __restrict__ wide_curves,
                                               const uint32_t* __restrict__ wide_curve_count, int part) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (part == 0) {
        const uint32_t c = tid / kMaxPieces;
        if (c < g.n_curves)
            merge_piece(g, offs, pieces, cbuf, rec, status, c, (int)(tid % kMaxPieces), curve_wide[c] != 0);
        return;
    }
    const uint32_t nw = imin((int32_t)*wide_curve_count, (int32_t)g.n_curves);
    for (uint32_t k = tid; k < nw * kMaxPieces; k += gridDim.x * blockDim.x)
        merge_piece(g, offs, pieces, cbuf, rec, status, wide_curves[k / kMaxPieces], (int)(k % kMaxPieces), false);
}

// Merge of one long piece by a CTA.  The chains are non-decreasing (each
// root is solved from the previous one, flag bits included); only the
// piece start t0 may exceed the first roots by less than 4 ulp, so the
// sequential merge is: the x roots <= t0, then t0, then the stable merge
// (x first on ties) of the remaining x roots with the y roots.  Each
// element's slot is its index plus its rank in the other chain.  The
// flag-OR of equal t values is then applied per element: record k of a
// run [s, e] of equal masked t ends as OR(v_s .. v_min(k+1,e)).
SR_DEV int32_t count_le(const int32_t* a, int32_t n, float v) {   // elements <= v
    int32_t lo = 0, hi = n;
    while (lo < hi) {
        int32_t mid = (lo + hi) >> 1;
        if (bitsf(a[mid]) <= v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}
SR_DEV int32_t count_lt(const int32_t* a, int32_t n, float v) {   // elements < v
    int32_t lo = 0, hi = n;
    while (lo < hi) {
        int32_t mid = (lo + hi) >> 1;
        if (bitsf(a[mid]) < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// A long piece merged by the CTA.  When its two chains fit in shared memory
// (cap elements) they are merged there: each thread writes one stretch of
// the output, its start found by a merge-path search (x first on ties), and
// the flag-OR reads shared memory.  Larger pieces use binary-search ranks in
// global memory.  Every thread of the CTA calls it with the same piece.
SR_DEV void merge_long_piece(uint32_t c, int32_t t0, int64_t base, int32_t nx, int32_t ny,
                             int32_t* __restrict__ cbuf, int2* __restrict__ rec, int32_t* sm, int32_t cap,
                             int32_t* s_i0) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const int32_t L = 1 + nx + ny;
    const int32_t* X = cbuf + base + 1;
    const int32_t* Y = X + nx;
    int2* R = rec + base;
    if (nx + ny <= cap) {
        int32_t* sin = sm;
        int32_t* sout = sm + cap;
        for (int32_t k = tid; k < nx + ny; k += nt) sin[k] = X[k];
        __syncthreads();
        const int32_t* sx = sin;
        const int32_t* sy = sin + nx;
        if (nx == 0 || ny == 0) {
            for (int32_t k = tid; k < L; k += nt) sout[k] = k == 0 ? t0 : sin[k - 1];
        } else {
            const int32_t i0 = count_le(sx, nx, bitsf(t0));
            for (int32_t k = tid; k < i0; k += nt) sout[k] = sx[k];
            if (tid == 0) sout[i0] = t0;
            // the merge of sx[i0..nx) with sy: this thread's stretch [d, d_end)
            const int32_t* xr = sx + i0;
            const int32_t nxr = nx - i0, M = nxr + ny;
            const int32_t per = (M + nt - 1) / nt;
            const int32_t d = imin(tid * per, M), d_end = imin(d + per, M);
            int32_t lo = imax(0, d - ny), hi = imin(d, nxr);
            while (lo < hi) {
                const int32_t mid = (lo + hi) >> 1;
                if (bitsf(xr[mid]) <= bitsf(sy[d - mid - 1])) lo = mid + 1;
                else hi = mid;
            }
            int32_t ia = lo, ib = d - lo;
            int32_t* o = sout + i0 + 1;
            for (int32_t k = d; k < d_end; ++k) {
                const bool take_x = ia < nxr && (ib >= ny || bitsf(xr[ia]) <= bitsf(sy[ib]));
                o[k] = take_x ? xr[ia++] : sy[ib++];
            }
        }
        __syncthreads();
        for (int32_t k = tid; k < L; k += nt) {
            const int32_t v = sout[k];
            int32_t acc = v;
            for (int32_t s2 = k - 1; s2 >= 0; --s2) {
                const int32_t u = sout[s2];
                if ((u & ~3) != (v & ~3)) break;
                acc |= u;
            }
            if (k + 1 < L) {
                const int32_t u = sout[k + 1];
                if ((u & ~3) == (v & ~3)) acc |= u;
            }
            R[k] = make_int2((int32_t)c, acc);
        }
        __syncthreads();
        return;
    }
    if (nx == 0 || ny == 0) {
        const int32_t* S = nx == 0 ? Y : X;
        for (int32_t k = tid; k < L; k += nt) R[k] = make_int2((int32_t)c, k == 0 ? t0 : S[k - 1]);
    } else {
        if (tid == 0) *s_i0 = count_le(X, nx, bitsf(t0));
        __syncthreads();
        const int32_t i0 = *s_i0;
        for (int32_t i = tid; i < nx; i += nt) {
            int32_t v = X[i];
            int32_t pos = i < i0 ? i : i0 + 1 + (i - i0) + count_lt(Y, ny, bitsf(v));
            R[pos] = make_int2((int32_t)c, v);
        }
        if (tid == 0) R[i0] = make_int2((int32_t)c, t0);
        for (int32_t j = tid; j < ny; j += nt) {
            int32_t v = Y[j];
            int32_t pos = i0 + 1 + j + count_le(X + i0, nx - i0, bitsf(v));
            R[pos] = make_int2((int32_t)c, v);
        }
    }
    __syncthreads();
    int32_t* T = cbuf + base;   // the chains are consumed: reuse as scratch
    for (int32_t k = tid; k < L; k += nt) {
        int32_t v = R[k].y, acc = v;
        for (int32_t s2 = k - 1; s2 >= 0; --s2) {
            int32_t u = R[s2].y;
            if ((u & ~3) != (v & ~3)) break;
            acc |= u;
        }
        if (k + 1 < L) {
            int32_t u = R[k + 1].y;
            if ((u & ~3) == (v & ~3)) acc |= u;
        }
        T[k] = acc;
    }
    __syncthreads();
    for (int32_t k = tid; k < L; k += nt) R[k].y = T[k];
    __syncthreads();
}

// Part 0: the long pieces of the list, a CTA each; those of wide curves are
// marked pending.  Part 1: the wide curves, a CTA each, merging their long
// pieces.
__global__ void __launch_bounds__(256) k_merge_long(const GeomArgs g, const int32_t* __restrict__ offs,
                                                    const uint4* __restrict__ pieces,
                                                    const uint32_t* __restrict__ long_list, uint32_t list_cap,
                                                    const uint32_t* __restrict__ long_count,
                                                    int32_t* __restrict__ cbuf, int2* __restrict__ rec,
                                                    const uint8_t* __restrict__ curve_wide,
                                                    const uint32_t* __restrict__ wide_curves,
                                                    const uint32_t* __restrict__ wide_curve_count, int part,
                                                    int32_t cap) {
    extern __shared__ int32_t sm_long[];   // [cap] chains in, [cap + 1] records out
    __shared__ int32_t s_i0;
    const int tid = threadIdx.x, nt = blockDim.x;
    if (part == 0) {
        const uint32_t n_long = imin((int32_t)*long_count, (int32_t)list_cap);
        for (uint32_t item = blockIdx.x; item < n_long; item += gridDim.x) {
            const uint32_t c = long_list[item] >> 3, piece = long_list[item] & 7u;
            const uint4* pt = pieces + (size_t)c * kMaxPieces;
            int64_t base = offs[c];
            for (uint32_t j = 0; j < piece; ++j) base += 1 + piece_nx(pt[j].x) + piece_ny(pt[j].x);
            const int32_t nx = piece_nx(pt[piece].x), ny = piece_ny(pt[piece].x);
            const int32_t L = 1 + nx + ny;
            if (base + L > g.rec_cap) continue;   // overflow: k_merge reports it
            if (curve_wide[c]) {   // merged by part 1: mark pending
                for (int32_t k = tid; k < L; k += nt) rec[base + k] = make_int2(kPendingCurve, 0);
                continue;
            }
            merge_long_piece(c, piece == 0 ? 0 : (int32_t)pt[piece - 1].y, base, nx, ny, cbuf, rec, sm_long, cap,
                             &s_i0);
        }
        return;
    }
    const uint32_t nw = imin((int32_t)*wide_curve_count, (int32_t)g.n_curves);
    for (uint32_t k = blockIdx.x; k < nw; k += gridDim.x) {
        const uint32_t c = wide_curves[k];
        const uint4* pt = pieces + (size_t)c * kMaxPieces;
        int64_t base = offs[c];
        const int64_t end = offs[c + 1];
        if (end > g.rec_cap) continue;   // overflow: k_merge reports it
        for (int j = 0; j < kMaxPieces && base < end; ++j) {
            const int32_t nx = piece_nx(pt[j].x), ny = piece_ny(pt[j].x);
            const int32_t L = 1 + nx + ny;
            if (base + L > end) break;   // k_merge reports the range error
            if (L >= kLongPiece)
                merge_long_piece(c, j == 0 ? 0 : (int32_t)pt[j - 1].y, base, nx, ny, cbuf, rec, sm_long, cap,
                                 &s_i0);
            base += L;
        }
    }
}

// ---------------------------------------------------------- fragment -----
// gen_fragment.comp:90-245, one thread per record: the piece between this
// record's t and the next record's t (t = 1 when the next record belongs to
// another curve), its cell, the 64-bit sort key, the winding change across
// the sample row and (pixel mode) the part of it left of the cell centre.
// Record i of curve r0.x: the piece runs to the next record's t when that
// record belongs to the same curve (i + 1 < offs[c + 1]), else to t = 1.
SR_DEV void fragment_record(const GeomArgs& g, const int2* __restrict__ rec, const int32_t* __restrict__ offs,
                            int64_t n, int64_t i, int2 r0, uint64_t* __restrict__ keys, uint8_t* __restrict__ wnp,
                            const DebugOut& dbg) {
    float t0 = gmax(bitsf(r0.y & ~3), 0.0f);
    uint32_t c = (uint32_t)r0.x;
    if (c >= g.n_curves) {
        // only in a frame whose records overflowed their capacity (the
        // frame is reported and discarded): never index with it
        keys[i] = ~0ull;
        if (wnp) wnp[i] = 0;
        return;
    }
    float t1 = 1.0f;
    if (i + 1 < n && i + 1 < (int64_t)offs[c + 1]) t1 = gmax(bitsf(rec[i + 1].y & ~3), 0.0f);
    uint32_t path = g.curve_path[c];
    int32_t yx = (int32_t)0xFFFEFFFE, wn = 0, left = 0;
    bool valid = false;
    int32_t pos_x = 0, pos_y = 0;
    if (t0 < t1) {
        uint32_t type = g.curve_type[c];
        CurvePts P;
        load_curve(g.tpos, g.curve_pos[c], type, P);
        float pfx = interp(type, t0, P.x), pfy = interp(type, t0, P.y);
        float plx = interp(type, t1, P.x), ply = interp(type, t1, P.y);
        const int32_t F = g.F;
        const SceneInfo& si = scene_of_path(g.st, path);
        const float invF = inv_F(F);
        int32_t rx = wmul(float2int_rd(__fmul_rn(__fmul_rn(__fadd_rn(pfx, plx), 0.5f), invF)), F);
        int32_t ry = wmul(float2int_rd(__fmul_rn(__fmul_rn(__fadd_rn(pfy, ply), 0.5f), invF)), F);
        pos_x = imin(imax(rx, -F), wadd(si.W & (int32_t)0xFFFFFFFE, F));
        pos_y = imin(imax(ry, -F), wadd(si.H & (int32_t)0xFFFFFFFE, F));
        if ((uint32_t)ry < (uint32_t)si.H) {
            valid = true;
            yx = (int32_t)(((uint32_t)wadd(pos_y, 0x7FFF) << 16) | ((uint32_t)wadd(pos_x, 0x7FFF) & 0xFFFFu));
        }
        // winding sample row cell_y + FRAG_SIZE/2 (gen_fragment.comp:188-199)
        float wn_y = __fadd_rn((float)pos_y, __fmul_rn(0.5f, (float)F));
        if (pfy == ply) wn = 0;
        else if (pfy < wn_y && wn_y <= ply) wn = -1;
        else if (ply < wn_y && wn_y <= pfy) wn = 1;
        if (g.pixel_mode && wn != 0) {
            float dyv = __fsub_rn(ply, pfy);
            float tc = __fdiv_rn(__fsub_rn(wn_y, pfy), dyv);
            float xc = __fadd_rn(pfx, __fmul_rn(tc, __fsub_rn(plx, pfx)));
            if (xc < __fadd_rn((float)pos_x, 0.5f)) left = wn;
        }
    }
    const uint32_t wbits = (uint32_t)((wn & 3) | ((left & 3) << 2));
    const uint64_t key = pack_key(g.L, path, valid, pos_y, pos_x);
    if (wnp) {
        keys[i] = key;
        wnp[i] = (uint8_t)wbits;
    } else {
        keys[i] = key | ((uint64_t)wbits << key_bits(g.L));   // winding bits ride above the key
    }
    if (dbg.fkey) {
        dbg.fkey[i] = yx;
        dbg.fwn[i] = wn;
        dbg.fleft[i] = left;
    }
}

// Part 0: every record but those of wide curves (pending, or already
// merged by part 1); part 1: the wide curves' records, a CTA per curve.
__global__ void __launch_bounds__(256) k_fragment(const GeomArgs g, const int2* __restrict__ rec,
                                                  const int32_t* __restrict__ offs, int64_t n_cap,
                                                  const uint32_t* __restrict__ n_dev, uint64_t* __restrict__ keys,
                                                  uint8_t* __restrict__ wnp, DebugOut dbg,
                                                  const uint8_t* __restrict__ curve_wide,
                                                  const uint32_t* __restrict__ wide_curves,
                                                  const uint32_t* __restrict__ wide_curve_count, int part) {
    const int64_t n = n_dev ? (int64_t)min((uint64_t)*n_dev, (uint64_t)n_cap) : n_cap;
    if (part == 0) {
        const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        if (i >= n) return;
        const int2 r0 = rec[i];
        if (r0.x == kPendingCurve) return;
        if ((uint32_t)r0.x < g.n_curves && curve_wide[r0.x]) return;
        fragment_record(g, rec, offs, n, i, r0, keys, wnp, dbg);
        return;
    }
    const uint32_t nw = imin((int32_t)*wide_curve_count, (int32_t)g.n_curves);
    for (uint32_t k = blockIdx.x; k < nw; k += gridDim.x) {
        const uint32_t c = wide_curves[k];
        const int64_t end = min((int64_t)offs[c + 1], n);
        for (int64_t i = (int64_t)offs[c] + threadIdx.x; i < end; i += blockDim.x)
            fragment_record(g, rec, offs, n, i, rec[i], keys, wnp, dbg);
    }
}

// -------------------------------------------------------------- launches --
void launch_arc_fixup(const uint32_t* curve_type, const uint32_t* curve_pos, const uint32_t* curve_path,
                      uint32_t n_curves, const float2* pos, const SceneTable& t, float2* tpos, int32_t* path_visible,
                      cudaStream_t st) {
    if (n_curves == 0) return;
    count_launches(1);
    k_arc_fixup<<<(n_curves + 255) / 256, 256, 0, st>>>(curve_type, curve_pos, curve_path, n_curves, pos, t, tpos,
                                                        path_visible);
}

void launch_transform(const float2* pos, const uint32_t* pos_path, uint32_t n_points, const SceneTable& t,
                      float2* tpos, int32_t* path_visible, cudaStream_t st) {
    if (n_points == 0) return;
    count_launches(1);
    k_transform<<<(n_points + 255) / 256, 256, 0, st>>>(pos, pos_path, n_points, t, tpos, path_visible);
}

static int sm_count_hint() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 148;
    }
    return n * 8;
}

size_t piece_table_bytes(uint32_t n_curves) { return sizeof(uint4) * kMaxPieces * (size_t)n_curves; }
uint32_t chain_list_capacity(uint32_t n_curves) { return 2u * kMaxPieces * n_curves; }

void launch_count(const GeomArgs& g, float* cut_cache, int32_t* count, const ChainWork& w, uint32_t* status,
                  cudaStream_t st) {
    if (g.n_curves == 0) return;
    count_launches(1);
    k_count<<<(g.n_curves + 255) / 256, 256, 0, st>>>(g, cut_cache, count, w.pieces, w.chain_items, w.chain_keys,
                                                      w.list_cap, w.chain_count, w.wide_count, w.curve_wide,
                                                      w.wide_curves, w.wide_curve_count, w.long_list, w.long_count,
                                                      status);
}

uint32_t chain_key_bits() { return kChainKeyBits; }

void launch_chains(const GeomArgs& g, const int32_t* offs, const ChainWork& w, int32_t* cbuf, int sm_count, int part,
                   cudaStream_t st) {
    if (g.n_curves == 0) return;
    count_launches(1);
    // Part 1 runs two CTAs (8 warps) an SM.  Fewer warps share each SM's
    // issue slots, so each group of chains, the longest first, finishes
    // sooner, and the wide chains beside them and the merge waiting on them
    // start earlier: on the 4096^2 frame its stage took 0.83 / 0.61 / 0.73 /
    // 0.75 / 0.78 ms at 1 / 2 / 4 / 8 / 16 CTAs an SM.
    if (part == 0)
        k_chains<<<sm_count * 4, 128, 0, st>>>(g, offs, w.pieces, w.sorted_items, w.sorted_keys, w.list_cap,
                                               w.chain_count, w.wide_count, w.wide_queue, cbuf, 0);
    else
        k_chains<<<sm_count * 2, 128, 0, st>>>(g, offs, w.pieces, w.sorted_items, w.sorted_keys, w.list_cap,
                                                w.chain_count, w.wide_count, w.chain_queue, cbuf, 1);
}

constexpr int32_t kLongCapMain = 3072, kLongCapSide = 12288;

cudaError_t geom_init() {
    return cudaFuncSetAttribute(k_merge_long, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(sizeof(int32_t) * (2 * (size_t)kLongCapSide + 1)));
}

void launch_merge(const GeomArgs& g, const int32_t* offs, const ChainWork& w, int32_t* cbuf, int2* rec,
                  uint32_t* status, int part, cudaStream_t st) {
    if (g.n_curves == 0) return;
    count_launches(2);
    const unsigned grid = part == 0 ? (unsigned)(((size_t)g.n_curves * kMaxPieces + 127) / 128)
                                    : (unsigned)sm_count_hint() / 8;
    k_merge<<<grid, 128, 0, st>>>(g, offs, w.pieces, cbuf, rec, status, w.curve_wide, w.wide_curves,
                                  w.wide_curve_count, part);
    // chains of up to 3 K elements in 25 KB of shared memory (eight CTAs an
    // SM) on the main stream; up to 12 K on the second stream, whose few
    // pieces are the longest
    const int32_t cap = part == 0 ? kLongCapMain : kLongCapSide;
    const size_t smem = sizeof(int32_t) * (2 * (size_t)cap + 1);
    k_merge_long<<<part == 0 ? sm_count_hint() : sm_count_hint() / 4, 256, smem, st>>>(
        g, offs, w.pieces, w.long_list, w.list_cap, w.long_count, cbuf, rec, w.curve_wide, w.wide_curves,
        w.wide_curve_count, part, cap);
}

void launch_fragment(const GeomArgs& g, const int2* rec, const int32_t* offs, int64_t n_cap, const uint32_t* n_dev,
                     uint64_t* keys, uint8_t* wnp, const DebugOut& dbg, const ChainWork& w, int part,
                     cudaStream_t st) {
    if (n_cap <= 0 || g.n_curves == 0) return;
    count_launches(1);
    const unsigned grid = part == 0 ? (unsigned)((n_cap + 255) / 256) : (unsigned)sm_count_hint() / 4;
    k_fragment<<<grid, 256, 0, st>>>(g, rec, offs, n_cap, n_dev, keys, wnp, dbg, w.curve_wide, w.wide_curves,
                                     w.wide_curve_count, part);
}

}  // namespace sr
