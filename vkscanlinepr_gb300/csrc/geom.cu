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
                                                   Mvp M, float fw, float fh, float2* __restrict__ tpos,
                                                   int32_t* __restrict__ path_visible) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t lane = lane_id();
    uint32_t pidx = 0xFFFFFFFFu;
    int32_t v = 0;
    if (i < n_points) {
        float2 p = pos[i];
        float o[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            // dot((x, y, 0, 1), m_r) summed left to right
            float acc = __fmul_rn(p.x, M.m[4 * r + 0]);
            acc = __fadd_rn(acc, __fmul_rn(p.y, M.m[4 * r + 1]));
            acc = __fadd_rn(acc, __fmul_rn(0.0f, M.m[4 * r + 2]));
            acc = __fadd_rn(acc, __fmul_rn(1.0f, M.m[4 * r + 3]));
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
        pidx = pos_path[i];
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

// ------------------------------------------------- shared curve helpers --
struct CurvePts {
    float x[4], y[4];
};

SR_DEV void load_curve(const float2* __restrict__ tpos, uint32_t first, uint32_t type, CurvePts& c) {
    uint32_t np = type & 7u;
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

// ---------------------------------------------------------------- K2 ----
// make_intersection_0.comp:226-411.  One thread per curve: path cull,
// monotonic cut points (cached, 5 floats per curve) and the number of
// intersection records the curve will emit.
__global__ void __launch_bounds__(256) k_count(const GeomArgs g, float* __restrict__ cut_cache,
                                               int32_t* __restrict__ count) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.n_curves) return;
    uint32_t type = g.curve_type[c];
    CurvePts P;
    load_curve(g.tpos, g.curve_pos[c], type, P);
    bool vis = path_visible_mask(g.path_visible[g.curve_path[c]]);
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
    int32_t pc = 0;
    for (uint32_t i = 0; i < n; ++i) {
        float t1 = q[i];
        float x1 = interp(type, t1, P.x), y1 = interp(type, t1, P.y);
        int32_t xb, xe, yb, ye;
        // get_xy_begin_end (make_intersection_0.comp:167-183)
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
        int32_t nx = cut_range(g.W, F, xb, xe);
        int32_t ny = cut_range(g.H, F, yb, ye);
        pc = wadd(pc, wadd(1, wadd(nx, ny)));
        x0 = x1;
        y0 = y1;
    }
    count[c] = pc;
}

// ---------------------------------------------------------- K4 + K5 -----
// Fragment of one record (gen_fragment.comp:100-200) given its piece
// [t0, t1) on curve P.  Returns the 64-bit sort key, the winding change and
// (pixel mode) the centre-sample part of the change.
struct FragOut {
    uint64_t key;
    int32_t yx;
    int32_t wn;
    int32_t left;
};

SR_DEV FragOut make_fragment(const GeomArgs& g, uint32_t path, float t0, float t1, float pfx, float pfy,
                             float plx, float ply) {
    FragOut o;
    o.yx = (int32_t)0xFFFEFFFE;
    o.wn = 0;
    o.left = 0;
    bool valid = false;
    int32_t pos_x = 0, pos_y = 0;
    if (t0 < t1) {
        const int32_t F = g.F;
        const float fF = (float)F;
        int32_t rx = wmul(float2int_rd(__fdiv_rn(__fmul_rn(__fadd_rn(pfx, plx), 0.5f), fF)), F);
        int32_t ry = wmul(float2int_rd(__fdiv_rn(__fmul_rn(__fadd_rn(pfy, ply), 0.5f), fF)), F);
        pos_x = imin(imax(rx, -F), wadd(g.W & (int32_t)0xFFFFFFFE, F));
        pos_y = imin(imax(ry, -F), wadd(g.H & (int32_t)0xFFFFFFFE, F));
        if ((uint32_t)ry < (uint32_t)g.H) {
            valid = true;
            o.yx = (int32_t)(((uint32_t)wadd(pos_y, 0x7FFF) << 16) | ((uint32_t)wadd(pos_x, 0x7FFF) & 0xFFFFu));
        }
        // winding sample row cell_y + FRAG_SIZE/2 (gen_fragment.comp:188-199)
        float wn_y = __fadd_rn((float)pos_y, __fmul_rn(0.5f, fF));
        if (pfy == ply) o.wn = 0;
        else if (pfy < wn_y && wn_y <= ply) o.wn = -1;
        else if (ply < wn_y && wn_y <= pfy) o.wn = 1;
        if (g.pixel_mode && o.wn != 0) {
            float dyv = __fsub_rn(ply, pfy);
            float tc = __fdiv_rn(__fsub_rn(wn_y, pfy), dyv);
            float xc = __fadd_rn(pfx, __fmul_rn(tc, __fsub_rn(plx, pfx)));
            if (xc < __fadd_rn((float)pos_x, 0.5f)) o.left = o.wn;
        }
    }
    o.key = pack_key(g.L, path, valid, pos_y, pos_x);
    return o;
}

// make_intersection_1.comp:217-447 fused with gen_fragment.comp:90-245.
// One thread per curve walks each monotonic piece across the FRAG_SIZE grid
// in t order, emitting the reference's intersection records; the fragment
// of record k is built when record k+1's t is known (the last record of a
// curve ends at t = 1).  Writes the sort key and packed winding bits of
// every record; debug pointers, when set, receive the reference layouts.
__global__ void __launch_bounds__(128) k_intersect_fragment(const GeomArgs g, const float* __restrict__ cut_cache,
                                                            const int32_t* __restrict__ offs,
                                                            uint64_t* __restrict__ keys,
                                                            uint8_t* __restrict__ wnp, DebugOut dbg,
                                                            uint32_t* __restrict__ status) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.n_curves) return;
    const int32_t F = g.F;
    uint32_t type = g.curve_type[c];
    uint32_t path = g.curve_path[c];
    CurvePts P;
    load_curve(g.tpos, g.curve_pos[c], type, P);
    bool vis = path_visible_mask(g.path_visible[path]);
    const float* cc = cut_cache + 5 * (size_t)c;
    float q[5] = {cc[0], cc[1], cc[2], cc[3], 0.0f};
    uint32_t n = __float_as_uint(cc[4]);
    if (n > 4) n = 4;
    if (vis) q[n++] = 1.0f;
    int64_t pc = offs[c];
    const int64_t end = offs[c + 1];
    if (pc >= end) return;

    float t0_ms = 0.0f;
    float x0m = P.x[0], y0m = P.y[0];
    const int32_t minus_one = fbits(-1.0f);
    // pending record: emitted, fragment not yet built
    bool have_prev = false;
    float prev_t = 0.0f, prev_x = 0.0f, prev_y = 0.0f;
    const float fF = (float)F;

    for (uint32_t i = 0; i < n; ++i) {
        float t1_ms = q[i];
        float x1m = interp(type, t1_ms, P.x), y1m = interp(type, t1_ms, P.y);
        int32_t tb = fbits(t1_ms) & ~3;
        tb |= (floorf(x1m) == x1m) ? 2 : 3;   // make_intersection_1.comp:271-276
        t1_ms = bitsf(tb);
        int32_t xb, xe, yb, ye;
        float dx, dy;
        // get_xy_begin_end_delta (make_intersection_1.comp:150-170)
        if (x0m <= x1m) {
            xb = wadd(wmul(float2int_rd(__fdiv_rn(x0m, fF)), F), F);
            xe = wmul(float2int_rd(__fdiv_rn(x1m, fF)), F);
            dx = fF;
        } else {
            xb = wadd(wmul(float2int_rd(__fdiv_rn(x1m, fF)), F), F);
            xe = wmul(float2int_rd(__fdiv_rn(x0m, fF)), F);
            dx = -fF;
        }
        if (y0m <= y1m) {
            yb = wadd(wmul(float2int_rd(__fdiv_rn(y0m, fF)), F), F);
            ye = wmul(float2int_rd(__fdiv_rn(y1m, fF)), F);
            dy = fF;
        } else {
            yb = wadd(wmul(float2int_rd(__fdiv_rn(y1m, fF)), F), F);
            ye = wmul(float2int_rd(__fdiv_rn(y0m, fF)), F);
            dy = -fF;
        }
        int32_t nx = cut_range(g.W, F, xb, xe);
        int32_t ny = cut_range(g.H, F, yb, ye);
        int32_t n_loop = nx + ny + 1;
        float x = (float)(dx < 0.0f ? xe : xb);
        float y = (float)(dy < 0.0f ? ye : yb);
        float tnx = t0_ms, tny = t0_ms;
        int32_t last = minus_one;
        for (int32_t it = -1; it < n_loop; ++it) {
            float t_solve = 0.0f, cval = 0.0f, t_min;
            int side = 0;
            if (it == -1) {
                t_min = tnx;
                if (nx == 0) { side = 0; t_solve = 2.0f; }
                else if (ny == 0) { side = 1; t_solve = 2.0f; }
                else { side = 0; --nx; cval = x; x = __fadd_rn(x, dx); }
            } else if (tnx <= tny) {
                t_min = tnx;
                side = 0;
                if (nx > 0) { --nx; cval = x; x = __fadd_rn(x, dx); }
                else t_solve = 2.0f;
            } else {
                t_min = tny;
                side = 1;
                if (ny > 0) { --ny; cval = y; y = __fadd_rn(y, dy); }
                else t_solve = 2.0f;
            }
            if (it >= 0) {
                // emit record (make_intersection_1.comp:361-375)
                int32_t out = fbits(t_min);
                if ((out & ~3) == (last & ~3)) {
                    out |= last;
                    if (dbg.inter) dbg.inter[pc - 1] = make_int2((int32_t)c, out);
                }
                if (pc >= end) {
                    set_error(status, ERR_RECORD_RANGE);
                    return;
                }
                if (dbg.inter) dbg.inter[pc] = make_int2((int32_t)c, out);
                last = out;
                float tcur = bitsf(out & ~3);
                tcur = gmax(tcur, 0.0f);
                float cx = interp(type, tcur, P.x), cy = interp(type, tcur, P.y);
                if (have_prev) {
                    FragOut fo = make_fragment(g, path, prev_t, tcur, prev_x, prev_y, cx, cy);
                    size_t k = (size_t)(pc - 1);
                    keys[k] = fo.key;
                    wnp[k] = (uint8_t)((fo.wn & 3) | ((fo.left & 3) << 2));
                    if (dbg.fkey) {
                        dbg.fkey[k] = fo.yx;
                        dbg.fwn[k] = fo.wn;
                        dbg.fleft[k] = fo.left;
                    }
                }
                have_prev = true;
                prev_t = tcur;
                prev_x = cx;
                prev_y = cy;
                ++pc;
            }
            if (t_solve < 2.0f) {
                const float* cv = side == 0 ? P.x : P.y;
                if (type == 2u) {
                    float a = __fsub_rn(cv[1], cv[0]);
                    a = (a != 0.0f) ? __fdiv_rn(1.0f, a) : 0.0f;
                    t_solve = gmin(gmax(__fmul_rn(__fsub_rn(cval, cv[0]), a), t_min), t1_ms);
                } else {
                    float ta = t_min, tb1 = t1_ms;
                    float vt0 = interp(type, ta, cv);
                    t_solve = ta;
                    if (vt0 != cval) {
                        float raw_t0 = ta, last_vtm = 0.0f;
#pragma unroll 4
                        for (int j = 0; j < 24; ++j) {
                            float tm = __fmul_rn(__fadd_rn(ta, tb1), 0.5f);
                            float vtm = interp(type, tm, cv);
                            t_solve = tm;
                            last_vtm = vtm;
                            if ((fbits(__fsub_rn(vtm, cval)) ^ fbits(__fsub_rn(vt0, cval))) >= 0) {
                                ta = tm;
                                vt0 = vtm;
                            } else {
                                tb1 = tm;
                            }
                        }
                        if (fabsf(__fsub_rn(last_vtm, cval)) > 1.0f) t_solve = raw_t0;
                    }
                }
            }
            int32_t nb = (fbits(t_solve) & ~3) | side;
            if (side == 0) tnx = bitsf(nb);
            else tny = bitsf(nb);
        }
        t0_ms = t1_ms;
        x0m = x1m;
        y0m = y1m;
    }
    if (pc != end) {
        set_error(status, ERR_RECORD_RANGE);
        return;
    }
    if (have_prev) {
        // last record of the curve: its piece ends at t = 1
        float cx = interp(type, 1.0f, P.x), cy = interp(type, 1.0f, P.y);
        FragOut fo = make_fragment(g, path, prev_t, 1.0f, prev_x, prev_y, cx, cy);
        size_t k = (size_t)(end - 1);
        keys[k] = fo.key;
        wnp[k] = (uint8_t)((fo.wn & 3) | ((fo.left & 3) << 2));
        if (dbg.fkey) {
            dbg.fkey[k] = fo.yx;
            dbg.fwn[k] = fo.wn;
            dbg.fleft[k] = fo.left;
        }
    }
}

// -------------------------------------------------------------- launches --
void launch_transform(const float2* pos, const uint32_t* pos_path, uint32_t n_points, const Mvp& M, float fw,
                      float fh, float2* tpos, int32_t* path_visible, cudaStream_t st) {
    if (n_points == 0) return;
    k_transform<<<(n_points + 255) / 256, 256, 0, st>>>(pos, pos_path, n_points, M, fw, fh, tpos, path_visible);
}

void launch_count(const GeomArgs& g, float* cut_cache, int32_t* count, cudaStream_t st) {
    if (g.n_curves == 0) return;
    k_count<<<(g.n_curves + 255) / 256, 256, 0, st>>>(g, cut_cache, count);
}

void launch_intersect_fragment(const GeomArgs& g, const float* cut_cache, const int32_t* offs, uint64_t* keys,
                               uint8_t* wnp, const DebugOut& dbg, uint32_t* status, cudaStream_t st) {
    if (g.n_curves == 0) return;
    k_intersect_fragment<<<(g.n_curves + 127) / 128, 128, 0, st>>>(g, cut_cache, offs, keys, wnp, dbg, status);
}

}  // namespace sr
