// host.cpp — scene sources behind sr.h: the seeded synthetic generator and
// an .rvg reader with the reference loader's behaviour (host code only).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/sr.h"
#include "synth.h"

struct sr_scene_buf {
    srsynth::Scene s;
    std::vector<sr_paint> paints;   // gradient paints (full RVG reader)
};

namespace {
thread_local std::string g_host_err;
}

extern "C" const char* sr_host_last_error(void) { return g_host_err.c_str(); }

extern "C" sr_status sr_synth_scene(const sr_synth_params* p, sr_scene_buf** out) {
    if (!p || !out) return SR_ERR_INVALID_ARG;
    if (p->struct_size < sizeof(sr_synth_params)) return SR_ERR_INVALID_ARG;
    if (p->preset < 0 || p->preset > 2) return SR_ERR_INVALID_ARG;
    srsynth::Params q;
    q.preset = p->preset;
    q.seed = p->seed;
    q.scene_index = p->scene_index;
    q.width = p->width;
    q.height = p->height;
    q.n_paths = p->n_paths;
    sr_scene_buf* b = new sr_scene_buf();
    srsynth::generate(q, b->s);
    *out = b;
    return SR_OK;
}

extern "C" sr_status sr_scene_buf_view(const sr_scene_buf* b, sr_scene_view* v) {
    if (!b || !v) return SR_ERR_INVALID_ARG;
    const auto& s = b->s;
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
    return SR_OK;
}

extern "C" void sr_scene_buf_free(sr_scene_buf* b) { delete b; }

extern "C" sr_status sr_scene_buf_paints(const sr_scene_buf* b, const sr_paint** paints, uint32_t* n) {
    if (!b || !paints || !n) return SR_ERR_INVALID_ARG;
    *paints = b->paints.empty() ? nullptr : b->paints.data();
    *n = (uint32_t)b->paints.size();
    return SR_OK;
}

extern "C" sr_status sr_scene_buf_size(const sr_scene_buf* b, uint32_t* wh) {
    if (!b || !wh) return SR_ERR_INVALID_ARG;
    wh[0] = b->s.width;
    wh[1] = b->s.height;
    return SR_OK;
}

// ------------------------------------------------------------- RVG ------
// The reference reader (core/vg/rvg.cpp:33-255) works on whitespace tokens;
// its asserts are compiled out in release builds, so a token it does not
// expect is simply consumed.  This reader consumes tokens the same way.
namespace {

struct Tok {
    std::istream& in;
    bool next(std::string& t) { return static_cast<bool>(in >> t); }
};

struct Pt {
    float x = 0.f, y = 0.f;
};

// read_point: commas and colons become blanks, then "%f %f"
Pt parse_point(std::string s) {
    for (char& ch : s)
        if (ch == ',' || ch == ':') ch = ' ';
    Pt p;
    float a = 0.f, b = 0.f;
    int got = std::sscanf(s.c_str(), "%f %f", &a, &b);
    if (got >= 1) p.x = a;
    if (got >= 2) p.y = b;
    return p;
}

struct PathRec {
    uint32_t first_curve;
    uint32_t rule = 0;
    float color[4] = {0.f, 0.f, 0.f, 1.f};
    float opacity = 0.f;
    bool gradient = false;   // a gradient paint (full reader)
    sr_paint paint{};
};

// The numbers of a token, brackets, parentheses, commas and colons taken as
// blanks: "(1,2)" -> 1 2, "dyn_affine([1,0,2],[0,1,3])" -> 1 0 2 0 1 3.
std::vector<float> token_numbers(const std::string& t) {
    std::string s = t;
    for (char& ch : s)
        if (ch == '(' || ch == ')' || ch == '[' || ch == ']' || ch == ',' || ch == ':') ch = ' ';
    std::vector<float> v;
    const char* p = s.c_str();
    while (*p) {
        char* end = nullptr;
        const float x = std::strtof(p, &end);
        if (end == p) {
            ++p;
            continue;
        }
        v.push_back(x);
        p = end;
    }
    return v;
}

}  // namespace

// full = false: exactly the reference reader's behaviour.  full = true adds
// what RVG::load leaves out (rvg.cpp:160-169, :234-251): 'A' (a rational
// quadratic, "A x,y,w x2,y2": the control point in homogeneous coordinates,
// then the end point) as SR_CURVE_ARC, 'Q' as SR_CURVE_QUADRIC, and linear
// and radial gradient paints, which are consumed whole.
static sr_status rvg_parse(const char* path, bool full, sr_scene_buf** out, float viewport[4]) {
    if (!path || !out) return SR_ERR_INVALID_ARG;
    std::ifstream fin(path);
    if (!fin.is_open()) {
        g_host_err = std::string("cannot open ") + path;
        return SR_ERR_INVALID_ARG;
    }
    Tok tk{fin};
    std::string t;
    // header: viewport x,y w,h / window x,y w,h / scene / dyn_identity
    float vp[4] = {0, 0, 0, 0};
    tk.next(t);
    {
        std::string a, b;
        tk.next(a);
        tk.next(b);
        Pt p0 = parse_point(a), p1 = parse_point(b);
        vp[0] = p0.x; vp[1] = p0.y; vp[2] = p1.x; vp[3] = p1.y;
    }
    tk.next(t);
    {
        std::string a, b;
        tk.next(a);
        tk.next(b);
    }
    tk.next(t);   // scene
    tk.next(t);   // dyn_identity
    if (viewport) std::memcpy(viewport, vp, sizeof vp);

    std::vector<Pt> pts;
    std::vector<uint32_t> curve_first, curve_type;
    std::vector<PathRec> paths;
    size_t last_path_points = (size_t)-1;

    auto add_curve = [&](uint32_t type, const Pt* p) {
        curve_first.push_back((uint32_t)pts.size());
        curve_type.push_back(type);
        const uint32_t np = type == SR_CURVE_ARC ? 4u : (type & 7u);
        for (uint32_t k = 0; k < np; ++k) pts.push_back(p[k]);
    };

    while (tk.next(t)) {
        if (t.size() >= 2 && t[0] == '/' && t[1] == '/') {
            std::string line;
            std::getline(fin, line);
            continue;
        }
        if (last_path_points != pts.size()) {
            last_path_points = pts.size();
            PathRec r;
            r.first_curve = (uint32_t)curve_type.size();
            paths.push_back(r);
        }
        PathRec& pr = paths.back();
        tk.next(t);   // "element"
        tk.next(t);   // fill rule
        if (t == "ofill") pr.rule = SR_FILL_EVENODD;
        else if (t == "nzfill") pr.rule = SR_FILL_NONZERO;
        else {
            tk.next(t);
            continue;
        }
        tk.next(t);   // dyn_concrete
        tk.next(t);
        tk.next(t);
        tk.next(t);   // three points, ignored
        Pt p[4];
        size_t contour_begin = pts.size();
        bool closed = false;
        while (tk.next(t)) {
            if (t != "fL" && t.size() != 1) break;
            char cmd = t[0];
            if (std::string(full ? "MmZzLlCcAaQq" : "MmZzLlCcAa").find(cmd) == std::string::npos && t != "fL") break;
            std::string a, b, c;
            if (full && cmd == 'A') {
                // control point (x, y, w) in homogeneous coordinates, then the end point
                tk.next(a);
                tk.next(b);
                for (char& ch : a)
                    if (ch == ',') ch = ' ';
                float hx = 0.f, hy = 0.f, hw = 1.f;
                std::sscanf(a.c_str(), "%f %f %f", &hx, &hy, &hw);
                Pt q[4] = {p[0], Pt{hx, hy}, parse_point(b), Pt{hw, hw}};
                add_curve(SR_CURVE_ARC, q);
                p[0] = q[2];
                continue;
            }
            if (full && cmd == 'Q') {
                tk.next(a);
                tk.next(b);
                p[1] = parse_point(a);
                p[2] = parse_point(b);
                add_curve(SR_CURVE_QUADRIC, p);
                p[0] = p[2];
                continue;
            }
            switch (cmd) {
                case 'M':
                    tk.next(a);
                    p[0] = parse_point(a);
                    contour_begin = pts.size();
                    closed = false;
                    break;
                case 'L':
                    tk.next(a);
                    p[1] = parse_point(a);
                    add_curve(SR_CURVE_LINE, p);
                    p[0] = p[1];
                    break;
                case 'C':
                    tk.next(a);
                    tk.next(b);
                    tk.next(c);
                    p[1] = parse_point(a);
                    p[2] = parse_point(b);
                    p[3] = parse_point(c);
                    add_curve(SR_CURVE_CUBIC, p);
                    p[0] = p[3];
                    break;
                case 'Z':
                    closed = true;
                    break;
                default:
                    if (t == "fL") {
                        tk.next(a);
                        p[0] = parse_point(a);
                    }
                    break;
            }
        }
        // the last contour, if open, is closed by a straight line (rvg.cpp:211-223)
        if (!closed && pts.size() > contour_begin) {
            // an arc's last slot is its weight: its end point is the slot before
            const bool arc_last = curve_type.back() == SR_CURVE_ARC && full;
            Pt first = pts[contour_begin], last = arc_last ? pts[pts.size() - 2] : pts.back();
            if (first.x != last.x || first.y != last.y) {
                Pt q[2] = {last, first};
                add_curve(SR_CURVE_LINE, q);
            }
        }
        // t now holds "dyn_identity"
        tk.next(t);   // dyn_paint
        {
            std::string o;
            tk.next(o);
            pr.opacity = (float)std::strtod(o.c_str(), nullptr);
        }
        tk.next(t);
        if (full && (t == "linear" || t == "radial")) {
            // linear gradient (x0,y0) (x1,y1) | radial gradient (cx,cy) (fx,fy) r,
            // then dyn_ramp, stops "offset:rgba(r,g,b,a)", the spread (pad,
            // repeat or reflect) and dyn_affine([a,b,c],[d,e,f]), which ends it
            pr.gradient = true;
            sr_paint& g = pr.paint;
            g.kind = t == "radial" ? SR_PAINT_RADIAL : SR_PAINT_LINEAR;
            g.opacity = pr.opacity;
            g.xf[0] = 1.f;
            g.xf[4] = 1.f;
            tk.next(t);   // gradient
            std::string a, b;
            tk.next(a);
            tk.next(b);
            std::vector<float> pa = token_numbers(a), pb = token_numbers(b);
            if (pa.size() >= 2) { g.p0[0] = pa[0]; g.p0[1] = pa[1]; }
            if (pb.size() >= 2) { g.p1[0] = pb[0]; g.p1[1] = pb[1]; }
            if (g.kind == SR_PAINT_RADIAL) {
                tk.next(a);
                g.radius = std::strtof(a.c_str(), nullptr);
            }
            while (tk.next(t) && t.compare(0, 10, "dyn_affine") != 0) {
                if (t == "pad") g.spread = SR_SPREAD_PAD;
                else if (t == "repeat") g.spread = SR_SPREAD_REPEAT;
                else if (t == "reflect") g.spread = SR_SPREAD_REFLECT;
                else if (t.find(':') != std::string::npos && g.n_stops < SR_PAINT_MAX_STOPS) {
                    std::vector<float> v = token_numbers(t);
                    const bool rgb = t.find("rgba") == std::string::npos;
                    if (v.size() >= (rgb ? 4u : 5u)) {
                        g.offset[g.n_stops] = v[0];
                        for (int q = 0; q < 3; ++q) g.rgba[g.n_stops][q] = v[1 + q];
                        g.rgba[g.n_stops][3] = rgb ? 1.f : v[4];
                        ++g.n_stops;
                    }
                }
            }
            std::vector<float> xf = token_numbers(t);
            if (xf.size() >= 6)
                for (int q = 0; q < 6; ++q) g.xf[q] = xf[q];
        } else if (t == "solid") {
            tk.next(t);
            std::string inner;
            bool rgba = t.compare(0, 4, "rgba") == 0;
            bool rgb = !rgba && t.compare(0, 3, "rgb") == 0;
            if (rgba && t.size() >= 6) inner = t.substr(5, t.size() - 6);
            else if (rgb && t.size() >= 6) inner = t.substr(4, t.size() - 6);   // as rvg.cpp:245
            if (rgba || rgb) {
                for (char& ch : inner)
                    if (ch == ',') ch = ' ';
                std::istringstream iss(inner);
                int nc = rgba ? 4 : 3;
                for (int k = 0; k < nc; ++k) {
                    float v;
                    if (!(iss >> v)) break;
                    pr.color[k] = v;
                }
            }
        }
    }

    // flatten (scanline_rasterizer.cpp:67-189)
    sr_scene_buf* bobj = new sr_scene_buf();
    srsynth::Scene& s = bobj->s;
    s.width = (uint32_t)vp[2];
    s.height = (uint32_t)vp[3];
    const uint32_t n_curves = (uint32_t)curve_type.size();
    for (uint32_t pi = 0; pi < paths.size(); ++pi) {
        const PathRec& pr = paths[pi];
        uint32_t cb = pr.first_curve;
        uint32_t ce = pi + 1 < paths.size() ? paths[pi + 1].first_curve : n_curves;
        float col[4] = {pr.color[0], pr.color[1], pr.color[2], pr.color[3] * pr.opacity};
        uint8_t b8[4];
        for (int k = 0; k < 4; ++k) {
            float v = col[k] * 255.0f;
            if (!(v > 0.0f)) v = 0.0f;
            if (v > 255.0f) v = 255.0f;
            b8[k] = (uint8_t)v;
        }
        uint32_t c = (uint32_t)b8[0] | ((uint32_t)b8[1] << 8) | ((uint32_t)b8[2] << 16) | ((uint32_t)b8[3] << 24);
        if (!(c & 0xFF000000u)) c = 0;
        if (pr.gradient) {
            c = pr.paint.n_stops ? SR_FILL_PAINT(bobj->paints.size()) : 0u;
            if (pr.paint.n_stops) bobj->paints.push_back(pr.paint);
        }
        s.fill_rule.push_back(pr.rule);
        s.fill_info.push_back(c);
        for (uint32_t ci = cb; ci < ce; ++ci) {
            uint32_t pb = curve_first[ci];
            uint32_t pe = ci + 1 < n_curves ? curve_first[ci + 1] : (uint32_t)pts.size();
            s.curve_pos.push_back(s.n_points());
            s.curve_type.push_back(curve_type[ci]);
            s.curve_path.push_back(pi);
            for (uint32_t k = pb; k < pe; ++k) {
                s.pos.push_back(pts[k].x);
                s.pos.push_back(pts[k].y);
                s.pos_path.push_back(pi);
            }
        }
    }
    // paths that received no curve still occupy a slot, like the reference
    *out = bobj;
    return SR_OK;
}

// Pinned host memory for callers that want asynchronous copies.
#include <cuda_runtime.h>
extern "C" void* sr_host_alloc(size_t bytes) {
    void* p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
    return p;
}
extern "C" void sr_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

extern "C" sr_status sr_rvg_load(const char* path, sr_scene_buf** out, float viewport[4]) {
    return rvg_parse(path, false, out, viewport);
}

extern "C" sr_status sr_rvg_load_full(const char* path, sr_scene_buf** out, float viewport[4]) {
    return rvg_parse(path, true, out, viewport);
}
