// synth.h — seeded synthetic scenes for the scanline renderer.
//
// The reference ships no benchmark scenes for its headline configurations
// (its large .rvg inputs are missing from the repository), so scenes are
// generated.  Every number is produced from a counter-based RNG (splitmix64)
// and from exp/log/sin/cos written here from their power series, in double
// precision with no fused multiply-add, so x86 and Arm hosts build the same
// float control points bit for bit.  Compile users of this header with
// -ffp-contract=off.
//
// Scene layout is the reference's flattened SoA (scanline_rasterizer.cpp:
// 67-189): each curve owns its control points (cubic 4, quadric 3, line 2).
#pragma once
#include <cstdint>
#include <cstring>
#include <vector>

namespace srsynth {

// ---------------------------------------------------------------- RNG ----
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uni() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }  // [0,1)
    uint32_t below(uint32_t n) { return (uint32_t)(uni() * (double)n); }
};

static inline uint64_t mix3(uint64_t a, uint64_t b, uint64_t c) {
    Rng r(a * 0x100000001B3ull ^ (b + 0x632BE59BD9B4E019ull));
    r.next();
    r.s ^= c * 0xD6E8FEB86659FD93ull;
    return r.next();
}

// ------------------------------------------------------ portable math ----
// Written from the Taylor / atanh series; accuracy ~1e-15 relative, which is
// far more than the distributions need.  What matters is that every step is
// a single IEEE operation, so results do not depend on the host's libm.
static const double kLn2 = 0.69314718055994530942;
static const double kPi = 3.14159265358979323846;

static inline double ldexp_exact(double x, int e) {
    // multiply by 2^e with exact power-of-two factors
    while (e > 0) { int k = e > 60 ? 60 : e; x *= (double)(1ull << k); e -= k; }
    while (e < 0) { int k = -e > 60 ? 60 : -e; x /= (double)(1ull << k); e += k; }
    return x;
}

static inline double pexp(double x) {
    if (x > 700.0) x = 700.0;
    if (x < -700.0) x = -700.0;
    double kf = x / kLn2;
    int k = (int)(kf >= 0 ? kf + 0.5 : kf - 0.5);
    double r = x - (double)k * kLn2;          // |r| <= ~0.35
    double term = 1.0, sum = 1.0;
    for (int i = 1; i <= 20; ++i) { term = term * r / (double)i; sum = sum + term; }
    return ldexp_exact(sum, k);
}

static inline double plog(double x) {
    if (!(x > 0.0)) return -745.0;
    int e = 0;
    while (x >= 1.4142135623730951) { x = x * 0.5; ++e; }
    while (x < 0.7071067811865476) { x = x * 2.0; --e; }
    double s = (x - 1.0) / (x + 1.0);
    double s2 = s * s, term = s, sum = 0.0;
    for (int i = 1; i <= 41; i += 2) { sum = sum + term / (double)i; term = term * s2; }
    return 2.0 * sum + (double)e * kLn2;
}

static inline void psincos(double x, double* sn, double* cs) {
    // reduce to [-pi, pi]
    double tp = 2.0 * kPi;
    double q = x / tp;
    long long qi = (long long)(q >= 0 ? q + 0.5 : q - 0.5);
    double r = x - (double)qi * tp;
    double r2 = r * r;
    double ts = r, ss = r, tc = 1.0, sc = 1.0;
    for (int i = 1; i <= 14; ++i) {
        ts = -ts * r2 / (double)((2 * i) * (2 * i + 1));
        ss = ss + ts;
        tc = -tc * r2 / (double)((2 * i - 1) * (2 * i));
        sc = sc + tc;
    }
    *sn = ss;
    *cs = sc;
}

static inline double pnormal(Rng& g) {
    // Box-Muller
    double u1 = g.uni(), u2 = g.uni();
    if (u1 < 1e-300) u1 = 1e-300;
    double rad = plog(u1) * -2.0;
    // sqrt is a single correctly rounded IEEE operation
    double m = __builtin_sqrt(rad);
    double s, c;
    psincos(2.0 * kPi * u2, &s, &c);
    return m * c;
}

// --------------------------------------------------------------- scene ----
struct Scene {
    uint32_t width = 0, height = 0;
    std::vector<float> pos;            // 2 per point
    std::vector<uint32_t> pos_path;
    std::vector<uint32_t> curve_pos, curve_type, curve_path;
    std::vector<uint32_t> fill_rule, fill_info;
    uint32_t n_points() const { return (uint32_t)pos_path.size(); }
    uint32_t n_curves() const { return (uint32_t)curve_type.size(); }
    uint32_t n_paths() const { return (uint32_t)fill_rule.size(); }

    void add_curve(uint32_t type, const double* xy, uint32_t path) {
        uint32_t np = type & 7u;
        curve_pos.push_back(n_points());
        curve_type.push_back(type);
        curve_path.push_back(path);
        for (uint32_t i = 0; i < np; ++i) {
            pos.push_back((float)xy[2 * i]);
            pos.push_back((float)xy[2 * i + 1]);
            pos_path.push_back(path);
        }
    }
};

struct Params {
    int preset = 0;           // 0 star cubics, 1 mixed, 2 one scene of a mixed batch
    uint64_t seed = 0;
    uint32_t scene_index = 0;
    uint32_t width = 1024, height = 1024;
    uint32_t n_paths = 500;
};

// Preset defaults (sizes named by the configurations they stand for):
//   preset 0: 1024x1024, 500 closed star paths of U{4..16} cubics,
//             radius lognormal(ln 60, 0.5), nonzero, alpha U[0.4,1].
//   preset 1: 4096x4096, 20000 paths, segments geometric(mean 12, cap 256),
//             60/30/10 cubic/quadric/line, 30% even-odd, 5% figure-eights
//             of 2 sub-contours, 2% full-canvas backgrounds, radius
//             lognormal(ln 40, 1.0) clipped to [1, side/2].
// Preset 2 (a batch of uneven scenes): scene `scene_index` of the batch has
// a square canvas with side uniform over {256, 512, 1024, 2048} and a path
// count lognormal(median 200, sigma 1) clipped to [10, 20000]; its paths are
// drawn with the preset-1 generator.
static inline void batch_scene_shape(uint64_t seed, uint32_t scene_index, uint32_t* side, uint32_t* paths) {
    Rng g(mix3(seed ^ 0xB47C4u, scene_index, 0x5CE7Eu));
    static const uint32_t sides[4] = {256, 512, 1024, 2048};
    *side = sides[g.below(4)];
    double p = pexp(plog(200.0) + pnormal(g));
    if (p < 10.0) p = 10.0;
    if (p > 20000.0) p = 20000.0;
    *paths = (uint32_t)p;
}

static inline void preset_defaults(Params& p) {
    if (p.preset == 2) {
        uint32_t side, paths;
        batch_scene_shape(p.seed, p.scene_index, &side, &paths);
        p.preset = 1;
        if (!p.width) p.width = side;
        if (!p.height) p.height = side;
        if (!p.n_paths) p.n_paths = paths;
        return;
    }
    if (p.preset == 0) {
        if (!p.width) p.width = 1024;
        if (!p.height) p.height = 1024;
        if (!p.n_paths) p.n_paths = 500;
    } else {
        if (!p.width) p.width = 4096;
        if (!p.height) p.height = 4096;
        if (!p.n_paths) p.n_paths = 20000;
    }
}

static inline uint32_t pack_color(Rng& g) {
    uint32_t r = g.below(256), gg = g.below(256), b = g.below(256);
    double a = 0.4 + 0.6 * g.uni();
    uint32_t ab = (uint32_t)(a * 255.0);   // truncation, like the reference's u8 cast
    if (ab > 255) ab = 255;
    return r | (gg << 8) | (b << 16) | (ab << 24);
}

// One star-shaped closed contour of n segments around (cx, cy).
static inline void star_contour(Scene& s, Rng& g, uint32_t path, double cx, double cy, double r,
                                uint32_t n, int preset) {
    std::vector<double> ang(n), rad(n);
    for (uint32_t k = 0; k < n; ++k) ang[k] = 2.0 * kPi * g.uni();
    // insertion sort (n <= 256) keeps the generator free of library sorts
    for (uint32_t i = 1; i < n; ++i) {
        double v = ang[i];
        uint32_t j = i;
        while (j > 0 && ang[j - 1] > v) { ang[j] = ang[j - 1]; --j; }
        ang[j] = v;
    }
    for (uint32_t k = 0; k < n; ++k) rad[k] = r * (1.0 + 0.4 * (g.uni() - 0.5));
    std::vector<double> vx(n), vy(n);
    for (uint32_t k = 0; k < n; ++k) {
        double sn, cs;
        psincos(ang[k], &sn, &cs);
        vx[k] = cx + rad[k] * cs;
        vy[k] = cy + rad[k] * sn;
    }
    double sd = 0.3 * r;
    for (uint32_t k = 0; k < n; ++k) {
        uint32_t k1 = (k + 1) % n;
        double x0 = vx[k], y0 = vy[k], x3 = vx[k1], y3 = vy[k1];
        uint32_t type = 4;
        if (preset != 0) {
            double u = g.uni();
            type = u < 0.6 ? 4u : (u < 0.9 ? 3u : 2u);
        }
        double xy[8];
        xy[0] = x0; xy[1] = y0;
        if (type == 4) {
            xy[2] = x0 + (x3 - x0) / 3.0 + sd * pnormal(g);
            xy[3] = y0 + (y3 - y0) / 3.0 + sd * pnormal(g);
            xy[4] = x0 + 2.0 * (x3 - x0) / 3.0 + sd * pnormal(g);
            xy[5] = y0 + 2.0 * (y3 - y0) / 3.0 + sd * pnormal(g);
            xy[6] = x3; xy[7] = y3;
        } else if (type == 3) {
            xy[2] = 0.5 * (x0 + x3) + sd * pnormal(g);
            xy[3] = 0.5 * (y0 + y3) + sd * pnormal(g);
            xy[4] = x3; xy[5] = y3;
        } else {
            xy[2] = x3; xy[3] = y3;
        }
        s.add_curve(type, xy, path);
    }
}

static inline void generate(const Params& in, Scene& s) {
    Params p = in;
    preset_defaults(p);
    s = Scene();
    s.width = p.width;
    s.height = p.height;
    const double W = (double)p.width, H = (double)p.height;
    const double side = W < H ? W : H;
    for (uint32_t pi = 0; pi < p.n_paths; ++pi) {
        Rng g(mix3(p.seed, p.scene_index, pi));
        uint32_t color = pack_color(g);
        double cx = g.uni() * W, cy = g.uni() * H;
        if (p.preset == 0) {
            uint32_t n = 4 + g.below(13);
            double r = pexp(plog(60.0) + 0.5 * pnormal(g));
            if (r < 1.0) r = 1.0;
            if (r > side * 0.5) r = side * 0.5;
            s.fill_rule.push_back(0);
            s.fill_info.push_back(color);
            star_contour(s, g, pi, cx, cy, r, n, 0);
            continue;
        }
        double u_kind = g.uni();
        uint32_t rule = g.uni() < 0.3 ? 1u : 0u;
        s.fill_rule.push_back(rule);
        s.fill_info.push_back(color);
        if (u_kind < 0.02) {
            // full-canvas background: rectangle one pixel outside the canvas
            double xs[5] = {-1.0, W + 1.0, W + 1.0, -1.0, -1.0};
            double ys[5] = {-1.0, -1.0, H + 1.0, H + 1.0, -1.0};
            for (int k = 0; k < 4; ++k) {
                double xy[4] = {xs[k], ys[k], xs[k + 1], ys[k + 1]};
                s.add_curve(2, xy, pi);
            }
            continue;
        }
        // geometric number of segments on {1,2,...} with mean 12, cap 256
        uint32_t n = 1;
        while (n < 256 && g.uni() >= 1.0 / 12.0) ++n;
        double r = pexp(plog(40.0) + 1.0 * pnormal(g));
        if (r < 1.0) r = 1.0;
        if (r > side * 0.5) r = side * 0.5;
        if (u_kind < 0.07) {
            // figure-eight: two overlapping sub-contours of the same orientation
            double sn, cs;
            psincos(2.0 * kPi * g.uni(), &sn, &cs);
            double dx = 0.5 * r * cs, dy = 0.5 * r * sn;
            uint32_t h = (n + 1) / 2;
            star_contour(s, g, pi, cx - dx, cy - dy, r, h, 1);
            star_contour(s, g, pi, cx + dx, cy + dy, r, h, 1);
        } else {
            star_contour(s, g, pi, cx, cy, r, n, 1);
        }
    }
}

}  // namespace srsynth
