// Seeded procedural room: the input fixture of the GI chain.
//
// The reference renders assimp scenes (CrytekSponza by default) through OpenGL rasterisation:
// RasterizationStage::render (RasterizationStage.cpp:151-277) writes the camera G-buffer and,
// with renderRSM = true, the light's reflective shadow map; the ISM points come from hardware
// tessellation (ism.tesc/ism.tese/ism.geom:49-70). None of that is graphics work we can run
// here, so this file ray-casts an analytic scene on the host instead and produces the same data
// contracts:
//   * G-buffer: FP32 window depth, octahedral normal (2 floats), RGBA8 albedo.
//   * RSM: FP32 window depth, RGB10_A2 UNORM normal (n*0.5+0.5), RGBA8 diffuse (the flux basis:
//     albedo * cos at the receiver, zero outside the spot cone).
//   * Points: area-uniform over every surface, bucketed round-robin, each packed as
//     vec4(pos, uintBitsToFloat(packUnorm4x8(n*0.5+0.5, r*sqrt(ismCount)/25))) (ism.geom:59-68).
// World units are centimetres (the room is 100 units on a side), which keeps the reference's
// scene-scale constants (radius/25 packing, radius*10 key byte, 0.02 shadow bias, 1/d^4 falloff
// with a 0.001 clamp) in their intended range.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "mlgi.h"
#include "room.h"

namespace {

struct D3 {
    double x, y, z;
};
inline D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 operator*(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 cross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline D3 normalize(D3 a) { return a * (1.0 / std::sqrt(dot(a, a))); }

// 4x4 column-major matrices in double.
struct M4 {
    double m[16];
    double& at(int r, int c) { return m[c * 4 + r]; }
    double at(int r, int c) const { return m[c * 4 + r]; }
};
M4 mul(const M4& a, const M4& b) {
    M4 r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            double s = 0;
            for (int k = 0; k < 4; ++k) s += a.at(i, k) * b.at(k, j);
            r.at(i, j) = s;
        }
    return r;
}
M4 identity() {
    M4 r;
    std::memset(r.m, 0, sizeof(r.m));
    for (int i = 0; i < 4; ++i) r.at(i, i) = 1;
    return r;
}
// Gauss-Jordan with partial pivoting.
M4 inverse(const M4& a) {
    double w[4][8];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            w[i][j] = a.at(i, j);
            w[i][j + 4] = (i == j) ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; ++c) {
        int p = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(w[r][c]) > std::fabs(w[p][c])) p = r;
        if (p != c)
            for (int j = 0; j < 8; ++j) std::swap(w[p][j], w[c][j]);
        double d = w[c][c];
        for (int j = 0; j < 8; ++j) w[c][j] /= d;
        for (int r = 0; r < 4; ++r) {
            if (r == c) continue;
            double f = w[r][c];
            for (int j = 0; j < 8; ++j) w[r][j] -= f * w[c][j];
        }
    }
    M4 r;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) r.at(i, j) = w[i][j + 4];
    return r;
}
// Right-handed view matrix (the glm lookAt convention the reference's cameras use).
M4 look_at(D3 eye, D3 center, D3 up) {
    D3 f = normalize(center - eye);
    D3 s = normalize(cross(f, up));
    D3 u = cross(s, f);
    M4 r = identity();
    r.at(0, 0) = s.x; r.at(0, 1) = s.y; r.at(0, 2) = s.z;
    r.at(1, 0) = u.x; r.at(1, 1) = u.y; r.at(1, 2) = u.z;
    r.at(2, 0) = -f.x; r.at(2, 1) = -f.y; r.at(2, 2) = -f.z;
    r.at(0, 3) = -dot(s, eye);
    r.at(1, 3) = -dot(u, eye);
    r.at(2, 3) = dot(f, eye);
    return r;
}
// OpenGL perspective projection, clip z in [-w, w]; `t` = cot(fovy / 2).
M4 perspective(double t, double aspect, double n, double f) {
    M4 r;
    std::memset(r.m, 0, sizeof(r.m));
    r.at(0, 0) = t / aspect;
    r.at(1, 1) = t;
    r.at(2, 2) = (f + n) / (n - f);
    r.at(2, 3) = 2 * f * n / (n - f);
    r.at(3, 2) = -1;
    return r;
}
void to_float(const M4& a, float* out) {
    for (int i = 0; i < 16; ++i) out[i] = (float)a.m[i];
}

struct Box {
    D3 lo, hi, albedo;
};
struct Sphere {
    D3 c;
    double r;
    D3 albedo;
};
struct Scene {
    D3 wall_albedo[5];  // floor, ceiling, back, left, right
    std::vector<Box> boxes;
    std::vector<Sphere> spheres;
};

constexpr double kRoom = 100.0;

struct Hit {
    double t;
    D3 n, albedo;
};

// Nearest intersection along o + t*d, t > tmin.
bool trace(const Scene& s, D3 o, D3 d, double tmin, Hit& h) {
    h.t = 1e30;
    bool any = false;
    // Room walls, seen from inside. plane axis, value, inward normal
    const int axis[5] = {1, 1, 2, 0, 0};
    const double val[5] = {0, kRoom, 0, 0, kRoom};
    const double nrm[5] = {1, -1, 1, 1, -1};
    for (int w = 0; w < 5; ++w) {
        double oa = axis[w] == 0 ? o.x : axis[w] == 1 ? o.y : o.z;
        double da = axis[w] == 0 ? d.x : axis[w] == 1 ? d.y : d.z;
        if (std::fabs(da) < 1e-300) continue;
        double t = (val[w] - oa) / da;
        if (t <= tmin || t >= h.t) continue;
        D3 p = o + d * t;
        double c[3] = {p.x, p.y, p.z};
        bool inside = true;
        for (int k = 0; k < 3; ++k) {
            if (k == axis[w]) continue;
            if (c[k] < 0 || c[k] > kRoom) inside = false;
        }
        if (!inside) continue;
        h.t = t;
        h.n = axis[w] == 0 ? D3{nrm[w], 0, 0} : axis[w] == 1 ? D3{0, nrm[w], 0} : D3{0, 0, nrm[w]};
        h.albedo = s.wall_albedo[w];
        any = true;
    }
    for (const Box& b : s.boxes) {
        double t0 = tmin, t1 = h.t;
        int enter_axis = -1;
        double enter_sign = 0;
        const double oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
        const double lo[3] = {b.lo.x, b.lo.y, b.lo.z}, hi[3] = {b.hi.x, b.hi.y, b.hi.z};
        bool miss = false;
        for (int k = 0; k < 3 && !miss; ++k) {
            if (std::fabs(dd[k]) < 1e-300) {
                if (oo[k] < lo[k] || oo[k] > hi[k]) miss = true;
                continue;
            }
            double ta = (lo[k] - oo[k]) / dd[k], tb = (hi[k] - oo[k]) / dd[k];
            double sgn = -1;  // entering through the lo face: outward normal is -axis
            if (ta > tb) { std::swap(ta, tb); sgn = 1; }
            if (ta > t0) { t0 = ta; enter_axis = k; enter_sign = sgn; }
            if (tb < t1) t1 = tb;
            if (t0 > t1) miss = true;
        }
        if (miss || enter_axis < 0 || t0 <= tmin || t0 >= h.t) continue;
        h.t = t0;
        h.n = enter_axis == 0 ? D3{enter_sign, 0, 0} : enter_axis == 1 ? D3{0, enter_sign, 0} : D3{0, 0, enter_sign};
        h.albedo = b.albedo;
        any = true;
    }
    for (const Sphere& sp : s.spheres) {
        D3 oc = o - sp.c;
        double b = dot(oc, d), c = dot(oc, oc) - sp.r * sp.r, a = dot(d, d);
        double disc = b * b - a * c;
        if (disc < 0) continue;
        double t = (-b - std::sqrt(disc)) / a;
        if (t <= tmin || t >= h.t) continue;
        h.t = t;
        h.n = normalize((o + d * t) - sp.c);
        h.albedo = sp.albedo;
        any = true;
    }
    return any;
}

Scene make_scene(const mlgi_scene_desc& d, D3 eye, D3 light) {
    std::mt19937_64 rng(d.seed);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    auto alb = [&]() { return D3{0.2 + 0.6 * U(rng), 0.2 + 0.6 * U(rng), 0.2 + 0.6 * U(rng)}; };
    Scene s;
    for (auto& a : s.wall_albedo) a = alb();
    auto clear_of = [&](D3 lo, D3 hi, D3 p, double m) {
        return p.x < lo.x - m || p.x > hi.x + m || p.y < lo.y - m || p.y > hi.y + m || p.z < lo.z - m || p.z > hi.z + m;
    };
    for (int i = 0; i < d.n_boxes; ++i) {
        for (int attempt = 0; attempt < 64; ++attempt) {
            D3 size{8 + 22 * U(rng), 8 + 22 * U(rng), 8 + 22 * U(rng)};
            D3 lo{(kRoom - size.x) * U(rng), (kRoom - size.y) * U(rng), (kRoom - size.z) * U(rng)};
            D3 hi = lo + size;
            D3 a = alb();
            if (clear_of(lo, hi, eye, 3) && clear_of(lo, hi, light, 3)) {
                s.boxes.push_back({lo, hi, a});
                break;
            }
        }
    }
    for (int i = 0; i < d.n_spheres; ++i) {
        for (int attempt = 0; attempt < 64; ++attempt) {
            double r = 4 + 8 * U(rng);
            D3 c{r + (kRoom - 2 * r) * U(rng), r + (kRoom - 2 * r) * U(rng), r + (kRoom - 2 * r) * U(rng)};
            D3 a = alb();
            D3 e = eye - c, l = light - c;
            if (std::sqrt(dot(e, e)) > r + 3 && std::sqrt(dot(l, l)) > r + 3) {
                s.spheres.push_back({c, r, a});
                break;
            }
        }
    }
    return s;
}

inline uint32_t rgba8(D3 c) {
    auto q = [](double v) {
        v = std::min(1.0, std::max(0.0, v));
        return (uint32_t)std::lround(v * 255.0);
    };
    return q(c.x) | (q(c.y) << 8) | (q(c.z) << 16) | (255u << 24);
}
inline uint32_t rgb10a2(D3 n) {
    auto q = [](double v) {
        v = std::min(1.0, std::max(0.0, v * 0.5 + 0.5));
        return (uint32_t)std::lround(v * 1023.0);
    };
    return q(n.x) | (q(n.y) << 10) | (q(n.z) << 20) | (3u << 30);
}
inline void oct_encode(D3 n, float* out) {
    double l1 = std::fabs(n.x) + std::fabs(n.y) + std::fabs(n.z);
    double x = n.x / l1, y = n.y / l1;
    if (n.z < 0) {
        double sx = x >= 0 ? 1 : -1, sy = y >= 0 ? 1 : -1;
        double nx = (1 - std::fabs(y)) * sx, ny = (1 - std::fabs(x)) * sy;
        x = nx;
        y = ny;
    }
    out[0] = (float)x;
    out[1] = (float)y;
}
inline uint32_t pack_unorm4x8(double a, double b, double c, double d) {
    auto q = [](double v) {
        v = std::min(1.0, std::max(0.0, v));
        return (uint32_t)std::lround(v * 255.0);
    };
    return q(a) | (q(b) << 8) | (q(c) << 16) | (q(d) << 24);
}

inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
inline double u01(uint64_t& state) {
    state = splitmix64(state);
    return (double)(state >> 11) * (1.0 / 9007199254740992.0);
}

// A sampleable surface patch: rectangle (origin, edge a, edge b) or sphere.
struct Patch {
    int kind;  // 0 rect, 1 sphere
    D3 o, a, b, n;
    double r;
    double area;
};

// sin and cos by their Taylor series (|x| <= pi/2 here), with plain multiplies and adds only, so
// the fixture is identical on every host (libm's trigonometric functions may differ in the last
// bit between platforms; this file is also built with -ffp-contract=off).
void sincos_series(double x, double& s, double& c) {
    double x2 = x * x, term = x, sum = x;
    for (int k = 1; k < 14; ++k) {
        term = -term * x2 / double((2 * k) * (2 * k + 1));
        sum = sum + term;
    }
    s = sum;
    term = 1.0;
    sum = 1.0;
    for (int k = 1; k < 14; ++k) {
        term = -term * x2 / double((2 * k - 1) * (2 * k));
        sum = sum + term;
    }
    c = sum;
}

// Rotate v about the y axis by angle (radians).
D3 rot_y(D3 v, double ang) {
    double c, s;
    sincos_series(ang, s, c);
    return {c * v.x + s * v.z, v.y, -s * v.x + c * v.z};
}

struct Setup {
    M4 view, proj, vp, inv_vp, lview, lproj, lvp, inv_biased, inv_lvp;
    D3 eye, lpos, ldir;
    Scene scene;
    std::vector<Patch> patches;
    std::vector<double> cdf;
    double total = 0, r_world = 0, r_boost = 0;
    int64_t stride = 0;
};

// Room objects from the seed, camera and light matrices, and the area table for point sampling.
Setup make_setup(const mlgi_scene_desc& d) {
    const double pi = 3.14159265358979323846;
    Setup S;
    // Camera: inside the open front of the room looking at the back wall, orbiting the room's
    // vertical axis by camera_orbit_deg.
    const D3 center{50, 50, 50};
    const double orbit = d.camera_orbit_deg * pi / 180.0;
    S.eye = center + rot_y(D3{0, 0, 46}, orbit);
    D3 target = center + rot_y(D3{0, 0, -50}, orbit);
    S.view = look_at(S.eye, target, D3{0, 1, 0});
    double aspect = d.height > 0 ? (double)d.width / d.height : 1.0;
    const double cot30 = std::sqrt(3.0);  // cot(60 degrees / 2)
    S.proj = perspective(cot30, aspect, d.z_near, d.z_far);
    S.vp = mul(S.proj, S.view);
    S.inv_vp = inverse(S.vp);
    // Spot light on the ceiling pointing down, direction jittered by yaw/pitch.
    S.lpos = D3{50, 96, 50};
    double yaw = d.light_yaw_deg * pi / 180.0, pitch = d.light_pitch_deg * pi / 180.0;
    double sp, cp, sy, cy;
    sincos_series(pitch, sp, cp);
    sincos_series(yaw, sy, cy);
    S.ldir = normalize(D3{sp * cy, -cp, sp * sy});
    S.lview = look_at(S.lpos, S.lpos + S.ldir, D3{0, 0, -1});
    S.lproj = perspective(cot30, 1.0, d.z_near, d.z_far);
    S.lvp = mul(S.lproj, S.lview);
    M4 bias = identity();
    bias.at(0, 0) = bias.at(1, 1) = bias.at(2, 2) = 0.5;
    bias.at(0, 3) = bias.at(1, 3) = bias.at(2, 3) = 0.5;
    S.inv_biased = inverse(mul(bias, S.lvp));  // VPLProcessor.cpp:76-82
    S.inv_lvp = inverse(S.lvp);
    S.scene = make_scene(d, S.eye, S.lpos);
    // Surface patches for area-uniform point sampling.
    auto rect = [&](D3 o, D3 a, D3 b, D3 n) {
        Patch p{0, o, a, b, n, 0, std::sqrt(dot(cross(a, b), cross(a, b)))};
        S.patches.push_back(p);
    };
    rect({0, 0, 0}, {kRoom, 0, 0}, {0, 0, kRoom}, {0, 1, 0});        // floor
    rect({0, kRoom, 0}, {kRoom, 0, 0}, {0, 0, kRoom}, {0, -1, 0});   // ceiling
    rect({0, 0, 0}, {kRoom, 0, 0}, {0, kRoom, 0}, {0, 0, 1});        // back
    rect({0, 0, 0}, {0, kRoom, 0}, {0, 0, kRoom}, {1, 0, 0});        // left
    rect({kRoom, 0, 0}, {0, kRoom, 0}, {0, 0, kRoom}, {-1, 0, 0});   // right
    for (const Box& b : S.scene.boxes) {
        D3 sz = b.hi - b.lo;
        rect(b.lo, {sz.x, 0, 0}, {0, sz.y, 0}, {0, 0, -1});
        rect({b.lo.x, b.lo.y, b.hi.z}, {sz.x, 0, 0}, {0, sz.y, 0}, {0, 0, 1});
        rect(b.lo, {0, sz.y, 0}, {0, 0, sz.z}, {-1, 0, 0});
        rect({b.hi.x, b.lo.y, b.lo.z}, {0, sz.y, 0}, {0, 0, sz.z}, {1, 0, 0});
        rect(b.lo, {sz.x, 0, 0}, {0, 0, sz.z}, {0, -1, 0});
        rect({b.lo.x, b.hi.y, b.lo.z}, {sz.x, 0, 0}, {0, 0, sz.z}, {0, 1, 0});
    }
    for (const Sphere& sph : S.scene.spheres) {
        Patch p{1, sph.c, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}, sph.r, 4 * pi * sph.r * sph.r};
        S.patches.push_back(p);
    }
    S.cdf.resize(S.patches.size());
    for (size_t i = 0; i < S.patches.size(); ++i) {
        S.total += S.patches[i].area;
        S.cdf[i] = S.total;
    }
    S.stride = d.n_points == 0 ? 0 : (d.n_points + d.n_buckets - 1) / d.n_buckets;
    S.r_world = d.n_points > 0 ? std::sqrt(S.total / ((double)d.n_points * pi)) : 0.0;
    S.r_boost = S.r_world * std::sqrt((double)d.ism_count);
    return S;
}

void fill_info(const mlgi_scene_desc& d, const Setup& S, mlgi_scene_info* info) {
    to_float(S.view, info->view);
    to_float(S.proj, info->proj);
    to_float(S.inv_vp, info->inv_view_proj);
    to_float(S.lview, info->light_view);
    to_float(S.lproj, info->light_proj);
    to_float(S.inv_biased, info->inv_biased_light_vp);
    info->eye[0] = (float)S.eye.x; info->eye[1] = (float)S.eye.y; info->eye[2] = (float)S.eye.z;
    info->light_pos[0] = (float)S.lpos.x; info->light_pos[1] = (float)S.lpos.y; info->light_pos[2] = (float)S.lpos.z;
    info->light_dir[0] = (float)S.ldir.x; info->light_dir[1] = (float)S.ldir.y; info->light_dir[2] = (float)S.ldir.z;
    info->z_near = d.z_near;
    info->z_far = d.z_far;
    info->total_area = (float)S.total;
    info->point_radius = (float)S.r_world;
    info->bucket_stride = S.stride;
}

bool bad_desc(const mlgi_scene_desc& d) {
    return d.width < 0 || d.height < 0 || d.rsm_width < 0 || d.rsm_height < 0 || d.n_points < 0 || d.n_buckets <= 0 ||
           d.z_near <= 0 || d.z_far <= d.z_near || d.ism_count <= 0;
}

}  // namespace

extern "C" mlgi_status mlgi_scene_generate(const mlgi_scene_desc* desc, mlgi_scene_info* info, float* gbuf_depth,
                                           float* gbuf_normal, uint32_t* gbuf_albedo, float* rsm_depth,
                                           uint32_t* rsm_normal, uint32_t* rsm_diffuse, float* points,
                                           uint32_t* counts) {
    if (!desc || !info) return MLGI_EINVAL;
    const mlgi_scene_desc& d = *desc;
    if (bad_desc(d)) return MLGI_EINVAL;
    const double pi = 3.14159265358979323846;
    const Setup S = make_setup(d);
    fill_info(d, S, info);
    const Scene& scene = S.scene;
    const M4& vp = S.vp;
    const M4& inv_vp = S.inv_vp;
    const M4& inv_lvp = S.inv_lvp;
    const M4& lproj = S.lproj;
    const M4& lview = S.lview;
    const D3 ldir = S.ldir;

    // Ray cast a view: pixel centres, row 0 at the bottom (GL window convention).
    auto cast = [&](const M4& inv, int w, int h, int x, int y, D3& o, D3& dir) {
        double nx = (x + 0.5) / w * 2 - 1, ny = (y + 0.5) / h * 2 - 1;
        double pn[4] = {nx, ny, -1, 1}, pf[4] = {nx, ny, 1, 1};
        double a[4] = {0, 0, 0, 0}, b[4] = {0, 0, 0, 0};
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) {
                a[r] += inv.at(r, c) * pn[c];
                b[r] += inv.at(r, c) * pf[c];
            }
        o = D3{a[0] / a[3], a[1] / a[3], a[2] / a[3]};
        D3 f{b[0] / b[3], b[1] / b[3], b[2] / b[3]};
        dir = normalize(f - o);
    };
    auto window_depth = [](const M4& m, D3 p) {
        double cz = m.at(2, 0) * p.x + m.at(2, 1) * p.y + m.at(2, 2) * p.z + m.at(2, 3);
        double cw = m.at(3, 0) * p.x + m.at(3, 1) * p.y + m.at(3, 2) * p.z + m.at(3, 3);
        return cz / cw * 0.5 + 0.5;
    };

    if (gbuf_depth || gbuf_normal || gbuf_albedo) {
#pragma omp parallel for schedule(dynamic, 4)
        for (int y = 0; y < d.height; ++y) {
            for (int x = 0; x < d.width; ++x) {
                D3 o, dir;
                cast(inv_vp, d.width, d.height, x, y, o, dir);
                Hit h;
                size_t i = (size_t)y * d.width + x;
                if (trace(scene, o, dir, 0.0, h)) {
                    D3 p = o + dir * h.t;
                    if (gbuf_depth) gbuf_depth[i] = (float)window_depth(vp, p);
                    if (gbuf_normal) oct_encode(h.n, gbuf_normal + 2 * i);
                    if (gbuf_albedo) gbuf_albedo[i] = rgba8(h.albedo);
                } else {
                    if (gbuf_depth) gbuf_depth[i] = 1.0f;
                    if (gbuf_normal) { gbuf_normal[2 * i] = 0.0f; gbuf_normal[2 * i + 1] = 0.0f; }
                    if (gbuf_albedo) gbuf_albedo[i] = 0u;
                }
            }
        }
    }
    if (rsm_depth || rsm_normal || rsm_diffuse) {
        const double cos_cone = std::sqrt(3.0) / 2.0;  // cos(30 degrees), the spot's half angle
#pragma omp parallel for schedule(dynamic, 4)
        for (int y = 0; y < d.rsm_height; ++y) {
            for (int x = 0; x < d.rsm_width; ++x) {
                D3 o, dir;
                cast(inv_lvp, d.rsm_width, d.rsm_height, x, y, o, dir);
                Hit h;
                size_t i = (size_t)y * d.rsm_width + x;
                if (trace(scene, o, dir, 0.0, h)) {
                    D3 p = o + dir * h.t;
                    double cosr = std::max(0.0, -dot(h.n, dir));
                    double in_cone = dot(dir, ldir) >= cos_cone ? 1.0 : 0.0;
                    if (rsm_depth) rsm_depth[i] = (float)window_depth(mul(lproj, lview), p);
                    if (rsm_normal) rsm_normal[i] = rgb10a2(h.n);
                    if (rsm_diffuse) rsm_diffuse[i] = rgba8(h.albedo * (cosr * in_cone));
                } else {
                    if (rsm_depth) rsm_depth[i] = 1.0f;
                    if (rsm_normal) rsm_normal[i] = 0u;
                    if (rsm_diffuse) rsm_diffuse[i] = 0u;
                }
            }
        }
    }

    const std::vector<Patch>& patches = S.patches;
    const std::vector<double>& cdf = S.cdf;
    const double total = S.total;
    const int64_t stride = S.stride;
    const double r_boost = S.r_boost;

    if (counts) {
        for (int b = 0; b < d.n_buckets; ++b) {
            int64_t c = d.n_points / d.n_buckets + (b < d.n_points % d.n_buckets ? 1 : 0);
            counts[b] = (uint32_t)c;
        }
    }
    if (points) {
        std::memset(points, 0, sizeof(float) * 4 * (size_t)stride * d.n_buckets);
        const uint64_t base = splitmix64(d.seed ^ 0x5EEDF00Dull);
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < d.n_points; ++k) {
            uint64_t st = base ^ ((uint64_t)k * 0xD1B54A32D192ED03ull);
            double u0 = u01(st) * total, u1 = u01(st), u2 = u01(st);
            size_t pi_ = (size_t)(std::lower_bound(cdf.begin(), cdf.end(), u0) - cdf.begin());
            if (pi_ >= patches.size()) pi_ = patches.size() - 1;
            const Patch& pt = patches[pi_];
            D3 pos, n;
            if (pt.kind == 0) {
                pos = pt.o + pt.a * u1 + pt.b * u2;
                n = pt.n;
            } else {
                // uniform direction by Marsaglia's method (rejection in the unit disk, sqrt only)
                double a = 2 * u1 - 1, b = 2 * u2 - 1, q = a * a + b * b;
                while (q >= 1.0 || q == 0.0) {
                    a = 2 * u01(st) - 1;
                    b = 2 * u01(st) - 1;
                    q = a * a + b * b;
                }
                const double r2 = 2 * std::sqrt(1 - q);
                n = D3{a * r2, b * r2, 1 - 2 * q};
                pos = pt.o + n * pt.r;
            }
            uint32_t w = pack_unorm4x8(n.x * 0.5 + 0.5, n.y * 0.5 + 0.5, n.z * 0.5 + 0.5, r_boost / 25.0);
            int64_t b = k % d.n_buckets, slot = k / d.n_buckets;
            float* e = points + 4 * (b * stride + slot);
            e[0] = (float)pos.x;
            e[1] = (float)pos.y;
            e[2] = (float)pos.z;
            std::memcpy(&e[3], &w, 4);
        }
    }
    return MLGI_OK;
}

namespace mlgi {

mlgi_status build_room(const mlgi_scene_desc& d, RoomGPU* room, mlgi_scene_info* info) {
    if (!room || bad_desc(d)) return MLGI_EINVAL;
    const Setup S = make_setup(d);
    if ((int)S.scene.boxes.size() > kRoomMaxBoxes || (int)S.scene.spheres.size() > kRoomMaxSpheres) return MLGI_EINVAL;
    std::memset(room, 0, sizeof(*room));
    auto put3 = [](float* o, D3 v) { o[0] = (float)v.x; o[1] = (float)v.y; o[2] = (float)v.z; };
    for (int w = 0; w < 5; ++w) put3(room->wall_albedo[w], S.scene.wall_albedo[w]);
    room->n_boxes = (int)S.scene.boxes.size();
    room->n_spheres = (int)S.scene.spheres.size();
    for (int i = 0; i < room->n_boxes; ++i) {
        put3(room->box_lo[i], S.scene.boxes[i].lo);
        put3(room->box_hi[i], S.scene.boxes[i].hi);
        put3(room->box_albedo[i], S.scene.boxes[i].albedo);
    }
    for (int i = 0; i < room->n_spheres; ++i) {
        put3(room->sph_c[i], S.scene.spheres[i].c);
        room->sph_r[i] = (float)S.scene.spheres[i].r;
        put3(room->sph_albedo[i], S.scene.spheres[i].albedo);
    }
    room->n_patches = (int)S.patches.size();
    for (int i = 0; i < room->n_patches; ++i) {
        const Patch& p = S.patches[i];
        put3(room->patch_o[i], p.o);
        put3(room->patch_a[i], p.a);
        put3(room->patch_b[i], p.b);
        put3(room->patch_n[i], p.n);
        room->patch_r[i] = (float)p.r;
        room->patch_kind[i] = p.kind;
        room->cdf[i] = (float)S.cdf[i];
    }
    to_float(S.vp, room->vp);
    to_float(S.inv_vp, room->inv_vp);
    to_float(S.lvp, room->lvp);
    to_float(S.inv_lvp, room->inv_lvp);
    put3(room->light_dir, S.ldir);
    room->cos_cone = (float)(std::sqrt(3.0) / 2.0);
    room->total_area = (float)S.total;
    room->r_boost = (float)S.r_boost;
    room->point_seed = splitmix64(d.seed ^ 0x5EEDF00Dull);
    if (info) fill_info(d, S, info);
    return MLGI_OK;
}

}  // namespace mlgi
