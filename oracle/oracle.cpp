// CPU oracle for the many-lights GI hot path -- TEST INFRASTRUCTURE ONLY.
//
// A C++ restatement of the reference's GLSL compute shaders, one function per shader, templated
// on the scalar type: T = float reproduces the reference's FP32 arithmetic in a fixed operation
// order (built with -ffp-contract=off, so every CUDA kernel that claims bit-exactness can be
// compared word for word), T = double is the FP64 oracle used for the radiance tolerance.
// Only the test suite, the smoke check and the benchmark's CPU-baseline leg load this library;
// the product never links it.
//
// Parity status: the reference ships no tests, fixtures or golden vectors for this path, so this
// restatement is pinned by hand-derived known answers (tests/test_oracle_kat.py) and, where the
// reference shaders compile as C++ through oracle/ref_shim.hpp, by the reference's own shader
// source (oracle/build_ref.py).
//
// Followed files (paths inside the reference project):
//   data/shaders/gi/vpl_processor.comp:41-72           -> vpl_process()
//   data/shaders/common/floatpacking.glsl:5-76         -> pack3SN / unpack3SN / half packing
//   data/shaders/ism/ism_utils.glsl:5-40               -> lookAtRH / paraboloid_project
//   data/shaders/ism/ism.comp:54-139                   -> ism_splat()
//   data/shaders/ism/pull.comp:20-126                  -> pull_level()
//   data/shaders/ism/push.comp:44-165                  -> push_level()
//   source/mfs-painters/multiframepainter/ImperfectShadowmap.cpp:121-192 -> pullpush()
//   data/shaders/gi/final_gathering.comp:63-135        -> final_gather()
//   source/mfs-painters/multiframepainter/GIStage.cpp:261-306 (dispatch geometry)
//
// Generalisations (each reduces to the reference for its constants):
//   * VPL count N replaces the constant 1024 (vpl_processor.comp:14, ism.comp:12, ...).
//   * The ISM grid is gx x gy tiles (the reference's ismIndices1d square grid when gx == gy),
//     the ISM size s replaces 2048/ismIndices1d, and the push ISM-border rule compares
//     floor(coord / (s >> (level+1))) -- push.comp:83 hard-codes s = 64 as a shift by 6-(level+1).
//   * The number of pull-push levels L replaces the constant 6 (ImperfectShadowmap.cpp:128,155).
//   * Interleave factor I replaces the constant 4 (final_gathering.comp:53), and class c reads the
//     VPL slice [c*N/I^2, (c+1)*N/I^2) (the "no culling" light list of final_gathering.comp:93-98).
//   * The G-buffer normal is octahedral-encoded (2 floats) instead of RGB10_A2 (n*0.5+0.5).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "glsl.hpp"

using namespace glsl;

namespace {

template <class T> using V2 = tvec2<T>;
template <class T> using V3 = tvec3<T>;
template <class T> using V4 = tvec4<T>;

// ---- floatpacking.glsl ----------------------------------------------------------------------
// pack3UNToFloat (floatpacking.glsl:26-38): 10:10:10 fields, z offset by +1.5 and scaled by 1021.
template <class T> uint pack3UN(V3<T> c) {
    uint u = to_uint(c.x * T(1023) + T(0.5));
    u |= to_uint(c.y * T(1023) + T(0.5)) << 10;
    u |= to_uint(c.z * T(1021) + T(1.5)) << 20;
    return u;
}
template <class T> uint pack3SN(V3<T> n) { return pack3UN(n * T(0.5) + T(0.5)); }
// unpack3UNFromFloat / unpack3SNFromFloat (floatpacking.glsl:46-66)
template <class T> V3<T> unpack3SN(uint u) {
    T a = T(u & 0x3FFu) / T(1023);
    T b = T((u >> 10) & 0x3FFu) / T(1023);
    T c = (T((u >> 20) & 0x3FFu) - T(1.5)) / T(1021);
    return V3<T>(a, b, c) * T(2) - T(1);
}

// ---- ism_utils.glsl -------------------------------------------------------------------------
template <class T> tmat3<T> lookAtRH(V3<T> n) {
    V3<T> up(T(0), T(1), T(0.01f));
    V3<T> f = n;
    V3<T> s = normalize(cross(f, up));
    V3<T> u = cross(s, f);
    return transpose(tmat3<T>(s, u, -f));
}

// paraboloid_project (ism_utils.glsl:15-40) with a gx x gy tile grid.
template <class T>
V3<T> paraboloid_project(V3<T> rel, T dist, V3<T> n, T zFar, T ismIndex, int gx, int gy, bool preserveSign) {
    tmat3<T> view = lookAtRH(n);
    V3<T> v = view * rel;
    T signOfV = gsign(v.z);
    v = v / dist;
    v.z = T(1) - v.z;
    v.x = v.x / v.z;
    v.y = v.y / v.z;
    v.z = dist / zFar;
    if (preserveSign) v.z = v.z * -signOfV;
    v.x = v.x + T(1);
    v.y = v.y + T(1);
    v.x = v.x / T(2);
    v.y = v.y / T(2);
    T y = T(to_int(ismIndex / T(gx)));
    int tx = to_int(ismIndex - y * T(gx));
    int ty = to_int(y);
    v.x = v.x + T(tx);
    v.y = v.y + T(ty);
    v.x = v.x / T(gx);
    v.y = v.y / T(gy);
    return v;
}

inline void atomic_min_u32(uint32_t* p, uint32_t v) {
    uint32_t cur = __atomic_load_n(p, __ATOMIC_RELAXED);
    while (v < cur && !__atomic_compare_exchange_n(p, &cur, v, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
    }
}

int set_threads(int threads) {
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
    return threads;
#else
    (void)threads;
    return 1;
#endif
}

// ---- S1: vpl_processor.comp:41-72 -----------------------------------------------------------
template <class T>
void vpl_process(int rsm_w, int rsm_h, const float* depth, const uint32_t* normal10, const uint32_t* diffuse8, int n,
                 const T* inv_bpv, T light_intensity, int shuffle, const int32_t* perm, T* pos_out, T* nrm_out,
                 T* col_out, uint32_t* packed_normal_out) {
    tmat4<T> m = tmat4<T>::from(inv_bpv);
    const uint s1d = to_uint(std::ceil(std::sqrt(T(n))));
    const uint work = (uint)n;  // dispatch n/64 groups of 64 invocations
    const uint ax = s1d, ay = work / s1d;
    for (int i = 0; i < n; ++i) {
        uint idx = (uint)i;
        uint tcx = (idx % ax) * (uint)rsm_w / ax;
        uint tcy = (idx / ax) * (uint)rsm_h / ay;
        T tfx = T(tcx) / T(rsm_w);
        T tfy = T(tcy) / T(rsm_h);
        V3<T> diffuse(T(0)), normal;
        T d = T(0);
        uint nbits = 0;
        if (tcx < (uint)rsm_w && tcy < (uint)rsm_h) {  // texelFetch out of range reads zero
            size_t t = (size_t)tcy * rsm_w + tcx;
            uint dw = diffuse8[t];
            diffuse = V3<T>(T(dw & 0xFFu) / T(255), T((dw >> 8) & 0xFFu) / T(255), T((dw >> 16) & 0xFFu) / T(255));
            nbits = normal10[t];
            d = T(depth[t]);
        }
        normal = V3<T>(T(nbits & 0x3FFu) / T(1023), T((nbits >> 10) & 0x3FFu) / T(1023),
                       T((nbits >> 20) & 0x3FFu) / T(1023)) * T(2) - T(1);
        V4<T> wc = m * V4<T>(tfx, tfy, d, T(1));
        V3<T> pos(wc.x / wc.w, wc.y / wc.w, wc.z / wc.w);
        V3<T> color = diffuse * light_intensity;
        uint ri = shuffle ? (uint)perm[i] : idx;
        uint pn = pack3SN(normal);
        V3<T> un = unpack3SN<T>(pn);
        pos_out[3 * ri + 0] = pos.x; pos_out[3 * ri + 1] = pos.y; pos_out[3 * ri + 2] = pos.z;
        nrm_out[3 * ri + 0] = un.x; nrm_out[3 * ri + 1] = un.y; nrm_out[3 * ri + 2] = un.z;
        col_out[3 * ri + 0] = color.x; col_out[3 * ri + 1] = color.y; col_out[3 * ri + 2] = color.z;
        packed_normal_out[ri] = pn;
    }
}

// ---- S3: ism.comp:54-139 --------------------------------------------------------------------
struct SplatParams {
    int n_vpl;             // totalVplCount
    int vpl_start, vpl_end;
    int scale_isms, points_only_scaled;
    int gx, gy, atlas_w, atlas_h;
    int64_t bucket_stride;  // imageSize(pointBuffer).x / sampledVplCount
    int n_groups;           // dispatched work groups (sampledVplCount)
    int64_t n_entries;      // imageSize(pointBuffer).x
};

// issued (optional): the number of imageAtomicMin calls that land inside the atlas.
template <class T>
void ism_splat(const float* points, const uint32_t* counts, const T* vpl_pos, const uint32_t* vpl_pn, const SplatParams& p,
               T zFar, uint32_t* atlas, int threads, int64_t* issued = nullptr) {
    const int vplCount = p.vpl_end - p.vpl_start;
    const int maxTest = 16, maxCollect = 4;
    int64_t n_issued = 0;
#pragma omp parallel for schedule(dynamic, 4) num_threads(set_threads(threads)) reduction(+ : n_issued)
    for (int wg = 0; wg < p.n_groups; ++wg) {
        if (p.points_only_scaled && wg > vplCount) continue;
        V3<T> vp[16];
        uint vn[16];
        int vid[16];
        for (int l = 0; l < maxTest; ++l) {
            int index = (wg + l) % p.n_vpl;
            if (p.points_only_scaled) {
                index %= vplCount;
                index += p.vpl_start;
            }
            vid[l] = index;
            vp[l] = V3<T>(vpl_pos[3 * index], vpl_pos[3 * index + 1], vpl_pos[3 * index + 2]);
            vn[l] = vpl_pn[index];
        }
        // A counter may run past its bucket (ism.geom:65-67 does not bound it): the loop then reads
        // the next buckets' entries, and past the end of the buffer an imageLoad returns zero. All
        // such points are the same zero point, and splatting it again changes no key (atomicMin),
        // so the loop stops after one of them.
        const int64_t first = (int64_t)wg * p.bucket_stride;
        const int64_t avail = std::max<int64_t>(0, p.n_entries - first);
        const uint cnt = (int64_t)counts[wg] > avail ? (uint)(avail + 1) : counts[wg];
        static const float zero[4] = {0.f, 0.f, 0.f, 0.f};
        for (uint j = 0; j < cnt; ++j) {
            const float* pt = (int64_t)j < avail ? points + 4 * (first + j) : zero;
            V3<T> position{T(pt[0]), T(pt[1]), T(pt[2])};
            V4<T> nr = unpackUnorm4x8<T>(floatBitsToUint(pt[3]));
            V3<T> pointNormal = V3<T>(nr.x, nr.y, nr.z) * T(2) - T(1);
            T pointRadius = nr.w * T(25);
            int used[4];
            int found = 0;
            for (int i = 0; i < maxTest; ++i) {
                V3<T> n2 = unpack3SN<T>(vn[i]);
                V3<T> rel = position - vp[i];
                bool cull = dot(n2, rel) < T(0) || dot(pointNormal, -rel) < T(0);
                if (!cull && found < maxCollect) used[found++] = i;
            }
            for (int k = 0; k < found; ++k) {
                int l = used[k];
                int gid = vid[l];
                V3<T> n2 = unpack3SN<T>(vn[l]);
                V3<T> rel = position - vp[l];
                T dist = length(rel);
                T ismIndex = p.scale_isms ? T(gid) - T(p.vpl_start) : T(gid);
                V3<T> v = paraboloid_project(rel, dist, n2, zFar, ismIndex, p.gx, p.gy, true);
                v.x = v.x * T(p.atlas_w);
                v.y = v.y * T(p.atlas_h);
                v.z = v.z * T(1 << 24);
                uint key = to_uint(v.z) << 8;
                key |= to_uint(pointRadius * T(10) / std::sqrt(T(maxCollect)));
                int tx = to_int(v.x), ty = to_int(v.y);
                if (tx < 0 || ty < 0 || tx >= p.atlas_w || ty >= p.atlas_h) continue;  // image op out of range: no-op
                atomic_min_u32(&atlas[(size_t)ty * p.atlas_w + tx], key);
                ++n_issued;
            }
        }
    }
    if (issued) *issued = n_issued;
}

// ---- S4/S5: pull.comp / push.comp driven by ImperfectShadowmap::pullpush --------------------
template <class T> struct Texel {
    T r, g, b;
    uint a;  // packHalf2x16 bits of the displacement vector
};

template <class T> inline T pow2neg(int level) { return std::ldexp(T(1), -level); }

template <class T>
void pull_level(int level, const uint32_t* keys, const Texel<T>* in, int in_w, Texel<T>* out, int out_w, int out_h,
                T zFar, int ismPixelSize, int threads) {
    static const int off[4][2] = {{0, 0}, {0, 1}, {1, 0}, {1, 1}};
#pragma omp parallel for schedule(static) num_threads(set_threads(threads))
    for (int oy = 0; oy < out_h; ++oy) {
        for (int ox = 0; ox < out_w; ++ox) {
            T depthSamples[4], maxDepths[4], radiuses[4];
            V2<T> disps[4];
            bool valid[4];
            for (int i = 0; i < 4; ++i) {
                int ix = ox * 2 + off[i][0], iy = oy * 2 + off[i][1];
                T depthSample, radius, maxDepth;
                V2<T> disp;
                if (level == 1) {
                    uint k = keys[(size_t)iy * in_w + ix];
                    depthSample = T(k >> 8) / T(1 << 24);
                    radius = T(k & 0xFFu) / T(10);
                    disp = V2<T>(T(0), T(0));
                    T magic = T(0.6f);
                    maxDepth = depthSample + (radius * T(2)) / zFar * magic;
                    T distToCamera = depthSample * zFar;
                    radius = radius / distToCamera / T(3.14f) * T(ismPixelSize);
                    radius = radius * T(1.3f);
                    radius = gmin(radius, T(15));
                } else {
                    const Texel<T>& t = in[(size_t)iy * in_w + ix];
                    depthSample = t.r;
                    maxDepth = t.g;
                    V2<float> d = unpackHalf2x16(t.a);
                    disp = V2<T>(T(d.x), T(d.y));
                    radius = t.b;
                }
                V2<T> nd((T(ix) + T(0.5) + disp.x) / T(2) - (T(ox) + T(0.5)),
                         (T(iy) + T(0.5) + disp.y) / T(2) - (T(oy) + T(0.5)));
                T dist = length(nd);
                T scaledRadius = radius * pow2neg<T>(level);
                bool pass = dist <= scaledRadius;
                depthSamples[i] = depthSample;
                maxDepths[i] = maxDepth;
                radiuses[i] = radius;
                disps[i] = nd;
                valid[i] = depthSample != T(1);
                valid[i] = valid[i] && pass;
            }
            T minimum = T(INFINITY);
            T maxDepth = T(0);  // read below only when some sample is valid
            for (int i = 0; i < 4; ++i) {
                if (!valid[i]) continue;
                minimum = gmin(depthSamples[i], minimum);
                if (minimum == depthSamples[i]) maxDepth = maxDepths[i];
            }
            for (int i = 0; i < 4; ++i)
                if (depthSamples[i] > maxDepth) valid[i] = false;
            T depthAcc = T(0), radiusAcc = T(0), maxValid = T(0);
            V2<T> dispAcc(T(0), T(0));
            uint numValid = 0;
            for (int i = 0; i < 4; ++i) {
                if (!valid[i]) continue;
                depthAcc = depthAcc + depthSamples[i];
                dispAcc = dispAcc + disps[i];
                radiusAcc = radiusAcc + radiuses[i];
                maxValid = gmax(maxValid, maxDepths[i]);
                numValid++;
            }
            Texel<T> r;
            if (numValid > 0) {
                T nv = T(numValid);
                r.r = depthAcc / nv;
                r.g = maxValid;
                r.b = radiusAcc / nv;
                r.a = packHalf2x16(float(dispAcc.x / nv), float(dispAcc.y / nv));
            } else {
                r.r = T(1); r.g = T(0); r.b = T(0); r.a = 0u;
            }
            out[(size_t)oy * out_w + ox] = r;
        }
    }
}

inline int floordiv(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

// push.comp:44-165 for one level. `same` is the pull level at this level (level >= 1), keys for
// level 0; `coarse` is the level+1 input (pull level L for the first push, else push level+1).
template <class T>
void push_level(int level, const uint32_t* keys, const Texel<T>* same, const Texel<T>* coarse, int c_w, int c_h,
                Texel<T>* out, T* final_out, int o_w, int o_h, int ism_size, int threads) {
    static const int off[4][2] = {{0, 0}, {0, 1}, {1, 1}, {1, 0}};
    static const int weightsX[4] = {9, 3, 1, 3};
    const int ismC = ism_size >> (level + 1);  // ISM width in texels at the coarser level
    const int ngx = o_w / 8 / 2 + 1, ngy = o_h / 8 / 2 + 1;  // ImperfectShadowmap.cpp:174
#pragma omp parallel for schedule(static) num_threads(set_threads(threads))
    for (int gy = 0; gy < ngy * 8; ++gy) {
        for (int gx = 0; gx < ngx * 8; ++gx) {
            const int cllx = gx - 1, clly = gy - 1;
            T depths[4], maxDepths[4], radiuses[4];
            V2<T> dispC[4];
            for (int i = 0; i < 4; ++i) {
                int cx = cllx + off[i][0], cy = clly + off[i][1];
                if (cx >= 0 && cy >= 0 && cx < c_w && cy < c_h) {  // imageLoad out of range reads zero
                    const Texel<T>& t = coarse[(size_t)cy * c_w + cx];
                    depths[i] = t.r; maxDepths[i] = t.g; radiuses[i] = t.b;
                    V2<float> d = unpackHalf2x16(t.a);
                    dispC[i] = V2<T>(T(d.x), T(d.y));
                } else {
                    depths[i] = T(0); maxDepths[i] = T(0); radiuses[i] = T(0);
                    dispC[i] = V2<T>(T(0), T(0));
                }
            }
            for (int op = 0; op < 4; ++op) {
                const int px = gx * 2 - 1 + off[op][0], py = gy * 2 - 1 + off[op][1];
                if (px < 0 || py < 0 || px >= o_w || py >= o_h) continue;  // imageStore out of range: no-op
                int w[4];
                for (int i = 0; i < 4; ++i) w[i] = weightsX[(i - op + 4) % 4];
                const int ox = px / 2, oy = py / 2;
                for (int i = 0; i < 4; ++i) {
                    int ix = cllx + off[i][0], iy = clly + off[i][1];
                    if (floordiv(ox, ismC) != floordiv(ix, ismC) || floordiv(oy, ismC) != floordiv(iy, ismC)) w[i] = 0;
                }
                for (int i = 0; i < 4; ++i)
                    if (depths[i] == T(1)) w[i] = 0;
                V2<T> dv[4];
                for (int i = 0; i < 4; ++i) {
                    V2<T> ct((T(cllx + off[i][0]) + T(0.5)) * T(2), (T(clly + off[i][1]) + T(0.5)) * T(2));
                    V2<T> tt(T(px) + T(0.5), T(py) + T(0.5));
                    dv[i] = ct - tt + dispC[i] * T(2);
                    T dist = length(dv[i]);
                    T radius = radiuses[i] * pow2neg<T>(level);
                    if (dist > radius) w[i] = 0;
                }
                T minimum = T(9001);
                T maxDepth = T(0);
                for (int i = 0; i < 4; ++i) {
                    if (w[i] == 0) continue;
                    minimum = gmin(depths[i], minimum);
                    if (minimum == depths[i]) maxDepth = maxDepths[i];
                }
                for (int i = 0; i < 4; ++i)
                    if (depths[i] > maxDepth) w[i] = 0;
                T depthAcc = T(0), radiusAcc = T(0), maxDepthAcc = T(0);
                V2<T> dispAcc(T(0), T(0));
                int weightAcc = 0;
                for (int i = 0; i < 4; ++i) {
                    T wf = T(w[i]);
                    depthAcc = depthAcc + depths[i] * wf;
                    maxDepthAcc = maxDepthAcc + maxDepths[i] * wf;
                    radiusAcc = radiusAcc + radiuses[i] * wf;
                    dispAcc = dispAcc + dv[i] * wf;
                    weightAcc += w[i];
                }
                Texel<T> r;
                T wa = T(weightAcc);
                r.r = depthAcc / wa;
                r.g = maxDepthAcc / wa;
                r.b = radiusAcc / wa;
                r.a = packHalf2x16(float(dispAcc.x / wa), float(dispAcc.y / wa));
                Texel<T> orig;
                if (level == 0) {
                    uint k = keys[(size_t)py * o_w + px];
                    orig.r = T(k >> 8) / T(1 << 24);
                    orig.g = T(0); orig.b = T(0); orig.a = 0u;
                } else {
                    orig = same[(size_t)py * o_w + px];
                }
                bool invalid = orig.r == T(1);
                bool occluded = false;
                for (int i = 0; i < 4; ++i) occluded = occluded || (w[i] > 0 && orig.r > maxDepths[i]);
                bool allInvalid = weightAcc <= 0;
                if (allInvalid || (!invalid && !occluded)) r = orig;
                if (level == 0)
                    final_out[(size_t)py * o_w + px] = r.r;
                else
                    out[(size_t)py * o_w + px] = r;
            }
        }
    }
}

template <class T>
void pullpush(const uint32_t* keys, int W, int H, int ism_size, int levels, T zFar, T* final_out, int threads) {
    std::vector<std::vector<Texel<T>>> pull(levels + 1), push(levels + 1);
    for (int l = 1; l <= levels; ++l) pull[l].resize((size_t)(W >> l) * (H >> l));
    for (int l = 1; l < levels; ++l) push[l].resize((size_t)(W >> l) * (H >> l));
    for (int l = 1; l <= levels; ++l)
        pull_level<T>(l, keys, l == 1 ? nullptr : pull[l - 1].data(), W >> (l - 1), pull[l].data(), W >> l, H >> l,
                      zFar, ism_size, threads);
    for (int l = levels - 1; l >= 0; --l) {
        const Texel<T>* coarse = (l == levels - 1) ? pull[l + 1].data() : push[l + 1].data();
        push_level<T>(l, keys, l == 0 ? nullptr : pull[l].data(), coarse, W >> (l + 1), H >> (l + 1),
                      l == 0 ? nullptr : push[l].data(), final_out, W >> l, H >> l, ism_size, threads);
    }
}

// ---- S7: final_gathering.comp:63-135 --------------------------------------------------------
struct FgParams {
    int width, height;
    int n_vpl;
    int vpl_count;        // vplEndIndex - vplStartIndex (normalisation)
    int ism_index_offset; // SCALE_ISMS ? vplStartIndex : 0
    int interleave;
    int shadowing;
    int gx, gy, atlas_w, atlas_h;
    int tile;             // 0: no culling; else tile edge in de-interleaved pixels
    double influence_cutoff;  // 0: no influence-radius culling
    int accurate_world;       // reconstruct world positions exactly rounded (see frag_world_rounded)
    // clustered culling: a pixel keeps the VPLs whose bit is set in its cluster's mask
    const uint32_t* cl_masks = nullptr;
    const uint8_t* cl_slice = nullptr;
    int cl_tiles_x = 0, cl_words = 0;
};

template <class T> V3<T> oct_decode(T ex, T ey) {
    V3<T> n(ex, ey, T(1) - std::fabs(ex) - std::fabs(ey));
    if (n.z < T(0)) {
        T sx = ex >= T(0) ? T(1) : T(-1), sy = ey >= T(0) ? T(1) : T(-1);
        n.x = (T(1) - std::fabs(ey)) * sx;
        n.y = (T(1) - std::fabs(ex)) * sy;
    }
    return normalize(n);
}

template <class T>
V3<T> frag_world(const FgParams& p, const tmat4<T>& inv_vp, const float* depth, int x, int y);

// World position evaluated exactly (in FP64) and rounded once to T: what a compensated FP32
// evaluation of inv_vp * ndc delivers. Used to state the error of the GPU's accurate
// reconstruction mode.
template <class T>
V3<T> frag_world_rounded(const FgParams& p, const tmat4<T>& inv_vp, const float* depth, int x, int y) {
    tmat4<double> m;
    for (int i = 0; i < 4; ++i)
        m.c[i] = tvec4<double>(double(inv_vp.c[i].x), double(inv_vp.c[i].y), double(inv_vp.c[i].z), double(inv_vp.c[i].w));
    tvec3<double> w = frag_world<double>(p, m, depth, x, y);
    return V3<T>(T(w.x), T(w.y), T(w.z));
}

template <class T>
V3<T> frag_world(const FgParams& p, const tmat4<T>& inv_vp, const float* depth, int x, int y) {
    T ux = T(x) / T(p.width), uy = T(y) / T(p.height);
    T d = T(depth[(size_t)y * p.width + x]);
    V4<T> ndc = V4<T>(ux, uy, d, T(1)) * T(2) - T(1);
    V4<T> w = inv_vp * ndc;
    return V3<T>(w.x / w.w, w.y / w.w, w.z / w.w);
}

template <class T>
void final_gather(const FgParams& p, const float* depth, const float* nrm_oct, const T* inv_vp16, const T* vpos,
                  const T* vnrm, const T* vcol, const float* atlas, T zFar, T gi_intensity, T clamp_value, T* out,
                  int threads) {
    const tmat4<T> inv_vp = tmat4<T>::from(inv_vp16);
    const int I = p.interleave, I2 = I * I;
    const int per_class = p.n_vpl / I2;
    const int sw = (p.width + I - 1) / I, sh = (p.height + I - 1) / I;  // de-interleaved sub-image bounds
    const int tile = p.tile > 0 ? p.tile : std::max(sw, sh);
    const int ntx = (sw + tile - 1) / tile, nty = (sh + tile - 1) / tile;
    const int ntiles = ntx * nty * I2;
#pragma omp parallel for schedule(dynamic, 1) num_threads(set_threads(threads))
    for (int t = 0; t < ntiles; ++t) {
        const int c = t / (ntx * nty);
        const int tt = t % (ntx * nty);
        const int tix = tt % ntx, tiy = tt / ntx;
        const int cx = c % I, cy = c / I;
        // pixels of class c in this tile
        std::vector<int> px, py;
        for (int j = tiy * tile; j < std::min(sh, (tiy + 1) * tile); ++j)
            for (int i = tix * tile; i < std::min(sw, (tix + 1) * tile); ++i) {
                int x = i * I + cx, y = j * I + cy;
                if (x < p.width && y < p.height) { px.push_back(x); py.push_back(y); }
            }
        if (px.empty()) continue;
        std::vector<V3<T>> world(px.size());
        for (size_t k = 0; k < px.size(); ++k)
            world[k] = p.accurate_world ? frag_world_rounded(p, inv_vp, depth, px[k], py[k])
                                        : frag_world(p, inv_vp, depth, px[k], py[k]);
        // per-tile VPL list (culling mirrors the CUDA kernel's rule; tile == 0 keeps every VPL)
        std::vector<int> list;
        V3<T> bmin = world[0], bmax = world[0];
        for (auto& w : world) {
            bmin = V3<T>(std::min(bmin.x, w.x), std::min(bmin.y, w.y), std::min(bmin.z, w.z));
            bmax = V3<T>(std::max(bmax.x, w.x), std::max(bmax.y, w.y), std::max(bmax.z, w.z));
        }
        for (int k = 0; k < per_class; ++k) {
            int vi = c * per_class + k;
            if (p.tile > 0) {
                V3<T> vp(vpos[3 * vi], vpos[3 * vi + 1], vpos[3 * vi + 2]);
                V3<T> vn(vnrm[3 * vi], vnrm[3 * vi + 1], vnrm[3 * vi + 2]);
                // hemisphere: the AABB corner farthest along the VPL normal
                V3<T> sup(vn.x > T(0) ? bmax.x : bmin.x, vn.y > T(0) ? bmax.y : bmin.y, vn.z > T(0) ? bmax.z : bmin.z);
                if (dot(vn, sup - vp) < T(-1e-3)) continue;
                if (p.influence_cutoff > 0) {
                    T fl = std::max(vcol[3 * vi], std::max(vcol[3 * vi + 1], vcol[3 * vi + 2]));
                    T r = std::sqrt(std::sqrt(fl / T(p.influence_cutoff)));
                    V3<T> q(std::min(std::max(vp.x, bmin.x), bmax.x), std::min(std::max(vp.y, bmin.y), bmax.y),
                            std::min(std::max(vp.z, bmin.z), bmax.z));
                    V3<T> dq = q - vp;
                    if (dot(dq, dq) > r * r) continue;
                }
            }
            list.push_back(vi);
        }
        for (size_t k = 0; k < px.size(); ++k) {
            const int x = px[k], y = py[k];
            const V3<T> fw = world[k];
            const size_t pix = (size_t)y * p.width + x;
            const V3<T> fn = oct_decode<T>(T(nrm_oct[2 * pix]), T(nrm_oct[2 * pix + 1]));
            V3<T> acc(T(0));
            const uint32_t* cl_row =
                p.cl_masks ? p.cl_masks + ((size_t)((y / 128) * p.cl_tiles_x + x / 128) * 16 + p.cl_slice[pix]) * p.cl_words
                           : nullptr;
            for (int vi : list) {
                if (cl_row && !((cl_row[vi >> 5] >> (vi & 31)) & 1u)) continue;
                V3<T> vp(vpos[3 * vi], vpos[3 * vi + 1], vpos[3 * vi + 2]);
                V3<T> vn(vnrm[3 * vi], vnrm[3 * vi + 1], vnrm[3 * vi + 2]);
                V3<T> vc(vcol[3 * vi], vcol[3 * vi + 1], vcol[3 * vi + 2]);
                V3<T> diff = fw - vp;
                T dist = length(diff);
                V3<T> nd = diff / dist;
                T angle = gmax(T(0), dot(vn, nd)) * gmax(T(0), dot(fn, -nd));
                if (angle <= T(0)) continue;
                T att = T(1) / std::pow(dist, T(4));
                T G = gmin(angle * att, clamp_value);
                if (p.shadowing) {
                    T ismIndex = T(vi) - T(p.ism_index_offset);
                    V3<T> v = paraboloid_project(diff, dist, vn, zFar, ismIndex, p.gx, p.gy, false);
                    // textureLod, nearest filter, GL_REPEAT wrap
                    long tx = (long)std::floor(v.x * T(p.atlas_w)), ty = (long)std::floor(v.y * T(p.atlas_h));
                    tx = ((tx % p.atlas_w) + p.atlas_w) % p.atlas_w;
                    ty = ((ty % p.atlas_h) + p.atlas_h) % p.atlas_h;
                    T occ = T(atlas[(size_t)ty * p.atlas_w + tx]);
                    T sv = v.z - occ;
                    sv = smoothstep(T(1) - T(0.02f), T(1), T(1) - sv);
                    G = G * sv;
                }
                acc = acc + vc * G;
            }
            V3<T> res = acc * gi_intensity / T(p.vpl_count) * T(I2);
            out[3 * pix + 0] = res.x;
            out[3 * pix + 1] = res.y;
            out[3 * pix + 2] = res.z;
        }
    }
}

}  // namespace

// ---- C entry points (ctypes) ----------------------------------------------------------------
namespace {

// ---- after the gathering -------------------------------------------------------------------
// R11G11B10F (GL_R11F_G11F_B10F, GIStage.cpp:470): one unsigned float channel with a 5-bit
// exponent (bias 15) and `mb` mantissa bits, restated in double arithmetic: round to nearest even
// (nearbyint in the default rounding mode), negatives and -0 to 0, finite overflow to the largest
// finite value, +Inf to Inf, NaN to NaN, denormals kept.
uint32_t uf_pack_ref(float x, int mb) {
    const uint32_t emax = 31u << mb, maxfin = (30u << mb) | ((1u << mb) - 1u);
    if (std::isnan(x)) return emax | (1u << (mb - 1));
    if (std::signbit(x) || x == 0.0f) return 0u;
    if (std::isinf(x)) return emax;
    const double v = x;
    if (v >= (2.0 - std::ldexp(1.0, -mb)) * 32768.0) return maxfin;
    int e2 = 0;
    std::frexp(v, &e2);  // v in [2^(e2-1), 2^e2)
    int E = e2 - 1;
    if (E < -14) return (uint32_t)std::nearbyint(v / std::ldexp(1.0, -14 - mb));  // denormal (or smallest normal)
    double q = std::nearbyint(v / std::ldexp(1.0, E - mb));                          // in [2^mb, 2^(mb+1)]
    if (q >= std::ldexp(1.0, mb + 1)) {
        q = q / 2.0;
        ++E;
    }
    if (E + 15 >= 31) return maxfin;
    return ((uint32_t)(E + 15) << mb) | ((uint32_t)q - (1u << mb));
}

float uf_unpack_ref(uint32_t v, int mb) {
    const uint32_t e = (v >> mb) & 31u, m = v & ((1u << mb) - 1u);
    if (e == 31u) return m ? std::numeric_limits<float>::quiet_NaN() : std::numeric_limits<float>::infinity();
    if (e == 0u) return (float)std::ldexp((double)m, -14 - mb);
    return (float)std::ldexp(1.0 + std::ldexp((double)m, -mb), (int)e - 15);
}

uint32_t pack_r11_ref(float r, float g, float b) {
    return uf_pack_ref(r, 6) | (uf_pack_ref(g, 6) << 11) | (uf_pack_ref(b, 5) << 22);
}
V3<float> unpack_r11_ref(uint32_t w) {
    return V3<float>(uf_unpack_ref(w & 0x7FFu, 6), uf_unpack_ref((w >> 11) & 0x7FFu, 6), uf_unpack_ref(w >> 22, 5));
}

// gi_blur.frag:24-72 as GIStage::blur runs it (GIStage.cpp:308-344): the X pass over the whole
// image into a temporary buffer, then the Y pass; with `packed`, every buffer is R11G11B10F.
// Samples outside the image are skipped.
// nrm_rgb (optional, in place of nrm_oct): normals stored as n*0.5+0.5 RGB, decoded as gi_blur.frag
// decodes its faceNormalSampler texels (rgb * 2 - 1) -- the reference G-buffer's format, for pinning
void gi_blur_ref(int w, int h, const float* depth, const float* nrm_oct, const void* gi_in, int packed, float A,
                 float B, void* gi_out, int threads, const float* nrm_rgb = nullptr) {
    const size_t n = (size_t)w * h;
    std::vector<float> lin(n);
    std::vector<V3<float>> nrm(n), src(n), tmp(n);
    for (size_t p = 0; p < n; ++p) {
        const float z_b = depth[p];
        const float z_n = 2.0f * z_b - 1.0f;
        lin[p] = -B / (A + z_n);  // reprojection.glsl:6-14
        nrm[p] = nrm_rgb ? V3<float>(nrm_rgb[3 * p] * 2.0f - 1.0f, nrm_rgb[3 * p + 1] * 2.0f - 1.0f,
                                     nrm_rgb[3 * p + 2] * 2.0f - 1.0f)
                         : oct_decode<float>(nrm_oct[2 * p], nrm_oct[2 * p + 1]);
        src[p] = packed ? unpack_r11_ref(static_cast<const uint32_t*>(gi_in)[p])
                        : V3<float>(static_cast<const float*>(gi_in)[3 * p], static_cast<const float*>(gi_in)[3 * p + 1],
                                    static_cast<const float*>(gi_in)[3 * p + 2]);
    }
    auto weight = [](float r, float depthDiff, float normalDiff) {
        const float factor = (3.0f - r + 1.0f) / 4.0f;  // (KERNEL_RADIUS - r + 1) / 4
        float wgt = factor - depthDiff * depthDiff - normalDiff * normalDiff;
        return glsl::gmax(0.0f, wgt);
    };
    auto pass = [&](const std::vector<V3<float>>& in, std::vector<V3<float>>& out, int dx, int dy) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(threads > 0 ? threads : omp_get_max_threads())
#endif
        for (int y = 0; y < h; ++y)
            for (int x = 0; x < w; ++x) {
                const size_t c = (size_t)y * w + x;
                const float d = lin[c];
                const V3<float> N = nrm[c];
                V3<float> acc(0.0f, 0.0f, 0.0f);
                float factorAcc = 0.0f;
                acc = acc + in[c];
                factorAcc = factorAcc + 1.0f;
                for (int side = -1; side <= 1; side += 2)
                    for (int i = 1; i <= 3; ++i) {
                        const int sx = x + side * dx * i, sy = y + side * dy * i;
                        if (sx < 0 || sy < 0 || sx >= w || sy >= h) continue;
                        const size_t sp = (size_t)sy * w + sx;
                        const float normalFactor = 1.0f - glsl::gmax(0.0f, dot(N, nrm[sp]));
                        const float depthDiff = (lin[sp] - d) / 1.0f;
                        const float factor = weight(float(i), depthDiff, normalFactor * 5.0f);
                        factorAcc = factorAcc + factor;
                        acc = acc + in[sp] * factor;
                    }
                V3<float> o = acc / factorAcc;
                if (packed) o = unpack_r11_ref(pack_r11_ref(o.x, o.y, o.z));
                out[c] = o;
            }
    };
    pass(src, tmp, 1, 0);
    pass(tmp, src, 0, 1);
    for (size_t p = 0; p < n; ++p) {
        if (packed) {
            static_cast<uint32_t*>(gi_out)[p] = pack_r11_ref(src[p].x, src[p].y, src[p].z);
        } else {
            float* o = static_cast<float*>(gi_out);
            o[3 * p] = src[p].x;
            o[3 * p + 1] = src[p].y;
            o[3 * p + 2] = src[p].z;
        }
    }
}

// clustering.comp:30-86 and light_lists.comp:42-126 (ClusteredShading::process), in FP32 with the
// shaders' operation order: used depth slices per 128-pixel tile, each pixel's slice, and per used
// cluster the VPLs for which any of the 8 corners (the reference's list, (left, top) twice) lies
// in front of the VPL's plane. Slice index clamped to 15.
void cluster_lights_ref(int w, int h, const float* depth, const float* inv_vp16, float A, float B, float zfar,
                        const float* vpos, const uint32_t* vpn_bits, int n_vpl, uint32_t* used, uint32_t* masks,
                        uint8_t* pixel_slice) {
    const int tx = (w + 127) / 128, ty = (h + 127) / 128, words = (n_vpl + 31) / 32;
    const float scale = float(16 + 3) / std::log2(zfar);
    auto lin_depth = [&](float z_b) { const float z_n = 2.0f * z_b - 1.0f; return -B / (A + z_n); };
    auto log_depth = [&](float z_e) { const float z_n = (1.0f / z_e * -B) - A; return (z_n + 1.0f) / 2.0f; };
    std::fill(used, used + (size_t)tx * ty, 0u);
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const float s = glsl::gmax(std::log2(-lin_depth(depth[(size_t)y * w + x])) * scale - 3.0f, 0.0f);
            const int slice = std::min(to_int(s), 15);
            pixel_slice[(size_t)y * w + x] = (uint8_t)slice;
            used[(y / 128) * tx + x / 128] |= 1u << slice;
        }
    const tmat4<float> m = tmat4<float>::from(inv_vp16);
    auto slice_to_z = [&](int sl) { return sl == 0 ? 0.05f : -std::pow(2.0f, float(sl + 3) / scale); };
    for (int t = 0; t < tx * ty; ++t)
        for (int sl = 0; sl < 16; ++sl) {
            if (!((used[t] >> sl) & 1u)) continue;
            const int cx = t % tx, cy = t / tx;
            const float zF = slice_to_z(sl), zB = slice_to_z(sl + 1);
            const float L = float(cx) * 128.0f / float(w), R = float(cx + 1) * 128.0f / float(w);
            const float Bo = float(cy) * 128.0f / float(h), To = float(cy + 1) * 128.0f / float(h);
            const float F = log_depth(zF), K = log_depth(zB);
            const float cs[8][3] = {{L, Bo, F}, {L, Bo, K}, {R, Bo, F}, {R, Bo, K}, {L, To, F}, {L, To, K}, {L, To, F}, {L, To, K}};
            V3<float> corner[8];
            for (int i = 0; i < 8; ++i) {
                V4<float> v(cs[i][0], cs[i][1], cs[i][2], 1.0f);
                v = v * 2.0f - V4<float>(1.0f, 1.0f, 1.0f, 1.0f);
                v = m * v;
                corner[i] = V3<float>(v.x, v.y, v.z) / v.w;
            }
            uint32_t* row = masks + ((size_t)t * 16 + sl) * words;
            std::fill(row, row + words, 0u);
            for (int vi = 0; vi < n_vpl; ++vi) {
                const V3<float> p(vpos[3 * vi], vpos[3 * vi + 1], vpos[3 * vi + 2]);
                const V3<float> n = unpack3SN<float>(vpn_bits[vi]);
                bool found = false;
                for (int j = 0; j < 8; ++j) found = found || (dot(corner[j] - p, n) >= 0.0f);
                if (found) row[vi >> 5] |= 1u << (vi & 31);
            }
        }
}

// deferredshading.frag:39-44, 69-80 (GI ambient + the caller's direct term, Reinhard, toSRGB with
// srgb_utils.glsl's gamma 2.2); albedo is RGBA8 UNORM.
void composite_ref(int w, int h, const void* gi, int packed, const uint32_t* albedo, const float* occ,
                   const float* direct, float exposure, float* out_rgb, uint32_t* out_rgba8) {
    const float gamma = 2.2f, inv_gamma = 1.0f / gamma;
    for (size_t p = 0; p < (size_t)w * h; ++p) {
        const V3<float> g = packed ? unpack_r11_ref(static_cast<const uint32_t*>(gi)[p])
                                   : V3<float>(static_cast<const float*>(gi)[3 * p], static_cast<const float*>(gi)[3 * p + 1],
                                               static_cast<const float*>(gi)[3 * p + 2]);
        const uint32_t al = albedo[p];
        const V3<float> diffuse(std::pow(float(al & 0xFFu) / 255.0f, gamma), std::pow(float((al >> 8) & 0xFFu) / 255.0f, gamma),
                                std::pow(float((al >> 16) & 0xFFu) / 255.0f, gamma));
        const float occlusion = occ ? occ[p] : 1.0f;
        V3<float> c = g * diffuse * occlusion;
        if (direct) c = c + V3<float>(direct[3 * p], direct[3 * p + 1], direct[3 * p + 2]);
        c = c * exposure;
        c = V3<float>(c.x / (1.0f + c.x), c.y / (1.0f + c.y), c.z / (1.0f + c.z));
        c = V3<float>(std::pow(c.x, inv_gamma), std::pow(c.y, inv_gamma), std::pow(c.z, inv_gamma));
        if (out_rgb) {
            out_rgb[3 * p] = c.x;
            out_rgb[3 * p + 1] = c.y;
            out_rgb[3 * p + 2] = c.z;
        }
        if (out_rgba8) {
            auto unorm = [](float v) { return to_uint(glsl::gmin(glsl::gmax(v, 0.0f), 1.0f) * 255.0f + 0.5f); };
            out_rgba8[p] = unorm(c.x) | (unorm(c.y) << 8) | (unorm(c.z) << 16) | 0xFF000000u;
        }
    }
}

}  // namespace

extern "C" {

int oracle_max_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_vpl_process_f32(int rsm_w, int rsm_h, const float* depth, const uint32_t* n10, const uint32_t* d8, int n,
                            const float* inv_bpv, float intensity, int shuffle, const int32_t* perm, float* pos,
                            float* nrm, float* col, uint32_t* pn) {
    vpl_process<float>(rsm_w, rsm_h, depth, n10, d8, n, inv_bpv, intensity, shuffle, perm, pos, nrm, col, pn);
}
void oracle_vpl_process_f64(int rsm_w, int rsm_h, const float* depth, const uint32_t* n10, const uint32_t* d8, int n,
                            const double* inv_bpv, double intensity, int shuffle, const int32_t* perm, double* pos,
                            double* nrm, double* col, uint32_t* pn) {
    vpl_process<double>(rsm_w, rsm_h, depth, n10, d8, n, inv_bpv, intensity, shuffle, perm, pos, nrm, col, pn);
}

static SplatParams make_splat(int n_vpl, int vpl_start, int vpl_end, int scale_isms, int points_only, int gx, int gy,
                              int aw, int ah, int64_t bucket_stride, int64_t n_entries, int n_groups) {
    SplatParams p;
    p.n_vpl = n_vpl; p.vpl_start = vpl_start; p.vpl_end = vpl_end;
    p.scale_isms = scale_isms; p.points_only_scaled = points_only;
    p.gx = gx; p.gy = gy; p.atlas_w = aw; p.atlas_h = ah;
    p.bucket_stride = bucket_stride; p.n_groups = n_groups; p.n_entries = n_entries;
    return p;
}

void oracle_ism_splat_f32(const float* points, const uint32_t* counts, int n_groups, int64_t bucket_stride, int64_t n_entries,
                          const float* vpl_pos, const uint32_t* vpl_pn, int n_vpl, int vpl_start, int vpl_end,
                          int scale_isms, int points_only, int gx, int gy, int aw, int ah, float zfar, uint32_t* atlas,
                          int threads) {
    SplatParams p = make_splat(n_vpl, vpl_start, vpl_end, scale_isms, points_only, gx, gy, aw, ah, bucket_stride, n_entries, n_groups);
    ism_splat<float>(points, counts, vpl_pos, vpl_pn, p, zfar, atlas, threads);
}
int64_t oracle_ism_splat_count_f32(const float* points, const uint32_t* counts, int n_groups, int64_t bucket_stride, int64_t n_entries,
                                   const float* vpl_pos, const uint32_t* vpl_pn, int n_vpl, int vpl_start, int vpl_end,
                                   int scale_isms, int points_only, int gx, int gy, int aw, int ah, float zfar,
                                   uint32_t* atlas, int threads) {
    SplatParams p = make_splat(n_vpl, vpl_start, vpl_end, scale_isms, points_only, gx, gy, aw, ah, bucket_stride, n_entries, n_groups);
    int64_t issued = 0;
    ism_splat<float>(points, counts, vpl_pos, vpl_pn, p, zfar, atlas, threads, &issued);
    return issued;
}
void oracle_ism_splat_f64(const float* points, const uint32_t* counts, int n_groups, int64_t bucket_stride, int64_t n_entries,
                          const double* vpl_pos, const uint32_t* vpl_pn, int n_vpl, int vpl_start, int vpl_end,
                          int scale_isms, int points_only, int gx, int gy, int aw, int ah, double zfar,
                          uint32_t* atlas, int threads) {
    SplatParams p = make_splat(n_vpl, vpl_start, vpl_end, scale_isms, points_only, gx, gy, aw, ah, bucket_stride, n_entries, n_groups);
    ism_splat<double>(points, counts, vpl_pos, vpl_pn, p, zfar, atlas, threads);
}

void oracle_pullpush_f32(const uint32_t* keys, int w, int h, int ism_size, int levels, float zfar, float* out,
                         int threads) {
    pullpush<float>(keys, w, h, ism_size, levels, zfar, out, threads);
}
void oracle_pullpush_f64(const uint32_t* keys, int w, int h, int ism_size, int levels, double zfar, double* out,
                         int threads) {
    pullpush<double>(keys, w, h, ism_size, levels, zfar, out, threads);
}

// One pull level or one push level on caller-provided texel planes (4 x uint32 per texel:
// r, g, b as float bits, a as packHalf2x16 bits). Used by the hand-derived known-answer tests.
void oracle_pull_level_f32(int level, const uint32_t* keys, const uint32_t* in, int in_w, uint32_t* out, int out_w,
                           int out_h, float zfar, int ism_pixel_size) {
    pull_level<float>(level, keys, reinterpret_cast<const Texel<float>*>(in), in_w, reinterpret_cast<Texel<float>*>(out),
                      out_w, out_h, zfar, ism_pixel_size, 1);
}
void oracle_push_level_f32(int level, const uint32_t* keys, const uint32_t* same, const uint32_t* coarse, int c_w,
                           int c_h, uint32_t* out, float* final_out, int o_w, int o_h, int ism_size) {
    push_level<float>(level, keys, reinterpret_cast<const Texel<float>*>(same),
                      reinterpret_cast<const Texel<float>*>(coarse), c_w, c_h, reinterpret_cast<Texel<float>*>(out),
                      final_out, o_w, o_h, ism_size, 1);
}

static FgParams make_fg(int w, int h, int n_vpl, int vpl_count, int ism_off, int interleave, int shadowing, int gx,
                        int gy, int aw, int ah, int tile, double cutoff) {
    FgParams p;
    p.width = w; p.height = h; p.n_vpl = n_vpl; p.vpl_count = vpl_count; p.ism_index_offset = ism_off;
    p.interleave = interleave; p.shadowing = shadowing; p.gx = gx; p.gy = gy; p.atlas_w = aw; p.atlas_h = ah;
    p.tile = tile; p.influence_cutoff = cutoff; p.accurate_world = 0;
    return p;
}

void oracle_final_gather_f32(int w, int h, const float* depth, const float* nrm_oct, const float* inv_vp, int n_vpl,
                             int vpl_count, int ism_off, const float* vpos, const float* vnrm, const float* vcol,
                             const float* atlas, int aw, int ah, int gx, int gy, float zfar, float gi, float clampv,
                             int interleave, int shadowing, int tile, double cutoff, float* out, int threads) {
    FgParams p = make_fg(w, h, n_vpl, vpl_count, ism_off, interleave, shadowing, gx, gy, aw, ah, tile, cutoff);
    final_gather<float>(p, depth, nrm_oct, inv_vp, vpos, vnrm, vcol, atlas, zfar, gi, clampv, out, threads);
}
void oracle_final_gather_f32_accurate_world(int w, int h, const float* depth, const float* nrm_oct,
                                            const float* inv_vp, int n_vpl, int vpl_count, int ism_off,
                                            const float* vpos, const float* vnrm, const float* vcol,
                                            const float* atlas, int aw, int ah, int gx, int gy, float zfar, float gi,
                                            float clampv, int interleave, int shadowing, int tile, double cutoff,
                                            float* out, int threads) {
    FgParams p = make_fg(w, h, n_vpl, vpl_count, ism_off, interleave, shadowing, gx, gy, aw, ah, tile, cutoff);
    p.accurate_world = 1;
    final_gather<float>(p, depth, nrm_oct, inv_vp, vpos, vnrm, vcol, atlas, zfar, gi, clampv, out, threads);
}
void oracle_final_gather_f64(int w, int h, const float* depth, const float* nrm_oct, const double* inv_vp, int n_vpl,
                             int vpl_count, int ism_off, const double* vpos, const double* vnrm, const double* vcol,
                             const float* atlas, int aw, int ah, int gx, int gy, double zfar, double gi, double clampv,
                             int interleave, int shadowing, int tile, double cutoff, double* out, int threads) {
    FgParams p = make_fg(w, h, n_vpl, vpl_count, ism_off, interleave, shadowing, gx, gy, aw, ah, tile, cutoff);
    final_gather<double>(p, depth, nrm_oct, inv_vp, vpos, vnrm, vcol, atlas, zfar, gi, clampv, out, threads);
}

// Exposed for unit tests of the shared math.
void oracle_pack_r11g11b10f(const float* rgb, uint32_t* words, int64_t n) {
    for (int64_t i = 0; i < n; ++i) words[i] = pack_r11_ref(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
}
void oracle_unpack_r11g11b10f(const uint32_t* words, float* rgb, int64_t n) {
    for (int64_t i = 0; i < n; ++i) {
        const V3<float> c = unpack_r11_ref(words[i]);
        rgb[3 * i] = c.x;
        rgb[3 * i + 1] = c.y;
        rgb[3 * i + 2] = c.z;
    }
}
void oracle_gi_blur(int w, int h, const float* depth, const float* nrm_oct, const void* gi_in, int packed, float A,
                    float B, void* gi_out, int threads) {
    gi_blur_ref(w, h, depth, nrm_oct, gi_in, packed, A, B, gi_out, threads);
}
void oracle_gi_blur_rgb_normals(int w, int h, const float* depth, const float* nrm_rgb, const float* gi_in, float A,
                                float B, float* gi_out, int threads) {
    gi_blur_ref(w, h, depth, nullptr, gi_in, 0, A, B, gi_out, threads, nrm_rgb);
}
void oracle_cluster_lights(int w, int h, const float* depth, const float* inv_vp, float A, float B, float zfar,
                           const float* vpos, const uint32_t* vpn_bits, int n_vpl, uint32_t* used, uint32_t* masks,
                           uint8_t* pixel_slice) {
    cluster_lights_ref(w, h, depth, inv_vp, A, B, zfar, vpos, vpn_bits, n_vpl, used, masks, pixel_slice);
}
void oracle_final_gather_f64_clustered(int w, int h, const float* depth, const float* nrm_oct, const double* inv_vp,
                                       int n_vpl, int vpl_count, int ism_off, const double* vpos, const double* vnrm,
                                       const double* vcol, const float* atlas, int aw, int ah, int gx, int gy,
                                       double zfar, double gi, double clampv, int interleave, int shadowing,
                                       const uint32_t* cl_masks, const uint8_t* cl_slice, double* out, int threads) {
    FgParams p = make_fg(w, h, n_vpl, vpl_count, ism_off, interleave, shadowing, gx, gy, aw, ah, 0, 0.0);
    p.cl_masks = cl_masks;
    p.cl_slice = cl_slice;
    p.cl_tiles_x = (w + 127) / 128;
    p.cl_words = (n_vpl + 31) / 32;
    final_gather<double>(p, depth, nrm_oct, inv_vp, vpos, vnrm, vcol, atlas, zfar, gi, clampv, out, threads);
}
void oracle_composite(int w, int h, const void* gi, int packed, const uint32_t* albedo, const float* occ,
                      const float* direct, float exposure, float* out_rgb, uint32_t* out_rgba8) {
    composite_ref(w, h, gi, packed, albedo, occ, direct, exposure, out_rgb, out_rgba8);
}

uint32_t oracle_pack3sn_f32(float x, float y, float z) { return pack3SN<float>(V3<float>(x, y, z)); }
void oracle_unpack3sn_f32(uint32_t u, float* out) {
    V3<float> v = unpack3SN<float>(u);
    out[0] = v.x; out[1] = v.y; out[2] = v.z;
}
uint32_t oracle_pack_half2x16(float a, float b) { return packHalf2x16(a, b); }
void oracle_paraboloid_project_f32(const float* rel, float dist, const float* n, float zfar, float ism_index, int gx,
                                   int gy, int preserve_sign, float* out) {
    V3<float> v = paraboloid_project<float>(V3<float>(rel[0], rel[1], rel[2]), dist, V3<float>(n[0], n[1], n[2]), zfar,
                                            ism_index, gx, gy, preserve_sign != 0);
    out[0] = v.x; out[1] = v.y; out[2] = v.z;
}

}  // extern "C"
