// Harness that runs the reference's own compute shaders (rewritten to C++ by build_ref.py) on
// the CPU -- TEST INFRASTRUCTURE ONLY, built into oracle/_ref/libref.so.
//
// It plays the role of the OpenGL driver and of the reference's host dispatch code: it binds
// images, samplers and buffers, sets uniforms and dispatches work groups with the group counts
// the reference's stages use (VPLProcessor.cpp:95-100, ImperfectShadowmap.cpp:121-182,249-257,
// GIStage.cpp:270-303). Work groups run in parallel (OpenMP); inside a group, invocations run as
// fibers (ucontext) so that barrier() holds.
#include <omp.h>
#include <ucontext.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

#include "glsl.hpp"
#include "ref_shim.hpp"

namespace glslref {

// packHalf2x16 / unpackHalf2x16 conversions: round to nearest even (the same rule the oracle's
// restatement and the CUDA kernels use).
uint16_t f2h_rne(float f) { return glsl::float_to_half_rne(f); }
float h2f(uint16_t h) { return glsl::half_to_float(h); }

thread_local std::map<std::string, std::vector<unsigned char>>* tl_shared_arena = nullptr;
thread_local ucontext_t* tl_sched = nullptr;
thread_local ucontext_t* tl_cur = nullptr;

void barrier() {
    if (tl_cur && tl_sched) swapcontext(tl_cur, tl_sched);
}

#define MLGI_REF_SHADER(NAME)                                     \
    struct NAME : RefShaderBase {                                 \
        explicit NAME(Bindings* b) : RefShaderBase(b) {}          \
        _Pragma("GCC diagnostic push")                            \
        _Pragma("GCC diagnostic ignored \"-Wall\"")
#define MLGI_REF_SHADER_END \
    _Pragma("GCC diagnostic pop") \
    }                       \
    ;

MLGI_REF_SHADER(Ref_vpl_processor)
#include "Ref_vpl_processor.inc"
MLGI_REF_SHADER_END
MLGI_REF_SHADER(Ref_ism)
#include "Ref_ism.inc"
MLGI_REF_SHADER_END
MLGI_REF_SHADER(Ref_pull_L0)
#include "Ref_pull_L0.inc"
MLGI_REF_SHADER_END
MLGI_REF_SHADER(Ref_pull)
#include "Ref_pull.inc"
MLGI_REF_SHADER_END
MLGI_REF_SHADER(Ref_push_L0)
#include "Ref_push_L0.inc"
MLGI_REF_SHADER_END
MLGI_REF_SHADER(Ref_push)
#include "Ref_push.inc"
MLGI_REF_SHADER_END
MLGI_REF_SHADER(Ref_final_gathering)
#include "Ref_final_gathering.inc"
MLGI_REF_SHADER_END
MLGI_REF_SHADER(Ref_gi_blur_x)
#include "Ref_gi_blur_x.inc"
MLGI_REF_SHADER_END
MLGI_REF_SHADER(Ref_gi_blur_y)
#include "Ref_gi_blur_y.inc"
MLGI_REF_SHADER_END
MLGI_REF_SHADER(Ref_clustering)
#include "Ref_clustering.inc"
MLGI_REF_SHADER_END
MLGI_REF_SHADER(Ref_light_lists)
#include "Ref_light_lists.inc"
MLGI_REF_SHADER_END

// ---- dispatch -----------------------------------------------------------------------------------
namespace {

struct Fiber {
    ucontext_t ctx;
    std::vector<char> stack;
    RefShaderBase* shader = nullptr;
    void (*run)(RefShaderBase*) = nullptr;
    bool done = false;
};

thread_local Fiber* tl_fiber = nullptr;

void fiber_entry() {
    Fiber* f = tl_fiber;
    f->run(f->shader);
    f->done = true;
}

template <class S>
void dispatch(Bindings& B, uvec3 groups, uvec3 local, bool fibers, int threads) {
    B.local_size = local;
    B.num_groups = groups;
    const int nloc = (int)(local.x * local.y * local.z);
    const long ng = (long)groups.x * groups.y * groups.z;
#pragma omp parallel num_threads(threads > 0 ? threads : omp_get_max_threads())
    {
        std::map<std::string, std::vector<unsigned char>> arena;
        tl_shared_arena = &arena;
        std::vector<std::unique_ptr<S>> inv;
        for (int i = 0; i < (fibers ? nloc : 1); ++i) inv.emplace_back(new S(&B));
        std::vector<Fiber> fib(fibers ? nloc : 0);
        for (auto& f : fib) f.stack.resize(1 << 16);
        ucontext_t sched;
#pragma omp for schedule(dynamic, 8)
        for (long g = 0; g < ng; ++g) {
            const uvec3 gid((uint)(g % groups.x), (uint)((g / groups.x) % groups.y), (uint)(g / ((long)groups.x * groups.y)));
            if (!fibers) {
                S& s = *inv[0];
                s.gl_WorkGroupID = gid;
                for (int l = 0; l < nloc; ++l) {
                    s.gl_LocalInvocationID = uvec3(l % local.x, (l / local.x) % local.y, l / (local.x * local.y));
                    s.main();
                }
                continue;
            }
            for (int l = 0; l < nloc; ++l) {
                S& s = *inv[l];
                s.gl_WorkGroupID = gid;
                s.gl_LocalInvocationID = uvec3(l % local.x, (l / local.x) % local.y, l / (local.x * local.y));
                Fiber& f = fib[l];
                f.shader = &s;
                f.run = [](RefShaderBase* p) { static_cast<S*>(p)->main(); };
                f.done = false;
                getcontext(&f.ctx);
                f.ctx.uc_stack.ss_sp = f.stack.data();
                f.ctx.uc_stack.ss_size = f.stack.size();
                f.ctx.uc_link = &sched;
                makecontext(&f.ctx, fiber_entry, 0);
            }
            tl_sched = &sched;
            bool any = true;
            while (any) {
                any = false;
                for (int l = 0; l < nloc; ++l) {
                    Fiber& f = fib[l];
                    if (f.done) continue;
                    tl_fiber = &f;
                    tl_cur = &f.ctx;
                    swapcontext(&sched, &f.ctx);
                    any = any || !f.done;
                }
            }
            tl_cur = nullptr;
            tl_sched = nullptr;
        }
    }
}

mat4 to_mat4(const float* m) {
    mat4 r;
    for (int c = 0; c < 4; ++c) r.c[c] = vec4(m[4 * c], m[4 * c + 1], m[4 * c + 2], m[4 * c + 3]);
    return r;
}

}  // namespace
}  // namespace glslref


using namespace glslref;

extern "C" {

// vpl_processor.comp driven as VPLProcessor::process does (N must be the shader's 1024).
// Outputs: vpl_out N x 9 floats (pos, normal, color), packed_out N x 4 floats.
void ref_vpl_process(int rsm_w, int rsm_h, const float* depth, const uint32_t* n10, const uint32_t* d8, int n,
                     const float* inv_bpv, float intensity, int shuffle, const int32_t* perm, float* vpl_out,
                     float* packed_out, int threads) {
    std::vector<float> diff((size_t)rsm_w * rsm_h * 4), nrm((size_t)rsm_w * rsm_h * 4), dep((size_t)rsm_w * rsm_h * 4);
    for (size_t t = 0; t < (size_t)rsm_w * rsm_h; ++t) {  // UNORM -> float as the texture unit returns it
        const uint32_t d = d8[t], nb = n10[t];
        diff[4 * t] = float(d & 0xFFu) / 255.0f;
        diff[4 * t + 1] = float((d >> 8) & 0xFFu) / 255.0f;
        diff[4 * t + 2] = float((d >> 16) & 0xFFu) / 255.0f;
        diff[4 * t + 3] = float(d >> 24) / 255.0f;
        nrm[4 * t] = float(nb & 0x3FFu) / 1023.0f;
        nrm[4 * t + 1] = float((nb >> 10) & 0x3FFu) / 1023.0f;
        nrm[4 * t + 2] = float((nb >> 20) & 0x3FFu) / 1023.0f;
        nrm[4 * t + 3] = float(nb >> 30) / 3.0f;
        dep[4 * t] = depth[t];
    }
    Bindings B;
    B.set("rsmDiffuseSampler", Sampler2D{diff.data(), nullptr, rsm_w, rsm_h, true});
    B.set("rsmNormalSampler", Sampler2D{nrm.data(), nullptr, rsm_w, rsm_h, true});
    B.set("rsmDepthSampler", Sampler2D{dep.data(), nullptr, rsm_w, rsm_h, true});
    B.set("biasedLightViewProjectionInverseMatrix", to_mat4(inv_bpv));
    B.set("lightIntensity", intensity);
    B.set("shuffleLights", shuffle != 0);
    std::vector<vec3> vpl((size_t)n * 3);
    std::vector<int32_t> sh(perm, perm + n);
    B.buffers["vplBuffer"] = vpl.data();
    B.buffers["packedVplBuffer"] = packed_out;
    B.buffers["shuffledIndicesBuffer"] = sh.data();
    dispatch<Ref_vpl_processor>(B, uvec3(n / 64, 1, 1), uvec3(64, 1, 1), false, threads);
    std::memcpy(vpl_out, vpl.data(), sizeof(float) * 9 * (size_t)n);
}

// ism.comp driven as ImperfectShadowmap::render does (1024 work groups of 128).
void ref_ism_splat(const float* points, int64_t n_points_total, const uint32_t* counts, int n_counts,
                   const float* packed_vpls, int n_vpl, int vpl_start, int vpl_end, int scale_isms, int points_only,
                   int atlas_w, int atlas_h, float zfar, uint32_t* keys, int threads) {
    for (size_t i = 0; i < (size_t)atlas_w * atlas_h; ++i) keys[i] = 0xFFFFFFFFu;  // ImperfectShadowmap.cpp:212
    std::vector<uint32_t> cnt(4096, 0u);                                           // 4*1024 counters (:110)
    for (int i = 0; i < n_counts; ++i) cnt[i] = counts[i];
    std::vector<vec4> pk(1024);
    std::memcpy(pk.data(), packed_vpls, sizeof(float) * 4 * (size_t)n_vpl);
    Bindings B;
    B.buffers["vplPositionNormalBuffer"] = pk.data();
    B.buffers["atomicCounter"] = cnt.data();
    B.set("softrenderBuffer", UImage2D{keys, atlas_w, atlas_h, 1});
    B.set("pointBuffer", ImageBuffer{const_cast<float*>(points), (int)n_points_total});
    B.set("viewport", ivec2(atlas_w, atlas_h));
    B.set("zFar", zfar);
    B.set("usePushPull", true);
    B.set("vplStartIndex", vpl_start);
    B.set("vplEndIndex", vpl_end);
    B.set("scaleISMs", scale_isms != 0);
    B.set("pointsOnlyIntoScaledISMs", points_only != 0);
    B.set("tessLevelFactor", 2.0f);
    dispatch<Ref_ism>(B, uvec3(1024, 1, 1), uvec3(128, 1, 1), true, threads);
}

// ImperfectShadowmap::pullpush (ImperfectShadowmap.cpp:121-182) with `levels` levels; the final
// result (the R16 image of the reference) is written as float.
void ref_pullpush(const uint32_t* keys, int w, int h, int ism_pixel_size, int levels, float zfar, float* out,
                  int threads) {
    std::vector<std::vector<float>> pull(levels + 1), push(levels + 1);
    for (int l = 0; l <= levels; ++l) {
        pull[l].assign((size_t)(w >> l) * (h >> l) * 4, 0.f);
        push[l].assign((size_t)(w >> l) * (h >> l) * 4, 0.f);
    }
    auto img = [&](std::vector<float>& v, int l) { return Image2D{v.data(), nullptr, w >> l, h >> l, 4}; };
    const USampler2D soft{keys, w, h};
    for (int i = 1; i <= levels; ++i) {
        Bindings B;
        B.set("softrenderBuffer", soft);
        B.set("ismDepthImage", img(pull[i - 1], i - 1));
        B.set("img_output", img(pull[i], i));
        B.set("level", i);
        B.set("ismPixelSize", ism_pixel_size);
        B.set("zFar", zfar);
        const uint gx = (uint)((w >> i) / 8), gy = (uint)((h >> i) / 8);
        if (i == 1)
            dispatch<Ref_pull_L0>(B, uvec3(gx, gy, 1), uvec3(8, 8, 1), false, threads);
        else
            dispatch<Ref_pull>(B, uvec3(gx, gy, 1), uvec3(8, 8, 1), false, threads);
    }
    Image2D last{out, nullptr, w, h, 1};
    for (int i = levels - 1; i >= 0; --i) {
        Bindings B;
        B.set("pullSameLevelTexture", soft);
        B.set("pullSameLevelImage", img(pull[i], i));
        B.set("coarserLevel", i == levels - 1 ? img(pull[i + 1], i + 1) : img(push[i + 1], i + 1));
        B.set("img_output", img(push[i], i));
        B.set("imgOutputLastStage", last);
        B.set("level", i);
        const uint gx = (uint)((w >> i) / 8 / 2 + 1), gy = (uint)((h >> i) / 8 / 2 + 1);
        if (i == 0)
            dispatch<Ref_push_L0>(B, uvec3(gx, gy, 1), uvec3(8, 8, 1), false, threads);
        else
            dispatch<Ref_push>(B, uvec3(gx, gy, 1), uvec3(8, 8, 1), false, threads);
    }
}

// final_gathering.comp driven as GIStage::compute_final_gathering does, with light lists that
// give interleave class c the VPLs [c*per_class, (c+1)*per_class) (per_class <= 63, the most a
// 64-entry sub-list holds). normal_rgb: width*height*3 floats of n*0.5+0.5.
void ref_final_gather(int w, int h, const float* depth, const float* normal_rgb, const float* inv_vp,
                      const float* proj, const float* vpl9, int n_vpl, int vpl_start, int vpl_end,
                      const float* atlas, int aw, int ah, float zfar, float znear, float gi, float clampv,
                      int per_class, float* out_rgb, int threads) {
    std::vector<float> dep((size_t)w * h * 4, 0.f), nrm((size_t)w * h * 4, 0.f), ism((size_t)aw * ah * 4, 0.f);
    for (size_t t = 0; t < (size_t)w * h; ++t) {
        dep[4 * t] = depth[t];
        nrm[4 * t] = normal_rgb[3 * t];
        nrm[4 * t + 1] = normal_rgb[3 * t + 1];
        nrm[4 * t + 2] = normal_rgb[3 * t + 2];
        nrm[4 * t + 3] = 1.f;
    }
    for (size_t t = 0; t < (size_t)aw * ah; ++t) ism[4 * t] = atlas[t];
    const int ncx = (w + 127) / 128, ncy = (h + 127) / 128;
    std::vector<uint32_t> ids((size_t)ncx * ncy * 16, 0u);  // every cluster uses light list 0
    std::vector<uint32_t> lists(1024 + 64, 0u);             // one R16UI column, 1024 rows
    for (int c = 0; c < 16; ++c) {
        lists[64 * c] = (uint32_t)per_class + 1u;
        for (int k = 0; k < per_class; ++k) lists[64 * c + 1 + k] = (uint32_t)(c * per_class + k);
    }
    std::vector<float> outv((size_t)w * h * 4, 0.f);
    std::vector<float> vpl((size_t)1024 * 9, 0.f);
    std::memcpy(vpl.data(), vpl9, sizeof(float) * 9 * (size_t)n_vpl);
    Bindings B;
    B.set("img_output", Image2D{outv.data(), nullptr, w, h, 4});
    B.set("lightListIds", Image3D{ids.data(), ncx, ncy, 16});
    B.set("lightLists", UImage2D{lists.data(), 1, 1024, 1});
    B.buffers["vplBuffer"] = vpl.data();
    B.set("faceNormalSampler", Sampler2D{nrm.data(), nullptr, w, h, true});
    B.set("depthSampler", Sampler2D{dep.data(), nullptr, w, h, true});
    B.set("ismDepthSampler", Sampler2D{ism.data(), nullptr, aw, ah, true});
    const mat4 P = to_mat4(proj), I4 = to_mat4(inv_vp);
    B.set("projectionMatrix", P);
    B.set("projectionInverseMatrix", I4);
    B.set("viewMatrix", I4);
    B.set("viewInvertedMatrix", I4);
    B.set("viewProjectionInvertedMatrix", I4);
    B.set("zFar", zfar);
    B.set("zNear", znear);
    B.set("viewport", ivec2(w, h));
    B.set("giIntensityFactor", gi);
    B.set("vplClampingValue", clampv);
    B.set("vplStartIndex", vpl_start);
    B.set("vplEndIndex", vpl_end);
    const int gx = (w + 31) / 32 * 4, gy = (h + 31) / 32 * 4;  // GIStage.cpp:297-301
    dispatch<Ref_final_gathering>(B, uvec3((uint)gx, (uint)gy, 1), uvec3(8, 8, 1), false, threads);
    for (size_t t = 0; t < (size_t)w * h; ++t)
        for (int k = 0; k < 3; ++k) out_rgb[3 * t + k] = outv[4 * t + k];
}

// ClusteredShading::process (ClusteredShading.cpp:70-112): clustering.comp over
// ceil(w/128) x ceil(h/128) groups of 128, then light_lists.comp over (clusters, 16) groups of 64.
// The projection matrix has only [2][2] = proj_a and [3][2] = proj_b set (the shaders read no
// other entry). Outputs: *n_used, and per used cluster (in the order the atomic counter gave):
// cluster_word[i] = x | y << 8 | slice << 16, and lists[i * 1024 .. +1024), the light-list column
// (entry 64 s is sub-list s's count + 1, its VPL ids follow). Runs work groups in dispatch order
// on one thread, so that a sub-list's count slot is written after the previous sub-list's entries.
void ref_cluster_lights(int w, int h, const float* depth, const float* inv_vp, float proj_a, float proj_b, float zfar,
                        const float* packed_vpls, int n_vpl, int* n_used, uint32_t* cluster_word, uint32_t* lists) {
    const int ncx = (w + 127) / 128, ncy = (h + 127) / 128, nclusters = ncx * ncy * 16;
    std::vector<float> dep((size_t)w * h * 4, 0.f);
    for (size_t t = 0; t < (size_t)w * h; ++t) dep[4 * t] = depth[t];
    mat4 P;
    for (int c = 0; c < 4; ++c) P.c[c] = vec4(0.f, 0.f, 0.f, 0.f);
    P.c[2].z = proj_a;
    P.c[3].z = proj_b;
    std::vector<uint32_t> compact((size_t)nclusters, 0u), list_ids((size_t)nclusters, 0u);
    std::vector<uint32_t> counter(4, 0u);
    {
        Bindings B;
        B.set("compactUsedIDs", UImage2D{compact.data(), nclusters, 1, 1});
        B.set("lightListIds", Image3D{list_ids.data(), ncx, ncy, 16});
        B.set("depthSampler", Sampler2D{dep.data(), nullptr, w, h, true});
        B.buffers["atomicCounter"] = counter.data();
        B.set("projectionMatrix", P);
        B.set("zFar", zfar);
        dispatch<Ref_clustering>(B, uvec3((uint)ncx, (uint)ncy, 1), uvec3(128, 1, 1), true, 1);
    }
    const int used = (int)counter[0];
    std::vector<vec4> pk(1024);
    std::memcpy(pk.data(), packed_vpls, sizeof(float) * 4 * (size_t)std::min(n_vpl, 1024));
    std::vector<uint32_t> ll((size_t)std::max(used, 1) * 1024, 0u);
    {
        Bindings B;
        B.set("compactUsedClusterIDs", UImage2D{compact.data(), nclusters, 1, 1});
        B.set("lightLists", UImage2D{ll.data(), std::max(used, 1), 1024, 1});
        B.set("clusterCorners", Image2D{nullptr, nullptr, 0, 0, 4});
        B.buffers["vplPositionNormalBuffer"] = pk.data();
        B.buffers["numUsedClusters"] = counter.data();
        B.set("viewport", ivec2(w, h));
        B.set("projectionMatrix", P);
        B.set("viewProjectionInverseMatrix", to_mat4(inv_vp));
        B.set("zFar", zfar);
        B.set("vplStartIndex", 0);
        B.set("vplEndIndex", 1024);
        dispatch<Ref_light_lists>(B, uvec3((uint)nclusters, 16, 1), uvec3(64, 1, 1), true, 1);
    }
    *n_used = used;
    for (int i = 0; i < used; ++i) {
        cluster_word[i] = compact[i];
        for (int r = 0; r < 1024; ++r) lists[(size_t)i * 1024 + r] = ll[(size_t)r * used + i];
    }
}

// GIStage::blur (GIStage.cpp:308-344): gi_blur.frag's X program over the screen-aligned quad into a
// temporary buffer, then its Y program; every buffer is float RGB here. normal_rgb: n*0.5+0.5.
void ref_gi_blur(int w, int h, const float* depth, const float* normal_rgb, const float* gi_rgb, float proj_a,
                 float proj_b, float* out_rgb, int threads) {
    std::vector<float> dep((size_t)w * h * 4, 0.f), nrm((size_t)w * h * 4, 0.f), gi((size_t)w * h * 4, 0.f),
        tmp((size_t)w * h * 4, 0.f);
    for (size_t t = 0; t < (size_t)w * h; ++t) {
        dep[4 * t] = depth[t];
        for (int k = 0; k < 3; ++k) {
            nrm[4 * t + k] = normal_rgb[3 * t + k];
            gi[4 * t + k] = gi_rgb[3 * t + k];
        }
    }
    mat4 P;
    for (int c = 0; c < 4; ++c) P.c[c] = vec4(0.f, 0.f, 0.f, 0.f);
    P.c[2].z = proj_a;
    P.c[3].z = proj_b;
    auto pass = [&](auto tag, const std::vector<float>& src, std::vector<float>& dst) {
        using S = typename decltype(tag)::type;
        Bindings B;
        B.set("giSampler", Sampler2D{src.data(), nullptr, w, h, true});
        B.set("faceNormalSampler", Sampler2D{nrm.data(), nullptr, w, h, true});
        B.set("depthSampler", Sampler2D{dep.data(), nullptr, w, h, true});
        B.set("projectionMatrix", P);
        B.set("projectionInverseMatrix", P);
#pragma omp parallel for schedule(static) num_threads(threads > 0 ? threads : omp_get_max_threads())
        for (int y = 0; y < h; ++y) {
            S sh(&B);
            for (int x = 0; x < w; ++x) {
                sh.gl_FragCoord = vec4(float(x) + 0.5f, float(y) + 0.5f, 0.f, 1.f);
                sh.v_uv = vec2((float(x) + 0.5f) / float(w), (float(y) + 0.5f) / float(h));
                sh.main();
                float* o = dst.data() + 4 * ((size_t)y * w + x);
                o[0] = sh.outColor.x;
                o[1] = sh.outColor.y;
                o[2] = sh.outColor.z;
            }
        }
    };
    struct X { using type = Ref_gi_blur_x; };
    struct Y { using type = Ref_gi_blur_y; };
    pass(X{}, gi, tmp);
    std::vector<float> res((size_t)w * h * 4, 0.f);
    pass(Y{}, tmp, res);
    for (size_t t = 0; t < (size_t)w * h; ++t)
        for (int k = 0; k < 3; ++k) out_rgb[3 * t + k] = res[4 * t + k];
}

}  // extern "C"
