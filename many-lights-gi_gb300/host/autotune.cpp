// Autotuner for a view's GI configuration: interleave factor I, ISM edge and pull-push levels,
// and the gathering tile. Candidates are timed on the GPU with the real kernels (mlgi_gi_frame on
// a device-generated room of the requested shape, best of three after one warm-up; a candidate
// whose warm-up is 3x slower than the best so far keeps its warm-up time) and cached per query.
// Two objectives:
//   budget_ms == 0: the fastest candidate that meets the quality floor
//                   (N / I^2 >= min_vpls_per_pixel, ISM edge >= min_ism_size);
//   budget_ms  > 0: among candidates meeting the floor, the highest quality (most VPLs per pixel,
//                   then the largest ISM) whose time fits the budget; the fastest one if none fits.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>

#include "kernels.h"
#include "mlgi.h"

namespace {

using Key = std::tuple<int, int, int, long long, int, int, int, int, float, int>;
std::mutex g_mu;
std::map<Key, mlgi_autotune_result> g_cache;

struct Cand {
    int I, s, levels, tile, gx, gy;
    float ms = 0.f;
};

int levels_for(int s) {
    int L = 0;
    while (L < 6 && s % (2 << L) == 0) ++L;
    return L;
}

struct DevBuf {
    void* p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    bool alloc(size_t bytes) {
        if (mlgi::dev_alloc(&p, std::max<size_t>(bytes, 16)) != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            return false;
        }
        return true;
    }
};

}  // namespace

extern "C" mlgi_status mlgi_autotune(mlgi_ctx* ctx, const mlgi_autotune_query* q, mlgi_autotune_result* out) {
    if (!ctx || !q || !out) return MLGI_EINVAL;
    if (q->width <= 0 || q->height <= 0 || q->n_vpl <= 0 || q->n_vpl % 64 || q->n_points < 0) return MLGI_EINVAL;
    const Key key{q->width, q->height, q->n_vpl, (long long)q->n_points, q->reduced, q->min_vpls_per_pixel,
                  q->min_ism_size, q->batched, q->budget_ms, q->rsm_size};
    {
        std::lock_guard<std::mutex> lock(g_mu);
        auto it = g_cache.find(key);
        if (it != g_cache.end()) {
            *out = it->second;
            return MLGI_OK;
        }
    }
    const int N = q->n_vpl;
    const int gx = 1 << (int)std::ceil(std::log2((double)N) / 2.0);
    const int gy = (N + gx - 1) / gx;
    // Interleave factors meeting the floor, largest first. Without a budget only the two largest are
    // timed: a smaller I evaluates at least 4x the pixel-VPL pairs with the same ISM work.
    std::vector<int> Is;
    for (int I : {16, 8, 4, 2, 1})
        if (N % (I * I) == 0 && N / (I * I) >= std::max(1, q->min_vpls_per_pixel)) Is.push_back(I);
    if (q->budget_ms <= 0.f && Is.size() > 2) Is.resize(2);
    std::vector<Cand> cands;
    for (int I : Is) {
        for (int s : {64, 96, 128}) {
            if (s < q->min_ism_size) continue;
            if ((long long)gx * s > 16384 || (long long)gy * s > 16384) continue;
            for (int tile : {8, 16}) {
                if (q->batched && tile != 16) continue;  // the batched gather uses 16 x 16 tiles
                cands.push_back(Cand{I, s, levels_for(s), tile, gx, gy});
            }
        }
    }
    if (cands.empty()) return MLGI_EINVAL;

    // One device-generated room of the requested shape; the inputs do not depend on the candidate.
    const int R = q->rsm_size > 0 ? q->rsm_size : 512;
    mlgi_scene_desc sd{};
    sd.seed = q->seed;
    sd.n_boxes = 16;
    sd.n_spheres = 8;
    sd.width = q->width;
    sd.height = q->height;
    sd.rsm_width = sd.rsm_height = R;
    sd.n_points = q->n_points;
    sd.n_buckets = N;
    sd.ism_count = N;
    sd.z_near = 1.f;
    sd.z_far = 400.f;
    mlgi_scene_info info{};
    const size_t px = (size_t)q->width * q->height;
    const int64_t stride = (q->n_points + N - 1) / N;
    DevBuf gd, gn, rd, rn, rf, pts, cnt, rgb;
    if (!gd.alloc(px * 4) || !gn.alloc(px * 8) || !rd.alloc((size_t)R * R * 4) || !rn.alloc((size_t)R * R * 4) ||
        !rf.alloc((size_t)R * R * 4) || !pts.alloc((size_t)N * stride * 16) || !cnt.alloc((size_t)N * 4) ||
        !rgb.alloc(px * 12))
        return MLGI_ENOMEM;
    cudaStream_t s = static_cast<cudaStream_t>(mlgi_ctx_stream(ctx));
    mlgi_status st = mlgi_scene_generate_device(&sd, &info, static_cast<float*>(gd.p), gn.p,
                                                q->reduced ? MLGI_F16 : MLGI_F32, nullptr, static_cast<float*>(rd.p),
                                                static_cast<uint32_t*>(rn.p), static_cast<uint32_t*>(rf.p),
                                                static_cast<float*>(pts.p), static_cast<uint32_t*>(cnt.p), s);
    if (st != MLGI_OK) return st;

    mlgi_frame_desc f{};
    f.rsm = mlgi_rsm_view{R, R, static_cast<float*>(rd.p), static_cast<uint32_t*>(rn.p), static_cast<uint32_t*>(rf.p)};
    f.vpl.count = N;
    f.vpl.light_intensity = 5.f;
    f.vpl.shuffle = 1;
    std::memcpy(f.vpl.inv_biased_light_vp, info.inv_biased_light_vp, sizeof(f.vpl.inv_biased_light_vp));
    f.points = mlgi_points{static_cast<float*>(pts.p), static_cast<uint32_t*>(cnt.p), N, stride};
    f.atlas_format = q->reduced ? MLGI_F16 : MLGI_F32;
    f.gbuffer = mlgi_gbuffer_view{q->width, q->height, static_cast<float*>(gd.p), gn.p, q->reduced ? MLGI_F16 : MLGI_F32};
    std::memcpy(f.fg.inv_view_proj, info.inv_view_proj, sizeof(f.fg.inv_view_proj));
    f.fg.z_far = 400.f;
    f.fg.gi_intensity = 3000.f;
    f.fg.clamp_value = 0.001f;
    f.fg.vpl_count = N;
    f.fg.vpl_start = 0;
    f.fg.vpl_end = N;
    f.fg.shadowing = 1;
    f.fg.cull = 1;
    f.fg.vpl_format = q->reduced ? MLGI_F16 : MLGI_F32;
    mlgi_radiance out_rgb{q->width, q->height, static_cast<float*>(rgb.p)};

    size_t max_texels = 0;
    for (const Cand& c : cands) max_texels = std::max(max_texels, (size_t)c.gx * c.gy * c.s * c.s);
    if ((st = mlgi_ctx_reserve(ctx, N, max_texels)) != MLGI_OK) return st;  // no allocation inside a timing
    float best_so_far = 1e30f;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (Cand& c : cands) {
        f.ism = mlgi_ism_params{0, N, 0, 0, c.s, c.gx, c.gy, c.levels, 400.f};
        f.fg.ism_size = c.s;
        f.fg.grid_x = c.gx;
        f.fg.grid_y = c.gy;
        f.fg.interleave = c.I;
        f.fg.tile = c.tile;
        float best = 1e30f;
        for (int rep = 0; rep < 4 && st == MLGI_OK; ++rep) {
            cudaEventRecord(e0, s);
            st = mlgi_gi_frame(ctx, &f, &out_rgb, s);
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep == 0) {  // warm-up; a candidate already 3x slower than the best so far is not refined
                if (ms > 3.f * best_so_far) {
                    best = ms;
                    break;
                }
                continue;
            }
            best = std::min(best, ms);
        }
        if (st != MLGI_OK) break;
        c.ms = best;
        best_so_far = std::min(best_so_far, best);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != MLGI_OK) return st;

    const Cand* pick = nullptr;
    auto fastest = [&]() {
        const Cand* b = &cands[0];
        for (const Cand& c : cands)
            if (c.ms < b->ms) b = &c;
        return b;
    };
    if (q->budget_ms > 0.f) {
        // quality order: VPLs per pixel (desc), ISM edge (desc); within a quality level the fastest tile
        for (const Cand& c : cands) {
            if (c.ms > q->budget_ms) continue;
            if (!pick || N / (c.I * c.I) > N / (pick->I * pick->I) ||
                (c.I == pick->I && (c.s > pick->s || (c.s == pick->s && c.ms < pick->ms))))
                pick = &c;
        }
    }
    if (!pick) pick = fastest();
    *out = mlgi_autotune_result{pick->I, pick->s, pick->gx, pick->gy, pick->levels, pick->tile, pick->ms,
                                (int)cands.size()};
    std::lock_guard<std::mutex> lock(g_mu);
    g_cache[key] = *out;
    return MLGI_OK;
}
