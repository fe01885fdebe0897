// Request server for GI frames on one GPU: continuous batching over in-flight slots.
//
// A request names a room (seed), a frame shape (resolution, VPL count, point count, precision)
// and a pose (light yaw/pitch jitter, camera orbit). The scheduler thread admits queued requests
// FIFO into free slots as soon as a slot and HBM budget are available, so frames of requests that
// arrive while others run overlap on the device (each slot is a context with its own stream and
// frame buffers). Per-room state -- the bucketed surface points of (seed, VPL count, point count)
// -- is generated on the GPU once and stays resident across requests, evicted least-recently-used
// under the budget. Each frame's G-buffer and RSM are ray-cast on the device for its pose, the
// chain runs with the autotuned configuration of its shape, and the radiance is reduced to an
// order-independent 64-bit digest and a fixed-order FP64 sum (optionally also copied to a host
// buffer). Latency runs from arrival to a host function queued behind the frame on its stream.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <mutex>
#include <random>
#include <thread>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>

#include "kernels.h"
#include "mlgi.h"

namespace {

using Clock = std::chrono::steady_clock;

double now_s() { return std::chrono::duration<double>(Clock::now().time_since_epoch()).count(); }

constexpr int kDigestBlocks = 608;  // 4 x 152 SMs
constexpr int kDigestThreads = 256;

// Per block: the sum over its elements of mix(i, bits(x_i)) mod 2^64 and the FP64 sum of the
// elements, both in a fixed order for a fixed grid.
__global__ void __launch_bounds__(kDigestThreads) digest_blocks_kernel(const float* rgb, size_t n,
                                                                        unsigned long long* part_h, double* part_s) {
    unsigned long long h = 0ull;
    double s = 0.0;
    for (size_t i = blockIdx.x * (size_t)kDigestThreads + threadIdx.x; i < n; i += (size_t)gridDim.x * kDigestThreads) {
        unsigned long long x = (unsigned long long)__float_as_uint(rgb[i]) + 0x9E3779B97F4A7C15ull * (i + 1);
        x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
        x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
        h += x ^ (x >> 31);
        s += (double)rgb[i];
    }
    for (int o = 16; o > 0; o >>= 1) {
        h += __shfl_xor_sync(0xffffffffu, h, o);
        s += __shfl_xor_sync(0xffffffffu, s, o);
    }
    __shared__ unsigned long long sh[kDigestThreads / 32];
    __shared__ double ss[kDigestThreads / 32];
    if ((threadIdx.x & 31) == 0) {
        sh[threadIdx.x >> 5] = h;
        ss[threadIdx.x >> 5] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kDigestThreads / 32; ++w) {
            h += sh[w];
            s += ss[w];
        }
        part_h[blockIdx.x] = h;
        part_s[blockIdx.x] = s;
    }
}

__global__ void digest_final_kernel(const unsigned long long* part_h, const double* part_s, int n,
                                    unsigned long long* out_h, double* out_s) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned long long h = 0ull;
    double s = 0.0;
    for (int b = 0; b < n; ++b) {
        h += part_h[b];
        s += part_s[b];
    }
    *out_h = h;
    *out_s = s;
}

struct ShapeKey {
    int w, h, n;
    long long pts;
    int reduced;
    bool operator<(const ShapeKey& o) const {
        return std::tie(w, h, n, pts, reduced) < std::tie(o.w, o.h, o.n, o.pts, o.reduced);
    }
};

struct RoomKey {
    unsigned long long seed;
    int n;
    long long pts;
    bool operator<(const RoomKey& o) const { return std::tie(seed, n, pts) < std::tie(o.seed, o.n, o.pts); }
};

struct RoomState {
    float* points = nullptr;
    uint32_t* counts = nullptr;
    size_t bytes = 0;
    long long stride = 0;
    cudaEvent_t ready = nullptr;
    int users = 0;
    std::list<RoomKey>::iterator lru;
};

struct Slot {
    mlgi_ctx* ctx = nullptr;
    cudaStream_t stream = nullptr;  // the context's stream
    float *gd = nullptr, *rd = nullptr, *rgb = nullptr;
    void* gn = nullptr;
    uint32_t *rn = nullptr, *rf = nullptr;
    unsigned long long* part_h = nullptr;  // kDigestBlocks digests, then the total
    double* part_s = nullptr;
    unsigned long long* h_out = nullptr;   // pinned: digest, sum
    cudaEvent_t done = nullptr;
    std::atomic<double> t_done{0.0};
    bool busy = false;
    mlgi_request req{};
    RoomKey room{};
    double t_admit = 0;
};

enum class Fit { kOk, kWait, kNoMem };

}  // namespace

struct mlgi_server {
    mlgi_server_desc desc{};
    std::vector<Slot*> slots;
    Slot* plain = nullptr;  // the plain arm's slot (created on first use)
    size_t slot_bytes = 0;  // per slot, frame buffers and reserved context buffers
    std::mutex mu;          // queue, completions, rooms
    std::condition_variable cv;
    std::deque<mlgi_request> queue;
    std::vector<mlgi_completion> done;
    std::map<RoomKey, RoomState> rooms;
    std::list<RoomKey> lru;  // front = most recently used
    size_t room_bytes = 0;
    std::mutex tune_mu;
    std::map<ShapeKey, mlgi_autotune_result> tuned;
    mlgi_ctx* tune_ctx = nullptr;
    int reserved_vpl = 0;
    size_t reserved_texels = 0;
    std::thread worker;
    std::atomic<bool> stop{false};
    std::atomic<long long> inflight{0}, pending{0};
    long long admitted = 0, budget_waits = 0, evictions = 0;
};

namespace {

size_t frame_bytes(int max_w, int max_h, int rsm) {
    const size_t px = (size_t)max_w * max_h, rt = (size_t)rsm * rsm;
    return px * (4 + 8 + 12) + rt * 12 + kDigestBlocks * 16 + 64;
}

bool dalloc(void** p, size_t bytes) {
    if (mlgi::dev_alloc(p, std::max<size_t>(bytes, 16)) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return false;
    }
    return true;
}

void free_slot(Slot* sl) {
    if (!sl) return;
    if (sl->stream) cudaStreamSynchronize(sl->stream);
    for (void* p : {(void*)sl->gd, sl->gn, (void*)sl->rd, (void*)sl->rn, (void*)sl->rf, (void*)sl->rgb,
                    (void*)sl->part_h})
        if (p) cudaFree(p);
    if (sl->h_out) cudaFreeHost(sl->h_out);
    if (sl->done) cudaEventDestroy(sl->done);
    if (sl->ctx) mlgi_destroy(sl->ctx);
    delete sl;
}

Slot* make_slot(mlgi_server* sv) {
    Slot* sl = new Slot();
    mlgi_ctx_desc cd{sv->desc.device, 0};
    const size_t px = (size_t)sv->desc.max_width * sv->desc.max_height;
    const size_t rt = (size_t)sv->desc.rsm_size * sv->desc.rsm_size;
    bool ok = mlgi_create(&sl->ctx, &cd) == MLGI_OK;
    if (ok) sl->stream = static_cast<cudaStream_t>(mlgi_ctx_stream(sl->ctx));
    ok = ok && dalloc((void**)&sl->gd, px * 4) && dalloc(&sl->gn, px * 8) && dalloc((void**)&sl->rgb, px * 12) &&
         dalloc((void**)&sl->rd, rt * 4) && dalloc((void**)&sl->rn, rt * 4) && dalloc((void**)&sl->rf, rt * 4) &&
         dalloc((void**)&sl->part_h, (kDigestBlocks + 1) * 16);
    ok = ok && mlgi::pinned_alloc((void**)&sl->h_out, 16) == cudaSuccess;
    ok = ok && cudaEventCreateWithFlags(&sl->done, cudaEventDisableTiming) == cudaSuccess;
    if (ok && sv->reserved_vpl > 0) ok = mlgi_ctx_reserve(sl->ctx, sv->reserved_vpl, sv->reserved_texels) == MLGI_OK;
    if (!ok) {
        cudaGetLastError();
        free_slot(sl);
        return nullptr;
    }
    sl->part_s = reinterpret_cast<double*>(sl->part_h + kDigestBlocks + 1);
    return sl;
}

mlgi_scene_desc scene_desc(const mlgi_server* sv, const mlgi_request& r) {
    mlgi_scene_desc d{};
    d.seed = r.room_seed;
    d.n_boxes = 16;
    d.n_spheres = 8;
    d.width = r.width;
    d.height = r.height;
    d.rsm_width = d.rsm_height = sv->desc.rsm_size;
    d.n_points = r.n_points;
    d.n_buckets = r.n_vpl;
    d.ism_count = r.n_vpl;
    d.light_yaw_deg = r.light_yaw_deg;
    d.light_pitch_deg = r.light_pitch_deg;
    d.camera_orbit_deg = r.camera_orbit_deg;
    d.z_near = 1.f;
    d.z_far = 400.f;
    return d;
}

void evict_room(mlgi_server* sv, std::list<RoomKey>::iterator it, cudaStream_t s) {
    const RoomKey k = *it;
    RoomState& st = sv->rooms[k];
    cudaStreamWaitEvent(s, st.ready, 0);
    cudaFreeAsync(st.points, s);
    cudaEventDestroy(st.ready);
    sv->room_bytes -= st.bytes;
    sv->evictions++;
    sv->lru.erase(it);
    sv->rooms.erase(k);
}

// The room state of request `r` (caller holds sv->mu), generated on stream `s` on first use.
Fit get_room(mlgi_server* sv, const mlgi_request& r, cudaStream_t s, RoomState** out) {
    const RoomKey k{r.room_seed, r.n_vpl, (long long)r.n_points};
    auto it = sv->rooms.find(k);
    if (it != sv->rooms.end()) {
        sv->lru.erase(it->second.lru);
        sv->lru.push_front(k);
        it->second.lru = sv->lru.begin();
        *out = &it->second;
        return Fit::kOk;
    }
    const long long stride = (k.pts + k.n - 1) / k.n;
    const size_t bytes = (size_t)k.n * stride * 16 + (size_t)k.n * 4;
    const size_t fixed = sv->slot_bytes * (sv->slots.size() + (sv->plain ? 1 : 0));
    if (fixed + bytes > sv->desc.hbm_budget) return Fit::kNoMem;  // would not fit in an empty server
    // evict unused rooms, least recently used first, until the new one fits
    auto v = sv->lru.end();
    while (fixed + sv->room_bytes + bytes > sv->desc.hbm_budget && v != sv->lru.begin()) {
        --v;
        if (sv->rooms[*v].users == 0) {
            auto victim = v++;
            evict_room(sv, victim, s);
        }
    }
    if (fixed + sv->room_bytes + bytes > sv->desc.hbm_budget) return Fit::kWait;
    RoomState st;
    void* p = nullptr;
    if (mlgi::dev_alloc_async(&p, bytes, s) != cudaSuccess) {
        cudaGetLastError();
        return Fit::kNoMem;
    }
    st.points = static_cast<float*>(p);
    st.counts = reinterpret_cast<uint32_t*>(static_cast<char*>(p) + (size_t)k.n * stride * 16);
    st.bytes = bytes;
    st.stride = stride;
    cudaMemsetAsync(st.points, 0, (size_t)k.n * stride * 16, s);
    mlgi_scene_desc d = scene_desc(sv, r);
    mlgi_scene_info info;
    if (mlgi_scene_generate_device(&d, &info, nullptr, nullptr, MLGI_F32, nullptr, nullptr, nullptr, nullptr, st.points,
                                   st.counts, s) != MLGI_OK) {
        cudaFreeAsync(p, s);
        return Fit::kNoMem;
    }
    cudaEventCreateWithFlags(&st.ready, cudaEventDisableTiming);
    cudaEventRecord(st.ready, s);
    sv->lru.push_front(k);
    st.lru = sv->lru.begin();
    sv->room_bytes += bytes;
    *out = &(sv->rooms[k] = st);
    return Fit::kOk;
}

mlgi_status tune(mlgi_server* sv, const mlgi_request& r, mlgi_autotune_result* out) {
    std::lock_guard<std::mutex> lock(sv->tune_mu);
    const ShapeKey sk{r.width, r.height, r.n_vpl, (long long)r.n_points, r.reduced};
    auto t = sv->tuned.find(sk);
    if (t != sv->tuned.end()) {
        *out = t->second;
        return MLGI_OK;
    }
    mlgi_autotune_query q{r.width, r.height, r.n_vpl, r.n_points, r.reduced, sv->desc.rsm_size, 16, 64, 0, 0.f, 1};
    const mlgi_status st = mlgi_autotune(sv->tune_ctx, &q, out);
    if (st == MLGI_OK) sv->tuned[sk] = *out;
    return st;
}

void CUDART_CB stamp_done(void* p) { static_cast<Slot*>(p)->t_done.store(now_s()); }

// Issue one request's frame on `sl` (the request is in sl->req).
mlgi_status issue(mlgi_server* sv, Slot* sl, const RoomState* room) {
    const mlgi_request& r = sl->req;
    mlgi_autotune_result tu;
    mlgi_status st = tune(sv, r, &tu);
    if (st != MLGI_OK) return st;
    const int R = sv->desc.rsm_size;
    const int fmt = r.reduced ? MLGI_F16 : MLGI_F32;
    mlgi_scene_desc d = scene_desc(sv, r);
    mlgi_scene_info info;
    cudaStreamWaitEvent(sl->stream, room->ready, 0);
    st = mlgi_scene_generate_device(&d, &info, sl->gd, sl->gn, fmt, nullptr, sl->rd, sl->rn, sl->rf, nullptr, nullptr,
                                    sl->stream);
    if (st != MLGI_OK) return st;
    mlgi_frame_desc f{};
    f.rsm = mlgi_rsm_view{R, R, sl->rd, sl->rn, sl->rf};
    f.vpl.count = r.n_vpl;
    f.vpl.light_intensity = 5.f;
    f.vpl.shuffle = 1;
    std::memcpy(f.vpl.inv_biased_light_vp, info.inv_biased_light_vp, sizeof(f.vpl.inv_biased_light_vp));
    f.points = mlgi_points{room->points, room->counts, r.n_vpl, room->stride};
    f.ism = mlgi_ism_params{0, r.n_vpl, 0, 0, tu.ism_size, tu.grid_x, tu.grid_y, tu.levels, 400.f};
    f.atlas_format = fmt;
    f.gbuffer = mlgi_gbuffer_view{r.width, r.height, sl->gd, sl->gn, fmt};
    std::memcpy(f.fg.inv_view_proj, info.inv_view_proj, sizeof(f.fg.inv_view_proj));
    f.fg.z_far = 400.f;
    f.fg.gi_intensity = 3000.f;
    f.fg.clamp_value = 0.001f;
    f.fg.vpl_count = r.n_vpl;
    f.fg.vpl_start = 0;
    f.fg.vpl_end = r.n_vpl;
    f.fg.scale_isms = 0;
    f.fg.ism_size = tu.ism_size;
    f.fg.grid_x = tu.grid_x;
    f.fg.grid_y = tu.grid_y;
    f.fg.interleave = tu.interleave;
    f.fg.shadowing = 1;
    f.fg.tile = tu.tile;
    f.fg.cull = 1;
    f.fg.vpl_format = fmt;
    mlgi_radiance out{r.width, r.height, sl->rgb};
    if ((st = mlgi_gi_frame(sl->ctx, &f, &out, sl->stream)) != MLGI_OK) return st;
    const size_t n = (size_t)r.width * r.height * 3;
    digest_blocks_kernel<<<kDigestBlocks, kDigestThreads, 0, sl->stream>>>(sl->rgb, n, sl->part_h, sl->part_s);
    digest_final_kernel<<<1, 32, 0, sl->stream>>>(sl->part_h, sl->part_s, kDigestBlocks, sl->part_h + kDigestBlocks,
                                                  sl->part_s + kDigestBlocks);
    cudaMemcpyAsync(sl->h_out, sl->part_h + kDigestBlocks, 8, cudaMemcpyDeviceToHost, sl->stream);
    cudaMemcpyAsync(sl->h_out + 1, sl->part_s + kDigestBlocks, 8, cudaMemcpyDeviceToHost, sl->stream);
    if (r.out_host) cudaMemcpyAsync(r.out_host, sl->rgb, n * 4, cudaMemcpyDeviceToHost, sl->stream);
    cudaLaunchHostFunc(sl->stream, stamp_done, sl);
    cudaEventRecord(sl->done, sl->stream);
    return cudaGetLastError() == cudaSuccess ? MLGI_OK : MLGI_ECUDA;
}

mlgi_completion completion_of(Slot* sl, mlgi_status launch_status, cudaError_t q) {
    mlgi_completion c{};
    c.id = sl->req.id;
    c.status = launch_status != MLGI_OK ? launch_status
               : q != cudaSuccess       ? MLGI_ECUDA
                                        : mlgi_check_device_status(sl->ctx, sl->stream);
    const double t_done = launch_status == MLGI_OK ? sl->t_done.load() : now_s();
    c.latency_ms = (t_done - sl->req.arrival_s) * 1e3;
    c.queue_ms = (sl->t_admit - sl->req.arrival_s) * 1e3;
    if (c.status == MLGI_OK) {
        std::memcpy(&c.digest, sl->h_out, 8);
        std::memcpy(&c.sum, sl->h_out + 1, 8);
    }
    return c;
}

void finish(mlgi_server* sv, Slot* sl, const mlgi_completion& c) {
    std::lock_guard<std::mutex> lock(sv->mu);
    sv->done.push_back(c);
    auto it = sv->rooms.find(sl->room);
    if (it != sv->rooms.end()) it->second.users--;
    sl->busy = false;
    sv->inflight--;
    sv->pending--;
}

// Caller holds sv->mu.
void complete_unissued(mlgi_server* sv, const mlgi_request& r, mlgi_status st) {
    mlgi_completion c{};
    c.id = r.id;
    c.status = st;
    c.latency_ms = (now_s() - r.arrival_s) * 1e3;
    sv->done.push_back(c);
    sv->pending--;
}

void worker_loop(mlgi_server* sv) {
    cudaSetDevice(sv->desc.device);
    const size_t max_px = (size_t)sv->desc.max_width * sv->desc.max_height;
    while (true) {
        bool progressed = false;
        for (Slot* sl : sv->slots) {
            if (!sl->busy) continue;
            const cudaError_t q = cudaEventQuery(sl->done);
            if (q == cudaErrorNotReady) continue;
            finish(sv, sl, completion_of(sl, MLGI_OK, q));
            progressed = true;
        }
        for (Slot* sl : sv->slots) {
            if (sl->busy) continue;
            RoomState* room = nullptr;
            {
                std::lock_guard<std::mutex> lock(sv->mu);
                while (!sv->queue.empty() && (size_t)sv->queue.front().width * sv->queue.front().height > max_px) {
                    complete_unissued(sv, sv->queue.front(), MLGI_EINVAL);
                    sv->queue.pop_front();
                    progressed = true;
                }
                if (sv->queue.empty()) break;
                const Fit fit = get_room(sv, sv->queue.front(), sl->stream, &room);
                if (fit == Fit::kNoMem || (fit == Fit::kWait && sv->inflight == 0)) {
                    complete_unissued(sv, sv->queue.front(), MLGI_ENOMEM);
                    sv->queue.pop_front();
                    progressed = true;
                    continue;
                }
                if (fit == Fit::kWait) {
                    sv->budget_waits++;
                    break;  // the head of the queue waits for completions to release rooms
                }
                room->users++;
                sl->req = sv->queue.front();
                sv->queue.pop_front();
                sl->room = RoomKey{sl->req.room_seed, sl->req.n_vpl, (long long)sl->req.n_points};
                sl->busy = true;
                sv->inflight++;
                sv->admitted++;
            }
            sl->t_admit = now_s();
            const mlgi_status st = issue(sv, sl, room);
            if (st != MLGI_OK) finish(sv, sl, completion_of(sl, st, cudaSuccess));
            progressed = true;
        }
        if (sv->stop && sv->pending == 0) break;
        if (!progressed) {
            std::unique_lock<std::mutex> lock(sv->mu);
            if (sv->queue.empty() && sv->inflight == 0 && !sv->stop)
                sv->cv.wait_for(lock, std::chrono::milliseconds(5));
            else
                sv->cv.wait_for(lock, std::chrono::microseconds(10));
        }
    }
}

}  // namespace

extern "C" {

mlgi_status mlgi_server_drain(mlgi_server* sv, double timeout_s) {
    if (!sv) return MLGI_EINVAL;
    const double t_end = now_s() + timeout_s;
    while (sv->pending > 0) {
        if (now_s() > t_end) return MLGI_ETIMEDOUT;
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    return MLGI_OK;
}

void mlgi_server_destroy(mlgi_server* sv) {
    if (!sv) return;
    if (sv->worker.joinable()) {
        mlgi_server_drain(sv, 600.0);
        sv->stop = true;
        sv->cv.notify_all();
        sv->worker.join();
    }
    cudaSetDevice(sv->desc.device);
    for (Slot* sl : sv->slots) free_slot(sl);
    free_slot(sv->plain);
    cudaDeviceSynchronize();
    for (auto& kv : sv->rooms) {
        cudaFree(kv.second.points);
        cudaEventDestroy(kv.second.ready);
    }
    if (sv->tune_ctx) mlgi_destroy(sv->tune_ctx);
    delete sv;
}

mlgi_status mlgi_server_create(const mlgi_server_desc* desc, mlgi_server** out) {
    if (!desc || !out || desc->slots <= 0 || desc->slots > 64 || desc->max_width <= 0 || desc->max_height <= 0)
        return MLGI_EINVAL;
    *out = nullptr;
    if (cudaSetDevice(desc->device) != cudaSuccess) {
        cudaGetLastError();
        return MLGI_ECUDA;
    }
    mlgi_server* sv = new mlgi_server();
    sv->desc = *desc;
    if (sv->desc.rsm_size <= 0) sv->desc.rsm_size = 512;
    sv->slot_bytes = frame_bytes(desc->max_width, desc->max_height, sv->desc.rsm_size);
    if (sv->slot_bytes * desc->slots > desc->hbm_budget) {
        delete sv;
        return MLGI_ENOMEM;
    }
    mlgi_ctx_desc cd{desc->device, 0};
    const mlgi_status cst = mlgi_create(&sv->tune_ctx, &cd);
    if (cst != MLGI_OK) {
        mlgi_server_destroy(sv);
        return cst;
    }
    for (int i = 0; i < desc->slots; ++i) {
        Slot* sl = make_slot(sv);
        if (!sl) {
            mlgi_server_destroy(sv);
            return MLGI_ENOMEM;
        }
        sv->slots.push_back(sl);
    }
    sv->worker = std::thread(worker_loop, sv);
    *out = sv;
    return MLGI_OK;
}

mlgi_status mlgi_server_prepare(mlgi_server* sv, const mlgi_request* shapes, int n) {
    if (!sv || n < 0 || (n > 0 && !shapes)) return MLGI_EINVAL;
    cudaSetDevice(sv->desc.device);
    int max_vpl = 64;
    size_t max_texels = 1;
    for (int i = 0; i < n; ++i) {
        if (shapes[i].n_vpl <= 0 || shapes[i].n_vpl % 64) return MLGI_EINVAL;
        mlgi_autotune_result tu;
        const mlgi_status st = tune(sv, shapes[i], &tu);
        if (st != MLGI_OK) return st;
        max_vpl = std::max(max_vpl, shapes[i].n_vpl);
        max_texels = std::max(max_texels, (size_t)tu.grid_x * tu.grid_y * tu.ism_size * tu.ism_size);
    }
    // buffers are resized only while nothing is in flight
    if (mlgi_server_drain(sv, 600.0) != MLGI_OK) return MLGI_ETIMEDOUT;
    sv->reserved_vpl = std::max(sv->reserved_vpl, max_vpl);
    sv->reserved_texels = std::max(sv->reserved_texels, max_texels);
    const size_t ctx_bytes = (size_t)sv->reserved_vpl * (48 + 16 + 24) + sv->reserved_texels * 8;
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        sv->slot_bytes = frame_bytes(sv->desc.max_width, sv->desc.max_height, sv->desc.rsm_size) + ctx_bytes;
    }
    for (Slot* sl : sv->slots) {
        const mlgi_status st = mlgi_ctx_reserve(sl->ctx, sv->reserved_vpl, sv->reserved_texels);
        if (st != MLGI_OK) return st;
    }
    if (sv->plain) return mlgi_ctx_reserve(sv->plain->ctx, sv->reserved_vpl, sv->reserved_texels);
    return MLGI_OK;
}

mlgi_status mlgi_server_submit(mlgi_server* sv, const mlgi_request* r) {
    if (!sv || !r) return MLGI_EINVAL;
    if (r->n_vpl <= 0 || r->n_vpl % 64 || r->width <= 0 || r->height <= 0 || r->n_points <= 0 ||
        (r->reduced != 0 && r->reduced != 1))
        return MLGI_EINVAL;
    {
        std::lock_guard<std::mutex> lock(sv->mu);
        sv->queue.push_back(*r);
        if (sv->queue.back().arrival_s <= 0) sv->queue.back().arrival_s = now_s();
        sv->pending++;
    }
    sv->cv.notify_all();
    return MLGI_OK;
}

int mlgi_server_poll(mlgi_server* sv, mlgi_completion* out, int max) {
    if (!sv || !out || max <= 0) return 0;
    std::lock_guard<std::mutex> lock(sv->mu);
    const int n = std::min<int>(max, (int)sv->done.size());
    std::copy(sv->done.begin(), sv->done.begin() + n, out);
    sv->done.erase(sv->done.begin(), sv->done.begin() + n);
    return n;
}

mlgi_status mlgi_server_cancel(mlgi_server* sv, uint64_t id) {
    if (!sv) return MLGI_EINVAL;
    std::lock_guard<std::mutex> lock(sv->mu);
    for (auto it = sv->queue.begin(); it != sv->queue.end(); ++it) {
        if (it->id != id) continue;
        complete_unissued(sv, *it, MLGI_ECANCELED);
        sv->queue.erase(it);
        return MLGI_OK;
    }
    return MLGI_EINVAL;
}

mlgi_status mlgi_server_stats_get(mlgi_server* sv, mlgi_server_stats* st) {
    if (!sv || !st) return MLGI_EINVAL;
    std::lock_guard<std::mutex> lock(sv->mu);
    st->queued = (int64_t)sv->queue.size();
    st->inflight = sv->inflight;
    st->admitted = sv->admitted;
    st->rooms_resident = (int64_t)sv->rooms.size();
    st->budget_waits = sv->budget_waits;
    st->evictions = sv->evictions;
    st->room_bytes = sv->room_bytes;
    st->slot_bytes = sv->slot_bytes * (sv->slots.size() + (sv->plain ? 1 : 0));
    return MLGI_OK;
}

mlgi_status mlgi_server_run_poisson(mlgi_server* sv, const mlgi_poisson_desc* pd, mlgi_completion* out, int max_out,
                                    int* n_out, double* wall_s) {
    if (!sv || !pd || !out || !n_out || max_out <= 0 || pd->n_shapes <= 0 || !pd->shapes || pd->rate_hz <= 0 ||
        pd->duration_s <= 0 || (pd->mode != 0 && pd->mode != 1))
        return MLGI_EINVAL;
    cudaSetDevice(sv->desc.device);
    // the request sequence is a function of the descriptor only
    std::mt19937_64 rng(pd->seed);
    std::exponential_distribution<double> gap(pd->rate_hz);
    std::uniform_int_distribution<int> pick(0, pd->n_shapes - 1), room(0, std::max(1, pd->n_rooms) - 1);
    std::uniform_real_distribution<double> jit(-pd->light_jitter_deg, pd->light_jitter_deg);
    std::vector<double> orbit(std::max(1, pd->n_rooms), 0.0);
    std::vector<mlgi_request> reqs;
    for (double t = gap(rng); t <= pd->duration_s; t += gap(rng)) {
        mlgi_request r = pd->shapes[pick(rng)];
        const int rm = room(rng);
        r.id = reqs.size();
        r.room_seed = pd->room_seed_base + (uint64_t)rm;
        r.light_yaw_deg = (float)jit(rng);
        r.light_pitch_deg = (float)jit(rng);
        orbit[rm] += pd->orbit_step_deg;
        if (orbit[rm] > 10.0) orbit[rm] -= 20.0;
        r.camera_orbit_deg = (float)orbit[rm];
        r.out_host = nullptr;
        r.arrival_s = t;  // relative until the run starts
        reqs.push_back(r);
    }
    const double drain = pd->drain_timeout_s > 0 ? pd->drain_timeout_s : 600.0;
    if (pd->mode == 1 && !sv->plain) {
        Slot* sl = make_slot(sv);
        if (!sl) return MLGI_ENOMEM;
        std::lock_guard<std::mutex> lock(sv->mu);
        sv->plain = sl;
    }
    int n = 0;
    mlgi_status result = MLGI_OK;
    const double t0 = now_s();
    if (pd->mode == 0) {
        for (mlgi_request& r : reqs) {
            r.arrival_s += t0;
            while (now_s() < r.arrival_s) {
                if (n < max_out) n += mlgi_server_poll(sv, out + n, max_out - n);
                std::this_thread::yield();
            }
            mlgi_server_submit(sv, &r);
        }
        result = mlgi_server_drain(sv, drain);
        if (n < max_out) n += mlgi_server_poll(sv, out + n, max_out - n);
    } else {
        Slot* sl = sv->plain;
        for (mlgi_request& r : reqs) {
            r.arrival_s += t0;
            while (now_s() < r.arrival_s) std::this_thread::yield();
            if (now_s() - t0 > pd->duration_s + drain) {
                result = MLGI_ETIMEDOUT;
                break;
            }
            RoomState* room = nullptr;
            Fit fit;
            {
                std::lock_guard<std::mutex> lock(sv->mu);
                fit = get_room(sv, r, sl->stream, &room);
                if (fit == Fit::kOk) room->users++;
            }
            mlgi_completion c{};
            if (fit != Fit::kOk) {
                c.id = r.id;
                c.status = MLGI_ENOMEM;
            } else {
                sl->req = r;
                sl->room = RoomKey{r.room_seed, r.n_vpl, (long long)r.n_points};
                sl->t_admit = now_s();
                const mlgi_status st = issue(sv, sl, room);
                const cudaError_t q = st == MLGI_OK ? cudaEventSynchronize(sl->done) : cudaSuccess;
                c = completion_of(sl, st, q);
                std::lock_guard<std::mutex> lock(sv->mu);
                room->users--;
            }
            if (n < max_out) out[n++] = c;
        }
    }
    *n_out = n;
    if (wall_s) *wall_s = now_s() - t0;
    return result;
}

}  // extern "C"
