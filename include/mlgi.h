/*
 * mlgi.h -- C ABI of the GB300 many-lights GI hot path.
 *
 * One entry point per painter stage of the reference (paths inside the reference project):
 *   mlgi_vpl_process   replaces VPLProcessor::process
 *                      (source/mfs-painters/multiframepainter/VPLProcessor.h:22, VPLProcessor.cpp:73-101)
 *                      and the compute pass data/shaders/gi/vpl_processor.comp:41-72
 *   mlgi_ism_splat     replaces ImperfectShadowmap::render's compute path
 *                      (ImperfectShadowmap.cpp:194-261: atlas clear :212, dispatch of ism.comp :257)
 *                      and data/shaders/ism/ism.comp:54-139
 *   mlgi_pullpush      replaces ImperfectShadowmap::pullpush (ImperfectShadowmap.cpp:121-182)
 *                      and data/shaders/ism/pull.comp:20-126 + push.comp:44-165
 *   mlgi_final_gather  replaces GIStage::compute_final_gathering (GIStage.h:66, GIStage.cpp:261-306)
 *                      and data/shaders/gi/final_gathering.comp:63-135
 *   mlgi_gi_frame      replaces GIStage::process's GI chain (GIStage.cpp:346-418: VPLP, ISM, FG)
 *
 * Conventions
 *   - The caller owns every buffer passed in; the library never frees them. A context owns its
 *     scratch space (pull-push pyramid, frame-level VPL buffers and atlas, shuffle tables).
 *   - Every call returns an mlgi_status; mlgi_last_error() gives the detail of the last failure.
 *   - Device calls are asynchronous on the given stream (NULL = the context's own stream).
 *   - A context is thread-compatible (one thread at a time); separate contexts are thread-safe.
 *   - Pointers marked "device" must be device memory of the context's GPU; "host" pointers are
 *     ordinary (preferably pinned) host memory.
 */
#ifndef MLGI_H
#define MLGI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t mlgi_status;
#define MLGI_OK 0
#define MLGI_EINVAL 1      /* bad argument or unsupported configuration */
#define MLGI_ENOMEM 2      /* device or host allocation failed, or admission over budget */
#define MLGI_ETIMEDOUT 3   /* a bounded device-side wait gave up */
#define MLGI_ECUDA 4       /* a CUDA runtime call failed */
#define MLGI_ECANCELED 5   /* a queued request was cancelled */
#define MLGI_EBOUNDS 6     /* bounds-checked library only: a kernel computed an index outside its buffer */

typedef struct mlgi_ctx mlgi_ctx;
typedef void* mlgi_stream; /* a cudaStream_t; NULL selects the context's stream */

/* storage formats */
#define MLGI_F32 0
#define MLGI_F16 1
#define MLGI_BF16 2
#define MLGI_R11G11B10F 3  /* one 32-bit word per pixel, as GL_R11F_G11F_B10F */
#define MLGI_RGBA8 4       /* one 32-bit word per pixel, UNORM, r in bits 0-7 */

typedef struct {
    int device;          /* CUDA device ordinal */
    uint32_t flags;      /* reserved, 0 */
} mlgi_ctx_desc;

mlgi_status mlgi_create(mlgi_ctx** out, const mlgi_ctx_desc* desc);
void mlgi_destroy(mlgi_ctx* ctx);
const char* mlgi_last_error(const mlgi_ctx* ctx);
const char* mlgi_status_string(mlgi_status s);
/* Default stream of the context (a cudaStream_t). */
mlgi_stream mlgi_ctx_stream(mlgi_ctx* ctx);

/* ---- VPL processor ------------------------------------------------------------------------ */

/* RSM of the light as RasterizationStage writes it with renderRSM = true
 * (RasterizationStage.cpp:139-149): device pointers, width*height texels each. */
typedef struct {
    int width, height;
    const float* depth;      /* window depth in [0,1] */
    const uint32_t* normal;  /* RGB10_A2 UNORM of n*0.5+0.5 (r in bits 0-9) */
    const uint32_t* diffuse; /* RGBA8 UNORM flux basis (r in bits 0-7) */
} mlgi_rsm_view;

typedef struct {
    int count;                      /* N VPLs; a multiple of 64 (one 64-wide group per 64 VPLs) */
    float light_intensity;          /* GIStage "LightIntensity" */
    int shuffle;                    /* GIStage "ShuffleLights" */
    float inv_biased_light_vp[16];  /* inverse(bias * P_light * V_light), column-major */
} mlgi_vpl_params;

/* VPL buffers (device). `vpl` and `packed` are the reference's vplBuffer and packedVplBuffer
 * (VPLProcessor.cpp:29-41). `reduced` (optional, may be NULL) receives the reduced-precision
 * gather record: float pos[3], half normal[3], bfloat16 flux[3] (24 bytes per VPL). */
typedef struct {
    int capacity;
    float* vpl;     /* capacity x 12 floats: pos, pad, normal, pad, flux, pad (48-byte stride) */
    float* packed;  /* capacity x 4 floats: pos, uintBitsToFloat(pack3SN(normal)) */
    void* reduced;  /* capacity x 24 bytes, 16-byte aligned, or NULL */
} mlgi_vpl_buf;

/* VPLProcessor::process: regular RSM sampling into the VPL buffers. */
mlgi_status mlgi_vpl_process(mlgi_ctx* ctx, const mlgi_rsm_view* rsm, const mlgi_vpl_params* params,
                             mlgi_vpl_buf* out, mlgi_stream stream);

/* Host: the fixed VPL shuffle of VPLProcessor.cpp:58-65 (std::iota, std::mt19937(1979982),
 * std::shuffle) for n entries. */
mlgi_status mlgi_shuffle_table(int n, int32_t* out_host);

/* ---- imperfect shadow maps ---------------------------------------------------------------- */

/* Bucketed point buffer: the contract the reference's ism.geom:59-69 produces. Bucket b holds
 * counts[b] points starting at entry b*bucket_stride. Each entry is 4 floats:
 * xyz position, uintBitsToFloat(packUnorm4x8(vec4(normal*0.5+0.5, radius/25))). */
typedef struct {
    const float* points;     /* device */
    const uint32_t* counts;  /* device, n_buckets entries */
    int n_buckets;           /* sampledVplCount */
    int64_t bucket_stride;   /* imageSize(pointBuffer) / sampledVplCount */
} mlgi_points;

typedef struct {
    int vpl_start, vpl_end;   /* GIStage VPLStartIndex / VPLEndIndex */
    int scale_isms;           /* GIStage ScaleISMs */
    int points_only_scaled;   /* GIStage PointsOnlyToScaledISMs */
    int ism_size;             /* texels per ISM edge (reference: 2048 / ismIndices1d) */
    int grid_x, grid_y;       /* ISM tile grid; the atlas is (grid_x*ism_size) x (grid_y*ism_size) */
    int levels;               /* pull-push levels; ism_size must be divisible by 2^levels */
    float z_far;              /* light projection far plane */
} mlgi_ism_params;

typedef struct {
    int width, height;   /* grid_x*ism_size, grid_y*ism_size */
    uint32_t* keys;      /* device: softrender keys (uint(depth*2^24) << 8 | radius byte) */
    void* depth;         /* device: pull-push result (final ISM depth) */
    int format;          /* MLGI_F32 or MLGI_F16 for `depth` */
} mlgi_atlas;

/* ImperfectShadowmap::render (compute path): clear keys to 0xFFFFFFFF, splat every bucketed
 * point into up to 4 of the 16 VPLs cached for its bucket by atomicMin. Bit-exact with the
 * reference's FP32 arithmetic. */
mlgi_status mlgi_ism_splat(mlgi_ctx* ctx, const mlgi_points* pts, const mlgi_vpl_buf* vpls, int n_vpl,
                           const mlgi_ism_params* params, mlgi_atlas* atlas, mlgi_stream stream);

/* ImperfectShadowmap::pullpush: fill holes of every ISM with the pull-push pyramid and write
 * atlas->depth. Bit-exact with the reference's FP32 arithmetic for the FP32 format. */
mlgi_status mlgi_pullpush(mlgi_ctx* ctx, mlgi_atlas* atlas, const mlgi_ism_params* params, mlgi_stream stream);

/* No counterpart in the reference: the pieces of mlgi_ism_splat + mlgi_pullpush for callers that
 * overlap them with their own uploads (mlgi_gi_frame_host does).
 *   mlgi_ism_clear        the key clear of mlgi_ism_splat.
 *   mlgi_ism_splat_range  the splat of buckets [bucket0, bucket0 + n_buckets) only, no clear.
 *                         After one clear, splatting every bucket once, in any partition and
 *                         order, gives mlgi_ism_splat's keys (atomicMin is order-independent).
 *   mlgi_pullpush_rows    the pull-push of ISM rows [row0, row1) of the grid. The pyramid of an
 *                         ISM reads only its own keys, so running every row once, in any
 *                         partition, gives mlgi_pullpush's atlas; runs of different rows may
 *                         execute concurrently on different streams. A row's keys are final once
 *                         every bucket that splats into the row or into a row next to it is done:
 *                         bucket b splats into the ISMs of VPLs b..b+15 (mod N), and rounding at
 *                         a paraboloid's rim can put a point on the border texels of a
 *                         neighbouring ISM; a point on a VPL's position lands on texel (0, 0). */
mlgi_status mlgi_ism_clear(mlgi_ctx* ctx, mlgi_atlas* atlas, mlgi_stream stream);
/* No counterpart in the reference: the number of atomicMin operations mlgi_ism_splat issues for
 * these inputs (projections that land inside the atlas, at most 4 per point), from the splat's own
 * cull and projection run without the atomics. Synchronous on the context's stream; for reporting
 * the splat's atomic rate. */
mlgi_status mlgi_ism_splat_count(mlgi_ctx* ctx, const mlgi_points* pts, const mlgi_vpl_buf* vpls, int n_vpl,
                                 const mlgi_ism_params* params, const mlgi_atlas* atlas, uint64_t* atomics);
mlgi_status mlgi_ism_splat_range(mlgi_ctx* ctx, const mlgi_points* pts, const mlgi_vpl_buf* vpls, int n_vpl,
                                 const mlgi_ism_params* params, mlgi_atlas* atlas, int bucket0, int n_buckets,
                                 mlgi_stream stream);
mlgi_status mlgi_pullpush_rows(mlgi_ctx* ctx, mlgi_atlas* atlas, const mlgi_ism_params* params, int row0, int row1,
                               mlgi_stream stream);
/* No counterpart in the reference: the number of kernel launches mlgi_pullpush issues for this
 * geometry -- 1 when each ISM's whole pyramid runs in one block (ISM edges up to 128 with two or
 * more levels, far plane in [2^-20, 2^20], and at most one wave of such blocks on this GPU: 3 per
 * SM for edges up to 64, else 2); otherwise the per-level launches, 4 (2 for one level), for each
 * half of the ISM rows when the grid has two or more rows (the halves run side by side on the
 * caller's stream and the context's stream); -1 for a geometry mlgi_pullpush refuses.
 * mlgi_pullpush_rows chooses between the two forms the same way for the ISMs of its rows, and
 * launches one sequence. With per-pass timing, a pull-push in one block or in two halves reports
 * its time in the last of its four slots. */
int mlgi_pullpush_launches(const mlgi_ism_params* params);

/* No counterpart in the reference. Allocation-free ISM rendering for callers that cannot
 * allocate device memory (their device memory is reserved up front by another allocator, or
 * they run in a plugin or callback that is only handed pre-allocated buffers): clears, splats
 * and pull-pushes like mlgi_ism_splat + mlgi_pullpush, but keeps its intermediates (the key
 * atlas and pull-push pyramid levels 1 and 2, the latter used only when an ISM's pyramid does not
 * run in one block) in fixed device arrays inside the library instead of allocating them. Needs no context; runs on
 * the current device and on `stream` (NULL = the legacy default stream).
 *   - Atlas limit: grid_x*ism_size * grid_y*ism_size <= 1,048,576 texels (e.g. 1024 x 1024);
 *     larger atlases, and any geometry mlgi_ism_splat refuses, return MLGI_EINVAL.
 *   - The arrays (4 MiB of keys, 5 MiB of pyramid levels) are reserved on a device by the first
 *     call on it (under the CUDA runtime's default lazy module loading; at context creation with
 *     CUDA_MODULE_LOADING=EAGER) and stay until the process exits. A caller whose own allocator
 *     reserves the device memory up front should make that first call before the reservation;
 *     without room for the arrays the first call returns MLGI_ENOMEM. The first call looks the
 *     arrays up with the device current; make it before any stream capture. The addresses are
 *     kept per device for the process's life: do not use this entry point on a device after
 *     cudaDeviceReset.
 *   - Every call shares the arrays (the keys are cleared at the start of each call); calls whose
 *     work overlaps on the GPU race on them.
 *   - Calls no cudaMalloc, cudaFree or allocating library routine. */
mlgi_status mlgi_ism_render_static(const mlgi_points* pts, const mlgi_vpl_buf* vpls, int n_vpl,
                                   const mlgi_ism_params* params, void* depth_out, int depth_format,
                                   mlgi_stream stream);

/* ---- final gathering ---------------------------------------------------------------------- */

typedef struct {
    int width, height;
    const float* depth;   /* device: FP32 window depth */
    const void* normal;   /* device: octahedral normal, 2 x FP32 or 2 x FP16 per pixel */
    int normal_format;    /* MLGI_F32 or MLGI_F16 */
} mlgi_gbuffer_view;

typedef struct {
    float inv_view_proj[16]; /* viewInverted * projectionInverted, column-major */
    float z_far;             /* ISM far plane (the light projection's) */
    float gi_intensity;      /* GIIntensityFactor */
    float clamp_value;       /* VPLClampingValue */
    int vpl_count;           /* N */
    int vpl_start, vpl_end;  /* final_gathering.comp:40-46 */
    int scale_isms;
    int ism_size, grid_x, grid_y; /* atlas layout (see mlgi_ism_params) */
    int interleave;          /* interleaved-sampling factor I (N must be a multiple of I*I) */
    int shadowing;           /* GIShadowing */
    int tile;                /* work tile edge in same-class pixels: 8 or 16 (0 selects 16) */
    int cull;                /* 0: none; 1: per-tile culling against the tile's world-space bounds;
                                2: reference-style clustered culling (mlgi_cluster_lights), which
                                needs proj_a, proj_b and camera_z_far below */
    float influence_cutoff;  /* with cull 1: flux/d^4 contribution below which a VPL is dropped; 0 = off */
    int vpl_format;          /* MLGI_F32: 48-byte records; MLGI_F16: 24-byte reduced records */
    float proj_a, proj_b;    /* cull 2: projectionMatrix[2][2] and [3][2] of the camera */
    float camera_z_far;      /* cull 2: the camera's far plane */
} mlgi_fg_params;

/* ClusteredShading::process (ClusteredShading.cpp:70-112) with clustering.comp and light_lists.comp:
 * clusters of 128 x 128 pixels times 16 logarithmic depth slices; a used cluster keeps the VPLs
 * for which any of its corners lies in front of the VPL's plane. Outputs (device): `used`, one
 * word per tile (bit s = slice s is used; tiles_x = ceil(width / 128) per row), `masks`, per
 * cluster (tile * 16 + slice) ceil(n_vpl / 32) words of keep bits (rows of unused clusters are
 * left as they are), and `pixel_slice`, the slice of each pixel. Kept from the reference: slice 0
 * starting at view z = +0.05 and its corner list, which has (left, top) twice in place of
 * (right, top). The slice index is clamped to 15 (the reference's formula reaches 16 at the far
 * plane). With cull == 2, mlgi_final_gather runs this itself with context scratch. */
typedef struct {
    float inv_view_proj[16];  /* inverse(projection * view), column-major */
    float proj_a, proj_b;     /* projectionMatrix[2][2], [3][2] */
    float z_far;              /* the camera's far plane */
} mlgi_cluster_params;
mlgi_status mlgi_cluster_lights(mlgi_ctx* ctx, const mlgi_gbuffer_view* gbuffer, const mlgi_vpl_buf* vpls, int n_vpl,
                                const mlgi_cluster_params* params, uint32_t* used, uint32_t* masks,
                                uint8_t* pixel_slice, mlgi_stream stream);

typedef struct {
    int width, height;
    float* rgb;          /* device: width*height*3 floats */
} mlgi_radiance;

mlgi_status mlgi_final_gather(mlgi_ctx* ctx, const mlgi_gbuffer_view* gbuf, const mlgi_vpl_buf* vpls,
                              const mlgi_atlas* atlas, const mlgi_fg_params* params, mlgi_radiance* out,
                              mlgi_stream stream);

/* ---- whole GI chain (GIStage::process) ---------------------------------------------------- */

typedef struct {
    mlgi_rsm_view rsm;
    mlgi_vpl_params vpl;
    mlgi_points points;
    mlgi_ism_params ism;
    int atlas_format;        /* MLGI_F32 or MLGI_F16 */
    mlgi_gbuffer_view gbuffer;
    mlgi_fg_params fg;
} mlgi_frame_desc;

/* VPL processing -> ISM splat -> pull-push -> final gathering on device buffers; the VPL
 * buffers and the atlas are context-owned. A call that repeats the previous call's frame
 * description and output replays a CUDA graph of the frame, captured from the context's stream by
 * the second such call and launched on `stream` (the buffers' contents are read when the frame
 * runs, so new input data needs no new call form). Calls with per-pass timing, with new arguments,
 * or after a context buffer was reallocated run directly. */
mlgi_status mlgi_gi_frame(mlgi_ctx* ctx, const mlgi_frame_desc* frame, mlgi_radiance* out, mlgi_stream stream);

/* ---- after the gathering: GI buffer format, bilateral blur, composite ------------------------ */

/* GIStage's GI buffers are GL_R11F_G11F_B10F (GIStage.cpp:470). Packing of n RGB triples (device)
 * into words with R in bits 0-10, G in 11-21, B in 22-31: unsigned floats with a 5-bit exponent
 * (bias 15) and 6/6/5 mantissa bits, rounded to nearest even; negatives and -0 give 0, finite
 * values beyond the largest (65024 / 65024 / 64512) give the largest, +Inf gives Inf, NaN gives
 * NaN; denormals are kept. Unpacking is exact. */
mlgi_status mlgi_pack_r11g11b10f(mlgi_ctx* ctx, const float* rgb, uint32_t* words, int64_t n, mlgi_stream stream);
mlgi_status mlgi_unpack_r11g11b10f(mlgi_ctx* ctx, const uint32_t* words, float* rgb, int64_t n, mlgi_stream stream);

/* GIStage::blur (GIStage.cpp:308-344) with gi_blur.frag:24-72: a separable 7-tap bilateral filter,
 * the X pass then the Y pass, weights max(0, (4 - i)/4 - dz^2 - (5 (1 - max(0, N.n)))^2) from the
 * linear depth difference dz (reprojection.glsl linearDepth) and the G-buffer normals. Both passes
 * run in one kernel (the X pass of a tile and its 3-pixel halo rows is kept on chip). With
 * format MLGI_R11G11B10F, input, intermediate and output are R11G11B10F words, as the reference's
 * buffers are; with MLGI_F32 they are RGB floats. Samples outside the image are skipped (the
 * reference's texelFetch there is undefined). */
typedef struct {
    float proj_a, proj_b;  /* projectionMatrix[2][2] and [3][2] (column-major [col][row]) */
    int format;            /* MLGI_F32 or MLGI_R11G11B10F */
} mlgi_blur_params;
mlgi_status mlgi_gi_blur(mlgi_ctx* ctx, const mlgi_gbuffer_view* gbuffer, const void* gi_in, void* gi_out,
                         const mlgi_blur_params* params, mlgi_stream stream);

/* The GI part of the deferred composite (deferredshading.frag:47-81): ambient = GI * toLinear(albedo)
 * * occlusion, plus the caller's direct term (diffuse + specular, which need the light's shadow
 * map and are not part of this path), Reinhard tone mapping with exposure, then toSRGB (gamma
 * 2.2, srgb_utils.glsl). albedo: RGBA8 UNORM words; occlusion and direct may be NULL (1 and 0).
 * Output: RGB floats (out_format MLGI_F32) or RGBA8 UNORM words with alpha 255 (MLGI_RGBA8). */
typedef struct {
    int width, height;
    float exposure;
    int gi_format;   /* MLGI_F32 or MLGI_R11G11B10F */
    int out_format;  /* MLGI_F32 or MLGI_RGBA8 */
} mlgi_composite_params;
mlgi_status mlgi_composite(mlgi_ctx* ctx, const void* gi, const uint32_t* albedo, const float* occlusion,
                           const float* direct_rgb, void* out, const mlgi_composite_params* params,
                           mlgi_stream stream);

/* ---- batched views ------------------------------------------------------------------------- */

/* A fixed set of independent views (each an mlgi_frame_desc on device buffers plus its radiance
 * output) rendered together: every pass is ONE persistent launch over a device-resident view table
 * (work items of all views interleaved across the whole GPU), and the five launches plus the
 * table upload are captured once into a CUDA graph that mlgi_batch_launch replays. Views may mix
 * sizes, VPL counts, ISM layouts and precisions (a view is either all FP32 or all reduced: F16
 * atlas, F16 normals, F16 VPL records). Gathering uses 16 x 16 tiles. The batch owns every
 * view's VPL buffers and atlas (one device arena). Each view's result equals mlgi_gi_frame's for
 * the same inputs bit for bit. */
typedef struct mlgi_batch mlgi_batch;
mlgi_status mlgi_batch_create(mlgi_ctx* ctx, int n_views, const mlgi_frame_desc* views, const mlgi_radiance* outputs,
                              mlgi_batch** out);
/* Replace view i's parameters and buffers (same sizes and formats as at creation); synchronises
 * the batch's previous launch, takes effect at the next mlgi_batch_launch. */
mlgi_status mlgi_batch_update_view(mlgi_batch* b, int view, const mlgi_frame_desc* desc, const mlgi_radiance* output);
mlgi_status mlgi_batch_launch(mlgi_batch* b, mlgi_stream stream);
void mlgi_batch_destroy(mlgi_batch* b);

/* Batch forms. PERSISTENT (mlgi_batch_create): one persistent launch per pass over all views --
 * or, with `streams` = G > 1, over each of G view groups (balanced by estimated cost), every group
 * on its own stream with persistent grids of 1/G of the GPU, so that different groups' passes run
 * side by side (9 G launches). CONCURRENT: each view's own single-frame kernels, the views spread
 * over `streams` CUDA streams (balanced the same way) and joined in one graph, so that the kernels
 * of different views overlap (filling each other's tail waves and launch gaps). All give results
 * bit-identical to mlgi_gi_frame on each view. */
#define MLGI_BATCH_PERSISTENT 0
#define MLGI_BATCH_CONCURRENT 1
typedef struct {
    int form;     /* MLGI_BATCH_PERSISTENT or MLGI_BATCH_CONCURRENT */
    int streams;  /* PERSISTENT: view groups (0 selects 1); CONCURRENT: streams (0 selects 4); at most 64 */
} mlgi_batch_opts;
mlgi_status mlgi_batch_create_ex(mlgi_ctx* ctx, int n_views, const mlgi_frame_desc* views,
                                 const mlgi_radiance* outputs, const mlgi_batch_opts* opts, mlgi_batch** out);
/* Kernels one mlgi_batch_launch runs. */
int mlgi_batch_kernel_launches(const mlgi_batch* b);

/* ---- autotuner ------------------------------------------------------------------------------ */

/* Picks the interleave factor, ISM edge (with its pull-push levels and a power-of-two-wide ISM
 * grid) and gathering tile for a view shape by timing candidates on this GPU with the real kernels
 * (on a device-generated seeded room of that shape). budget_ms == 0: the fastest candidate meeting
 * the quality floor (n_vpl / I^2 >= min_vpls_per_pixel, ISM edge >= min_ism_size); budget_ms > 0:
 * the highest-quality candidate (most VPLs per pixel, then largest ISM) that fits the budget, or
 * the fastest if none does. batched != 0 restricts the tile to the batched gather's 16. Results
 * are cached per query for the life of the process. Synchronises the context's stream. */
typedef struct {
    int width, height, n_vpl;
    int64_t n_points;
    int reduced;
    int rsm_size;            /* 0 selects 512 */
    int min_vpls_per_pixel;  /* e.g. 16 */
    int min_ism_size;        /* e.g. 64 */
    int batched;
    float budget_ms;
    uint64_t seed;
} mlgi_autotune_query;

typedef struct {
    int interleave, ism_size, grid_x, grid_y, levels, tile;
    float ms;                /* measured frame time of the pick */
    int candidates_timed;
} mlgi_autotune_result;

mlgi_status mlgi_autotune(mlgi_ctx* ctx, const mlgi_autotune_query* query, mlgi_autotune_result* result);

/* Size the context's frame buffers (VPL records, key and depth atlases) for frames of up to
 * max_vpl VPLs and max_atlas_texels atlas texels, so that later frames within those bounds
 * allocate nothing. Synchronous. */
mlgi_status mlgi_ctx_reserve(mlgi_ctx* ctx, int max_vpl, size_t max_atlas_texels);

/* ---- request server ------------------------------------------------------------------------- */

/* Continuous-batching server of GI frames on one GPU (the served form of mlgi_gi_frame; the
 * reference renders one view per frame and has no server). A request names a room seed, a frame
 * shape and a pose; a scheduler thread admits queued requests FIFO into free slots (each slot a
 * context with its own stream and per-frame buffers), so frames of different requests overlap on
 * the device. Per-room state -- the bucketed surface points of (room seed, VPL count, point
 * count) -- is generated on the GPU on first use and stays resident, evicted least-recently-used
 * when the HBM budget (slots + resident rooms) would be exceeded; a request waits in the queue
 * while its room does not fit. Each frame's G-buffer and RSM are ray-cast on the device for its
 * pose, the chain runs with the autotuned configuration of its shape (16 VPLs per pixel floor,
 * 64^2 ISM floor; per-tile culling), and the radiance is reduced to an order-independent 64-bit
 * digest and an FP64 sum, and optionally copied to the request's host buffer. The results of a
 * request do not depend on what else is in flight. */
typedef struct mlgi_server mlgi_server;

typedef struct {
    int device;
    int slots;                  /* frames in flight */
    int max_width, max_height;  /* largest frame a request may ask for */
    int rsm_size;               /* 0 selects 512 */
    size_t hbm_budget;          /* bytes for slots + resident rooms */
} mlgi_server_desc;

typedef struct {
    uint64_t id;
    uint64_t room_seed;
    int width, height, n_vpl;   /* n_vpl a multiple of 64 */
    int64_t n_points;
    int reduced;                /* FP16 atlas, G-buffer normals and VPL attributes */
    float light_yaw_deg, light_pitch_deg, camera_orbit_deg;
    double arrival_s;           /* steady-clock seconds; <= 0 takes the submit time */
    float* out_host;            /* optional: width*height*3 floats, written before completion */
} mlgi_request;

typedef struct {
    uint64_t id;
    mlgi_status status;         /* MLGI_ECANCELED for a cancelled request */
    double latency_ms;          /* arrival -> completion observed by the scheduler */
    double queue_ms;            /* arrival -> admission */
    uint64_t digest;            /* order-independent digest of the radiance bits */
    double sum;                 /* FP64 sum of the radiance components */
} mlgi_completion;

typedef struct {
    int64_t queued, inflight, admitted, rooms_resident, budget_waits, evictions;
    size_t room_bytes, slot_bytes;
} mlgi_server_stats;

/* Create the server and its slots (allocations sized by max_width/max_height and rsm_size). */
mlgi_status mlgi_server_create(const mlgi_server_desc* desc, mlgi_server** out);
/* Autotune the given shapes (width, height, n_vpl, n_points, reduced of each entry) and reserve
 * every slot's buffers for the largest, so that serving allocates nothing but room state. */
mlgi_status mlgi_server_prepare(mlgi_server* sv, const mlgi_request* shapes, int n);
/* Queue a request (copied). MLGI_EINVAL for a malformed request; a frame larger than the
 * server's maximum completes with MLGI_EINVAL. */
mlgi_status mlgi_server_submit(mlgi_server* sv, const mlgi_request* req);
/* Cancel a request still in the queue (completes with MLGI_ECANCELED); MLGI_EINVAL if it is
 * unknown or already admitted. */
mlgi_status mlgi_server_cancel(mlgi_server* sv, uint64_t id);
/* Move up to `max` completions into `out`; returns how many. */
int mlgi_server_poll(mlgi_server* sv, mlgi_completion* out, int max);
/* Wait until every submitted request has completed (MLGI_ETIMEDOUT after timeout_s). */
mlgi_status mlgi_server_drain(mlgi_server* sv, double timeout_s);
mlgi_status mlgi_server_stats_get(mlgi_server* sv, mlgi_server_stats* stats);
/* Drains, then frees everything. */
void mlgi_server_destroy(mlgi_server* sv);

/* Open-loop Poisson load: arrivals at rate_hz for duration_s (seeded exponential gaps), each
 * request a shape drawn uniformly from `shapes`, a room drawn uniformly from n_rooms seeds
 * (room_seed_base + k), light yaw and pitch uniform in +-light_jitter_deg, and the room's camera
 * orbit advanced by orbit_step_deg per request (wrapping within +-10 degrees). Requests are
 * submitted at their arrival times from the calling thread; completions go to `out` (capacity
 * max_out). mode 0 serves through the server; mode 1 is the plain arm on the same request
 * sequence: one frame at a time on one stream, each issued when it has arrived and the previous
 * one has completed. */
typedef struct {
    uint64_t seed;
    double rate_hz, duration_s;
    const mlgi_request* shapes;
    int n_shapes;
    int n_rooms;
    uint64_t room_seed_base;
    float light_jitter_deg, orbit_step_deg;
    double drain_timeout_s;     /* 0 selects 600 */
    int mode;
} mlgi_poisson_desc;
mlgi_status mlgi_server_run_poisson(mlgi_server* sv, const mlgi_poisson_desc* desc, mlgi_completion* out,
                                    int max_out, int* n_out, double* wall_s);

/* Sizes of the host buffers mlgi_gi_frame_host reads, in bytes. */
typedef struct {
    size_t rsm_depth, rsm_normal, rsm_diffuse;
    size_t points, counts;
    size_t gbuf_depth, gbuf_normal;
    size_t radiance;
} mlgi_frame_host_sizes;
mlgi_status mlgi_frame_host_sizes_get(const mlgi_frame_desc* frame, mlgi_frame_host_sizes* sizes);

/* The same chain from HOST buffers: every pointer in `frame` is a host pointer; the call copies
 * the inputs to context-owned device buffers, runs the chain and copies the radiance back to
 * `rgb_host` before returning. Copies overlap the passes: point bucket ranges are splatted as they
 * arrive, the ISM rows a range completes are pulled and pushed before the next range, and the
 * gathering runs in bands of rows whose radiance is copied back while the next band runs. The
 * result equals mlgi_gi_frame's bit for bit. Pinned host memory gives the full copy bandwidth.
 * A call whose `frame` (every pointer and parameter) and `rgb_host` equal the previous call's, with
 * every host buffer pinned, captures the frame into a CUDA graph, and the calls after it replay
 * the graph (one launch instead of about a hundred API calls); each replay copies what the host
 * buffers hold at that time. A bucket count above bucket_stride (the bucket reads the next
 * buckets' entries, as the reference's splat does) makes the frame upload every point first. */
mlgi_status mlgi_gi_frame_host(mlgi_ctx* ctx, const mlgi_frame_desc* frame, float* rgb_host);

/* Per-pass device times (ms) of the last mlgi_gi_frame / mlgi_gi_frame_host call when timing is
 * enabled, named after the reference's PerfCounter passes:
 * [0] VPLP, [1] ISM clear, [2] ISM CS (splat), [3] pull-push, [4] FG, [5] H2D, [6] D2H, then the
 * pull-push pass's launches: [7] pull level 1, [8] middle levels, [9] push level 1, [10] push level 0.
 * After mlgi_gi_frame_host the passes overlap the copies: [2] spans the splat of every point range,
 * [3] the pull-push of the ISM rows finished by the last range (rows finished earlier run on a
 * second stream during [2]), [4] the banded gathering, [5] the whole upload, [6] the part of the
 * download left after the last band, and [7..10] are 0. Reading them synchronises the context's
 * stream. */
mlgi_status mlgi_set_timing(mlgi_ctx* ctx, int enabled);
mlgi_status mlgi_last_timings(mlgi_ctx* ctx, float* ms, int n);

/* Synchronise `stream` and report device-side errors recorded since the last check
 * (MLGI_ETIMEDOUT when a bounded wait inside a kernel gave up). Clears the error word. In the
 * bounds-checked library it first synchronises the device and reports MLGI_EBOUNDS when any
 * kernel of the process met an index outside its buffer since the last check (mlgi_last_error
 * names the source line and the index); those records are cleared too. */
mlgi_status mlgi_check_device_status(mlgi_ctx* ctx, mlgi_stream stream);

/* No counterpart in the reference (its only error handling is ModelLoadingStage.cpp:92-97): the
 * allocation-failure hook. With after >= 0 the library's next `after` device or pinned host
 * allocations succeed and every later one fails as out of memory, without asking CUDA, until the
 * hook is reset with -1 (the default). Calls whose allocation fails return MLGI_ENOMEM and leave
 * their context usable; a server request whose room cannot be allocated completes with
 * MLGI_ENOMEM. Process-wide; for tests. */
mlgi_status mlgi_set_alloc_fault(int64_t after);

/* The bounds-checked library, libmlgi_checked.so, is this library built with -DMLGI_CHECKS: its
 * kernels check the indices they compute against the extents of the buffers they address, record
 * the first one outside (its source line and value, per translation unit), and use index 0 in its
 * place, so that the access stays inside the buffer. 1 in that library, 0 in the normal one. */
int mlgi_checks_enabled(void);
/* Test of the checks themselves: reads element `index` of a device array of `extent` >= 1 floats
 * through a checked index. In the checked library an index outside [0, extent) is recorded (the
 * read goes to element 0) and mlgi_check_device_status then reports MLGI_EBOUNDS; the normal
 * library, whose index is unchecked, refuses it with MLGI_EINVAL and launches nothing. */
mlgi_status mlgi_check_index_selftest(mlgi_ctx* ctx, int64_t index, int64_t extent);
/* No counterpart in the reference: exercises the bounded device wait. The gathering stages each
 * VPL slice with a bulk copy completed on an mbarrier, and waits for it at most `wait_cycles` SM
 * cycles (0 restores the default, about 2^31; else 1000..2^31). A nonzero `extra_tx_bytes` (test
 * only, at most 4096) makes each block's first staging wait expect that many bytes more than its
 * copy delivers, so that the wait runs out: the block sets the status word, retires the surplus,
 * lets its copy land and returns, and mlgi_check_device_status then reports MLGI_ETIMEDOUT. The
 * settings apply to the context's later mlgi_final_gather calls; set (0, 0) to return to normal. */
mlgi_status mlgi_set_gather_wait_test(mlgi_ctx* ctx, int64_t wait_cycles, uint32_t extra_tx_bytes);

/* ---- scene fixture (host) ----------------------------------------------------------------- */

/* Seeded Cornell-style room: a 100 x 100 x 100 world-unit box (1 unit = 1 cm) with floor,
 * ceiling, back, left and right walls, n_boxes axis-aligned boxes and n_spheres spheres, a
 * ceiling spot light with a 60 degree cone and a pinhole camera. Stands in for the reference's
 * model loading and rasterisation stages, which are graphics-API code. */
typedef struct {
    uint64_t seed;
    int n_boxes, n_spheres;
    int width, height;          /* camera G-buffer */
    int rsm_width, rsm_height;  /* light RSM */
    int64_t n_points;           /* surface points, area-uniform */
    int n_buckets;              /* point buckets (sampledVplCount), round-robin assignment */
    int ism_count;              /* ISMs, for the sqrt(ismCount) point-radius boost (ism.geom:63) */
    float light_yaw_deg, light_pitch_deg;  /* jitter of the spot light direction */
    float camera_orbit_deg;     /* camera orbit around the room's vertical axis */
    float z_near, z_far;
} mlgi_scene_desc;

typedef struct {
    float view[16], proj[16], inv_view_proj[16];               /* camera, column-major */
    float light_view[16], light_proj[16], inv_biased_light_vp[16];
    float eye[3], light_pos[3], light_dir[3];
    float z_near, z_far;
    float total_area, point_radius;                            /* world units */
    int64_t bucket_stride;
} mlgi_scene_info;

/* Fill the host buffers that are not NULL:
 *   gbuf_depth  width*height floats         gbuf_normal width*height*2 floats (octahedral)
 *   gbuf_albedo width*height RGBA8 words
 *   rsm_depth   rsm_width*rsm_height floats rsm_normal / rsm_diffuse rsm_width*rsm_height words
 *   points      n_buckets*bucket_stride*4 floats; counts n_buckets words
 * bucket_stride = ceil(n_points / n_buckets). Runs on all host threads. */
mlgi_status mlgi_scene_generate(const mlgi_scene_desc* desc, mlgi_scene_info* info, float* gbuf_depth,
                                float* gbuf_normal, uint32_t* gbuf_albedo, float* rsm_depth, uint32_t* rsm_normal,
                                uint32_t* rsm_diffuse, float* points, uint32_t* counts);

/* The same seeded room generated on the device: the G-buffer and the RSM ray-cast by CUDA
 * kernels (FP32) and the bucketed points sampled on the GPU, so that a frame needs no host upload.
 * Buffers are device pointers (any may be NULL); gbuf_normal is 2 x FP32 or 2 x FP16 per pixel
 * (gbuf_normal_format). The objects and matrices are those of mlgi_scene_generate for the same
 * descriptor; values agree with the host fixture to FP32 rounding. At most 32 boxes and 16
 * spheres. Asynchronous on `stream`; allocates nothing. */
mlgi_status mlgi_scene_generate_device(const mlgi_scene_desc* desc, mlgi_scene_info* info, float* gbuf_depth,
                                       void* gbuf_normal, int gbuf_normal_format, uint32_t* gbuf_albedo,
                                       float* rsm_depth, uint32_t* rsm_normal, uint32_t* rsm_diffuse,
                                       float* points, uint32_t* counts, mlgi_stream stream);

#ifdef __cplusplus
}
#endif

#endif /* MLGI_H */
