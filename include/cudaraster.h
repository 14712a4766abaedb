/*
 * cudaraster.h -- C ABI of the GB300 sort-middle rasterizer.
 *
 * Every entry point takes plain pointers and sizes (device pointers where
 * noted) and returns a cr_status. The C++ drop-in classes in
 * include/cudaraster/CudaRaster.hpp are a header-only layer over this file.
 *
 * Threading: a cr_context is not thread-safe -- one host thread at a time
 * per context, as with the reference's CudaRaster; separate contexts may be
 * used from separate threads. Work is ordered on the stream each call takes
 * (NULL: the legacy default stream).
 *
 * Reference interface replaced (tcoppex/cudaraster-linux):
 *   CudaRaster::init                 src/cudaraster/CudaRaster.cpp:98-128      -> cr_create
 *   CudaRaster::~CudaRaster          src/cudaraster/CudaRaster.cpp:80-94       -> cr_destroy
 *   CudaRaster::setSurfaces          src/cudaraster/CudaRaster.cpp:132-170     -> cr_set_surfaces
 *   CudaRaster::deferredClear        src/cudaraster/CudaRaster.cpp:174-179     -> cr_deferred_clear
 *   CudaRaster::setPixelPipe         src/cudaraster/CudaRaster.cpp:183-216     -> cr_set_pixel_pipe
 *   CudaRaster::setVertexBuffer      src/cudaraster/CudaRaster.cpp:220-224     -> cr_set_vertex_buffer
 *   CudaRaster::setIndexBuffer       src/cudaraster/CudaRaster.cpp:228-233     -> cr_set_index_buffer
 *   CudaRaster::drawTriangles        src/cudaraster/CudaRaster.cpp:237-342     -> cr_draw_triangles
 *   CudaRaster::getStats             src/cudaraster/CudaRaster.cpp:346-363     -> cr_get_stats
 *   CudaRaster::getProfilingInfo     src/cudaraster/CudaRaster.cpp:367-497     -> cr_get_profiling_info
 *   CudaRaster::setDebugParams       src/cudaraster/CudaRaster.hpp:53-67,168   -> cr_set_debug_params
 *   g_crAtomics read-back            src/cudaraster/CudaRaster.cpp:326         -> cr_get_counters
 *   CudaModule::getKernel/getGlobal  src/framework/gpu/CudaModule.cpp:161-261  -> cr_pipe_count/cr_pipe_info
 *   encodeDepth / Vec4f::toABGR      src/cudaraster/cuda/Util.hpp:290-298,
 *                                    src/framework/base/Math.cpp:41-48         -> cr_encode_depth / cr_color_to_abgr
 */
#ifndef CUDARASTER_H
#define CUDARASTER_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CR_ABI_VERSION 1

typedef enum cr_status {
    CR_OK = 0,
    CR_ERR_INVALID_ARGUMENT = 1, /* bad pointer, size, sample count, name ...            */
    CR_ERR_INVALID_STATE = 2,    /* e.g. drawTriangles before surfaces / pipe are set   */
    CR_ERR_NO_PIPE = 3,          /* setPixelPipe with an unknown name                    */
    CR_ERR_PIPE_MISMATCH = 4,    /* pipe sample count differs from the surfaces          */
    CR_ERR_CAPACITY = 5,         /* a hard limit was exceeded (triangles, viewport ...) */
    CR_ERR_CUDA = 6,             /* a CUDA runtime call failed (see cr_last_error)       */
    CR_ERR_TIMEOUT = 7,          /* a device-side bounded wait gave up                   */
    CR_ERR_OUT_OF_MEMORY = 8,
    CR_ERR_UNSUPPORTED = 9       /* feature not supported by this library                 */
} cr_status;

/* Render mode flags, as RenderModeFlag_* in src/cudaraster/cuda/PixelPipe.hpp:30-35. */
#define CR_RENDER_DEPTH 1u
#define CR_RENDER_LERP  2u
#define CR_RENDER_QUADS 4u

/* Limits. The reference caps the viewport at 2048 px and subtriangles at 2^24
 * (Constants.hpp:21, 38); here the viewport may reach 4095 px (snapped vertex
 * coordinates must stay in S16) and subtriangle slots 2^29 (list entries
 * hold triangleIndex << 3 | subtriangleIndex in 32 bits). */
#define CR_MAX_VIEWPORT      4095
#define CR_MAX_TRIANGLES     ((1 << 29) - 1)
#define CR_TILE_SIZE_PX      8

typedef struct cr_context cr_context;

/* Per-stage times of the last draw in seconds (CudaRaster.hpp:45-51). */
typedef struct cr_stats {
    float setup_time;
    float bin_time;
    float coarse_time;
    float fine_time;
} cr_stats;

/* Device counters of the last draw (the reference's CRAtomics, PrivateDefs.hpp:123-143),
 * plus the capacities that were in force and how many reruns the draw took. */
typedef struct cr_counters {
    int64_t num_tris;
    int64_t num_subtris;          /* subtriangle slots used (num_tris + clip extras)  */
    int64_t bin_entries;          /* (bin, subtriangle) list entries                  */
    int64_t tile_entries;         /* (tile, subtriangle) list entries                 */
    int64_t coarse_units;         /* coarse work units                                */
    int64_t max_subtris;
    int64_t max_bin_entries;
    int64_t max_tile_entries;
    int32_t reruns;               /* overflow-detect-and-rerun iterations of the draw */
    int32_t overflow;             /* nonzero if the last launch overflowed            */
    int32_t num_bins;
    int32_t num_tiles;
} cr_counters;

/* Static description of a compiled pixel pipe (the reference's PixelPipeSpec,
 * PrivateDefs.hpp:147-154). */
typedef struct cr_pipe_info {
    char     name[64];
    int32_t  samples_log2;
    int32_t  vertex_struct_size;
    uint32_t render_mode_flags;
    int32_t  profiling_mode;
    char     blend_shader_name[64];
    char     fragment_shader_name[64];
} cr_pipe_info;

/* Debug parameters (CudaRaster.hpp:53-67). Host emulation of stages is not
 * part of this library: setting any flag returns CR_ERR_UNSUPPORTED. */
typedef struct cr_debug_params {
    int32_t emulate_triangle_setup;
    int32_t emulate_bin_raster;
    int32_t emulate_coarse_raster;
    int32_t emulate_fine_raster;
} cr_debug_params;

/* Tuning knobs (the reference's compile-time CR_* constants turned run-time).
 * Any value <= 0 keeps the default. Output bits do not depend on them. */
typedef struct cr_tuning {
    int32_t bin_log2;             /* tiles per bin side, log2: 3, 4 (default) or 5    */
    int32_t bin_chunk_tris;       /* triangles per bin-stage work chunk               */
    int32_t coarse_unit_entries;  /* bin entries per coarse work unit                 */
    int32_t fine_warps;           /* warps per fine-raster CTA                        */
    int32_t fine_ctas_per_sm;     /* resident fine CTAs per SM                        */
    int32_t fine_self_pixels;     /* fine stage: triangles whose pixel box in a tile  */
                                  /* has at most this many pixels are rasterized      */
                                  /* pixel by pixel by the lanes, larger ones by the  */
                                  /* whole warp (default 16)                          */
} cr_tuning;

/* One scene of a batched draw (cr_draw_batch). All pointers are device pointers. */
typedef struct cr_instance {
    const char* pipe;             /* pixel pipe name                                  */
    void*       color;            /* RGBA8 surface, reference layout                  */
    void*       depth;            /* DEPTH32 surface, reference layout                */
    int32_t     width, height, num_samples;
    const void* vertices;         /* vertex records of the pipe's vertex struct       */
    const void* indices;          /* int32 triplets                                   */
    int32_t     num_tris;
    int32_t     deferred_clear;   /* 1 => clear before drawing                        */
    uint32_t    clear_color;      /* ABGR8                                            */
    uint32_t    clear_depth;      /* encoded (cr_encode_depth)                        */
} cr_instance;

/* ---- Lifecycle ---- */
cr_status   cr_create(cr_context** out);
cr_status   cr_destroy(cr_context* ctx);
const char* cr_status_string(cr_status s);
const char* cr_last_error(const cr_context* ctx);
int32_t     cr_abi_version(void);

/* ---- State (CudaRaster.hpp:147-168) ---- */
/* color / depth: device pointers to surfaces of the reference's layout:
 * rounded_height rows of (rounded_width * num_samples) 32-bit words, where
 * rounded_* = size rounded up to 8, and sample i of pixel (x, y) at word
 * y * (rounded_width * num_samples) + (x / 8) * 8 * num_samples + i * 8 + x % 8. */
cr_status cr_set_surfaces(cr_context* ctx, void* color, void* depth,
                          int32_t width, int32_t height, int32_t num_samples);
cr_status cr_deferred_clear(cr_context* ctx, float r, float g, float b, float a, float depth);
cr_status cr_deferred_clear_raw(cr_context* ctx, uint32_t abgr, uint32_t encoded_depth);
cr_status cr_set_pixel_pipe(cr_context* ctx, const char* name);
cr_status cr_set_vertex_buffer(cr_context* ctx, const void* vertices, int64_t offset_bytes);
/* Inspection of the last single draw's setup output (the intermediate
 * buffers the reference exposed for its per-stage debugging, CudaRaster.hpp:
 * 53-67): per triangle its subtriangle count [num_tris], then every slot's
 * CRTriangleHeader (4 words) and CRTriangleData (16 words) -- slot t for
 * triangle t, and for a clipped triangle with several subtriangles slots
 * header[t].w + k. Host buffers of at least *num_slots slots (any may be
 * NULL); synchronous. Fails after an overflowing draw. */
cr_status cr_read_setup_output(cr_context* ctx, uint8_t* tri_subtris, uint32_t* tri_header, uint32_t* tri_data,
                               int64_t max_slots, int64_t* num_tris, int64_t* num_slots);

/* Inspection of the last single draw's bin and tile queues (the intermediate
 * lists the reference exposed only through its host emulation of the bin and
 * coarse stages, CudaRaster.hpp:53-67, BinRaster.inl:381-418,
 * CoarseRaster.inl:561-680): for every bin (row-major over the viewport's
 * bins of 8 << bin_log2 pixels) the start and length of its list in
 * bin_list, likewise for every 8x8 tile in tile_list. Entries are
 * triangle << 3 | subtriangle (7 = the triangle's only subtriangle) in
 * submission order. Host buffers: bin_start / bin_count of num_bins entries,
 * tile_start / tile_count of num_tiles (cr_get_counters), the lists of at
 * least *num_bin_entries / *num_tile_entries words (any pointer may be NULL to
 * query the sizes). Synchronous. Fails after an overflowing draw or a batch. */
cr_status cr_read_queue_output(cr_context* ctx, int32_t* bin_start, int32_t* bin_count, uint32_t* bin_list,
                               int64_t max_bin_entries, int32_t* tile_start, int32_t* tile_count,
                               uint32_t* tile_list, int64_t max_tile_entries, int64_t* num_bin_entries,
                               int64_t* num_tile_entries);

/* Fused vertex transform (no counterpart in the reference): while set, the
 * setup stage of cr_draw_triangles / _async takes each vertex's clip position
 * as mvp * (model[i].xyz, 1) -- vertexShader_passthrough (test/shader/
 * PassThrough.cu:16-35) with the same operation order, so the output bits are
 * those of running that shader first -- instead of reading the vertex
 * record's clipPos; the records still supply the varyings. model: device
 * array, model_stride floats per vertex (>= 3); mvp: 16 row-major floats,
 * copied. model NULL turns it off. Batched and static draws ignore it. */
cr_status cr_set_vertex_transform(cr_context* ctx, const float* model, int32_t model_stride,
                                  const float* mvp_row_major);
cr_status cr_set_index_buffer(cr_context* ctx, const void* indices, int64_t offset_bytes,
                              int32_t num_tris);
cr_status cr_set_tuning(cr_context* ctx, const cr_tuning* tuning);
cr_status cr_set_debug_params(cr_context* ctx, const cr_debug_params* params);
/* Per-stage timing of getStats (CudaRaster.cpp:346-363): on by default, as in
 * the reference, each draw records a CUDA event between its stages. Off, the
 * stages launch back to back with no event between them, so each stage's
 * launch overlaps the end of the previous one, and cr_get_stats reports zeros. */
cr_status cr_set_stage_timing(cr_context* ctx, int32_t enabled);
/* Queue capacities (elements) for the next draws. All zero keeps the
 * reference-style estimates (CudaRaster.cpp:263-275); otherwise the given
 * sizes are used as they are (a predictor's sizing) and, when a draw
 * overflows them, grown by the rerun loop. Capacities never shrink. */
cr_status cr_set_capacity(cr_context* ctx, int64_t max_subtris, int64_t max_bin_entries,
                          int64_t max_tile_entries);

/* ---- Drawing ---- */
/* Draws the current index buffer on `stream` (a cudaStream_t; NULL = legacy
 * default stream). Like the reference it checks the device counters after the
 * draw and reruns with larger queues on overflow, so it synchronises with the
 * stream before returning. */
cr_status cr_draw_triangles(cr_context* ctx, void* stream);
/* Asynchronous variant: no host synchronisation and no rerun. The caller
 * checks cr_get_counters().overflow after synchronising. */
cr_status cr_draw_triangles_async(cr_context* ctx, void* stream);
/* Several independent scenes in one set of launches. */
cr_status cr_draw_batch(cr_context* ctx, const cr_instance* instances, int32_t count, void* stream);
cr_status cr_draw_batch_async(cr_context* ctx, const cr_instance* instances, int32_t count, void* stream);

/* Batched draw captured into a CUDA graph (no counterpart in the reference).
 * Capture fixes the batch (surfaces, buffers, triangle counts, pipes) and the
 * queue capacities of `ctx` at that moment; replays are asynchronous. A
 * replay whose queues overflow skips the frame (surfaces untouched) and sets
 * `overflow` in cr_batch_graph_counters: grow the capacities
 * (cr_set_capacity) and recapture. While a graph is alive, other draws on the
 * same context must not need larger queues (they would reallocate them). */
typedef struct cr_batch_graph cr_batch_graph;
cr_status cr_batch_graph_create(cr_context* ctx, const cr_instance* instances, int32_t count, void* stream,
                                cr_batch_graph** out);
cr_status cr_batch_graph_launch(cr_batch_graph* graph, void* stream);
cr_status cr_batch_graph_counters(cr_batch_graph* graph, void* stream, cr_counters* out);
cr_status cr_batch_graph_destroy(cr_batch_graph* graph);

/* No counterpart in the reference. The same draw as cr_draw_triangles for
 * callers that may not allocate memory while they run (a host application
 * that owns a fixed memory budget, a real-time loop where cudaMalloc would
 * stall the frame, a plugin that only receives device pointers): no context,
 * no cudaMalloc/cudaFree, no pinned host buffers. The intermediate queues
 * live in one static array of about 13 MiB compiled into this library, held
 * by every GPU that loads it until the process exits, and shared by every
 * call: calls that overlap on the GPU race, so order them on one stream.
 * Limits: num_tris <= 65536, width and height <= 1024, fixed queue sizes;
 * larger draws return CR_ERR_CAPACITY (surfaces untouched) with a message in
 * `error` (may be NULL). The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress) with that device current; make it
 * before any stream capture. Synchronises with `stream` before returning. */
cr_status cr_draw_triangles_static(const char* pipe, void* color, void* depth, int32_t width, int32_t height,
                                   int32_t num_samples, const void* vertices, const void* indices,
                                   int32_t num_tris, int32_t deferred_clear, uint32_t clear_color,
                                   uint32_t clear_depth, void* stream, char* error, int64_t error_size);

/* ---- Vertex stage ---- */
/* The reference's vertexShader_passthrough (test/shader/PassThrough.cu:16-35):
 * out[i].clipPos = MVP * (model[i].xyz, 1), Mat4f * Vec4f accumulated in the
 * framework's order (Math.hpp:990-1001). model: float triplets at
 * model_stride floats; colors (optional, may be NULL): RGBA floats at
 * color_stride copied behind the position; out: 16- or 32-byte records
 * (ShadedVertexBase / GouraudVertex). Device pointers; asynchronous. */
cr_status cr_vertex_shader_passthrough(const float* model, int32_t model_stride, const float* colors,
                                       int32_t color_stride, void* out_vertices, int32_t out_stride_bytes,
                                       int64_t num_vertices, const float* mvp_row_major, void* stream);

/* The reference's Constants (test/shader/Shaders.hpp) for its vertex shaders:
 * row-major matrices. */
typedef struct cr_vertex_constants {
    float pos_to_clip[16];
    float pos_to_camera[16];
    float normal_to_camera[9];
} cr_vertex_constants;

/* The reference's vertexShader_gouraud (test/shader/Shaders.cu:55-82) with
 * evaluateLighting (Shaders.cu:37-50). in_vertices: InputVertex records of 8
 * floats (modelPos xyz, modelNormal xyz, texCoord uv); materials: num_materials
 * records material_stride_bytes apart (0 = 32) that start with diffuse rgba,
 * specular rgb, glossiness -- the reference's Material (cr_material, 576
 * bytes) or just its first 32 bytes; vertex_material_idx: one index per
 * vertex (clamped to the table); out_vertices: GouraudVertex records (clipPos,
 * colour rgb + diffuse alpha). Arithmetic as the framework's C, one rounded
 * operation at a time; sqrt is IEEE and powf an exactly specified power
 * (cr_pow_exact) where the reference used fast-math approximations. Device
 * pointers; asynchronous. No counterpart call in the reference's host code. */
cr_status cr_vertex_shader_gouraud(const void* in_vertices, int64_t num_vertices,
                                   const cr_vertex_constants* constants, const void* materials,
                                   int32_t material_stride_bytes, int32_t num_materials,
                                   const int32_t* vertex_material_idx, void* out_vertices, void* stream);

/* The reference's vertexShader_texPhong (test/shader/Shaders.cu:86-108):
 * InputVertex records -> ShadedVertex_texPhong records of 16 floats (clipPos,
 * cameraPos, cameraNormal with w 0, texCoord with z 0 and w 1). */
cr_status cr_vertex_shader_tex_phong(const void* in_vertices, int64_t num_vertices,
                                    const cr_vertex_constants* constants, void* out_vertices, void* stream);

/* ---- Textured Phong pipe (PixelPipe_texPhong*) ----
 * The reference's TextureSpec and Material (test/shader/Shaders.hpp), field
 * for field: a texture's size in texels (0 = no texture) and per mip level
 * (scaleX, scaleY, biasX, biasY) mapping [0, 1)^2 into the atlas. */
typedef struct cr_texture_spec {
    float size[2];
    uint32_t pad[2];
    float mip_levels[16][4];
} cr_texture_spec;

typedef struct cr_material {
    float diffuse_color[4];
    float specular_color[3];
    float glossiness;
    cr_texture_spec diffuse_texture;
    cr_texture_spec alpha_texture;
} cr_material;

/* The fragment shader's inputs, which the reference kept in c_constants
 * (materials, triangleMaterialIdx) and the texture reference t_textureAtlas:
 * materials: device array of num_materials cr_material; triangle_material_idx:
 * device array of num_triangle_material_idx indices, one per triangle of the
 * draw (a triangle past the end uses the last entry; indices are clamped to
 * the table); atlas: device RGBA8 texels (R in the low byte), atlas_width x
 * atlas_height, sampled bilinearly with wrapped, normalized coordinates.
 * Stream-ordered: draws on `stream` after this call read these values. One
 * set is current at a time, as with the reference's module constants. */
cr_status cr_set_tex_phong_constants(const cr_material* materials, int32_t num_materials,
                                     const int32_t* triangle_material_idx, int64_t num_triangle_material_idx,
                                     const uint32_t* atlas, int32_t atlas_width, int32_t atlas_height,
                                     void* stream);

/* The texture filter of the textured pipe over arrays: out[4 i + c] = channel c
 * of the atlas filtered at (uv[2 i], uv[2 i + 1]) -- linear filtering, wrap
 * addressing, normalized coordinates, 8-bit fractional weights rounded to
 * nearest, the weighted integer sum divided by 255 * 65536 (the reference's
 * tex2D on t_textureAtlas, test/shader/Shaders.cu:141-142, with its result
 * specified). Device arrays; asynchronous. */
cr_status cr_texture_sample(const uint32_t* atlas, int32_t atlas_width, int32_t atlas_height, const float* uv,
                            float* out, int64_t n, void* stream);

/* The same lookups through the GPU's texture unit (an RGBA8 CUDA array read as
 * normalized floats, linear filter, wrap, normalized coordinates), for
 * comparing cr_texture_sample with the hardware filter the reference used.
 * Synchronises with `stream`. */
cr_status cr_texture_sample_hw(const uint32_t* atlas, int32_t atlas_width, int32_t atlas_height, const float* uv,
                               float* out, int64_t n, void* stream);

/* The exact power the Gouraud vertex shader uses: out[i] = x[i]^y[i] for
 * x >= 0, within about 1e-5 relative of pow (device arrays; asynchronous). */
cr_status cr_pow_exact(const float* x, const float* y, float* out, int64_t n, void* stream);

/* ---- MSAA resolve ----
 * The reference's CudaSurface::resolveToScreen (CudaSurface.hpp:73) is
 * commented out and drew through GL. This averages each pixel's samples per
 * channel, rounding half up ((sum + S/2) >> log2 S), into a row-major image of
 * one RGBA8 word per pixel (R in the low byte); with one sample it copies the
 * pixels without the 8x8 tile padding. color: a colour surface of width x
 * height with num_samples samples (device); out: device, out_row_bytes per row
 * (>= 4 * width, multiple of 4). Asynchronous on stream. */
cr_status cr_resolve_color(const void* color, int32_t width, int32_t height, int32_t num_samples, void* out,
                           int64_t out_row_bytes, void* stream);

/* ---- Queue occupancy and the learned queue predictor ----
 * No reference counterpart: the reference sizes its queues from the previous
 * draw and grows them on overflow (CudaRaster.cpp:263-275, 325-342), which
 * stays the fallback and the check of every prediction made here. */

/* Bin and tile grid of the last draw (of its first instance for a batch). */
typedef struct cr_queue_layout {
    int32_t bins_x, bins_y;       /* bins of (8 << bin_log2) pixels */
    int32_t tiles_x, tiles_y;     /* 8x8-pixel tiles                */
    int32_t bin_log2;
    int32_t num_bins, num_tiles;  /* totals over all instances      */
    int32_t num_instances;
} cr_queue_layout;
cr_status cr_get_queue_layout(cr_context* ctx, cr_queue_layout* out);
/* Device pointers to the last draw's per-bin counts [num_bins], per-tile
 * counts [num_tiles] and 8 counters, valid until the next draw on ctx. */
cr_status cr_get_queue_buffers(cr_context* ctx, const int32_t** bin_counts, const int32_t** tile_counts,
                               const int32_t** counters);

/* Device-to-device copies, ordered on `stream` after the last draw, of its
 * per-bin bin-queue entry counts [num_bins], per-tile tile-queue entry counts
 * [num_tiles] and its 8 device counters (extra subtriangles, bin entries,
 * coarse units, tile entries, fine tiles taken, overflow flags, and the two
 * coarse work counters).
 * Any of the three pointers may be NULL. After an overflow the counts of the
 * overflowing stage and later ones are incomplete. */
cr_status cr_queue_counts(cr_context* ctx, int32_t* bin_counts, int32_t num_bins, int32_t* tile_counts,
                          int32_t num_tiles, int32_t* counters, void* stream);

/* Predictor input: x[cy*16+cx] = 0.125 * mean of log1p(count) over the bins
 * (bx, by) with bx*16/bins_x == cx and by*16/bins_y == cy, x[256..261] =
 * camera_delta (6 host floats). x: 262 device floats. */
cr_status cr_queue_features(const int32_t* bin_counts, int32_t bins_x, int32_t bins_y, const float* camera_delta,
                            float* x, void* stream);
/* logs[b] = log1p(bin entries of bin b), logs[nb + b] = log1p(sum of the tile
 * entries of bin b's tiles), logs[2nb] / logs[2nb + 1] = log1p of the bin /
 * tile entry totals; nb = bins_x * bins_y. logs: 2nb + 6 device floats,
 * 8-byte aligned (the last four are scratch for the 64-bit totals). */
cr_status cr_queue_log_counts(const int32_t* bin_counts, const int32_t* tile_counts, int32_t bins_x, int32_t bins_y,
                              int32_t tiles_x, int32_t tiles_y, int32_t bin_log2, float* logs, void* stream);
/* The network's regression target: target[i] = logs_cur[i] - logs_prev[i],
 * minus (logs_prev[i] - logs_prevprev[i]) for the last n_trend entries when
 * logs_prevprev is given (the total heads learn corrections to the trend). */
cr_status cr_queue_targets(const float* logs_prevprev, const float* logs_prev, const float* logs_cur, int32_t n,
                           int32_t n_trend, float* target, void* stream);
/* Occupancy predicted from the last logs and the network output (2nb + 2
 * values): per_bin[i] = max(expm1(logs_prev[i] + prediction[i]), 0) for
 * i < 2nb (may be NULL); totals[0] / totals[1] = predicted bin / tile entry
 * totals from the total heads, expm1(logs_prev[h] + (logs_prev[h] -
 * logs_prevprev[h]) + prediction[h]) (no trend term when logs_prevprev is
 * NULL); totals[2] / totals[3] = sums of the per-bin predictions (device
 * doubles). */
cr_status cr_queue_plan(const float* logs_prevprev, const float* logs_prev, const float* prediction,
                        int32_t num_bins, float* per_bin, double* totals, void* stream);

/* The network: inputs -> hidden1 -> hidden2 -> outputs, GELU after both
 * hidden layers. Parameters are held in FP32 (Adam master copy) and used in
 * BF16; every product is accumulated in FP32. Flat parameter layout:
 * W1[hidden1][inputs], b1[hidden1], W2[hidden2][hidden1], b2[hidden2],
 * W3[outputs][hidden2], b3[outputs]. Loss: mean squared error over the
 * batch's outputs. A predictor's calls must be ordered (one stream): they
 * share its activation buffers. All data pointers are device pointers. */
typedef struct cr_predictor cr_predictor;
cr_status cr_predictor_create(cr_predictor** out, int32_t inputs, int32_t hidden1, int32_t hidden2, int32_t outputs,
                              int32_t max_batch);
void      cr_predictor_destroy(cr_predictor* p);
int64_t   cr_predictor_num_params(const cr_predictor* p);
int64_t   cr_predictor_steps(const cr_predictor* p);
/* Host FP32 parameters in; the BF16 copy is rounded to nearest even and the
 * Adam state reset. Synchronous. */
cr_status cr_predictor_set_params(cr_predictor* p, const float* host, int64_t n);
cr_status cr_predictor_get_params(const cr_predictor* p, float* host, int64_t n);
cr_status cr_predictor_get_params_bf16(const cr_predictor* p, uint16_t* host, int64_t n);
/* y[batch][outputs] = network(x[batch][inputs]). */
cr_status cr_predictor_forward(cr_predictor* p, const float* x, int32_t batch, float* y, void* stream);
/* Gradients of the loss over rows `rows[0..batch)` of the sample pools of
 * pool_rows rows each (rows NULL: rows 0..batch-1) into grads[num_params]
 * (may be NULL) and the loss into *loss (device float, may be NULL);
 * parameters unchanged. A row index outside the pool reads row 0 instead
 * and raises the flag that cr_predictor_bad_rows returns. */
cr_status cr_predictor_gradients(cr_predictor* p, const float* x_pool, const float* target_pool, int32_t pool_rows,
                                 const int32_t* rows, int32_t batch, float* grads, float* loss, void* stream);
/* One Adam step (bias-corrected) on the gradients of those rows. */
cr_status cr_predictor_train_step(cr_predictor* p, const float* x_pool, const float* target_pool, int32_t pool_rows,
                                  const int32_t* rows, int32_t batch, float lr, float beta1, float beta2, float eps,
                                  float* loss, void* stream);
/* One frame k of the online predictor in a single launch, for a network with
 * 262 inputs (16x16 histogram + camera delta) and 2nb + 2 outputs predicting
 * `ahead` frames on. From the draw's counts (bin_counts, tile_counts,
 * counters: device pointers, e.g. from cr_get_queue_buffers) it writes
 *   - logs_cur: frame k's logs (as cr_queue_log_counts, 2nb + 2 floats);
 *   - target: the target of the sample that frame k completes, whose input
 *     was frame k - ahead (logs_target_base; logs_target_trend = frame
 *     k - ahead - 1, may be NULL): logs_cur - base, and for the two total
 *     heads also - ahead * (base - trend); skipped when target or
 *     logs_target_base is NULL (cr_queue_targets for ahead = 1);
 *   - x_next[262]: frame k's pooled histogram and camera_delta_ahead (the
 *     camera move from k to k + ahead), bit for bit as cr_queue_features;
 *   - the network's prediction for frame k + ahead and its plan (as
 *     cr_queue_plan with frame k as the base, the total heads on the trend
 *     expm1(cur + ahead * (cur - logs_prev) + y); per_bin may be NULL);
 *   - fetch (device, 64 bytes, 8-byte aligned): the 4 predicted totals
 *     (doubles), then the draw's 8 counters (int32), for one copy to host. */
cr_status cr_predictor_frame(cr_predictor* p, const int32_t* bin_counts, const int32_t* tile_counts,
                             const int32_t* counters, const cr_queue_layout* layout, int32_t ahead,
                             const float* logs_prev, float* logs_cur, const float* logs_target_base,
                             const float* logs_target_trend, float* target, const float* camera_delta_ahead,
                             float* x_next, float* per_bin, void* fetch, void* stream);
/* Per-output loss weights w (outputs values >= 0, sum > 0; NULL restores
 * equal weights): loss = sum_b sum_o w_o (y - t)^2 / (batch * sum_o w_o).
 * Copied; synchronous. Available for networks within the fused training
 * step's sizes (inputs <= 320, hidden layers <= 64, max_batch <= 64), which
 * every gradient and training call of such a network uses: four launches
 * per step. */
cr_status cr_predictor_set_loss_weights(cr_predictor* p, const float* weights, int64_t n);
/* *flag = nonzero if a batch since the last reset named a row outside its
 * pool; reset != 0 clears it. Synchronous. */
cr_status cr_predictor_bad_rows(cr_predictor* p, int32_t* flag, int32_t reset);

/* ---- Results ---- */
cr_status cr_get_stats(cr_context* ctx, cr_stats* out);
cr_status cr_get_counters(cr_context* ctx, cr_counters* out);
cr_status cr_get_profiling_info(cr_context* ctx, char* buffer, int64_t size);

/* ---- Pipes ---- */
int32_t   cr_pipe_count(void);
cr_status cr_pipe_info_at(int32_t index, cr_pipe_info* out);
cr_status cr_pipe_info_by_name(const char* name, cr_pipe_info* out);

/* ---- Host helpers matching the reference's host arithmetic ---- */
uint32_t cr_color_to_abgr(float r, float g, float b, float a);   /* Math.cpp:41-48      */
uint32_t cr_encode_depth(uint32_t depth);                         /* Util.hpp:290-298    */
uint32_t cr_decode_depth(uint32_t depth);                         /* Util.hpp:302-310    */
uint32_t cr_clear_depth_from_float(float depth);                  /* CudaRaster.cpp:178  */

#ifdef __cplusplus
}
#endif
#endif
