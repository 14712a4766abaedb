/*
 * cr_oracle.h -- C interface of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY. This is a scalar restatement of the reference
 * rasterizer's device arithmetic (tcoppex/cudaraster-linux,
 * src/cudaraster/cuda/*.inl) used as the checker for the GPU pipeline.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it. The product library never links or calls it.
 *
 * Normative semantics the oracle encodes (the GPU pipeline must match bit
 * for bit):
 *   - triangle setup exactly as TriangleSetup.inl:19-417, with binary32
 *     arithmetic evaluated operation by operation (no FMA contraction),
 *     IEEE division, and PTX cvt saturation rules for float->int casts;
 *   - per-sample coverage by exact 64-bit edge functions with the fill rule
 *     of Util.inl:100 (dy > 0 || (dy == 0 && dx <= 0) => exclusive);
 *   - fragments applied per pixel / per sample in submission order
 *     (triangle index, then subtriangle index), depth test LESS with write,
 *     blend after the depth test (FineRaster.inl:433-495, 758-851 with the
 *     warp races resolved in submission order).
 */
#ifndef CR_ORACLE_H
#define CR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Render mode flags (PixelPipe.hpp:30-35). */
#define OR_DEPTH 1
#define OR_LERP  2
#define OR_QUADS 4

/* Blend shaders (PixelPipe.hpp:145-175). */
#define OR_BLEND_REPLACE   0
#define OR_BLEND_SRCOVER   1
#define OR_BLEND_ADDITIVE  2
#define OR_BLEND_DEPTHONLY 3

/* Fragment shaders known to the oracle. */
#define OR_SHADER_GOURAUD     0 /* toABGR(varying 0 at the centroid), PixelPipe.inl:65-69 */
#define OR_SHADER_RED         1 /* constant red, test/shader/PassThrough.cu:44-54          */
#define OR_SHADER_TRIHASH     2 /* ABGR from a hash of the triangle index (ordering probe)  */
#define OR_SHADER_DERIV       3 /* colour from barycentric derivatives (quad mode probe)    */
#define OR_SHADER_TEXPHONG    4 /* test/shader/Shaders.cu:117-193, inputs from or_set_tex_phong */

typedef struct or_pipe {
    int32_t  width, height;       /* viewport = surface size in pixels            */
    int32_t  samples_log2;        /* 0..3                                          */
    uint32_t render_mode;         /* OR_DEPTH | OR_LERP | OR_QUADS                 */
    int32_t  blend;               /* OR_BLEND_*                                    */
    int32_t  shader;              /* OR_SHADER_*                                   */
    int32_t  vertex_stride;       /* bytes, multiple of 16, >= 16                  */
    int32_t  deferred_clear;      /* 1 => clear every tile before drawing          */
    uint32_t clear_color;         /* ABGR8                                         */
    uint32_t clear_depth;         /* encoded depth                                 */
} or_pipe;

typedef struct or_stats {
    int64_t num_subtris;          /* emitted subtriangles                          */
    int64_t num_clipped;          /* triangles that took the clip path             */
    int64_t num_fragments;        /* covered (pixel, subtri) pairs                 */
    int64_t zmin_violations;      /* covered samples whose depth < header zmin     */
    int64_t tile_entries;         /* (tile, subtri) pairs after bbox binning       */
} or_stats;

/* Triangle setup of a whole draw. Outputs follow CRTriangleHeader /
 * CRTriangleData layouts (PrivateDefs.hpp:26-62): headers are 4 words per
 * slot, data 16 words per slot. Subtriangles of clipped triangles that emit
 * more than one are stored from slot num_tris on, in triangle order.
 * Returns the number of slots used, or -1 when max_subtris is too small. */
int64_t or_setup(const or_pipe* p, const float* vertices, const int32_t* indices,
                 int64_t num_tris, uint8_t* tri_subtris, uint32_t* headers,
                 uint32_t* data, int64_t max_subtris);

/* Full frame. color/depth hold rounded_h x (rounded_w << samples_log2)
 * words in the reference surface layout (CudaSurface.hpp:65) and are updated
 * in place. num_threads <= 0 uses the OpenMP default. */
int or_render(const or_pipe* p, const float* vertices, const int32_t* indices,
              int64_t num_tris, uint32_t* color, uint32_t* depth,
              int num_threads, or_stats* stats);

/* Per-stage queue model of one draw (bins of 8 << bin_log2 pixels, 8x8 tiles)
 * as CSR arrays over cells in row-major order: kind 0 / 2 = the exact bin /
 * tile lists (entries covering a sample of the cell), kind 1 / 3 = the lists
 * the GPU's conservative binning rule keeps. Entries are triangle << 3 |
 * subtriangle (7 = the triangle's only subtriangle) in submission order.
 * offsets has num_cells + 1 entries; both arrays are filled only when the
 * total fits cap. Returns the total, or -1 on bad arguments. */
int64_t or_queue_lists(const or_pipe* p, const float* vertices, const int32_t* indices, int64_t num_tris,
                       int bin_log2, int kind, int64_t* offsets, uint32_t* entries, int64_t cap);

/* ---- Single-function entry points used by the known-answer tests. ---- */
int32_t  or_f32_to_s32_sat(float a);
uint32_t or_f32_to_u32_sat(float a);
uint32_t or_f32_to_u32_sat_rmi(float a);
int64_t  or_f32_to_s64(float a);
uint32_t or_f32_to_u32_rz(float a);
uint32_t or_to_abgr(float r, float g, float b, float a);
uint32_t or_host_to_abgr(float r, float g, float b, float a);
uint32_t or_encode_depth(uint32_t d);
uint32_t or_decode_depth(uint32_t d);
uint32_t or_clear_depth(float depth);
uint32_t or_blend(int blend, uint32_t src, uint32_t dst, int* write_color);
uint32_t or_select_flips(int32_t dx, int32_t dy);
int      or_select_msaa_centroid(int samples_log2, uint32_t mask);
void     or_centroid_lut(int samples_log2, uint8_t* lut);
void     or_setup_pleq(const float values[3], const int32_t v0[2], const int32_t d1[2],
                       const int32_t d2[2], float area_rcp, int samples_log2, uint32_t out[3]);
int      or_clip_triangle(float* bary18, const float v0[4], const float v1[4], const float v2[4],
                          const float d1[4], const float d2[4]);
uint64_t or_cover8x8_exact(int32_t ox, int32_t oy, int32_t dx, int32_t dy);
uint64_t or_cover8x8_conservative(int32_t ox, int32_t oy, int32_t dx, int32_t dy);
uint32_t or_cover_msaa(int samples_log2, int32_t ox, int32_t oy, int32_t dx, int32_t dy);
uint64_t or_triangle_pixel_coverage(const uint32_t header[4], int tile_x, int tile_y,
                                    int width, int height, int samples_log2);
uint32_t or_triangle_sample_coverage(const uint32_t header[4], int px, int py,
                                     int width, int height, int samples_log2);
void     or_compute_barys(int samples_log2, const int32_t w[3], const int32_t u[3],
                          const int32_t v[3], int32_t sx, int32_t sy, float out[9]);
int      or_find_bit(uint64_t mask, int idx, int quads);
/* Inputs of the textured Phong shader (the reference's c_constants and
 * t_textureAtlas): materials as 576-byte Material records (144 floats), one
 * material index per triangle, an RGBA8 atlas. The pointers are kept, not
 * copied, until the next call. */
void     or_set_tex_phong(const float* materials, int num_materials, const int32_t* triangle_material_idx,
                          int64_t num_triangle_material_idx, const uint32_t* atlas, int atlas_width,
                          int atlas_height);
/* The atlas filter (bilinear, wrap, normalized coordinates, 8-bit weights). */
void     or_texture_sample(const uint32_t* atlas, int atlas_width, int atlas_height, const float* uv,
                           float* out, int64_t n);
/* Differences between the GPU filter's division-free normalisation and the
 * specified division, over every weighted sum the filter can form (0 expected). */
int64_t  or_tex_normalize_mismatches(void);
/* The exactly specified power / log2 and evaluateLighting (Shaders.cu:37-50). */
float    or_pow_exact(float x, float y);
float    or_log2_exact(float x);
void     or_evaluate_lighting(const float camera_pos[3], const float camera_normal[3], const float specular[3],
                              float glossiness, const float diffuse[3], float out[3]);
/* Fragment shader of pipe p for one pixel (FineRaster.inl:48-119). */
uint32_t or_fragment(const or_pipe* p, const uint32_t data16[16], const float* vertices,
                     int32_t tri_idx, int32_t px, int32_t py, uint32_t centroid);
void     or_perspective(float fov_deg, float near_z, float far_z, float out16[16]);

#ifdef __cplusplus
}
#endif
#endif
