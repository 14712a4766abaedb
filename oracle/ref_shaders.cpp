/*
 * ref_shaders.cpp -- compiles the reference's example shaders
 * (tcoppex/cudaraster-linux, test/shader/Shaders.cu: evaluateLighting, the
 * Gouraud and texPhong vertex shaders, FragmentShader_texPhong) for the host,
 * in place, as a second translation unit of the reference harness, and runs
 * them per vertex / per fragment through a C interface.
 *
 * TEST INFRASTRUCTURE ONLY (oracle/_ref). The reference's shaders call
 * log2f, powf and tex2D on a texture reference, whose results nvcc does not
 * specify; here they are bound to the exactly specified versions the
 * pipeline uses (shader_math.h: the atanh-series log2, the power built on it,
 * and the 8-bit-weight RGBA8 atlas filter), so that everything else -- the
 * level-of-detail choice, mip selection, the two lookups and their lerp, the
 * alpha test, the lighting, the vertex transforms -- is the reference's own
 * source, compared with the oracle's restatement.
 */
#include "ref_shim.h"
#include "shader_math.h"

// The reference compiles Shaders.cu once per pipe configuration; its pipe
// definitions at the end need these, though no pipe kernel is run here.
#define SAMPLES_LOG2 0
#define RENDER_MODE_FLAGS 3
#define BLEND_SHADER BlendReplace

#include "Shaders.hpp"

namespace {
const uint32_t* g_atlas = nullptr;
int g_atlasW = 1, g_atlasH = 1;
}  // namespace

namespace FW {
// Declared by Shaders.hpp only under nvcc.
extern "C" {
Constants c_constants;
texture<float4, 2> t_textureAtlas;
void vertexShader_gouraud(const InputVertex* inPtr, ShadedVertex_gouraud* outPtr, int numVertices);
void vertexShader_texPhong(const InputVertex* inPtr, ShadedVertex_texPhong* outPtr, int numVertices);
}
Vec3f evaluateLighting(Vec3f cameraPos, Vec3f cameraNormal, const Material& material, Vec3f diffuseColor);

// FragmentShaderBase declares dFdx / dFdy only under nvcc; the shader's quad
// branch that calls them is compiled but not taken here (no quads).
inline Vec2f dFdx(const Vec2f&) { return Vec2f(0.0f); }
inline Vec2f dFdy(const Vec2f&) { return Vec2f(0.0f); }

// tex2D on t_textureAtlas: the pipeline's atlas filter.
inline float4 tex2D(const texture<float4, 2>&, float u, float v) {
    float c[4];
    crsm::tex2d(g_atlas, g_atlasW, g_atlasH, u, v, c);
    return make_float4(c[0], c[1], c[2], c[3]);
}
}  // namespace FW

inline float harness_log2f(float x) { return crsm::log2_full(x); }
inline float harness_powf(float x, float y) { return crsm::pow_exact(x, y); }
#define log2f harness_log2f
#define powf harness_powf
// PixelPipe.inl, which Shaders.cu includes, defines the global c_zero; the
// harness's first translation unit already holds one.
#define c_zero ref_shaders_c_zero

#include "Shaders.cu"

#undef log2f
#undef powf
#undef c_zero

using namespace FW;

namespace {
void set_matrices(const float* posToClip, const float* posToCamera, const float* normalToCamera) {
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) {
            c_constants.posToClip.get(r, c) = posToClip[r * 4 + c];
            c_constants.posToCamera.get(r, c) = posToCamera[r * 4 + c];
        }
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) c_constants.normalToCamera.get(r, c) = normalToCamera[r * 3 + c];
}

// One thread per vertex: vidx = blockIdx.x with one-thread blocks.
template <class F>
void for_each_vertex(int n, F&& f) {
    blockDim = dim3(1, 1, 1);
    gridDim = dim3((unsigned)n, 1, 1);
    threadIdx = make_uint3(0, 0, 0);
    for (int v = 0; v < n; v++) {
        blockIdx = make_uint3((unsigned)v, 0, 0);
        f();
    }
}

template <int S, U32 F>
U32 run_tex_phong(int triIdx, int px, int py, U32 centroid, bool* discard) {
    static volatile U32 shared[32];
    threadIdx = make_uint3(0, 0, 0);
    FragmentShader_texPhong fs;
    runFragmentShader<ShadedVertex_texPhong, FragmentShader_texPhong, S, F>(fs, triIdx, 0, px, py, centroid, shared);
    *discard = fs.m_discard;
    return fs.m_color;
}
}  // namespace

extern "C" {

// vertexShader_gouraud (Shaders.cu:56-84). materials: 576-byte Material records.
void ref_vertex_gouraud(const float* in, int n, const float* posToClip, const float* posToCamera,
                        const float* normalToCamera, const void* materials, const int* vertexMaterialIdx, float* out) {
    set_matrices(posToClip, posToCamera, normalToCamera);
    c_constants.materials = (CUdeviceptr)(uintptr_t)materials;
    c_constants.vertexMaterialIdx = (CUdeviceptr)(uintptr_t)vertexMaterialIdx;
    for_each_vertex(n, [&] {
        vertexShader_gouraud((const InputVertex*)in, (ShadedVertex_gouraud*)out, n);
    });
}

// vertexShader_texPhong (Shaders.cu:86-108).
void ref_vertex_tex_phong(const float* in, int n, const float* posToClip, const float* posToCamera,
                          const float* normalToCamera, float* out) {
    set_matrices(posToClip, posToCamera, normalToCamera);
    for_each_vertex(n, [&] {
        vertexShader_texPhong((const InputVertex*)in, (ShadedVertex_texPhong*)out, n);
    });
}

// The texPhong shader's inputs: Material records, one material per triangle, an RGBA8 atlas.
void ref_set_tex_phong(const void* materials, const int* triangleMaterialIdx, const uint32_t* atlas, int atlasW,
                       int atlasH) {
    c_constants.materials = (CUdeviceptr)(uintptr_t)materials;
    c_constants.triangleMaterialIdx = (CUdeviceptr)(uintptr_t)triangleMaterialIdx;
    g_atlas = atlas;
    g_atlasW = atlasW;
    g_atlasH = atlasH;
}

// runFragmentShader (FineRaster.inl:48-119) + FragmentShader_texPhong::run (Shaders.cu:149-193),
// without quads (their derivatives need the four lanes of a quad). triData: the
// triangle's 16 data words; vertices: ShadedVertex_texPhong records.
unsigned int ref_tex_phong_fragment(int s, const unsigned int* triData, const float* vertices, int triIdx, int px,
                                    int py, unsigned int centroid, int* discard) {
    t_triData.ptr = (const uint4*)triData;
    t_vertexBuffer.ptr = (const float4*)vertices;
    bool d = false;
    U32 c;
    switch (s) {
    case 0: c = run_tex_phong<0, 3>(triIdx, px, py, centroid, &d); break;
    case 1: c = run_tex_phong<1, 3>(triIdx, px, py, centroid, &d); break;
    case 2: c = run_tex_phong<2, 3>(triIdx, px, py, centroid, &d); break;
    default: c = run_tex_phong<3, 3>(triIdx, px, py, centroid, &d); break;
    }
    *discard = d ? 1 : 0;
    return c;
}

}  // extern "C"
