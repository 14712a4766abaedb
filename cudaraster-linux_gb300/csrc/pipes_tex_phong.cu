// pipes_tex_phong.cu -- the reference's textured Phong pipe
// (test/shader/Shaders.cu:117-199, PixelPipe_texPhong): per-fragment lighting
// of interpolated camera-space position and normal, a diffuse and an alpha
// texture sampled from one atlas with a level of detail chosen from the
// texture-coordinate derivatives (analytic at the centroid, or numerical
// across the 2x2 quad in quad mode), and an alpha test that discards.
//
// The reference sampled a legacy texture reference with the texture unit's
// filter and called log2f, powf and a reciprocal square root; here the atlas
// is filtered by crTex2D and the rest is crLog2 / crPow / crNormalize
// (ShaderMath.hpp), so every output bit is specified and the CPU oracle
// reproduces it. The shader reads its constants from c_texPhong, which
// cr_set_tex_phong_constants fills, as the reference read c_constants and
// t_textureAtlas.
#include "cudaraster.h"
#include "cudaraster/PixelPipe.inl"
#include "cudaraster/ShaderMath.hpp"

namespace FW {

// Shaders.hpp: TextureSpec and Material, field for field.
struct TextureSpec {
    Vec2f size;
    U32 pad[2];
    Vec4f mipLevels[16];  // scaleX, scaleY, biasX, biasY
};

struct Material {
    Vec4f diffuseColor;
    Vec3f specularColor;
    F32 glossiness;
    TextureSpec diffuseTexture;
    TextureSpec alphaTexture;
};

static_assert(sizeof(TextureSpec) == sizeof(cr_texture_spec), "TextureSpec layout");
static_assert(sizeof(Material) == sizeof(cr_material) && sizeof(Material) == 576, "Material layout");

struct TexPhongConstants {
    const Material* materials;
    const S32* triangleMaterialIdx;
    S64 numTriangleMaterialIdx;
    S32 numMaterials;
    TextureAtlas atlas;
};

__constant__ TexPhongConstants c_texPhong;

struct ShadedVertex_texPhong : ShadedVertexBase {
    Vec4f cameraPos;     // varying 0
    Vec4f cameraNormal;  // varying 1
    Vec4f texCoord;      // varying 2
};

// kQuads: the pipe's RenderModeFlag_EnableQuads, which the reference's shader
// read from its compile-time RENDER_MODE_FLAGS.
template <bool kQuads>
class TexPhongShader : public FragmentShaderBase {
public:
    // Two bilinear lookups in adjacent mip levels, blended by the fraction of
    // the level of detail (Shaders.cu:123-147).
    __device__ __forceinline__ Vec4f texture2D(const TextureSpec& spec, const Vec2f& tex, const Vec2f& texDX,
                                               const Vec2f& texDY) {
        const F32 sx = spec.size.x, sy = spec.size.y;
        const F32 ax = __fmul_rn(texDX.x, sx), ay = __fmul_rn(texDX.y, sy);
        const F32 bx = __fmul_rn(texDY.x, sx), by = __fmul_rn(texDY.y, sy);
        const F32 dxlen = __fadd_rn(__fmul_rn(ax, ax), __fmul_rn(ay, ay));
        const F32 dylen = __fadd_rn(__fmul_rn(bx, bx), __fmul_rn(by, by));
        const F32 lod = fminf(fmaxf(__fmul_rn(crLog2(fmaxf(dxlen, dylen)), 0.5f), 0.0f), 14.0f);
        const int levelIdx = (int)lod;
        const Vec4f m0 = spec.mipLevels[levelIdx + 0];
        const Vec4f m1 = spec.mipLevels[levelIdx + 1];
        const F32 tx = __fsub_rn(tex.x, floorf(tex.x));
        const F32 ty = __fsub_rn(tex.y, floorf(tex.y));
        const Vec4f v0 = crTex2D(c_texPhong.atlas, __fadd_rn(__fmul_rn(tx, m0.x), m0.z), __fadd_rn(__fmul_rn(ty, m0.y), m0.w));
        const Vec4f v1 = crTex2D(c_texPhong.atlas, __fadd_rn(__fmul_rn(tx, m1.x), m1.z), __fadd_rn(__fmul_rn(ty, m1.y), m1.w));
        const F32 t = __fsub_rn(lod, (F32)levelIdx);
        return v0 * __fsub_rn(1.0f, t) + v1 * t;  // lerp (Math.hpp: a * (1 - t) + b * t)
    }

    __device__ __forceinline__ void run(void) {
        const Vec4f cp = interpolateVarying(0, m_centroid);
        const Vec4f cn = interpolateVarying(1, m_centroid);
        Vec2f tex, texDX, texDY;
        if (!kQuads) {
            // Sampled at the centroid with analytic derivatives.
            const Vec4f t = interpolateVarying(2, m_centroid);
            const Vec4f tdx = interpolateVarying(2, m_centroidDX);
            const Vec4f tdy = interpolateVarying(2, m_centroidDY);
            tex = Vec2f(t.x, t.y);
            texDX = Vec2f(tdx.x, tdx.y);
            texDY = Vec2f(tdy.x, tdy.y);
        } else {
            // Sampled at the pixel centre with numerical derivatives.
            const Vec4f t = interpolateVarying(2, m_center);
            tex = Vec2f(t.x, t.y);
            texDX = dFdx(tex);
            texDY = dFdy(tex);
        }

        const TexPhongConstants& k = c_texPhong;
        if (k.numMaterials <= 0) {  // no constants set yet: nothing to read
            m_discard = true;
            return;
        }
        const S64 slot = min((S64)m_triIdx, k.numTriangleMaterialIdx - 1);
        const S32 materialIdx = min(max(__ldg(k.triangleMaterialIdx + slot), 0), k.numMaterials - 1);
        const Material& material = k.materials[materialIdx];
        Vec4f diffuseColor = material.diffuseColor;
        if (material.diffuseTexture.size.x != 0.0f) {
            const Vec4f c = texture2D(material.diffuseTexture, tex, texDX, texDY);
            diffuseColor = Vec4f(c.x, c.y, c.z, diffuseColor.w);
        }
        if (material.alphaTexture.size.x != 0.0f) diffuseColor.w = texture2D(material.alphaTexture, tex, texDX, texDY).y;

        // Alpha test.
        if (diffuseColor.w < 0.5f) {
            m_discard = true;
            return;
        }
        const Vec3f color = evaluateLighting(Vec3f(cp.x, cp.y, cp.z), Vec3f(cn.x, cn.y, cn.z), material.specularColor,
                                             material.glossiness, Vec3f(diffuseColor.x, diffuseColor.y, diffuseColor.z));
        m_color = toABGR(Vec4f(color, diffuseColor.w));
    }
};

typedef TexPhongShader<false> FragmentShader_texPhong;
typedef TexPhongShader<true> FragmentShader_texPhong_quads;

}  // namespace FW

using namespace FW;

CR_DEFINE_PIXEL_PIPE(PixelPipe_texPhong, ShadedVertex_texPhong, FragmentShader_texPhong, BlendReplace, 0,
                     RenderModeFlag_EnableDepth | RenderModeFlag_EnableLerp)
CR_DEFINE_PIXEL_PIPE(PixelPipe_texPhong_quads, ShadedVertex_texPhong, FragmentShader_texPhong_quads, BlendReplace, 0,
                     RenderModeFlag_EnableDepth | RenderModeFlag_EnableLerp | RenderModeFlag_EnableQuads)
CR_DEFINE_PIXEL_PIPE(PixelPipe_texPhong_srcover, ShadedVertex_texPhong, FragmentShader_texPhong, BlendSrcOver, 0,
                     RenderModeFlag_EnableDepth | RenderModeFlag_EnableLerp)
CR_DEFINE_PIXEL_PIPE(PixelPipe_texPhong_msaa4, ShadedVertex_texPhong, FragmentShader_texPhong, BlendReplace, 2,
                     RenderModeFlag_EnableDepth | RenderModeFlag_EnableLerp)

extern "C" cr_status cr_set_tex_phong_constants(const cr_material* materials, int32_t num_materials,
                                                const int32_t* triangle_material_idx,
                                                int64_t num_triangle_material_idx, const uint32_t* atlas,
                                                int32_t atlas_width, int32_t atlas_height, void* stream) {
    if (!materials || num_materials < 1 || !triangle_material_idx || num_triangle_material_idx < 1 || !atlas ||
        atlas_width < 1 || atlas_height < 1 || atlas_width > 65536 || atlas_height > 65536 ||
        ((uintptr_t)materials & 3) || ((uintptr_t)triangle_material_idx & 3) || ((uintptr_t)atlas & 3))
        return CR_ERR_INVALID_ARGUMENT;
    FW::TexPhongConstants k;
    k.materials = (const FW::Material*)materials;
    k.triangleMaterialIdx = triangle_material_idx;
    k.numTriangleMaterialIdx = num_triangle_material_idx;
    k.numMaterials = num_materials;
    k.atlas = FW::TextureAtlas{atlas, atlas_width, atlas_height};
    // From pageable host memory: the copy has read `k` when the call returns.
    const cudaError_t e = cudaMemcpyToSymbolAsync(FW::c_texPhong, &k, sizeof(k), 0, cudaMemcpyHostToDevice,
                                                  (cudaStream_t)stream);
    return e == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}
