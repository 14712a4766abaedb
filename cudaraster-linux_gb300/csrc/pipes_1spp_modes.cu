// Built-in single-sample pipes covering the remaining render modes and blends.
#include "cudaraster/PixelPipe.inl"
#include "shaders.cuh"

using namespace FW;

CR_DEFINE_PIXEL_PIPE(PixelPipe_gouraud_additive, GouraudVertex, GouraudShader, BlendAdditive, 0,
                     RenderModeFlag_EnableDepth | RenderModeFlag_EnableLerp)
CR_DEFINE_PIXEL_PIPE(PixelPipe_gouraud_depthonly, GouraudVertex, GouraudShader, BlendDepthOnly, 0,
                     RenderModeFlag_EnableDepth | RenderModeFlag_EnableLerp)
CR_DEFINE_PIXEL_PIPE(PixelPipe_gouraud_nodepth, GouraudVertex, GouraudShader, BlendSrcOver, 0,
                     RenderModeFlag_EnableLerp)
CR_DEFINE_PIXEL_PIPE(PixelPipe_gouraud_flat, GouraudVertex, GouraudShader, BlendReplace, 0,
                     RenderModeFlag_EnableDepth)
CR_DEFINE_PIXEL_PIPE(PixelPipe_trihash_srcover, GouraudVertex, TriHashShader, BlendSrcOver, 0, 0)
CR_DEFINE_PIXEL_PIPE(PixelPipe_deriv_quads, GouraudVertex, DerivShader, BlendReplace, 0,
                     RenderModeFlag_EnableDepth | RenderModeFlag_EnableLerp | RenderModeFlag_EnableQuads)
