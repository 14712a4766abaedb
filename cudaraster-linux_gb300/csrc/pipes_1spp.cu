// Built-in single-sample pixel pipes.
#include "cudaraster/PixelPipe.inl"
#include "shaders.cuh"

using namespace FW;

CR_DEFINE_PIXEL_PIPE(PixelPipe_gouraud, GouraudVertex, GouraudShader, BlendReplace, 0,
                     RenderModeFlag_EnableDepth | RenderModeFlag_EnableLerp)
CR_DEFINE_PIXEL_PIPE(PixelPipe_gouraud_srcover, GouraudVertex, GouraudShader, BlendSrcOver, 0,
                     RenderModeFlag_EnableDepth | RenderModeFlag_EnableLerp)
CR_DEFINE_PIXEL_PIPE(PixelPipe_passthrough, ShadedVertexBase, FragmentShader_passthrough, BlendReplace, 0,
                     RenderModeFlag_EnableDepth | RenderModeFlag_EnableLerp)
