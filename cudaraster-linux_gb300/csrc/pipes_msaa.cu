// Built-in multisample pixel pipes.
#include "cudaraster/PixelPipe.inl"
#include "shaders.cuh"

using namespace FW;

CR_DEFINE_PIXEL_PIPE(PixelPipe_gouraud_msaa2, GouraudVertex, GouraudShader, BlendReplace, 1,
                     RenderModeFlag_EnableDepth | RenderModeFlag_EnableLerp)
CR_DEFINE_PIXEL_PIPE(PixelPipe_gouraud_msaa4, GouraudVertex, GouraudShader, BlendReplace, 2,
                     RenderModeFlag_EnableDepth | RenderModeFlag_EnableLerp)
CR_DEFINE_PIXEL_PIPE(PixelPipe_gouraud_msaa8, GouraudVertex, GouraudShader, BlendReplace, 3,
                     RenderModeFlag_EnableDepth | RenderModeFlag_EnableLerp)
CR_DEFINE_PIXEL_PIPE(PixelPipe_gouraud_srcover_msaa4, GouraudVertex, GouraudShader, BlendSrcOver, 2,
                     RenderModeFlag_EnableDepth | RenderModeFlag_EnableLerp)
CR_DEFINE_PIXEL_PIPE(PixelPipe_trihash_srcover_msaa4, GouraudVertex, TriHashShader, BlendSrcOver, 2, 0)
