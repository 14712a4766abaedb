// CudaRaster.hpp -- the reference's host classes as a header-only layer over
// the C ABI in cudaraster.h, for C++ callers of the rasterizer.
//
// Same names, arguments and error behaviour as tcoppex/cudaraster-linux:
//   FW::CudaRaster   src/cudaraster/CudaRaster.hpp:42-190 (init, setSurfaces,
//                    deferredClear, setPixelPipe, setVertexBuffer,
//                    setIndexBuffer, drawTriangles, getStats,
//                    getProfilingInfo, setDebugParams)
//   FW::CudaSurface  src/cudaraster/CudaSurface.hpp:39-71 (RGBA8 / DEPTH32,
//                    1-8 samples, sizes rounded up to 8x8 tiles)
//   FW::Buffer       the parts of src/framework/gpu/Buffer.hpp the raster
//                    path uses (resizeDiscard, setRange, getCudaPtr)
// A failed call prints the library's message and exits, as the reference's
// fail() does (src/framework/base/Defs.hpp:107-117); define
// CR_THROW_ON_ERROR to get a std::runtime_error instead.
//
// Differences from the reference, by design:
//   - pixel pipes are compiled ahead of time and registered by
//     CR_DEFINE_PIXEL_PIPE (PixelPipe.inl), so setPixelPipe's module argument
//     is accepted and ignored (pass nullptr);
//   - surfaces are plain device memory (no GL texture or CUDA array):
//     getDevicePtr() and download() take the place of getGLTexture() and
//     getCudaArray();
//   - draws go to a caller-chosen CUDA stream (setStream; default: the
//     legacy default stream, as the reference).
//
// Build: any C++17 compiler; include <repo>/include and the CUDA include
// directory, link libcudaraster_gb300.so and libcudart.
#pragma once

#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>

#include "../cudaraster.h"
#include "Types.hpp"

namespace FW {

typedef std::string String;
class CudaModule;  // pipes are linked in; see setPixelPipe

namespace crdetail {
[[noreturn]] inline void fail(const std::string& msg) {
#if defined(CR_THROW_ON_ERROR)
    throw std::runtime_error(msg);
#else
    std::fprintf(stderr, "%s\n", msg.c_str());
    std::exit(EXIT_FAILURE);
#endif
}
inline void check(cr_status st, cr_context* ctx) {
    if (st == CR_OK) return;
    const char* m = ctx ? cr_last_error(ctx) : nullptr;
    fail(m && *m ? std::string(m) : std::string("CudaRaster: ") + cr_status_string(st));
}
inline void checkCuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) fail(std::string(what) + " failed: " + cudaGetErrorString(e));
}
}  // namespace crdetail

// ------------------------------------------------------------------ Buffer
class Buffer {
public:
    Buffer() = default;
    explicit Buffer(S64 size) { resizeDiscard(size); }
    ~Buffer() { release(); }
    Buffer(const Buffer&) = delete;
    Buffer& operator=(const Buffer&) = delete;

    S64 getSize() const { return m_size; }
    // Reallocates without keeping the contents.
    void resizeDiscard(S64 size) {
        if (size < 0) crdetail::fail("Buffer: negative size!");
        if (size == m_size) return;
        release();
        if (size) crdetail::checkCuda(cudaMalloc(&m_ptr, (size_t)size), "cudaMalloc");
        m_size = size;
    }
    // Host -> device copy of `size` bytes at byte offset `ofs`.
    void setRange(S64 ofs, const void* src, S64 size) {
        if (ofs < 0 || size < 0 || ofs + size > m_size) crdetail::fail("Buffer: range out of bounds!");
        crdetail::checkCuda(cudaMemcpy((char*)m_ptr + ofs, src, (size_t)size, cudaMemcpyHostToDevice), "cudaMemcpy");
    }
    void getRange(void* dst, S64 ofs, S64 size) const {
        if (ofs < 0 || size < 0 || ofs + size > m_size) crdetail::fail("Buffer: range out of bounds!");
        crdetail::checkCuda(cudaMemcpy(dst, (const char*)m_ptr + ofs, (size_t)size, cudaMemcpyDeviceToHost),
                            "cudaMemcpy");
    }
    void* getMutableCudaPtr(S64 ofs = 0) { return (char*)m_ptr + ofs; }
    const void* getCudaPtr(S64 ofs = 0) const { return (const char*)m_ptr + ofs; }

private:
    void release() {
        if (m_ptr) cudaFree(m_ptr);
        m_ptr = nullptr;
        m_size = 0;
    }
    void* m_ptr = nullptr;
    S64 m_size = 0;
};

// ------------------------------------------------------------- CudaSurface
class CudaSurface {
public:
    enum Format { FORMAT_RGBA8, FORMAT_DEPTH32 };

    // Validation and messages as CudaSurface.cpp:44-62.
    CudaSurface(const Vec2i& size, Format format, int numSamples = 1)
        : m_size(size), m_format(format), m_numSamples(numSamples) {
        if (size.x <= 0 || size.y <= 0) crdetail::fail("CudaSurface: Size must be positive!");
        if (size.x > CR_MAX_VIEWPORT || size.y > CR_MAX_VIEWPORT)
            crdetail::fail("CudaSurface: CR_MAXVIEWPORT_SIZE exceeded!");
        if (numSamples > 8) crdetail::fail("CudaSurface: numSamples cannot exceed 8!");
        if (numSamples < 1 || (numSamples & (numSamples - 1)))
            crdetail::fail("CudaSurface: numSamples must be a power of two!");
        m_samplesLog2 = 0;
        while ((1 << m_samplesLog2) < numSamples) m_samplesLog2++;
        m_roundedSize = Vec2i((size.x + CR_TILE_SIZE_PX - 1) & ~(CR_TILE_SIZE_PX - 1),
                              (size.y + CR_TILE_SIZE_PX - 1) & ~(CR_TILE_SIZE_PX - 1));
        m_textureSize = Vec2i(m_roundedSize.x * numSamples, m_roundedSize.y);
        crdetail::checkCuda(cudaMalloc(&m_ptr, getNumBytes()), "cudaMalloc");
        crdetail::checkCuda(cudaMemset(m_ptr, 0, getNumBytes()), "cudaMemset");
    }
    ~CudaSurface() {
        if (m_ptr) cudaFree(m_ptr);
    }
    CudaSurface(const CudaSurface&) = delete;
    CudaSurface& operator=(const CudaSurface&) = delete;

    Vec2i getSize() const { return m_size; }
    Vec2i getRoundedSize() const { return m_roundedSize; }
    Vec2i getTextureSize() const { return m_textureSize; }
    Format getFormat() const { return m_format; }
    int getNumSamples() const { return m_numSamples; }
    int getSamplesLog2() const { return m_samplesLog2; }
    // Row-major 32-bit words, getTextureSize().x words per row; sample i of
    // pixel (x, y) at word (x >> 3) * 8 * S + i * 8 + (x & 7) of row y.
    void* getDevicePtr() const { return m_ptr; }
    size_t getNumBytes() const { return (size_t)m_textureSize.x * m_textureSize.y * 4; }
    void download(void* host) const {
        crdetail::checkCuda(cudaMemcpy(host, m_ptr, getNumBytes(), cudaMemcpyDeviceToHost), "cudaMemcpy");
    }

private:
    Vec2i m_size, m_roundedSize, m_textureSize;
    Format m_format;
    int m_numSamples = 1, m_samplesLog2 = 0;
    void* m_ptr = nullptr;
};

// -------------------------------------------------------------- CudaRaster
class CudaRaster {
public:
    struct Stats {  // seconds, CudaRaster.hpp:45-51
        F32 setupTime = 0.0f, binTime = 0.0f, coarseTime = 0.0f, fineTime = 0.0f;
    };
    struct DebugParams {  // CudaRaster.hpp:53-67
        bool emulateTriangleSetup = false, emulateBinRaster = false, emulateCoarseRaster = false,
             emulateFineRaster = false;
    };

    CudaRaster() = default;
    ~CudaRaster() {
        if (m_ctx) cr_destroy(m_ctx);
    }
    CudaRaster(const CudaRaster&) = delete;
    CudaRaster& operator=(const CudaRaster&) = delete;

    // CudaRaster.cpp:98-128.
    void init() {
        if (m_ctx) return;
        cr_status st = cr_create(&m_ctx);
        if (st == CR_ERR_CUDA) crdetail::fail("CudaRaster: No CUDA-capable devices found!");
        if (st == CR_ERR_UNSUPPORTED) crdetail::fail("CudaRaster: Compute capability 10.x or better is required!");
        crdetail::check(st, nullptr);
    }

    // CudaRaster.cpp:132-170; both null unbinds.
    void setSurfaces(CudaSurface* color, CudaSurface* depth) {
        needInit();
        if (!color && !depth) {
            crdetail::check(cr_set_surfaces(m_ctx, nullptr, nullptr, 0, 0, 0), m_ctx);
            return;
        }
        if (!color) crdetail::fail("CudaRaster: No color buffer specified!");
        if (!depth) crdetail::fail("CudaRaster: No depth buffer specified!");
        if (color->getFormat() != CudaSurface::FORMAT_RGBA8)
            crdetail::fail("CudaRaster: Unsupported color buffer format!");
        if (depth->getFormat() != CudaSurface::FORMAT_DEPTH32)
            crdetail::fail("CudaRaster: Unsupported depth buffer format!");
        if (color->getSize() != depth->getSize()) crdetail::fail("CudaRaster: Mismatch in size between surfaces!");
        if (color->getNumSamples() != depth->getNumSamples())
            crdetail::fail("CudaRaster: Mismatch in multisampling between surfaces!");
        crdetail::check(cr_set_surfaces(m_ctx, color->getDevicePtr(), depth->getDevicePtr(), color->getSize().x,
                                        color->getSize().y, color->getNumSamples()),
                        m_ctx);
    }

    // CudaRaster.cpp:174-179: applied by the next draw.
    void deferredClear(const Vec4f& color = Vec4f(0.0f), F32 depth = 1.0f) {
        needInit();
        crdetail::check(cr_deferred_clear(m_ctx, color.x, color.y, color.z, color.w, depth), m_ctx);
    }

    // CudaRaster.cpp:183-216: `name` is a pipe defined with CR_DEFINE_PIXEL_PIPE.
    void setPixelPipe(CudaModule* module, const String& name) {
        (void)module;
        needInit();
        crdetail::check(cr_set_pixel_pipe(m_ctx, name.c_str()), m_ctx);
    }

    // CudaRaster.cpp:220-233: byte offsets into device buffers.
    void setVertexBuffer(Buffer* buf, S64 ofs) {
        needInit();
        crdetail::check(cr_set_vertex_buffer(m_ctx, buf ? buf->getCudaPtr() : nullptr, ofs), m_ctx);
    }
    void setIndexBuffer(Buffer* buf, S64 ofs, int numTris) {
        needInit();
        crdetail::check(cr_set_index_buffer(m_ctx, buf ? buf->getCudaPtr() : nullptr, ofs, numTris), m_ctx);
    }
    // Beyond the reference: vertexShader_passthrough fused into setup
    // (cr_set_vertex_transform). `model` holds xyz at modelStride floats per
    // vertex; mvpRowMajor is 16 floats; a null model turns it off.
    void setVertexTransform(Buffer* model, int modelStride, const float* mvpRowMajor) {
        needInit();
        crdetail::check(cr_set_vertex_transform(m_ctx, model ? (const float*)model->getCudaPtr() : nullptr,
                                                modelStride, mvpRowMajor),
                        m_ctx);
    }

    // CudaRaster.cpp:237-342: draws, reads the overflow counters back and
    // reruns with grown queues until nothing overflowed.
    void drawTriangles() {
        needInit();
        crdetail::check(cr_draw_triangles(m_ctx, m_stream), m_ctx);
    }
    // No read-back: the caller reads the counters later (cr_get_counters).
    void drawTrianglesAsync() {
        needInit();
        crdetail::check(cr_draw_triangles_async(m_ctx, m_stream), m_ctx);
    }

    // CudaRaster.cpp:346-363.
    Stats getStats() {
        needInit();
        cr_stats s;
        crdetail::check(cr_get_stats(m_ctx, &s), m_ctx);
        Stats out;
        out.setupTime = s.setup_time;
        out.binTime = s.bin_time;
        out.coarseTime = s.coarse_time;
        out.fineTime = s.fine_time;
        return out;
    }

    // CudaRaster.cpp:367-497.
    String getProfilingInfo() {
        needInit();
        char buf[4096];
        crdetail::check(cr_get_profiling_info(m_ctx, buf, sizeof(buf)), m_ctx);
        return String(buf);
    }

    // CudaRaster.hpp:53-67, 168: host emulation of the stages is not
    // provided, so any emulation flag fails.
    void setDebugParams(const DebugParams& p) {
        needInit();
        cr_debug_params d;
        d.emulate_triangle_setup = p.emulateTriangleSetup;
        d.emulate_bin_raster = p.emulateBinRaster;
        d.emulate_coarse_raster = p.emulateCoarseRaster;
        d.emulate_fine_raster = p.emulateFineRaster;
        crdetail::check(cr_set_debug_params(m_ctx, &d), m_ctx);
    }

    // -------- beyond the reference
    void setStream(cudaStream_t stream) { m_stream = stream; }
    cr_counters getCounters() {
        needInit();
        cr_counters c;
        crdetail::check(cr_get_counters(m_ctx, &c), m_ctx);
        return c;
    }
    void setTuning(const cr_tuning& t) {
        needInit();
        crdetail::check(cr_set_tuning(m_ctx, &t), m_ctx);
    }
    void setCapacity(S64 maxSubtris, S64 maxBinEntries, S64 maxTileEntries) {
        needInit();
        crdetail::check(cr_set_capacity(m_ctx, maxSubtris, maxBinEntries, maxTileEntries), m_ctx);
    }
    cr_context* handle() const { return m_ctx; }

private:
    void needInit() const {
        if (!m_ctx) crdetail::fail("CudaRaster: init() has not been called!");
    }
    cr_context* m_ctx = nullptr;
    cudaStream_t m_stream = nullptr;
};

}  // namespace FW
