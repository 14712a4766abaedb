// static_draw.cu -- cr_draw_triangles_static: one draw whose intermediate
// queues live in a fixed array compiled into this library, so the call never
// allocates device or host memory.
//
// Who needs it: callers that are not allowed to allocate once they are
// running -- a host application that hands the rasterizer a fixed memory
// budget and owns every allocation itself, a real-time render loop where an
// allocation (and the implicit device synchronisation cudaMalloc/cudaFree can
// cause) would stall the frame, or a plugin that only receives raw device
// pointers from its host. cr_draw_triangles cannot serve them because its
// context grows its queues with cudaMalloc.
//
// Limits: at most kStaticMaxTris triangles, viewport at most
// kStaticMaxViewport pixels on each side, and fixed queue capacities (see
// below); a draw that needs more returns CR_ERR_CAPACITY and leaves the
// surfaces untouched.
//
// Sharing: the array is one per GPU and per process for the lifetime of the
// library, and every call reuses it. Calls that overlap on the GPU (issued on
// different streams, or from different host threads, without ordering
// between them) race on it and corrupt each other's output; order them on
// one stream. The array keeps the last call's contents; each call clears the
// counters it depends on.
//
// Set-up: the first call on a device, with that device current, looks up the
// array's device address with cudaGetSymbolAddress (a host-side name of a
// __device__ array is not a device address). Make that first call before any
// stream capture on the device.
#include "cudaraster.h"
#include "cudaraster/detail/device.cuh"
#include "cudaraster/detail/pipe_registry.h"

#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <mutex>

namespace cr {
cudaError_t launchBinning(const DrawDev& d, int maxBins, int numSMs, cudaStream_t stream, cudaEvent_t evCoarse);
}
namespace cr {
const PipeDesc* findRegisteredPipe(const char* name);
}

using namespace cr;

namespace {

constexpr int kStaticMaxTris = 65536;
constexpr int kStaticMaxViewport = 1024;
constexpr int kStaticBinLog2 = 4;
constexpr int kStaticChunkTris = 1024;
constexpr int kStaticUnitEntries = 512;
constexpr int kStaticMaxTiles = (kStaticMaxViewport / 8) * (kStaticMaxViewport / 8);
constexpr int kStaticMaxBins = (kStaticMaxViewport / 128) * (kStaticMaxViewport / 128);
constexpr int kStaticMaxChunks = kStaticMaxTris / kStaticChunkTris;
constexpr int64_t kStaticMaxSubtris = kStaticMaxTris + 16384;
constexpr int64_t kStaticMaxBinEntries = 4 * kStaticMaxTris;
constexpr int64_t kStaticMaxTileEntries = 16 * kStaticMaxTris;
constexpr int64_t kStaticMaxUnits = kStaticMaxBinEntries / kStaticUnitEntries + kStaticMaxBins + 1;
constexpr int kStaticTilesPerBin = 1 << (2 * kStaticBinLog2);

constexpr size_t alignUp(size_t v) { return (v + 255) & ~(size_t)255; }

// Byte layout of the array.
constexpr size_t kOffCounters = 0;
constexpr size_t kOffFine = alignUp(kOffCounters + sizeof(Counters));
constexpr size_t kOffInst = alignUp(kOffFine + sizeof(int32_t));
constexpr size_t kOffPrefix = alignUp(kOffInst + sizeof(InstanceDev));
constexpr size_t kOffSubtris = alignUp(kOffPrefix + 64);
constexpr size_t kOffHeader = alignUp(kOffSubtris + kStaticMaxTris);
constexpr size_t kOffData = alignUp(kOffHeader + 16 * kStaticMaxSubtris);
constexpr size_t kOffChunkCount = alignUp(kOffData + 64 * kStaticMaxSubtris);
constexpr size_t kOffChunkOffset = alignUp(kOffChunkCount + 4 * (size_t)kStaticMaxChunks * kStaticMaxBins);
constexpr size_t kOffBinCount = alignUp(kOffChunkOffset + 4 * (size_t)kStaticMaxChunks * kStaticMaxBins);
constexpr size_t kOffBinStart = alignUp(kOffBinCount + 4 * kStaticMaxBins);
constexpr size_t kOffBinUnitFirst = alignUp(kOffBinStart + 4 * kStaticMaxBins);
constexpr size_t kOffBinList = alignUp(kOffBinUnitFirst + 4 * kStaticMaxBins);
constexpr size_t kOffUnitTileCount = alignUp(kOffBinList + 4 * kStaticMaxBinEntries);
constexpr size_t kOffTileCount = alignUp(kOffUnitTileCount + 4 * (size_t)kStaticMaxUnits * kStaticTilesPerBin);
constexpr size_t kOffTileStart = alignUp(kOffTileCount + 4 * kStaticMaxTiles);
constexpr size_t kOffTileList = alignUp(kOffTileStart + 4 * kStaticMaxTiles);
constexpr size_t kStaticScratchBytes = alignUp(kOffTileList + 4 * kStaticMaxTileEntries);

}  // namespace

// The scratch array (about 13 MiB, held by every GPU that loads the library).
static __device__ __align__(256) unsigned char g_staticScratch[kStaticScratchBytes];

namespace {

std::mutex g_setupMutex;
void* g_scratchPtr[256];
int g_numSMs[256];

cr_status report(char* err, int64_t errSize, cr_status s, const char* fmt, ...) {
    if (err && errSize > 0) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(err, (size_t)errSize, fmt, ap);
        va_end(ap);
    }
    return s;
}

}  // namespace

extern "C" cr_status cr_draw_triangles_static(const char* pipe_name, void* color, void* depth, int32_t width,
                                              int32_t height, int32_t num_samples, const void* vertices,
                                              const void* indices, int32_t num_tris, int32_t deferred_clear,
                                              uint32_t clear_color, uint32_t clear_depth, void* stream, char* error,
                                              int64_t error_size) {
    if (error && error_size > 0) error[0] = 0;
    const PipeDesc* pipe = pipe_name ? findRegisteredPipe(pipe_name) : nullptr;
    if (!pipe) return report(error, error_size, CR_ERR_NO_PIPE, "cr_draw_triangles_static: unknown pixel pipe");
    if (!color || !depth) return report(error, error_size, CR_ERR_INVALID_ARGUMENT, "cr_draw_triangles_static: no surfaces");
    if (width <= 0 || height <= 0)
        return report(error, error_size, CR_ERR_INVALID_ARGUMENT, "cr_draw_triangles_static: size must be positive");
    if (width > kStaticMaxViewport || height > kStaticMaxViewport)
        return report(error, error_size, CR_ERR_CAPACITY,
                      "cr_draw_triangles_static: viewport %dx%d exceeds the static limit of %dx%d pixels", width, height,
                      kStaticMaxViewport, kStaticMaxViewport);
    if (num_tris < 0) return report(error, error_size, CR_ERR_INVALID_ARGUMENT, "cr_draw_triangles_static: negative triangle count");
    if (num_tris > kStaticMaxTris)
        return report(error, error_size, CR_ERR_CAPACITY,
                      "cr_draw_triangles_static: %d triangles exceed the static limit of %d", num_tris, kStaticMaxTris);
    if (num_samples < 1 || num_samples > 8 || (num_samples & (num_samples - 1)))
        return report(error, error_size, CR_ERR_INVALID_ARGUMENT, "cr_draw_triangles_static: numSamples must be 1, 2, 4 or 8");
    int samplesLog2 = 0;
    while ((1 << samplesLog2) < num_samples) samplesLog2++;
    if (pipe->samplesLog2 != samplesLog2)
        return report(error, error_size, CR_ERR_PIPE_MISMATCH,
                      "cr_draw_triangles_static: Mismatch in multisampling between pixel pipe and surface!");
    if (num_tris > 0 && (!vertices || !indices))
        return report(error, error_size, CR_ERR_INVALID_ARGUMENT, "cr_draw_triangles_static: no vertex or index buffer");
    if (((uintptr_t)vertices & 15) || ((uintptr_t)indices & 3) || ((uintptr_t)color & 3) || ((uintptr_t)depth & 3))
        return report(error, error_size, CR_ERR_INVALID_ARGUMENT, "cr_draw_triangles_static: misaligned buffer");

    // Per-device set-up: the array's device address, with the device current.
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256)
        return report(error, error_size, CR_ERR_CUDA, "cr_draw_triangles_static: no current CUDA device");
    unsigned char* scratch;
    int numSMs;
    {
        std::lock_guard<std::mutex> lock(g_setupMutex);
        if (!g_scratchPtr[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_staticScratch);
            if (e != cudaSuccess || !p)
                return report(error, error_size, CR_ERR_CUDA, "cr_draw_triangles_static: cudaGetSymbolAddress failed: %s",
                              cudaGetErrorString(e));
            int sms = 0;
            e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (e != cudaSuccess)
                return report(error, error_size, CR_ERR_CUDA, "cr_draw_triangles_static: %s", cudaGetErrorString(e));
            g_numSMs[dev] = sms;
            g_scratchPtr[dev] = p;
        }
        scratch = (unsigned char*)g_scratchPtr[dev];
        numSMs = g_numSMs[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;

    // One instance covering the whole draw.
    InstanceDev in;
    memset(&in, 0, sizeof(in));
    in.vertices = (const float4*)vertices;
    in.indices = (const int*)indices;
    in.color = (uint32_t*)color;
    in.depth = (uint32_t*)depth;
    in.stride4 = pipe->vertexStructSize / 16;
    in.numTris = num_tris;
    in.width = width;
    in.height = height;
    in.samplesLog2 = samplesLog2;
    in.deferredClear = deferred_clear ? 1 : 0;
    in.clearColor = clear_color;
    in.clearDepth = clear_depth;
    in.widthTiles = (width + 7) >> 3;
    in.heightTiles = (height + 7) >> 3;
    const int side = 1 << kStaticBinLog2;
    in.widthBins = (in.widthTiles + side - 1) / side;
    in.heightBins = (in.heightTiles + side - 1) / side;
    in.rowWords = (int64_t)(in.widthTiles * 8) << samplesLog2;
    in.chunkTris = kStaticChunkTris;
    in.numChunks = (num_tris + kStaticChunkTris - 1) / kStaticChunkTris;
    const int numBins = in.widthBins * in.heightBins;
    const int numTiles = in.widthTiles * in.heightTiles;

    // Descriptor block: instance, then prefixes (tri int64[2], chunk/bin/tile int32[2] each).
    struct Prefixes {
        int64_t tri[2];
        int32_t chunk[2], bin[2], tile[2];
    };
    Prefixes pref = {{0, num_tris}, {0, in.numChunks}, {0, numBins}, {0, numTiles}};
    static_assert(sizeof(pref) <= 64, "prefix block");

    DrawDev d;
    memset(&d, 0, sizeof(d));
    d.inst = (const InstanceDev*)(scratch + kOffInst);
    d.numInstances = 1;
    d.binLog2 = kStaticBinLog2;
    d.totalBins = numBins;
    d.totalTiles = numTiles;
    d.totalChunks = in.numChunks;
    d.unitEntries = kStaticUnitEntries;
    d.totalTris = num_tris;
    d.triSubtris = scratch + kOffSubtris;
    d.triHeader = (uint4*)(scratch + kOffHeader);
    d.triData = (uint4*)(scratch + kOffData);
    d.maxSubtris = kStaticMaxSubtris;
    d.chunkBinCount = (int32_t*)(scratch + kOffChunkCount);   // zero at load; each bin scan clears it again
    d.chunkBinOffset = (int32_t*)(scratch + kOffChunkOffset);
    d.maxBins = numBins;
    d.fineSelfPixels = 0;
    d.model = nullptr;
    d.modelStride = 0;
    d.modelVec4 = 0;
    d.binCount = (int32_t*)(scratch + kOffBinCount);
    d.binStart = (int32_t*)(scratch + kOffBinStart);
    d.binUnitFirst = (int32_t*)(scratch + kOffBinUnitFirst);
    d.binList = (uint32_t*)(scratch + kOffBinList);
    d.maxBinEntries = kStaticMaxBinEntries;
    d.unitTileCount = (int32_t*)(scratch + kOffUnitTileCount);
    d.maxUnits = kStaticMaxUnits;
    d.tileCount = (int32_t*)(scratch + kOffTileCount);
    d.tileStart = (int32_t*)(scratch + kOffTileStart);
    d.tileList = (uint32_t*)(scratch + kOffTileList);
    d.maxTileEntries = kStaticMaxTileEntries;
    d.triPrefix = (const int64_t*)(scratch + kOffPrefix);
    d.chunkPrefix = (const int32_t*)(scratch + kOffPrefix + offsetof(Prefixes, chunk));
    d.binPrefix = (const int32_t*)(scratch + kOffPrefix + offsetof(Prefixes, bin));
    d.tilePrefix = (const int32_t*)(scratch + kOffPrefix + offsetof(Prefixes, tile));
    d.counters = (Counters*)(scratch + kOffCounters);
    d.fineTileCounter = (int32_t*)(scratch + kOffFine);

#define CR_STATIC_CUDA(call)                                                                                   \
    do {                                                                                                       \
        cudaError_t e_ = (call);                                                                               \
        if (e_ != cudaSuccess)                                                                                 \
            return report(error, error_size, CR_ERR_CUDA, "cr_draw_triangles_static: %s", cudaGetErrorString(e_)); \
    } while (0)

    // Pageable host sources: the copies are staged by the driver before these calls return.
    CR_STATIC_CUDA(cudaMemcpyAsync(scratch + kOffInst, &in, sizeof(in), cudaMemcpyHostToDevice, s));
    CR_STATIC_CUDA(cudaMemcpyAsync(scratch + kOffPrefix, &pref, sizeof(pref), cudaMemcpyHostToDevice, s));
    // Counters and the fine work counter must start at zero on every call.
    CR_STATIC_CUDA(cudaMemsetAsync(scratch + kOffCounters, 0, kOffInst - kOffCounters, s));

    CR_STATIC_CUDA(pipe->launchSetup(d, 0, 1, 0, num_tris, s));
    CR_STATIC_CUDA(launchBinning(d, numBins, numSMs, s, nullptr));
    const int warps = 8;
    CR_STATIC_CUDA(pipe->launchFine(d, 0, 0, numTiles, warps, pipe->fineOccupancy(warps), numSMs, s));

    Counters c;
    CR_STATIC_CUDA(cudaMemcpyAsync(&c, scratch + kOffCounters, sizeof(c), cudaMemcpyDeviceToHost, s));
    CR_STATIC_CUDA(cudaStreamSynchronize(s));
    if (c.overflow)
        return report(error, error_size, CR_ERR_CAPACITY,
                      "cr_draw_triangles_static: the draw needs more than the static queues hold "
                      "(%lld subtriangle slots, %lld bin entries, %lld tile entries); surfaces left untouched",
                      (long long)kStaticMaxSubtris, (long long)kStaticMaxBinEntries, (long long)kStaticMaxTileEntries);
#undef CR_STATIC_CUDA
    return CR_OK;
}
