// runtime.cu -- host side of the C ABI (include/cudaraster.h).
//
// Mirrors the reference's CudaRaster host class (src/cudaraster/CudaRaster.cpp):
// state setters with the same validation messages, the queue-capacity
// estimate and the overflow-detect-and-rerun loop of drawTriangles
// (CudaRaster.cpp:237-342), per-stage CUDA events for getStats
// (CudaRaster.cpp:346-363). Errors are returned as cr_status codes with a
// message in cr_last_error() instead of exiting the process; the C++
// wrapper (CudaRaster.hpp) turns them into the reference's fail().
#include "cudaraster.h"
#include "cudaraster/detail/device.cuh"
#include "cudaraster/detail/launch.h"
#include "cudaraster/detail/pipe_registry.h"

#include <algorithm>
#include <cstddef>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace cr {
cudaError_t launchBinning(const DrawDev& d, int maxBins, int numSMs, cudaStream_t stream, cudaEvent_t evCoarse);
}

using namespace cr;

// ------------------------------------------------------------ pipe registry
namespace {
std::vector<PipeDesc>& registry() {
    static std::vector<PipeDesc> r;
    return r;
}
std::mutex& registryMutex() {
    static std::mutex m;
    return m;
}
const PipeDesc* findPipe(const char* name) {
    std::lock_guard<std::mutex> lock(registryMutex());
    for (const PipeDesc& p : registry())
        if (strncmp(p.name, name, sizeof(p.name)) == 0) return &p;
    return nullptr;
}
}  // namespace

namespace cr {
// Pipe lookup for other translation units of the library.
const PipeDesc* findRegisteredPipe(const char* name) { return findPipe(name); }
}  // namespace cr

extern "C" void cr_register_pipe(const cr::PipeDesc* desc) {
    std::lock_guard<std::mutex> lock(registryMutex());
    for (PipeDesc& p : registry())
        if (strncmp(p.name, desc->name, sizeof(p.name)) == 0) { p = *desc; return; }
    registry().push_back(*desc);
}

// ---------------------------------------------------------- device buffers
namespace {
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    // Grows only. A regrow takes a quarter more than asked, so queues whose
    // capacity creeps up from draw to draw (e.g. sized by a predictor) are
    // not reallocated -- and the device synchronised -- every draw.
    cudaError_t ensure(size_t need) {
        if (need <= bytes) return cudaSuccess;
        const bool regrow = ptr != nullptr;
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
        size_t alloc = std::max<size_t>(regrow ? need + need / 4 : need, 256);
        cudaError_t e = cudaMalloc(&ptr, alloc);
        if (e == cudaSuccess) bytes = alloc;
        return e;
    }
    // As ensure, and a new allocation starts zeroed.
    cudaError_t ensureZeroed(size_t need) {
        if (need <= bytes) return cudaSuccess;
        cudaError_t e = ensure(need);
        return e == cudaSuccess ? cudaMemset(ptr, 0, bytes) : e;
    }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    template <class T> T* as() const { return (T*)ptr; }
};

struct HostInstance {
    const PipeDesc* pipe;
    InstanceDev dev;
};
}  // namespace

struct cr_context {
    std::string lastError;
    // Surfaces (CudaRaster.cpp:132-170).
    void* color = nullptr;
    void* depth = nullptr;
    int width = 0, height = 0, numSamples = 0, samplesLog2 = 0;
    bool surfacesSet = false;
    // Deferred clear (CudaRaster.cpp:174-179).
    bool deferredClear = false;
    uint32_t clearColor = 0, clearDepth = 0;
    // Pipe and buffers.
    const PipeDesc* pipe = nullptr;
    const void* vertices = nullptr;
    const void* indices = nullptr;
    int numTris = 0;
    bool vertexSet = false, indexSet = false;
    // Fused vertex transform (cr_set_vertex_transform).
    const float* model = nullptr;
    int modelStride = 0;
    float mvp[16] = {};
    cr_tuning tuning{};
    // Capacities (elements), grown by the rerun loop and kept across draws.
    int64_t maxSubtris = 0, maxBinEntries = 0, maxTileEntries = 0;
    bool userCapacity = false;  // capacities set by cr_set_capacity replace the estimates
    // Device memory.
    DevBuf triSubtris, triHeader, triData, chunkBinCount, chunkBinOffset, binCount, binStart, binUnitFirst, binList;
    DevBuf unitTileCount, tileCount, tileStart, tileList;
    DevBuf binStage, binStageCount;     // bin pairs recorded by the count pass (DrawDev::binStage)
    DevBuf tileStage, tileStageCount;   // tile pairs recorded by the coarse count pass (DrawDev::tileStage)
    // Per-draw block, written by one copy per draw: the zeroed Counters and one
    // fine-stage tile counter per pipe group, then the instance descriptors
    // and the prefix arrays.
    DevBuf drawBlock;
    // Pinned staging.
    // Descriptor staging for asynchronous draws: a ring of pinned slots, each
    // reused only after the copy that read it has run (stageDone), so a host
    // that queues draw after draw never rewrites descriptors still in flight.
    static constexpr int kStageSlots = 4;
    void* hostStage[kStageSlots] = {};
    size_t hostStageBytes = 0;                // per slot
    cudaEvent_t stageDone[kStageSlots] = {};
    bool stageUsed[kStageSlots] = {};
    int stageNext = 0;
    Counters* hostCounters = nullptr;
    cudaEvent_t ev[5] = {};
    bool stageTiming = true;      // record the per-stage events of getStats
    bool eventsRecorded = false;  // the last draw recorded them
    bool drawn = false;           // a draw was enqueued (its counters are copied to hostCounters)
    int numSMs = 0;
    int device = 0;
    // Last draw.
    cr_counters last{};
    cr_queue_layout lastLayout{};
};

namespace {
cr_status fail(cr_context* ctx, cr_status s, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (ctx) ctx->lastError = buf;
    return s;
}
cr_status cudaFail(cr_context* ctx, cudaError_t e, const char* what) {
    return fail(ctx, e == cudaErrorMemoryAllocation ? CR_ERR_OUT_OF_MEMORY : CR_ERR_CUDA, "CudaRaster: %s failed: %s",
                what, cudaGetErrorString(e));
}
#define CR_CUDA(call, what)                              \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cudaFail(ctx, e_, what); \
    } while (0)

int ilog2(int v) {
    int r = 0;
    while ((1 << r) < v) r++;
    return r;
}

// Host arithmetic of the reference.
uint32_t hostChannel(float c) {  // Math.cpp:41-48
    float cl = std::fmin(std::fmax(c, 0.0f), 1.0f);
    uint64_t t = (uint64_t)((double)cl * std::exp2(56.0));
    return (uint32_t)((((t * 255) >> 55) + 1) >> 1);
}
uint32_t encodeDepth(uint32_t depth) {  // Util.hpp:290-298
    double v = (double)depth;
    v /= 65536.0 * 65536.0 - 1.0;
    v = std::min(std::max(v, 0.0), 1.0);
    v *= (double)(kDepthMax - kDepthMin);
    v += (double)kDepthMin;
    return (uint32_t)v;
}
}  // namespace

// ================================================================ C API
extern "C" {

int32_t cr_abi_version(void) { return CR_ABI_VERSION; }

const char* cr_status_string(cr_status s) {
    switch (s) {
    case CR_OK: return "CR_OK";
    case CR_ERR_INVALID_ARGUMENT: return "CR_ERR_INVALID_ARGUMENT";
    case CR_ERR_INVALID_STATE: return "CR_ERR_INVALID_STATE";
    case CR_ERR_NO_PIPE: return "CR_ERR_NO_PIPE";
    case CR_ERR_PIPE_MISMATCH: return "CR_ERR_PIPE_MISMATCH";
    case CR_ERR_CAPACITY: return "CR_ERR_CAPACITY";
    case CR_ERR_CUDA: return "CR_ERR_CUDA";
    case CR_ERR_TIMEOUT: return "CR_ERR_TIMEOUT";
    case CR_ERR_OUT_OF_MEMORY: return "CR_ERR_OUT_OF_MEMORY";
    case CR_ERR_UNSUPPORTED: return "CR_ERR_UNSUPPORTED";
    }
    return "CR_ERR_UNKNOWN";
}

const char* cr_last_error(const cr_context* ctx) { return ctx ? ctx->lastError.c_str() : ""; }

uint32_t cr_color_to_abgr(float r, float g, float b, float a) {
    return hostChannel(r) | (hostChannel(g) << 8) | (hostChannel(b) << 16) | (hostChannel(a) << 24);
}
uint32_t cr_encode_depth(uint32_t d) { return encodeDepth(d); }
uint32_t cr_decode_depth(uint32_t depth) {  // Util.hpp:302-310
    double v = (double)depth;
    v -= (double)kDepthMin;
    v *= 1.0 / (double)(kDepthMax - kDepthMin);
    v = std::min(std::max(v, 0.0), 1.0);
    v *= 65536.0 * 65536.0 - 1.0;
    return (uint32_t)v;
}
uint32_t cr_clear_depth_from_float(float depth) {  // CudaRaster.cpp:178
    double v = (double)depth * std::exp2(32.0);
    uint64_t t;
    if (!(v > 0.0)) t = 0;
    else if (v >= 18446744073709551616.0) t = UINT64_MAX;
    else t = (uint64_t)v;
    return encodeDepth((uint32_t)std::min<uint64_t>(t, 0xFFFFFFFFull));
}

cr_status cr_create(cr_context** out) {
    if (!out) return CR_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return CR_ERR_CUDA;  // "No CUDA-capable devices found!"
    cr_context* ctx = new cr_context();
    cudaGetDevice(&ctx->device);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, ctx->device) != cudaSuccess) { delete ctx; return CR_ERR_CUDA; }
    if (prop.major < 10) {  // the kernels are built for sm_103a only
        delete ctx;
        return CR_ERR_UNSUPPORTED;
    }
    ctx->numSMs = prop.multiProcessorCount;
    for (int i = 0; i < 5; i++) {
        if (cudaEventCreate(&ctx->ev[i]) != cudaSuccess) { delete ctx; return CR_ERR_CUDA; }
    }
    if (cudaMallocHost(&ctx->hostCounters, sizeof(Counters)) != cudaSuccess) { delete ctx; return CR_ERR_CUDA; }
    memset(ctx->hostCounters, 0, sizeof(Counters));
    *out = ctx;
    return CR_OK;
}

cr_status cr_destroy(cr_context* ctx) {
    if (!ctx) return CR_ERR_INVALID_ARGUMENT;
    cudaDeviceSynchronize();
    DevBuf* bufs[] = {&ctx->triSubtris, &ctx->triHeader, &ctx->triData, &ctx->chunkBinCount, &ctx->chunkBinOffset,
                      &ctx->binCount,
                      &ctx->binStart, &ctx->binUnitFirst, &ctx->binList, &ctx->unitTileCount,
                      &ctx->tileCount, &ctx->tileStart, &ctx->tileList, &ctx->binStage, &ctx->binStageCount,
                      &ctx->tileStage, &ctx->tileStageCount, &ctx->drawBlock};
    for (DevBuf* b : bufs) b->release();
    for (int i = 0; i < cr_context::kStageSlots; i++) {
        if (ctx->hostStage[i]) cudaFreeHost(ctx->hostStage[i]);
        if (ctx->stageDone[i]) cudaEventDestroy(ctx->stageDone[i]);
    }
    if (ctx->hostCounters) cudaFreeHost(ctx->hostCounters);
    for (int i = 0; i < 5; i++)
        if (ctx->ev[i]) cudaEventDestroy(ctx->ev[i]);
    delete ctx;
    return CR_OK;
}

cr_status cr_set_surfaces(cr_context* ctx, void* color, void* depth, int32_t width, int32_t height, int32_t num_samples) {
    if (!ctx) return CR_ERR_INVALID_ARGUMENT;
    if (!color && !depth) {
        ctx->surfacesSet = false;
        ctx->color = ctx->depth = nullptr;
        return CR_OK;
    }
    if (!color) return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaRaster: No color buffer specified!");
    if (!depth) return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaRaster: No depth buffer specified!");
    if (width <= 0 || height <= 0) return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaSurface: Size must be positive!");
    if (width > CR_MAX_VIEWPORT || height > CR_MAX_VIEWPORT)
        return fail(ctx, CR_ERR_CAPACITY, "CudaSurface: CR_MAXVIEWPORT_SIZE exceeded!");
    if (num_samples > 8) return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaSurface: numSamples cannot exceed 8!");
    if (num_samples < 1 || (num_samples & (num_samples - 1)))
        return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaSurface: numSamples must be a power of two!");
    if (((uintptr_t)color & 3) || ((uintptr_t)depth & 3))
        return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaRaster: surfaces must be 4-byte aligned!");
    ctx->color = color;
    ctx->depth = depth;
    ctx->width = width;
    ctx->height = height;
    ctx->numSamples = num_samples;
    ctx->samplesLog2 = ilog2(num_samples);
    ctx->surfacesSet = true;
    return CR_OK;
}

cr_status cr_deferred_clear(cr_context* ctx, float r, float g, float b, float a, float depth) {
    if (!ctx) return CR_ERR_INVALID_ARGUMENT;
    ctx->deferredClear = true;
    ctx->clearColor = cr_color_to_abgr(r, g, b, a);
    ctx->clearDepth = cr_clear_depth_from_float(depth);
    return CR_OK;
}

cr_status cr_deferred_clear_raw(cr_context* ctx, uint32_t abgr, uint32_t encoded_depth) {
    if (!ctx) return CR_ERR_INVALID_ARGUMENT;
    ctx->deferredClear = true;
    ctx->clearColor = abgr;
    ctx->clearDepth = encoded_depth;
    return CR_OK;
}

cr_status cr_set_pixel_pipe(cr_context* ctx, const char* name) {
    if (!ctx) return CR_ERR_INVALID_ARGUMENT;
    if (!name) {
        ctx->pipe = nullptr;
        return CR_OK;
    }
    const PipeDesc* p = findPipe(name);
    if (!p) return fail(ctx, CR_ERR_NO_PIPE, "CudaRaster: Invalid pixel pipe!");
    ctx->pipe = p;
    return CR_OK;
}

cr_status cr_set_vertex_buffer(cr_context* ctx, const void* vertices, int64_t offset_bytes) {
    if (!ctx) return CR_ERR_INVALID_ARGUMENT;
    if (!vertices) {
        ctx->vertexSet = false;
        ctx->vertices = nullptr;
        return CR_OK;
    }
    const char* p = (const char*)vertices + offset_bytes;
    if ((uintptr_t)p & 15) return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaRaster: vertex buffer must be 16-byte aligned!");
    ctx->vertices = p;
    ctx->vertexSet = true;
    return CR_OK;
}

cr_status cr_read_setup_output(cr_context* ctx, uint8_t* tri_subtris, uint32_t* tri_header, uint32_t* tri_data,
                               int64_t max_slots, int64_t* num_tris, int64_t* num_slots) {
    if (!ctx || !num_tris || !num_slots || max_slots < 0) return CR_ERR_INVALID_ARGUMENT;
    const int64_t t = ctx->last.num_tris, n = ctx->last.num_subtris;
    *num_tris = t;
    *num_slots = n;
    if (ctx->last.overflow) return fail(ctx, CR_ERR_INVALID_STATE, "CudaRaster: the last draw overflowed");
    if (n > max_slots) return fail(ctx, CR_ERR_CAPACITY, "CudaRaster: %lld setup slots do not fit", (long long)n);
    if (n == 0) return CR_OK;
    CR_CUDA(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    if (tri_subtris) CR_CUDA(cudaMemcpy(tri_subtris, ctx->triSubtris.ptr, (size_t)t, cudaMemcpyDeviceToHost), "cudaMemcpy");
    if (tri_header) CR_CUDA(cudaMemcpy(tri_header, ctx->triHeader.ptr, (size_t)n * 16, cudaMemcpyDeviceToHost), "cudaMemcpy");
    if (tri_data) CR_CUDA(cudaMemcpy(tri_data, ctx->triData.ptr, (size_t)n * 64, cudaMemcpyDeviceToHost), "cudaMemcpy");
    return CR_OK;
}

cr_status cr_read_queue_output(cr_context* ctx, int32_t* bin_start, int32_t* bin_count, uint32_t* bin_list,
                               int64_t max_bin_entries, int32_t* tile_start, int32_t* tile_count,
                               uint32_t* tile_list, int64_t max_tile_entries, int64_t* num_bin_entries,
                               int64_t* num_tile_entries) {
    if (!ctx || !num_bin_entries || !num_tile_entries || max_bin_entries < 0 || max_tile_entries < 0)
        return CR_ERR_INVALID_ARGUMENT;
    if (ctx->lastLayout.num_instances != 1)
        return fail(ctx, CR_ERR_INVALID_STATE, "CudaRaster: queue output is kept for single draws only");
    cr_counters c;
    cr_status st = cr_get_counters(ctx, &c);
    if (st != CR_OK) return st;
    *num_bin_entries = c.bin_entries;
    *num_tile_entries = c.tile_entries;
    if (c.overflow) return fail(ctx, CR_ERR_INVALID_STATE, "CudaRaster: the last draw overflowed");
    if ((bin_list && c.bin_entries > max_bin_entries) || (tile_list && c.tile_entries > max_tile_entries))
        return fail(ctx, CR_ERR_CAPACITY, "CudaRaster: %lld bin / %lld tile entries do not fit",
                    (long long)c.bin_entries, (long long)c.tile_entries);
    CR_CUDA(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    const size_t nb = (size_t)c.num_bins, nt = (size_t)c.num_tiles;
    if (bin_start) CR_CUDA(cudaMemcpy(bin_start, ctx->binStart.ptr, nb * 4, cudaMemcpyDeviceToHost), "cudaMemcpy");
    if (bin_count) CR_CUDA(cudaMemcpy(bin_count, ctx->binCount.ptr, nb * 4, cudaMemcpyDeviceToHost), "cudaMemcpy");
    if (tile_start) CR_CUDA(cudaMemcpy(tile_start, ctx->tileStart.ptr, nt * 4, cudaMemcpyDeviceToHost), "cudaMemcpy");
    if (tile_count) CR_CUDA(cudaMemcpy(tile_count, ctx->tileCount.ptr, nt * 4, cudaMemcpyDeviceToHost), "cudaMemcpy");
    if (bin_list && c.bin_entries > 0)
        CR_CUDA(cudaMemcpy(bin_list, ctx->binList.ptr, (size_t)c.bin_entries * 4, cudaMemcpyDeviceToHost), "cudaMemcpy");
    if (tile_list && c.tile_entries > 0)
        CR_CUDA(cudaMemcpy(tile_list, ctx->tileList.ptr, (size_t)c.tile_entries * 4, cudaMemcpyDeviceToHost),
                "cudaMemcpy");
    return CR_OK;
}

cr_status cr_set_vertex_transform(cr_context* ctx, const float* model, int32_t model_stride,
                                  const float* mvp_row_major) {
    if (!ctx) return CR_ERR_INVALID_ARGUMENT;
    if (!model) {
        ctx->model = nullptr;
        ctx->modelStride = 0;
        return CR_OK;
    }
    if (!mvp_row_major || model_stride < 3 || ((uintptr_t)model & 3))
        return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaRaster: bad vertex transform (model stride >= 3 floats, "
                                                  "4-byte aligned, 16 matrix entries)");
    ctx->model = model;
    ctx->modelStride = model_stride;
    memcpy(ctx->mvp, mvp_row_major, sizeof(ctx->mvp));
    return CR_OK;
}

cr_status cr_set_index_buffer(cr_context* ctx, const void* indices, int64_t offset_bytes, int32_t num_tris) {
    if (!ctx) return CR_ERR_INVALID_ARGUMENT;
    if (!indices) {
        ctx->indexSet = false;
        ctx->indices = nullptr;
        return CR_OK;
    }
    if (num_tris < 0 || num_tris > CR_MAX_TRIANGLES)
        return fail(ctx, CR_ERR_CAPACITY, "CudaRaster: CR_MAXSUBTRIS_SIZE exceeded!");
    const char* p = (const char*)indices + offset_bytes;
    if ((uintptr_t)p & 3) return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaRaster: index buffer must be 4-byte aligned!");
    ctx->indices = p;
    ctx->numTris = num_tris;
    ctx->indexSet = true;
    return CR_OK;
}

cr_status cr_set_tuning(cr_context* ctx, const cr_tuning* t) {
    if (!ctx) return CR_ERR_INVALID_ARGUMENT;
    if (!t) {
        ctx->tuning = cr_tuning{};
        return CR_OK;
    }
    if (t->bin_log2 > 0 && (t->bin_log2 < 3 || t->bin_log2 > 5))
        return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaRaster: bin_log2 must be 3, 4 or 5");
    if (t->fine_warps > 0 && (t->fine_warps > 8 || (t->fine_warps & (t->fine_warps - 1))))
        return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaRaster: fine_warps must be 1, 2, 4 or 8");
    if (t->fine_self_pixels < 0 || t->fine_self_pixels > 64)
        return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaRaster: fine_self_pixels must be in [0, 64]");
    if (t->bin_chunk_tris > 0 && (t->bin_chunk_tris % 32))
        return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaRaster: bin_chunk_tris must be a multiple of 32");
    ctx->tuning = *t;
    return CR_OK;
}

cr_status cr_set_debug_params(cr_context* ctx, const cr_debug_params* p) {
    if (!ctx) return CR_ERR_INVALID_ARGUMENT;
    if (p && (p->emulate_triangle_setup || p->emulate_bin_raster || p->emulate_coarse_raster || p->emulate_fine_raster))
        return fail(ctx, CR_ERR_UNSUPPORTED, "CudaRaster: host emulation of pipeline stages is not provided");
    return CR_OK;
}

cr_status cr_set_stage_timing(cr_context* ctx, int32_t enabled) {
    if (!ctx) return CR_ERR_INVALID_ARGUMENT;
    ctx->stageTiming = enabled != 0;
    return CR_OK;
}

cr_status cr_set_capacity(cr_context* ctx, int64_t ms, int64_t mb, int64_t mt) {
    if (!ctx) return CR_ERR_INVALID_ARGUMENT;
    if (ms < 0 || mb < 0 || mt < 0) return CR_ERR_INVALID_ARGUMENT;
    ctx->maxSubtris = ms;
    ctx->maxBinEntries = mb;
    ctx->maxTileEntries = mt;
    ctx->userCapacity = (ms | mb | mt) != 0;
    return CR_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ drawing
namespace {

// Prefix arrays staged behind the instance descriptors, numInstances + 1
// entries each: triangles (8 bytes), chunks, bins, tiles.
constexpr size_t kPrefixBytesPerInstance = 8 + 3 * 4;

struct Plan {
    std::vector<HostInstance> inst;
    std::vector<int32_t> chunkPrefix, binPrefix, tilePrefix;
    std::vector<int64_t> triPrefix;
    struct Group { const PipeDesc* pipe; int instBegin, instEnd; int64_t triBegin, triEnd; int32_t tileBegin, tileEnd; };
    std::vector<Group> groups;
    int64_t totalTris = 0, chunkCountEntries = 0;
    int32_t totalBins = 0, totalTiles = 0, totalChunks = 0, maxBins = 0, maxChunkTris = 0;
    int binLog2 = 4, unitEntries = 0;
    // Fused vertex transform (single draws only).
    const float* model = nullptr;
    int modelStride = 0;
    float mvp[16] = {};
};

// Coarse units a draw may use. A unit size set by the caller bounds them by
// the bin capacity; units sized on the device (unitEntries 0, at least 64
// entries each) are also capped at 8M per-unit tile counters, and the device
// grows the unit size until the draw's bin entries fit.
// Bin pairs a chunk may record for the scatter pass: twice its triangles (a
// chunk of small triangles makes about one bin entry per live triangle), at
// most 1024; chunks with more are walked again by the scatter pass.
int binStageCap(const Plan& plan) {
    const int cap = std::min(2 * plan.maxChunkTris, 1024);
    return (cap + 31) & ~31;
}

// Coarse units that record their tile pairs (units are sized on the device
// to about two per resident coarse warp), and the pairs each may record;
// later units and fuller ones are walked again by the coarse scatter pass.
constexpr int kTileStageUnits = 16384;
constexpr int kTileStageCap = 1024;

int64_t unitCapacity(int64_t maxBinEntries, int unitEntries, int32_t totalBins, int tpb) {
    if (unitEntries > 0) return maxBinEntries / unitEntries + totalBins + 1;
    return std::min<int64_t>(maxBinEntries / 64, std::max<int64_t>(4096, (8 << 20) / tpb)) + totalBins + 1;
}

cr_status buildPlan(cr_context* ctx, const std::vector<HostInstance>& in, Plan& plan) {
    plan.binLog2 = ctx->tuning.bin_log2 > 0 ? ctx->tuning.bin_log2 : 4;
    plan.unitEntries = std::max(0, ctx->tuning.coarse_unit_entries);   // 0: sized on the device
    // Group instances by pipe, keeping first-seen pipe order (outputs do not depend on it).
    std::vector<const PipeDesc*> order;
    for (const HostInstance& h : in)
        if (std::find(order.begin(), order.end(), h.pipe) == order.end()) order.push_back(h.pipe);
    for (const PipeDesc* p : order)
        for (const HostInstance& h : in)
            if (h.pipe == p) plan.inst.push_back(h);
    const int side = 1 << plan.binLog2;
    // Bin chunks are taken by warps, in order: about 80 per SM (two per
    // resident bin warp), of at most 65536 triangles and at least 256 (fewer,
    // down to 32, for draws under 128K triangles, whose chunks would
    // otherwise be too few to keep the warps busy), a multiple of 32.
    int64_t allTris = 0;
    for (const HostInstance& h : plan.inst) allTris += h.dev.numTris;
    const int64_t wantChunks = std::max<int64_t>(1, (int64_t)ctx->numSMs * 80);
    const int64_t floorChunk = std::min<int64_t>(256, std::max<int64_t>(32, allTris / 512));
    int64_t chunk = std::min<int64_t>(std::max<int64_t>((allTris + wantChunks - 1) / wantChunks, floorChunk), 65536);
    const int autoChunk = (int)((chunk + 31) & ~(int64_t)31);
    int64_t tri = 0;
    int32_t bins = 0, tiles = 0, chunks = 0;
    int64_t countBase = 0;
    for (size_t i = 0; i < plan.inst.size(); i++) {
        InstanceDev& d = plan.inst[i].dev;
        d.widthTiles = (d.width + 7) >> 3;
        d.heightTiles = (d.height + 7) >> 3;
        d.widthBins = (d.widthTiles + side - 1) / side;
        d.heightBins = (d.heightTiles + side - 1) / side;
        int nb = d.widthBins * d.heightBins;
        if (nb > 1024)
            return fail(ctx, CR_ERR_CAPACITY, "CudaRaster: %d bins exceed 1024; use a larger bin_log2", nb);
        plan.maxBins = std::max(plan.maxBins, nb);
        d.rowWords = (int64_t)(d.widthTiles * 8) << d.samplesLog2;
        d.triBase = tri;
        d.binBase = bins;
        d.tileBase = tiles;
        int chunkTris = ctx->tuning.bin_chunk_tris;
        if (chunkTris <= 0) chunkTris = autoChunk;
        d.chunkTris = chunkTris;
        d.numChunks = (d.numTris + chunkTris - 1) / chunkTris;
        plan.maxChunkTris = std::max(plan.maxChunkTris, chunkTris);
        d.chunkBase = chunks;
        d.chunkCountBase = countBase;
        countBase += (int64_t)d.numChunks * nb;
        tri += d.numTris;
        bins += nb;
        tiles += d.widthTiles * d.heightTiles;
        chunks += d.numChunks;
        if (tri > CR_MAX_TRIANGLES) return fail(ctx, CR_ERR_CAPACITY, "CudaRaster: CR_MAXSUBTRIS_SIZE exceeded!");
    }
    plan.totalTris = tri;
    plan.totalBins = bins;
    plan.totalTiles = tiles;
    plan.totalChunks = chunks;
    plan.chunkCountEntries = countBase;
    for (const HostInstance& h : plan.inst) {
        plan.chunkPrefix.push_back(h.dev.chunkBase);
        plan.binPrefix.push_back(h.dev.binBase);
        plan.tilePrefix.push_back(h.dev.tileBase);
        plan.triPrefix.push_back(h.dev.triBase);
    }
    plan.chunkPrefix.push_back(chunks);
    plan.binPrefix.push_back(bins);
    plan.tilePrefix.push_back(tiles);
    plan.triPrefix.push_back(tri);
    for (size_t i = 0; i < plan.inst.size();) {
        size_t j = i;
        while (j < plan.inst.size() && plan.inst[j].pipe == plan.inst[i].pipe) j++;
        Plan::Group g;
        g.pipe = plan.inst[i].pipe;
        g.instBegin = (int)i;
        g.instEnd = (int)j;
        g.triBegin = plan.inst[i].dev.triBase;
        g.triEnd = (j < plan.inst.size()) ? plan.inst[j].dev.triBase : tri;
        g.tileBegin = plan.inst[i].dev.tileBase;
        g.tileEnd = (j < plan.inst.size()) ? plan.inst[j].dev.tileBase : tiles;
        for (size_t k = i; k < j; k++) plan.inst[k].dev.pipeGroup = (int)plan.groups.size();
        plan.groups.push_back(g);
        i = j;
    }
    return CR_OK;
}

// Bytes of the per-draw block: the counters (256-byte aligned), then the
// instance descriptors and the prefix arrays.
size_t counterBytes(const Plan& plan) {
    return (sizeof(Counters) + sizeof(int32_t) * std::max<size_t>(plan.groups.size(), 1) + 255) & ~(size_t)255;
}
size_t drawBlockBytes(const Plan& plan) {
    return counterBytes(plan) + sizeof(InstanceDev) * plan.inst.size() +
           kPrefixBytesPerInstance * (plan.inst.size() + 1) + 64;
}

cr_status ensureCapacity(cr_context* ctx, const Plan& plan) {
    int64_t T = plan.totalTris;
    // Initial sizes in the spirit of CudaRaster.cpp:263-275 (subtriangle
    // slack 4096; queues scaled with the triangle count), grown on overflow.
    if (ctx->userCapacity) {
        // Capacities chosen by the caller (e.g. a predictor): only the
        // triangle slots themselves are guaranteed.
        ctx->maxSubtris = std::max<int64_t>(ctx->maxSubtris, T);
        ctx->maxBinEntries = std::max<int64_t>(ctx->maxBinEntries, 1);
        ctx->maxTileEntries = std::max<int64_t>(ctx->maxTileEntries, 1);
    } else {
        ctx->maxSubtris = std::max<int64_t>(ctx->maxSubtris, T + 4096);
        ctx->maxBinEntries = std::max<int64_t>(ctx->maxBinEntries, 2 * T + 65536);
        ctx->maxTileEntries = std::max<int64_t>(ctx->maxTileEntries, 4 * T + 65536);
    }
    const int tpb = 1 << (2 * plan.binLog2);
    const int64_t maxUnits = unitCapacity(ctx->maxBinEntries, plan.unitEntries, plan.totalBins, tpb);
    CR_CUDA(ctx->triSubtris.ensure((size_t)std::max<int64_t>(T, 1)), "cudaMalloc");
    CR_CUDA(ctx->triHeader.ensure((size_t)ctx->maxSubtris * 16), "cudaMalloc");
    CR_CUDA(ctx->triData.ensure((size_t)ctx->maxSubtris * 64), "cudaMalloc");
    CR_CUDA(ctx->chunkBinCount.ensureZeroed((size_t)std::max<int64_t>(plan.chunkCountEntries, 1) * 4), "cudaMalloc");
    CR_CUDA(ctx->chunkBinOffset.ensure((size_t)std::max<int64_t>(plan.chunkCountEntries, 1) * 4), "cudaMalloc");
    CR_CUDA(ctx->binCount.ensure((size_t)plan.totalBins * 4), "cudaMalloc");
    CR_CUDA(ctx->binStart.ensure((size_t)plan.totalBins * 4), "cudaMalloc");
    CR_CUDA(ctx->binUnitFirst.ensure((size_t)plan.totalBins * 4), "cudaMalloc");
    CR_CUDA(ctx->binList.ensure((size_t)ctx->maxBinEntries * 4), "cudaMalloc");
    CR_CUDA(ctx->unitTileCount.ensure((size_t)maxUnits * tpb * 4), "cudaMalloc");
    CR_CUDA(ctx->tileCount.ensure((size_t)plan.totalTiles * 4), "cudaMalloc");
    CR_CUDA(ctx->tileStart.ensure((size_t)plan.totalTiles * 4), "cudaMalloc");
    CR_CUDA(ctx->tileList.ensure((size_t)ctx->maxTileEntries * 4), "cudaMalloc");
    const int stageCap = binStageCap(plan);
    CR_CUDA(ctx->binStage.ensure((size_t)std::max(plan.totalChunks, 1) * stageCap * 8), "cudaMalloc");
    CR_CUDA(ctx->binStageCount.ensure((size_t)std::max(plan.totalChunks, 1) * 4), "cudaMalloc");
    const int64_t stageUnits = std::min<int64_t>(maxUnits, kTileStageUnits);
    CR_CUDA(ctx->tileStage.ensure((size_t)stageUnits * kTileStageCap * 8), "cudaMalloc");
    CR_CUDA(ctx->tileStageCount.ensure((size_t)stageUnits * 4), "cudaMalloc");
    const size_t stage = drawBlockBytes(plan);
    CR_CUDA(ctx->drawBlock.ensure(stage), "cudaMalloc");
    if (stage > ctx->hostStageBytes) {
        for (int i = 0; i < cr_context::kStageSlots; i++) {
            if (ctx->stageUsed[i]) CR_CUDA(cudaEventSynchronize(ctx->stageDone[i]), "cudaEventSynchronize");
            ctx->stageUsed[i] = false;
            if (ctx->hostStage[i]) cudaFreeHost(ctx->hostStage[i]);
            ctx->hostStage[i] = nullptr;
        }
        ctx->hostStageBytes = 0;
        for (int i = 0; i < cr_context::kStageSlots; i++) {
            CR_CUDA(cudaMallocHost(&ctx->hostStage[i], stage * 2), "cudaMallocHost");
            if (!ctx->stageDone[i])
                CR_CUDA(cudaEventCreateWithFlags(&ctx->stageDone[i], cudaEventDisableTiming), "cudaEventCreate");
        }
        ctx->hostStageBytes = stage * 2;
    }
    return CR_OK;
}

DrawDev makeDrawDev(cr_context* ctx, const Plan& plan) {
    DrawDev d{};
    const size_t cb = counterBytes(plan);
    d.inst = (const InstanceDev*)(ctx->drawBlock.as<char>() + cb);
    d.numInstances = (int)plan.inst.size();
    d.binLog2 = plan.binLog2;
    d.totalBins = plan.totalBins;
    d.totalTiles = plan.totalTiles;
    d.totalChunks = plan.totalChunks;
    d.unitEntries = plan.unitEntries;
    d.totalTris = plan.totalTris;
    d.model = plan.model;
    d.modelStride = plan.modelStride;
    d.modelVec4 = plan.model && plan.modelStride == 4 && ((uintptr_t)plan.model & 15) == 0;
    memcpy(d.mvp, plan.mvp, sizeof(d.mvp));
    d.triSubtris = ctx->triSubtris.as<uint8_t>();
    d.triHeader = ctx->triHeader.as<uint4>();
    d.triData = ctx->triData.as<uint4>();
    d.maxSubtris = ctx->maxSubtris;
    d.chunkBinCount = ctx->chunkBinCount.as<int32_t>();
    d.chunkBinOffset = ctx->chunkBinOffset.as<int32_t>();
    d.maxBins = plan.maxBins;
    d.fineSelfPixels = ctx->tuning.fine_self_pixels;
    d.binCount = ctx->binCount.as<int32_t>();
    d.binStart = ctx->binStart.as<int32_t>();
    d.binUnitFirst = ctx->binUnitFirst.as<int32_t>();
    d.binList = ctx->binList.as<uint32_t>();
    d.maxBinEntries = ctx->maxBinEntries;
    d.unitTileCount = ctx->unitTileCount.as<int32_t>();
    d.maxUnits = unitCapacity(ctx->maxBinEntries, plan.unitEntries, plan.totalBins, 1 << (2 * plan.binLog2));
    d.tileCount = ctx->tileCount.as<int32_t>();
    d.tileStart = ctx->tileStart.as<int32_t>();
    d.tileList = ctx->tileList.as<uint32_t>();
    d.maxTileEntries = ctx->maxTileEntries;
    char* pref = ctx->drawBlock.as<char>() + cb + sizeof(InstanceDev) * plan.inst.size();
    size_t n1 = plan.inst.size() + 1;
    d.triPrefix = (const int64_t*)pref;
    d.chunkPrefix = (const int32_t*)(pref + 8 * n1);
    d.binPrefix = d.chunkPrefix + n1;
    d.tilePrefix = d.binPrefix + n1;
    d.counters = ctx->drawBlock.as<Counters>();
    d.fineTileCounter = (int32_t*)(ctx->drawBlock.as<char>() + sizeof(Counters));
    d.binStage = ctx->binStage.as<U64>();
    d.binStageCount = ctx->binStageCount.as<int32_t>();
    d.binStageCap = binStageCap(plan);
    d.tileStage = ctx->tileStage.as<U64>();
    d.tileStageCount = ctx->tileStageCount.as<int32_t>();
    d.tileStageCap = kTileStageCap;
    d.tileStageUnits = (int32_t)std::min<int64_t>(d.maxUnits, kTileStageUnits);
    return d;
}

static_assert(sizeof(InstanceDev) % 8 == 0, "the prefix arrays follow the descriptors with 8-byte alignment");
static_assert(offsetof(Counters, coarseWork) == 6 * sizeof(int32_t) && sizeof(Counters) >= 8 * sizeof(int32_t),
              "cr_queue_counts exports the first 8 words of Counters");

// A draw's block (zeroed counters, instance descriptors, prefix arrays) as a
// kernel parameter: one CTA writes it to the device. Unlike a host-to-device
// copy it lets the setup kernels, launched as programmatic dependents, be
// scheduled behind it (they wait for it before their first access). It needs
// an SM slot, though: a queued draw whose stream runs beside another stream's
// persistent fine kernel would wait for that kernel, where a copy would not,
// so only blocking draws use it.
template <int N>
struct BlockWords {
    uint32_t w[N];
};
template <int N>
__global__ void __launch_bounds__(256) writeBlockKernel(const __grid_constant__ BlockWords<N> b, uint32_t* dst, int n) {
    pdlTrigger();
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = b.w[i];
}
template <int N>
cudaError_t writeBlock(const void* src, void* dst, size_t bytes, cudaStream_t stream) {
    BlockWords<N> b;
    memcpy(b.w, src, bytes);
    return launchKernel(writeBlockKernel<N>, 1, 256, 0, stream, false, b, (uint32_t*)dst, (int)(bytes / 4));
}

bool capturing(cudaStream_t s) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &st) != cudaSuccess) {
        cudaGetLastError();
        return true;
    }
    return st != cudaStreamCaptureStatusNone;
}

// Enqueues one draw of `plan` on `stream`. `stage` is pinned host memory for
// the descriptors (the copy node reads it when a captured graph replays;
// with `writeKernel` a blocking draw's block goes as a kernel parameter) and
// `hostCounters` (pinned) receives the device counters, written by the first
// fine launch or copied after the draw; with `events` false no stage
// events are recorded (graph capture).
cr_status launchDrawWith(cr_context* ctx, const Plan& plan, cudaStream_t stream, void* stage, Counters* hostCounters,
                         bool events, bool writeKernel) {
    DrawDev d = makeDrawDev(ctx, plan);
    // Stage the zeroed counters and the descriptors through pinned memory;
    // for a blocking draw a kernel parameter carries them to the device, else
    // (and for blocks above 8 KB) a copy; in a graph capture the copy node
    // reads the stage at every replay.
    size_t n1 = plan.inst.size() + 1;
    size_t instBytes = sizeof(InstanceDev) * plan.inst.size();
    const size_t cb = counterBytes(plan);
    memset(stage, 0, cb);
    char* hs = (char*)stage + cb;
    for (size_t i = 0; i < plan.inst.size(); i++) memcpy(hs + i * sizeof(InstanceDev), &plan.inst[i].dev, sizeof(InstanceDev));
    char* hp = hs + instBytes;
    memcpy(hp, plan.triPrefix.data(), 8 * n1);
    memcpy(hp + 8 * n1, plan.chunkPrefix.data(), 4 * n1);
    memcpy(hp + 12 * n1, plan.binPrefix.data(), 4 * n1);
    memcpy(hp + 16 * n1, plan.tilePrefix.data(), 4 * n1);
    const size_t blockBytes = cb + instBytes + kPrefixBytesPerInstance * n1;
    writeKernel = writeKernel && !capturing(stream);
    if (writeKernel && blockBytes <= 1024)
        CR_CUDA(writeBlock<256>(stage, ctx->drawBlock.ptr, blockBytes, stream), "block write");
    else if (writeKernel && blockBytes <= 8192)
        CR_CUDA(writeBlock<2048>(stage, ctx->drawBlock.ptr, blockBytes, stream), "block write");
    else
        CR_CUDA(cudaMemcpyAsync(ctx->drawBlock.ptr, stage, blockBytes, cudaMemcpyHostToDevice, stream),
                "cudaMemcpyAsync");

    if (events) CR_CUDA(cudaEventRecord(ctx->ev[0], stream), "cudaEventRecord");
    for (const Plan::Group& g : plan.groups)
        CR_CUDA(g.pipe->launchSetup(d, g.instBegin, g.instEnd, g.triBegin, g.triEnd, stream), "setup launch");
    if (events) CR_CUDA(cudaEventRecord(ctx->ev[1], stream), "cudaEventRecord");
    CR_CUDA(launchBinning(d, plan.maxBins, ctx->numSMs, stream, events ? ctx->ev[2] : nullptr), "bin/coarse launch");
    if (events) CR_CUDA(cudaEventRecord(ctx->ev[3], stream), "cudaEventRecord");
    // The first fine launch that has tiles writes the counters into the
    // pinned host buffer (its device address); without one, a copy follows.
    Counters* devHostCounters = nullptr;
    if (cudaHostGetDevicePointer((void**)&devHostCounters, hostCounters, 0) != cudaSuccess) {
        cudaGetLastError();
        devHostCounters = nullptr;
    }
    bool written = false;
    int warps = ctx->tuning.fine_warps > 0 ? ctx->tuning.fine_warps : 8;
    for (size_t gi = 0; gi < plan.groups.size(); gi++) {
        const Plan::Group& g = plan.groups[gi];
        int ctas = ctx->tuning.fine_ctas_per_sm > 0 ? ctx->tuning.fine_ctas_per_sm : g.pipe->fineOccupancy(warps);
        DrawDev dg = d;
        if (!written && devHostCounters && g.tileEnd > g.tileBegin) {
            dg.hostCounters = devHostCounters;
            written = true;
        }
        CR_CUDA(g.pipe->launchFine(dg, (int)gi, g.tileBegin, g.tileEnd, warps, ctas, ctx->numSMs, stream), "fine launch");
    }
    if (events) CR_CUDA(cudaEventRecord(ctx->ev[4], stream), "cudaEventRecord");
    ctx->eventsRecorded = events;
    if (!written)
        CR_CUDA(cudaMemcpyAsync(hostCounters, ctx->drawBlock.ptr, sizeof(Counters), cudaMemcpyDeviceToHost, stream),
                "cudaMemcpyAsync");
    return CR_OK;
}

cr_status launchDraw(cr_context* ctx, const Plan& plan, cudaStream_t stream, bool sync) {
    const int slot = ctx->stageNext;
    ctx->stageNext = (slot + 1) % cr_context::kStageSlots;
    if (ctx->stageUsed[slot]) CR_CUDA(cudaEventSynchronize(ctx->stageDone[slot]), "cudaEventSynchronize");
    cr_status st = launchDrawWith(ctx, plan, stream, ctx->hostStage[slot], ctx->hostCounters, ctx->stageTiming, sync);
    if (st != CR_OK) return st;
    ctx->drawn = true;
    CR_CUDA(cudaEventRecord(ctx->stageDone[slot], stream), "cudaEventRecord");
    ctx->stageUsed[slot] = true;
    return CR_OK;
}

void recordCounters(cr_context* ctx, const Plan& plan, int reruns) {
    const Counters& c = *ctx->hostCounters;
    ctx->last.num_tris = plan.totalTris;
    ctx->last.num_subtris = plan.totalTris + c.extraSubtris;
    ctx->last.bin_entries = c.binEntries;
    ctx->last.tile_entries = c.tileEntries;
    ctx->last.coarse_units = c.numUnits;
    ctx->last.max_subtris = ctx->maxSubtris;
    ctx->last.max_bin_entries = ctx->maxBinEntries;
    ctx->last.max_tile_entries = ctx->maxTileEntries;
    ctx->last.reruns = reruns;
    ctx->last.overflow = c.overflow;
    ctx->last.num_bins = plan.totalBins;
    ctx->last.num_tiles = plan.totalTiles;
}

// Overflow-detect-and-rerun (CudaRaster.cpp:277-339).
cr_status drawPlan(cr_context* ctx, const Plan& plan, cudaStream_t stream, bool sync) {
    cr_status st = ensureCapacity(ctx, plan);
    if (st != CR_OK) return st;
    const InstanceDev& first = plan.inst[0].dev;
    ctx->lastLayout = cr_queue_layout{first.widthBins, first.heightBins, first.widthTiles, first.heightTiles,
                                      plan.binLog2, plan.totalBins, plan.totalTiles, (int32_t)plan.inst.size()};
    ctx->last.num_bins = plan.totalBins;
    ctx->last.num_tiles = plan.totalTiles;
    for (int reruns = 0;; reruns++) {
        st = launchDraw(ctx, plan, stream, sync);
        if (st != CR_OK) return st;
        if (!sync) {
            ctx->last.reruns = 0;
            return CR_OK;
        }
        CR_CUDA(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
        recordCounters(ctx, plan, reruns);
        const Counters& c = *ctx->hostCounters;
        if (!c.overflow) return CR_OK;
        if (reruns >= 16) return fail(ctx, CR_ERR_CAPACITY, "CudaRaster: queues keep overflowing");
        int64_t subtris = plan.totalTris + c.extraSubtris;
        if (c.overflow & kOverflowSubtris) ctx->maxSubtris = std::max(ctx->maxSubtris, subtris + 4096);
        if (c.overflow & kOverflowBin) ctx->maxBinEntries = std::max<int64_t>(ctx->maxBinEntries, (int64_t)c.binEntries + 65536);
        if (c.overflow & kOverflowTile) ctx->maxTileEntries = std::max<int64_t>(ctx->maxTileEntries, (int64_t)c.tileEntries + 65536);
        if (ctx->maxSubtris > (int64_t)CR_MAX_TRIANGLES)
            return fail(ctx, CR_ERR_CAPACITY, "CudaRaster: CR_MAXSUBTRIS_SIZE exceeded!");
        st = ensureCapacity(ctx, plan);
        if (st != CR_OK) return st;
    }
}

cr_status drawCurrent(cr_context* ctx, void* stream, bool sync) {
    if (!ctx) return CR_ERR_INVALID_ARGUMENT;
    if (!ctx->surfacesSet) return fail(ctx, CR_ERR_INVALID_STATE, "CudaRaster: Surfaces not set!");
    if (!ctx->pipe) return fail(ctx, CR_ERR_INVALID_STATE, "CudaRaster: Pixel pipe not set!");
    if (!ctx->vertexSet) return fail(ctx, CR_ERR_INVALID_STATE, "CudaRaster: Vertex buffer not set!");
    if (!ctx->indexSet) return fail(ctx, CR_ERR_INVALID_STATE, "CudaRaster: Index buffer not set!");
    if (ctx->pipe->samplesLog2 != ctx->samplesLog2)
        return fail(ctx, CR_ERR_PIPE_MISMATCH, "CudaRaster: Mismatch in multisampling between pixel pipe and surface!");
    HostInstance h;
    memset(&h.dev, 0, sizeof(h.dev));
    h.pipe = ctx->pipe;
    h.dev.vertices = (const float4*)ctx->vertices;
    h.dev.indices = (const int*)ctx->indices;
    h.dev.color = (uint32_t*)ctx->color;
    h.dev.depth = (uint32_t*)ctx->depth;
    h.dev.stride4 = ctx->pipe->vertexStructSize / 16;
    h.dev.numTris = ctx->numTris;
    h.dev.width = ctx->width;
    h.dev.height = ctx->height;
    h.dev.samplesLog2 = ctx->samplesLog2;
    h.dev.deferredClear = ctx->deferredClear ? 1 : 0;
    h.dev.clearColor = ctx->clearColor;
    h.dev.clearDepth = ctx->clearDepth;
    Plan plan;
    std::vector<HostInstance> v{h};
    cr_status st = buildPlan(ctx, v, plan);
    if (st != CR_OK) return st;
    if (ctx->model) {
        plan.model = ctx->model;
        plan.modelStride = ctx->modelStride;
        memcpy(plan.mvp, ctx->mvp, sizeof(plan.mvp));
    }
    st = drawPlan(ctx, plan, (cudaStream_t)stream, sync);
    if (st == CR_OK) ctx->deferredClear = false;  // CudaRaster.cpp:341
    return st;
}

cr_status batchInstances(cr_context* ctx, const cr_instance* instances, int32_t count, std::vector<HostInstance>& v) {
    if (!ctx || (!instances && count > 0) || count < 0) return CR_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < count; i++) {
        const cr_instance& s = instances[i];
        const PipeDesc* p = s.pipe ? findPipe(s.pipe) : nullptr;
        if (!p) return fail(ctx, CR_ERR_NO_PIPE, "CudaRaster: Invalid pixel pipe! (instance %d)", i);
        if (!s.color || !s.depth) return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaRaster: instance %d has no surfaces", i);
        if (s.width <= 0 || s.height <= 0 || s.width > CR_MAX_VIEWPORT || s.height > CR_MAX_VIEWPORT)
            return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaSurface: bad size in instance %d", i);
        int ns = s.num_samples;
        if (ns < 1 || ns > 8 || (ns & (ns - 1))) return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaSurface: bad sample count in instance %d", i);
        if (p->samplesLog2 != ilog2(ns))
            return fail(ctx, CR_ERR_PIPE_MISMATCH, "CudaRaster: Mismatch in multisampling between pixel pipe and surface! (instance %d)", i);
        if (s.num_tris < 0 || (s.num_tris > 0 && (!s.vertices || !s.indices)))
            return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaRaster: instance %d has no geometry", i);
        if (((uintptr_t)s.vertices & 15) || ((uintptr_t)s.indices & 3))
            return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaRaster: misaligned buffers in instance %d", i);
        HostInstance h;
        memset(&h.dev, 0, sizeof(h.dev));
        h.pipe = p;
        h.dev.vertices = (const float4*)s.vertices;
        h.dev.indices = (const int*)s.indices;
        h.dev.color = (uint32_t*)s.color;
        h.dev.depth = (uint32_t*)s.depth;
        h.dev.stride4 = p->vertexStructSize / 16;
        h.dev.numTris = s.num_tris;
        h.dev.width = s.width;
        h.dev.height = s.height;
        h.dev.samplesLog2 = ilog2(ns);
        h.dev.deferredClear = s.deferred_clear ? 1 : 0;
        h.dev.clearColor = s.clear_color;
        h.dev.clearDepth = s.clear_depth;
        v.push_back(h);
    }
    return CR_OK;
}

cr_status drawBatch(cr_context* ctx, const cr_instance* instances, int32_t count, void* stream, bool sync) {
    std::vector<HostInstance> v;
    cr_status st = batchInstances(ctx, instances, count, v);
    if (st != CR_OK || v.empty()) return st;
    Plan plan;
    st = buildPlan(ctx, v, plan);
    if (st != CR_OK) return st;
    return drawPlan(ctx, plan, (cudaStream_t)stream, sync);
}

}  // namespace

// A batched draw captured once into a CUDA graph and replayed per frame
// (the descriptor copy with the counter resets and every kernel are graph
// nodes; the first fine kernel writes the counters into pinned host memory). Overflow cannot rerun inside a graph: the kernels skip the
// frame and raise a flag, and cr_batch_graph_counters reports it so the host
// grows the queues and recaptures.
struct cr_batch_graph {
    cr_context* ctx = nullptr;
    Plan plan;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    void* stage = nullptr;
    Counters* counters = nullptr;
};

extern "C" {

cr_status cr_draw_triangles(cr_context* ctx, void* stream) { return drawCurrent(ctx, stream, true); }

cr_status cr_batch_graph_create(cr_context* ctx, const cr_instance* instances, int32_t count, void* stream,
                                cr_batch_graph** out) {
    if (!ctx || !out) return CR_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    std::vector<HostInstance> v;
    cr_status st = batchInstances(ctx, instances, count, v);
    if (st != CR_OK) return st;
    if (v.empty()) return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaRaster: empty batch");
    cr_batch_graph* g = new cr_batch_graph();
    g->ctx = ctx;
    st = buildPlan(ctx, v, g->plan);
    if (st == CR_OK) st = ensureCapacity(ctx, g->plan);
    if (st != CR_OK) { delete g; return st; }
    size_t stageBytes = drawBlockBytes(g->plan);
    cudaError_t e = cudaMallocHost(&g->stage, stageBytes);
    if (e == cudaSuccess) e = cudaMallocHost(&g->counters, sizeof(Counters));
    if (e != cudaSuccess) {
        if (g->stage) cudaFreeHost(g->stage);
        delete g;
        return cudaFail(ctx, e, "cudaMallocHost");
    }
    memset(g->counters, 0, sizeof(Counters));
    // Capture on a private stream ordered after `stream`.
    cudaStream_t cap;
    e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) { cr_batch_graph_destroy(g); return cudaFail(ctx, e, "cudaStreamCreate"); }
    cudaStreamSynchronize((cudaStream_t)stream);
    e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        st = launchDrawWith(ctx, g->plan, cap, g->stage, g->counters, false, false);
        cudaError_t e2 = cudaStreamEndCapture(cap, &g->graph);
        if (st == CR_OK && e2 != cudaSuccess) st = cudaFail(ctx, e2, "cudaStreamEndCapture");
    } else {
        st = cudaFail(ctx, e, "cudaStreamBeginCapture");
    }
    cudaStreamDestroy(cap);
    if (st == CR_OK) {
        e = cudaGraphInstantiate(&g->exec, g->graph, 0);
        if (e != cudaSuccess) st = cudaFail(ctx, e, "cudaGraphInstantiate");
    }
    if (st != CR_OK) { cr_batch_graph_destroy(g); return st; }
    *out = g;
    return CR_OK;
}

cr_status cr_batch_graph_launch(cr_batch_graph* g, void* stream) {
    if (!g) return CR_ERR_INVALID_ARGUMENT;
    cudaError_t e = cudaGraphLaunch(g->exec, (cudaStream_t)stream);
    if (e != cudaSuccess) return cudaFail(g->ctx, e, "cudaGraphLaunch");
    return CR_OK;
}

cr_status cr_batch_graph_counters(cr_batch_graph* g, void* stream, cr_counters* out) {
    if (!g || !out) return CR_ERR_INVALID_ARGUMENT;
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cudaFail(g->ctx, e, "cudaStreamSynchronize");
    const Counters& c = *g->counters;
    memset(out, 0, sizeof(*out));
    out->num_tris = g->plan.totalTris;
    out->num_subtris = g->plan.totalTris + c.extraSubtris;
    out->bin_entries = c.binEntries;
    out->tile_entries = c.tileEntries;
    out->coarse_units = c.numUnits;
    out->max_subtris = g->ctx->maxSubtris;
    out->max_bin_entries = g->ctx->maxBinEntries;
    out->max_tile_entries = g->ctx->maxTileEntries;
    out->overflow = c.overflow;
    out->num_bins = g->plan.totalBins;
    out->num_tiles = g->plan.totalTiles;
    return CR_OK;
}

cr_status cr_batch_graph_destroy(cr_batch_graph* g) {
    if (!g) return CR_ERR_INVALID_ARGUMENT;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    if (g->stage) cudaFreeHost(g->stage);
    if (g->counters) cudaFreeHost(g->counters);
    delete g;
    return CR_OK;
}
cr_status cr_draw_triangles_async(cr_context* ctx, void* stream) { return drawCurrent(ctx, stream, false); }
cr_status cr_draw_batch(cr_context* ctx, const cr_instance* inst, int32_t n, void* stream) {
    return drawBatch(ctx, inst, n, stream, true);
}
cr_status cr_draw_batch_async(cr_context* ctx, const cr_instance* inst, int32_t n, void* stream) {
    return drawBatch(ctx, inst, n, stream, false);
}

cr_status cr_get_stats(cr_context* ctx, cr_stats* out) {
    if (!ctx || !out) return CR_ERR_INVALID_ARGUMENT;
    memset(out, 0, sizeof(*out));
    if (!ctx->eventsRecorded) return CR_OK;
    CR_CUDA(cudaEventSynchronize(ctx->ev[4]), "cudaEventSynchronize");
    float t[4] = {0, 0, 0, 0};
    for (int i = 0; i < 4; i++) cudaEventElapsedTime(&t[i], ctx->ev[i], ctx->ev[i + 1]);
    out->setup_time = t[0] * 1e-3f;
    out->bin_time = t[1] * 1e-3f;
    out->coarse_time = t[2] * 1e-3f;
    out->fine_time = t[3] * 1e-3f;
    return CR_OK;
}

cr_status cr_get_queue_layout(cr_context* ctx, cr_queue_layout* out) {
    if (!ctx || !out) return CR_ERR_INVALID_ARGUMENT;
    *out = ctx->lastLayout;
    return CR_OK;
}

cr_status cr_get_queue_buffers(cr_context* ctx, const int32_t** bin_counts, const int32_t** tile_counts,
                               const int32_t** counters) {
    if (!ctx || !bin_counts || !tile_counts || !counters) return CR_ERR_INVALID_ARGUMENT;
    if (ctx->lastLayout.num_bins == 0) return fail(ctx, CR_ERR_INVALID_STATE, "CudaRaster: no draw to take queue counts from");
    *bin_counts = ctx->binCount.as<int32_t>();
    *tile_counts = ctx->tileCount.as<int32_t>();
    *counters = ctx->drawBlock.as<int32_t>();
    return CR_OK;
}

cr_status cr_queue_counts(cr_context* ctx, int32_t* bin_counts, int32_t num_bins, int32_t* tile_counts,
                          int32_t num_tiles, int32_t* counters, void* stream) {
    if (!ctx) return CR_ERR_INVALID_ARGUMENT;
    const cr_queue_layout& l = ctx->lastLayout;
    if (l.num_bins == 0) return fail(ctx, CR_ERR_INVALID_STATE, "CudaRaster: no draw to take queue counts from");
    if ((bin_counts && num_bins != l.num_bins) || (tile_counts && num_tiles != l.num_tiles))
        return fail(ctx, CR_ERR_INVALID_ARGUMENT, "CudaRaster: queue count sizes %d/%d, last draw has %d bins, %d tiles",
                    num_bins, num_tiles, l.num_bins, l.num_tiles);
    cudaStream_t s = (cudaStream_t)stream;
    if (bin_counts)
        CR_CUDA(cudaMemcpyAsync(bin_counts, ctx->binCount.ptr, (size_t)num_bins * 4, cudaMemcpyDeviceToDevice, s),
                "cudaMemcpyAsync");
    if (tile_counts)
        CR_CUDA(cudaMemcpyAsync(tile_counts, ctx->tileCount.ptr, (size_t)num_tiles * 4, cudaMemcpyDeviceToDevice, s),
                "cudaMemcpyAsync");
    if (counters)   // the 8 counters the header documents (the first 8 words of Counters), no more
        CR_CUDA(cudaMemcpyAsync(counters, ctx->drawBlock.ptr, 8 * sizeof(int32_t), cudaMemcpyDeviceToDevice, s),
                "cudaMemcpyAsync");
    return CR_OK;
}

cr_status cr_get_counters(cr_context* ctx, cr_counters* out) {
    if (!ctx || !out) return CR_ERR_INVALID_ARGUMENT;
    if (ctx->drawn) {
        // The last draw's counters copy is enqueued on its stream.
        CR_CUDA(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
        const Counters& c = *ctx->hostCounters;
        ctx->last.num_subtris = ctx->last.num_tris + c.extraSubtris;
        ctx->last.bin_entries = c.binEntries;
        ctx->last.tile_entries = c.tileEntries;
        ctx->last.coarse_units = c.numUnits;
        ctx->last.overflow = c.overflow;
    }
    *out = ctx->last;
    return CR_OK;
}

cr_status cr_get_profiling_info(cr_context* ctx, char* buffer, int64_t size) {
    if (!ctx || !buffer || size <= 0) return CR_ERR_INVALID_ARGUMENT;
    cr_stats s;
    cr_status st = cr_get_stats(ctx, &s);
    if (st != CR_OK) return st;
    cr_counters c{};
    cr_get_counters(ctx, &c);
    // Format follows getProfilingInfo's default mode (CudaRaster.cpp:367-421):
    // stage times, then the memory footprint of the intermediate queues.
    double mb = 1.0 / (1024.0 * 1024.0);
    snprintf(buffer, (size_t)size,
             "Setup  %8.3f ms\nBin    %8.3f ms\nCoarse %8.3f ms\nFine   %8.3f ms\nTotal  %8.3f ms\n"
             "Triangles     %lld\nSubtriangles  %lld (%.1f MB)\nBin entries   %lld (%.1f MB)\n"
             "Tile entries  %lld (%.1f MB)\nCoarse units  %lld\nReruns        %d\n",
             s.setup_time * 1e3, s.bin_time * 1e3, s.coarse_time * 1e3, s.fine_time * 1e3,
             (s.setup_time + s.bin_time + s.coarse_time + s.fine_time) * 1e3, (long long)c.num_tris,
             (long long)c.num_subtris, c.num_subtris * 81.0 * mb, (long long)c.bin_entries, c.bin_entries * 4.0 * mb,
             (long long)c.tile_entries, c.tile_entries * 4.0 * mb, (long long)c.coarse_units, c.reruns);
    return CR_OK;
}

int32_t cr_pipe_count(void) {
    std::lock_guard<std::mutex> lock(registryMutex());
    return (int32_t)registry().size();
}

static void fillInfo(const PipeDesc& p, cr_pipe_info* out) {
    memset(out, 0, sizeof(*out));
    strncpy(out->name, p.name, sizeof(out->name) - 1);
    out->samples_log2 = p.samplesLog2;
    out->vertex_struct_size = p.vertexStructSize;
    out->render_mode_flags = p.renderModeFlags;
    out->profiling_mode = p.profilingMode;
    strncpy(out->blend_shader_name, p.blendShaderName, sizeof(out->blend_shader_name) - 1);
    strncpy(out->fragment_shader_name, p.fragmentShaderName, sizeof(out->fragment_shader_name) - 1);
}

cr_status cr_pipe_info_at(int32_t index, cr_pipe_info* out) {
    if (!out) return CR_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(registryMutex());
    if (index < 0 || index >= (int32_t)registry().size()) return CR_ERR_INVALID_ARGUMENT;
    fillInfo(registry()[index], out);
    return CR_OK;
}

cr_status cr_pipe_info_by_name(const char* name, cr_pipe_info* out) {
    if (!out || !name) return CR_ERR_INVALID_ARGUMENT;
    const PipeDesc* p = findPipe(name);
    if (!p) return CR_ERR_NO_PIPE;
    fillInfo(*p, out);
    return CR_OK;
}

}  // extern "C"
