// Draws one scene read from a file through the C++ drop-in classes
// (include/cudaraster/CudaRaster.hpp) and writes the colour and depth
// surfaces out; the GPU tests compare them with the CPU oracle.
//
//   draw_file <scene.bin> <out.bin>
//
// scene.bin (little endian): int32 width, height, samples, numVerts,
// vertexBytes, numTris, clear (0/1), float clearRGBA[4], clearDepth,
// char pipe[64], then numVerts * vertexBytes vertex bytes and numTris * 3
// int32 indices. out.bin: the colour words then the depth words.
#include <cudaraster/CudaRaster.hpp>

#include <cstdint>
#include <cstdio>
#include <vector>

using namespace FW;

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s scene.bin out.bin\n", argv[0]);
        return 2;
    }
    std::FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t hdr[7];
    float clear[5];
    char pipe[64];
    if (std::fread(hdr, 4, 7, f) != 7 || std::fread(clear, 4, 5, f) != 5 || std::fread(pipe, 1, 64, f) != 64) return 2;
    pipe[63] = 0;
    const int width = hdr[0], height = hdr[1], samples = hdr[2], numVerts = hdr[3], vertexBytes = hdr[4],
              numTris = hdr[5], doClear = hdr[6];
    std::vector<char> verts((size_t)numVerts * vertexBytes);
    std::vector<int32_t> idx((size_t)numTris * 3);
    if (std::fread(verts.data(), 1, verts.size(), f) != verts.size() ||
        std::fread(idx.data(), 4, idx.size(), f) != idx.size())
        return 2;
    std::fclose(f);

    CudaRaster raster;
    raster.init();
    CudaSurface color(Vec2i(width, height), CudaSurface::FORMAT_RGBA8, samples);
    CudaSurface depth(Vec2i(width, height), CudaSurface::FORMAT_DEPTH32, samples);
    Buffer vb((S64)verts.size()), ib((S64)idx.size() * 4);
    vb.setRange(0, verts.data(), (S64)verts.size());
    ib.setRange(0, idx.data(), (S64)idx.size() * 4);

    raster.setSurfaces(&color, &depth);
    raster.setPixelPipe(nullptr, pipe);
    raster.setVertexBuffer(&vb, 0);
    raster.setIndexBuffer(&ib, 0, numTris);
    if (doClear) raster.deferredClear(Vec4f(clear[0], clear[1], clear[2], clear[3]), clear[4]);
    raster.drawTriangles();
    CudaRaster::Stats st = raster.getStats();
    std::printf("setup %.6f bin %.6f coarse %.6f fine %.6f\n", st.setupTime, st.binTime, st.coarseTime,
                st.fineTime);
    std::printf("%s", raster.getProfilingInfo().c_str());

    std::vector<uint32_t> c(color.getNumBytes() / 4), d(depth.getNumBytes() / 4);
    color.download(c.data());
    depth.download(d.data());
    std::FILE* o = std::fopen(argv[2], "wb");
    if (!o) return 2;
    std::fwrite(c.data(), 4, c.size(), o);
    std::fwrite(d.data(), 4, d.size(), o);
    std::fclose(o);
    return 0;
}
