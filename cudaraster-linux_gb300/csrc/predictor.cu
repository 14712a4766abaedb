/*
 * predictor.cu -- learned queue-occupancy predictor.
 *
 * A small multilayer perceptron (inputs -> h1 -> h2 -> outputs, GELU on the
 * hidden layers) whose parameters are used in BF16 and whose products are
 * accumulated in FP32, trained online with Adam (FP32 master parameters and
 * moments). Its inputs are a 16x16 pooling of the previous frame's per-bin
 * queue histogram and a 6-float camera delta; its outputs are per-bin log
 * ratios of this frame's queue occupancy to the previous frame's (bin queues
 * and, per bin, the sum of its tile queues) and two heads for the log ratios
 * of the bin- and tile-entry totals, learned as corrections to the previous
 * frame's trend. The training targets are the counts the rasterizer itself
 * emits (cr_queue_counts).
 *
 * The reference has no counterpart: it sizes its queues on the host from the
 * previous draw and grows them when a draw overflows (CudaRaster.cpp:263-275,
 * 325-342). That grow-and-rerun path stays the fallback and the check of
 * every prediction; a prediction can cost a rerun, never an output bit.
 */
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>

#include "cudaraster.h"
#include "cudaraster/detail/launch.h"
#include "cudaraster/detail/per_device.h"

namespace cr {
namespace predictor {

constexpr int kTile = 32;          // GEMM output tile (rows x cols) and k-slab
constexpr int kGemmThreads = 256;  // 32 columns x 8 row groups, 4 rows per thread
constexpr int kHistCells = 16;     // input histogram is kHistCells x kHistCells
constexpr float kHistScale = 0.125f;

enum Epilogue { kEpiPlain = 0, kEpiBias = 1, kEpiBiasGelu = 2, kEpiGeluGrad = 3 };

__device__ __forceinline__ float toF(float v) { return v; }
__device__ __forceinline__ float toF(__nv_bfloat16 v) { return __bfloat162float(v); }

// GELU(z) = z * Phi(z), Phi the standard normal CDF.
__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
// d/dz GELU(z) = Phi(z) + z * phi(z).
__device__ __forceinline__ float geluGrad(float z) {
    return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

// C(m, n) = sum_k A(m, k) B(k, n) with A(m, k) = A[m*sam + k*sak] and
// B(k, n) = B[k*sbk + n*sbn]; FP32 products accumulated in increasing k by one
// thread per output, so results do not depend on the launch. Epilogues add
// a BF16 bias, apply GELU (C = pre-activation, C2 = activation), or multiply
// by GELU'(aux) (backward through the activation).
template <class TA, class TB, int EPI>
__global__ void __launch_bounds__(kGemmThreads) gemmKernel(int M, int N, int K,
                                                           const TA* __restrict__ A, long long sam, long long sak,
                                                           const TB* __restrict__ B, long long sbk, long long sbn,
                                                           float* __restrict__ C, long long ldc,
                                                           const __nv_bfloat16* __restrict__ bias,
                                                           const float* __restrict__ aux, long long ldaux,
                                                           float* __restrict__ C2) {
    __shared__ float As[kTile][kTile + 1];
    __shared__ float Bs[kTile][kTile + 1];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int m0 = blockIdx.y * kTile, n0 = blockIdx.x * kTile;
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int k0 = 0; k0 < K; k0 += kTile) {
        for (int r = ty; r < kTile; r += 8) {
            const int m = m0 + r, k = k0 + tx;
            As[r][tx] = (m < M && k < K) ? toF(A[(long long)m * sam + (long long)k * sak]) : 0.0f;
            const int kk = k0 + r, n = n0 + tx;
            Bs[r][tx] = (kk < K && n < N) ? toF(B[(long long)kk * sbk + (long long)n * sbn]) : 0.0f;
        }
        __syncthreads();
        const int kn = min(kTile, K - k0);
        for (int kk = 0; kk < kn; kk++) {
            const float b = Bs[kk][tx];
#pragma unroll
            for (int i = 0; i < 4; i++) acc[i] = fmaf(As[ty + 8 * i][kk], b, acc[i]);
        }
        __syncthreads();
    }
    const int n = n0 + tx;
    if (n >= N) return;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int m = m0 + ty + 8 * i;
        if (m >= M) continue;
        float v = acc[i];
        if (EPI == kEpiBias || EPI == kEpiBiasGelu) v += __bfloat162float(bias[n]);
        if (EPI == kEpiGeluGrad) v *= geluGrad(aux[(long long)m * ldaux + n]);
        C[(long long)m * ldc + n] = v;
        if (EPI == kEpiBiasGelu) C2[(long long)m * ldc + n] = gelu(v);
    }
}

template <class TA, class TB, int EPI>
void gemm(cudaStream_t s, int M, int N, int K, const TA* A, long long sam, long long sak, const TB* B, long long sbk,
          long long sbn, float* C, long long ldc, const __nv_bfloat16* bias = nullptr, const float* aux = nullptr,
          long long ldaux = 0, float* C2 = nullptr) {
    dim3 grid((N + kTile - 1) / kTile, (M + kTile - 1) / kTile);
    gemmKernel<TA, TB, EPI><<<grid, kGemmThreads, 0, s>>>(M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, bias, aux, ldaux,
                                                          C2);
}

__device__ float blockSum1024(float v, float* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    float t = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
    return t;
}

// Mean squared error over n outputs and its gradient: dY = 2 (Y - T) / n.
__global__ void __launch_bounds__(1024) mseKernel(const float* __restrict__ Y, const float* __restrict__ T, int n,
                                                  float* __restrict__ dY, float* __restrict__ loss) {
    __shared__ float red[32];
    const float inv = 1.0f / (float)n;
    float l = 0.0f;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float e = Y[i] - T[i];
        dY[i] = 2.0f * e * inv;
        l = fmaf(e, e, l);
    }
    const float s = blockSum1024(l, red);
    if (threadIdx.x == 0 && loss) *loss = s * inv;
}

// Bias gradients: out[n] = sum over rows m (in order) of dZ[m * ld + n].
__global__ void colSumKernel(const float* __restrict__ dZ, int M, int N, long long ld, float* __restrict__ out) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.0f;
    for (int m = 0; m < M; m++) s += dZ[(long long)m * ld + n];
    out[n] = s;
}

// Rows of a sample pool gathered into the batch buffer (rows == NULL: 0..batch-1).
// A row index outside [0, poolRows) reads row 0 instead and sets *badRows.
__global__ void gatherRowsKernel(const float* __restrict__ pool, int poolRows, const int32_t* __restrict__ rows,
                                 int batch, int width, float* __restrict__ out, int* __restrict__ badRows) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)batch * width) return;
    const int b = (int)(i / width), c = (int)(i % width);
    long long r = rows ? rows[b] : b;
    if (r < 0 || r >= poolRows) {
        if (c == 0) atomicOr(badRows, 1);
        r = 0;
    }
    out[i] = pool[r * width + c];
}

__global__ void adamKernel(float* __restrict__ w, __nv_bfloat16* __restrict__ w16, const float* __restrict__ g,
                           float* __restrict__ m, float* __restrict__ v, long long n, float lr, float b1, float b2,
                           float eps, float c1, float c2) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    w16[i] = __float2bfloat16_rn(wi);
}

__global__ void roundBf16Kernel(const float* __restrict__ w, __nv_bfloat16* __restrict__ w16, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) w16[i] = __float2bfloat16_rn(w[i]);
}

// ------------------------------------------------------ fused training step
// One training step (or one gradient evaluation) in four launches instead of
// a gather, six GEMMs, three bias reductions, the loss and Adam:
//   F  (one CTA per 8 units of hidden layer 1): gathers the batch and runs
//      hidden layer 1 (z1, a1 into global memory);
//   A  (one CTA per 32 outputs): hidden layer 2 (small, so every CTA runs
//      it), its slice of the output layer, the weighted
//      squared error and dY, the gradient of its rows of W3 / b3 (and their
//      Adam update), and its part of dL/da2 = dY . W3 over its rows;
//   B  (one CTA per batch row): dL/da2 summed over the A CTAs in CTA order, dz2,
//      da1 = dz2 . W2, dz1, and the loss;
//   C  (one thread per parameter of the hidden layers): the gradients of W1,
//      b1, W2, b2 (and their Adam update).
// No launch reads a parameter that another CTA of the same launch updates:
// W3 rows are read only by the CTA that owns them, W2 and b2 are read by A
// and B and updated by C, W1 and b1 are read by F only. Every sum runs
// in a fixed order, so results do not depend on timing. Sizes: inputs <=
// kFusedMaxIn, hidden layers <= kFusedMaxHidden, batch <= kFusedMaxBatch.
constexpr int kFusedMaxIn = 320;
constexpr int kFusedMaxHidden = 64;
constexpr int kFusedMaxBatch = 64;
constexpr int kFusedOutSlice = 32;
constexpr int kFusedThreads = 1024;

struct FusedNet {
    int in, h1, h2, out, batch;
    long long oW1, ob1, oW2, ob2, oW3, ob3;
    const __nv_bfloat16* w16;       // parameters used (BF16)
    __nv_bfloat16* w16Out;          // the same array, written by the Adam updates
    float* master;                  // FP32 parameters (Adam master copy)
    float* grad;                    // gradients [numParams]
    float* adamM;
    float* adamV;
    int adam;                       // 0: gradients only
    float lr, b1, b2, eps, c1, c2;
    const float* xPool;
    const float* tPool;
    int poolRows;
    const int32_t* rows;            // or NULL: rows 0..batch-1
    const float* outWeights;        // per-output loss weights, or NULL (all 1)
    float lossScale;                // 1 / (batch * sum of the output weights)
    float* x;                       // [batch][in] gathered inputs
    float* z1;                      // [batch][h1]
    float* a1;
    float* z2;                      // [batch][h2]
    float* dz1;
    float* dz2;
    float* da2Part;                 // [numOutSlices][batch][h2]
    float* lossPart;                // [numOutSlices]
    float* loss;
    int* badRows;
};

__device__ __forceinline__ void adamUpdate(const FusedNet& n, long long i, float g) {
    n.grad[i] = g;
    if (!n.adam) return;
    const float mi = n.b1 * n.adamM[i] + (1.0f - n.b1) * g;
    const float vi = n.b2 * n.adamV[i] + (1.0f - n.b2) * g * g;
    n.adamM[i] = mi;
    n.adamV[i] = vi;
    const float wi = n.master[i] - n.lr * (mi / n.c1) / (sqrtf(vi / n.c2) + n.eps);
    n.master[i] = wi;
    n.w16Out[i] = __float2bfloat16_rn(wi);
}

// Pool row of batch row b; a row outside the pool reads row 0.
__device__ __forceinline__ long long poolRow(const FusedNet& n, int b) {
    const long long r = n.rows ? n.rows[b] : b;
    return (r < 0 || r >= n.poolRows) ? 0 : r;
}

// Rows in shared memory are padded to a multiple of 8 elements (16 bytes of
// BF16): 128-bit loads, and consecutive rows start on different banks.
__host__ __device__ constexpr int padRow(int n) { return (n + 7) & ~7; }
__host__ __device__ constexpr int padRowOdd(int n) { return padRow(n) + 8; }   // 16 bytes more: 4 banks apart

// Shared memory of kernel F: inputs [B][padRow(in)] (floats), its W1 rows [kFusedUnits][padRow(in)] (BF16).
constexpr int kFusedUnits = 8;   // hidden-layer-1 units per kernel F CTA
__host__ __device__ constexpr size_t fusedSmemF(int in, int batch) {
    return sizeof(float) * (size_t)batch * padRow(in) + sizeof(__nv_bfloat16) * (size_t)kFusedUnits * padRow(in);
}
// Shared memory of kernel A: a1 [B][padRowOdd(h1)], a2 [B][padRowOdd(h2)], dY [B][32] (floats),
// W2 [h2][padRowOdd(h1)] and the W3 slice [32][padRowOdd(h2)] (BF16).
__host__ __device__ constexpr size_t fusedSmemA(int h1, int h2, int batch) {
    return sizeof(float) * ((size_t)batch * padRowOdd(h1) + (size_t)batch * padRowOdd(h2) +
                            (size_t)batch * kFusedOutSlice) +
           sizeof(__nv_bfloat16) * ((size_t)h2 * padRowOdd(h1) + (size_t)kFusedOutSlice * padRowOdd(h2));
}
static_assert(fusedSmemF(kFusedMaxIn, kFusedMaxBatch) <= 227 * 1024, "kernel F's shared memory must fit one CTA");
static_assert(fusedSmemA(kFusedMaxHidden, kFusedMaxHidden, kFusedMaxBatch) <= 227 * 1024,
              "kernel A's shared memory must fit one CTA");

// Eight BF16 values (16 bytes) as floats.
__device__ __forceinline__ void bf16x8(const __nv_bfloat16* p, float* f) {
    const uint4 v = *reinterpret_cast<const uint4*>(p);
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int i = 0; i < 4; i++) {
        f[2 * i] = __uint_as_float(w[i] << 16);
        f[2 * i + 1] = __uint_as_float(w[i] & 0xFFFF0000u);
    }
}

// Dot product of a BF16 weight row and a float row of n elements (both padded
// with zeros to a multiple of 8, 16-byte aligned), accumulated in increasing k.
__device__ __forceinline__ float dotRow(const __nv_bfloat16* w, const float* x, int n) {
    float s = 0.0f;
    for (int k = 0; k < n; k += 8) {
        float wf[8];
        bf16x8(w + k, wf);
        const float4 x0 = *reinterpret_cast<const float4*>(x + k);
        const float4 x1 = *reinterpret_cast<const float4*>(x + k + 4);
        s = fmaf(wf[0], x0.x, s);
        s = fmaf(wf[1], x0.y, s);
        s = fmaf(wf[2], x0.z, s);
        s = fmaf(wf[3], x0.w, s);
        s = fmaf(wf[4], x1.x, s);
        s = fmaf(wf[5], x1.y, s);
        s = fmaf(wf[6], x1.z, s);
        s = fmaf(wf[7], x1.w, s);
    }
    return s;
}

// Hidden layer 1: CTA c computes units kFusedUnits * c ... + kFusedUnits - 1
// for every batch row (thread t: unit t % kFusedUnits, rows t / kFusedUnits,
// + blockDim / kFusedUnits, ...); zero padding adds nothing to the sums. CTA 0
// also keeps the gathered inputs for the weight gradients.
__global__ void __launch_bounds__(256) trainForwardKernel(FusedNet n) {
    extern __shared__ __align__(16) unsigned char smemRaw[];
    __shared__ long long rowOf[kFusedMaxBatch];
    const int B = n.batch, IN = n.in, H1 = n.h1;
    const int INP = padRow(IN);
    float* xs = reinterpret_cast<float*>(smemRaw);
    __nv_bfloat16* w1 = reinterpret_cast<__nv_bfloat16*>(xs + (size_t)B * INP);
    pdlWait();
    pdlTrigger();
    const int t = threadIdx.x, nt = blockDim.x;
    const int j0 = blockIdx.x * kFusedUnits;
    if (t < B) {
        const long long r = n.rows ? n.rows[t] : t;
        if (blockIdx.x == 0 && (r < 0 || r >= n.poolRows)) atomicOr(n.badRows, 1);
        rowOf[t] = poolRow(n, t);
    }
    __syncthreads();
    for (int i = t; i < B * INP; i += nt) {
        const int b = i / INP, k = i - b * INP;
        const float v = k < IN ? n.xPool[rowOf[b] * IN + k] : 0.0f;
        xs[i] = v;
        if (blockIdx.x == 0 && k < IN) n.x[(size_t)b * IN + k] = v;
    }
    for (int i = t; i < kFusedUnits * INP; i += nt) {
        const int u = i / INP, k = i - u * INP;
        w1[i] = (k < IN && j0 + u < H1) ? n.w16[n.oW1 + (long long)(j0 + u) * IN + k] : __float2bfloat16_rn(0.0f);
    }
    __syncthreads();
    const int u = t % kFusedUnits, j = j0 + u;
    if (j >= H1) return;
    const float bias = __bfloat162float(n.w16[n.ob1 + j]);
    for (int b = t / kFusedUnits; b < B; b += nt / kFusedUnits) {
        const float z = dotRow(w1 + (size_t)u * INP, xs + (size_t)b * INP, INP) + bias;
        n.z1[b * H1 + j] = z;
        n.a1[b * H1 + j] = gelu(z);
    }
}

// One CTA per 32 outputs: lane q owns output o0 + q.
__global__ void __launch_bounds__(kFusedThreads) trainOutputKernel(FusedNet n) {
    extern __shared__ __align__(16) unsigned char smemRaw[];
    __shared__ float red[kFusedThreads / 32];
    __shared__ long long rowOf[kFusedMaxBatch];
    const int B = n.batch, H1 = n.h1, H2 = n.h2, H1P = padRowOdd(H1), H2P = padRowOdd(H2);
    float* a1 = reinterpret_cast<float*>(smemRaw);                                            // [B][H1P]
    float* a2 = a1 + (size_t)B * H1P;                                                         // [B][H2P]
    float* dy = a2 + (size_t)B * H2P;                                                         // [B][32]
    __nv_bfloat16* w2 = reinterpret_cast<__nv_bfloat16*>(dy + (size_t)B * kFusedOutSlice);   // [H2][H1P]
    __nv_bfloat16* w3 = w2 + (size_t)H2 * H1P;                                                // [32][H2P]
    pdlWait();
    pdlTrigger();
    const int t = threadIdx.x, nt = blockDim.x, lane = t & 31, warp = t >> 5, nw = nt >> 5;
    const int o0 = blockIdx.x * kFusedOutSlice;
    const int no = min(kFusedOutSlice, n.out - o0);
    if (t < B) rowOf[t] = poolRow(n, t);
    for (int i = t; i < B * H1P; i += nt) {
        const int b = i / H1P, k = i - b * H1P;
        a1[i] = k < H1 ? n.a1[b * H1 + k] : 0.0f;
    }
    for (int i = t; i < H2 * H1P; i += nt) {
        const int j = i / H1P, k = i - j * H1P;
        w2[i] = k < H1 ? n.w16[n.oW2 + (long long)j * H1 + k] : __float2bfloat16_rn(0.0f);
    }
    for (int i = t; i < kFusedOutSlice * H2P; i += nt) {
        const int q = i / H2P, k = i - q * H2P;
        w3[i] = (q < no && k < H2) ? n.w16[n.oW3 + (long long)(o0 + q) * H2 + k] : __float2bfloat16_rn(0.0f);
    }
    __syncthreads();
    // Hidden layer 2 (every CTA; CTA 0 keeps z2 for the backward pass).
    for (int i = t; i < B * H2P; i += nt) {
        const int b = i / H2P, j = i - b * H2P;
        float a = 0.0f;
        if (j < H2) {
            const float z = dotRow(w2 + (size_t)j * H1P, a1 + (size_t)b * H1P, H1P) + __bfloat162float(n.w16[n.ob2 + j]);
            a = gelu(z);
            if (blockIdx.x == 0) n.z2[b * H2 + j] = z;
        }
        a2[i] = a;
    }
    __syncthreads();
    // y, the weighted error and dY = 2 w (y - t) * lossScale for (batch row b, output lane).
    float l = 0.0f;
    const int q = lane;
    const float wo = (q < no && n.outWeights) ? n.outWeights[o0 + q] : 1.0f;
    const float bias = q < no ? __bfloat162float(n.w16[n.ob3 + o0 + q]) : 0.0f;
    for (int b = warp; b < B; b += nw) {
        float d = 0.0f;
        if (q < no) {
            const float y = dotRow(w3 + (size_t)q * H2P, a2 + (size_t)b * H2P, H2P) + bias;
            const float e = y - n.tPool[rowOf[b] * n.out + o0 + q];
            d = 2.0f * wo * e * n.lossScale;
            l = fmaf(wo * e, e, l);
        }
        dy[b * kFusedOutSlice + q] = d;
    }
    // The slice's loss, summed in a fixed order.
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xFFFFFFFFu, l, o);
    if (lane == 0) red[warp] = l;
    __syncthreads();
    if (t == 0) {
        float sum = 0.0f;
        for (int w = 0; w < nw; w++) sum += red[w];
        n.lossPart[blockIdx.x] = sum;
    }
    // dL/da2 over this slice's rows: part[b][j] = sum_q dY[b][q] W3[q][j].
    for (int b = warp; b < B; b += nw)
        for (int jj = lane; jj < H2; jj += 32) {
            float sum = 0.0f;
            for (int qq = 0; qq < no; qq++)
                sum = fmaf(dy[b * kFusedOutSlice + qq], __bfloat162float(w3[(size_t)qq * H2P + jj]), sum);
            n.da2Part[((size_t)blockIdx.x * B + b) * H2 + jj] = sum;
        }
    // Gradients of the slice's rows of W3 and b3 (batch order), then Adam:
    // warp w takes row q = w (and its bias), its lanes the row's columns.
    for (int qq = warp; qq < no; qq += nw) {
        for (int jj = lane; jj <= H2; jj += 32) {
            float g = 0.0f;
            if (jj < H2) {
                for (int b = 0; b < B; b++) g = fmaf(dy[b * kFusedOutSlice + qq], a2[(size_t)b * H2P + jj], g);
                adamUpdate(n, n.oW3 + (long long)(o0 + qq) * H2 + jj, g);
            } else {
                for (int b = 0; b < B; b++) g += dy[b * kFusedOutSlice + qq];
                adamUpdate(n, n.ob3 + o0 + qq, g);
            }
        }
    }
}

// Backward through the hidden layers, one CTA per batch row b (thread = unit):
// dz2 = (sum over slices, in slice order, of dL/da2) * GELU'(z2),
// dz1 = (dz2 . W2) * GELU'(z1); CTA 0 also sums the loss.
__global__ void __launch_bounds__(kFusedMaxHidden) trainHiddenKernel(FusedNet n, int slices) {
    __shared__ float dz2s[kFusedMaxHidden];
    pdlWait();
    pdlTrigger();
    const int B = n.batch, H1 = n.h1, H2 = n.h2;
    const int t = threadIdx.x, b = blockIdx.x;
    if (t < H2) {
        const int i = b * H2 + t;
        float sum = 0.0f;
        for (int g = 0; g < slices; g++) sum += n.da2Part[(size_t)g * B * H2 + i];
        const float d = sum * geluGrad(n.z2[i]);
        dz2s[t] = d;
        n.dz2[i] = d;
    }
    __syncthreads();
    if (t < H1) {
        float sum = 0.0f;
        for (int j = 0; j < H2; j++) sum = fmaf(dz2s[j], __bfloat162float(n.w16[n.oW2 + j * H1 + t]), sum);
        n.dz1[b * H1 + t] = sum * geluGrad(n.z1[b * H1 + t]);
    }
    if (b == 0 && t == 0) {
        float sum = 0.0f;
        for (int g = 0; g < slices; g++) sum += n.lossPart[g];
        *n.loss = sum * n.lossScale;
    }
}

// One thread per parameter of the hidden layers: W1, b1, W2, b2 in layout order.
__global__ void __launch_bounds__(256) trainWeightsKernel(FusedNet n) {
    pdlWait();
    pdlTrigger();
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int B = n.batch, IN = n.in, H1 = n.h1, H2 = n.h2;
    if (i >= n.oW3) return;
    float g = 0.0f;
    if (i < n.ob1) {
        const int j = (int)(i / IN), k = (int)(i - (long long)j * IN);
        for (int b = 0; b < B; b++) g = fmaf(n.dz1[b * H1 + j], n.x[(size_t)b * IN + k], g);
    } else if (i < n.oW2) {
        const int j = (int)(i - n.ob1);
        for (int b = 0; b < B; b++) g += n.dz1[b * H1 + j];
    } else if (i < n.ob2) {
        const int j = (int)((i - n.oW2) / H1), k = (int)((i - n.oW2) - (long long)j * H1);
        for (int b = 0; b < B; b++) g = fmaf(n.dz2[b * H2 + j], n.a1[b * H1 + k], g);
    } else {
        const int j = (int)(i - n.ob2);
        for (int b = 0; b < B; b++) g += n.dz2[b * H2 + j];
    }
    adamUpdate(n, i, g);
}

// ---------------------------------------------------------------- features
struct Cam6 {
    float v[6];
};

// x[cy*16 + cx] = kHistScale * mean of log1p(count) over the bins (bx, by)
// with bx*16/wb == cx and by*16/hb == cy (0 for cells that no bin maps to);
// x[256..261] = camera delta.
__global__ void queueFeaturesKernel(const int32_t* __restrict__ binCounts, int wb, int hb, Cam6 cam,
                                    float* __restrict__ x) {
    const int c = threadIdx.x;
    if (c < kHistCells * kHistCells) {
        const int cx = c % kHistCells, cy = c / kHistCells;
        const int bx0 = (cx * wb + kHistCells - 1) / kHistCells, bx1 = ((cx + 1) * wb + kHistCells - 1) / kHistCells;
        const int by0 = (cy * hb + kHistCells - 1) / kHistCells, by1 = ((cy + 1) * hb + kHistCells - 1) / kHistCells;
        float s = 0.0f;
        int n = 0;
        for (int by = by0; by < by1; by++)
            for (int bx = bx0; bx < bx1; bx++) {
                s += log1pf((float)binCounts[by * wb + bx]);
                n++;
            }
        x[c] = n ? s / (float)n * kHistScale : 0.0f;
    }
    if (c < 6) x[kHistCells * kHistCells + c] = cam.v[c];
}

// logs[b] = log1p(bin queue entries of bin b), logs[nb + b] = log1p(sum of
// the tile queue entries of the tiles of bin b). One warp per bin; the bin
// and tile totals are accumulated into totals[2] (zeroed by the caller).
__global__ void queueLogKernel(const int32_t* __restrict__ binCounts, const int32_t* __restrict__ tileCounts, int wb,
                               int hb, int wt, int ht, int binLog2, float* __restrict__ logs,
                               unsigned long long* __restrict__ totals) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int nb = wb * hb;
    if (warp >= nb) return;
    const int bx = warp % wb, by = warp / wb, side = 1 << binLog2;
    long long s = 0;
    for (int t = lane; t < side * side; t += 32) {
        const int tx = (bx << binLog2) + (t & (side - 1)), ty = (by << binLog2) + (t >> binLog2);
        if (tx < wt && ty < ht) s += tileCounts[ty * wt + tx];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
    if (lane == 0) {
        const int32_t b = binCounts[warp];
        logs[warp] = log1pf((float)b);
        logs[nb + warp] = log1pf((float)s);
        atomicAdd(&totals[0], (unsigned long long)b);
        atomicAdd(&totals[1], (unsigned long long)s);
    }
}

__global__ void totalLogKernel(const unsigned long long* __restrict__ totals, float* __restrict__ out) {
    if (threadIdx.x < 2) out[threadIdx.x] = (float)log1p((double)totals[threadIdx.x]);
}

// target[i] = cur[i] - prev[i]; for the last nTrend entries the trend of the
// previous step is taken off as well: - (prev[i] - prevprev[i]) when
// prevprev is given.
__global__ void targetsKernel(const float* __restrict__ prevprev, const float* __restrict__ prev,
                              const float* __restrict__ cur, int n, int nTrend, float* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float t = cur[i] - prev[i];
    if (i >= n - nTrend && prevprev) t -= prev[i] - prevprev[i];
    out[i] = t;
}

// Predicted occupancy: per_bin[i] = max(expm1(prev[i] + y[i]), 0) for the
// 2nb per-bin outputs; totals[0..1] from the two total heads on top of the
// previous step's trend: expm1(prev + (prev - prevprev) + y) (no trend
// without prevprev); totals[2..3] = sums of the per-bin predictions.
__global__ void __launch_bounds__(1024) queuePlanKernel(const float* __restrict__ prevprev,
                                                        const float* __restrict__ prev, const float* __restrict__ y,
                                                        int nb, float* __restrict__ perBin, double* __restrict__ totals) {
    __shared__ double red[2][32];
    double s[2] = {0.0, 0.0};
    for (int i = threadIdx.x; i < 2 * nb; i += blockDim.x) {
        const float p = fmaxf(expm1f(prev[i] + y[i]), 0.0f);
        if (perBin) perBin[i] = p;
        s[i >= nb] += (double)p;
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = 0; k < 2; k++) {
        double v = s[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
        if (lane == 0) red[k][w] = v;
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += red[threadIdx.x][i];
        totals[2 + threadIdx.x] = t;
        const int h = 2 * nb + threadIdx.x;
        const double base = (double)prev[h] + (prevprev ? (double)prev[h] - (double)prevprev[h] : 0.0);
        totals[threadIdx.x] = fmax(expm1(base + (double)y[h]), 0.0);
    }
}

// ------------------------------------------------------- fused frame step
struct FrameArgs {
    const int32_t* binCounts;     // the draw's per-bin bin-entry counts [nb]
    const int32_t* tileCounts;    // per-tile tile-entry counts [tiles_x * tiles_y]
    const int32_t* counters;      // the draw's 8 device counters
    int wb, hb, wt, ht, binLog2;
    float ahead;                  // frames between a sample's input and its target
    const float* logsPrev;        // previous frame's logs: the trend of this frame's prediction (or NULL)
    float* logsCur;               // this frame's logs [2nb + 2]
    const float* logsTgtBase;     // logs of the frame `ahead` back, whose sample this frame completes
    const float* logsTgtTrend;    // logs of the frame before that (its trend) or NULL
    float* target;                // target of that sample or NULL
    float* xNext;                 // input of this frame's sample / prediction [262]
    Cam6 camNext;                 // camera move from this frame to the predicted one
    float* perBin;                // predicted per-bin occupancy of the next frame [2nb] or NULL
    double* fetch;                // 4 doubles (predicted totals) then 8 int32 (this frame's counters)
};

// One frame of the online predictor in one CTA: this frame's logs (as
// queueLogKernel/totalLogKernel), the target of the sample that this frame
// completes (the frame `ahead` back: cur - base, and for the total heads
// also - ahead * (base - trend), as targetsKernel for ahead = 1), the next
// input (as queueFeaturesKernel, bit for bit), the network's forward pass on
// it (warp-split dot products in FP32 over the BF16 parameters) and the
// occupancy plan of the frame `ahead` on (as queuePlanKernel with this frame
// as the base and heads expm1(cur + ahead * (cur - prev) + y)), plus a copy
// of the counters into the fetch block.
__global__ void __launch_bounds__(1024) predictorFrameKernel(FrameArgs a, const __nv_bfloat16* __restrict__ w, int in,
                                                             int h1, int h2, int out, long long oW1, long long ob1,
                                                             long long oW2, long long ob2, long long oW3,
                                                             long long ob3) {
    __shared__ unsigned long long sTot[32][2];
    __shared__ double sPlan[32][2];
    __shared__ float sx[kHistCells * kHistCells + 6];
    __shared__ float sh1[256];
    __shared__ float sh2[256];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int nb = a.wb * a.hb, side = 1 << a.binLog2;
    // 1. Per-bin logs and the entry totals.
    unsigned long long tb = 0, tt = 0;
    for (int b = warp; b < nb; b += nw) {
        const int bx = b % a.wb, by = b / a.wb;
        long long sum = 0;
        for (int t = lane; t < side * side; t += 32) {
            const int tx = (bx << a.binLog2) + (t & (side - 1)), ty = (by << a.binLog2) + (t >> a.binLog2);
            if (tx < a.wt && ty < a.ht) sum += a.tileCounts[ty * a.wt + tx];
        }
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xFFFFFFFFu, sum, o);
        if (lane == 0) {
            const int32_t c = a.binCounts[b];
            a.logsCur[b] = log1pf((float)c);
            a.logsCur[nb + b] = log1pf((float)sum);
            tb += (unsigned long long)c;
            tt += (unsigned long long)sum;
        }
    }
    if (lane == 0) {
        sTot[warp][0] = tb;
        sTot[warp][1] = tt;
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        unsigned long long t = 0;
        for (int i = 0; i < nw; i++) t += sTot[i][threadIdx.x];
        a.logsCur[2 * nb + threadIdx.x] = (float)log1p((double)t);
    }
    __syncthreads();
    const int n2 = 2 * nb + 2;
    // 2. Target of the pending sample.
    if (a.target && a.logsTgtBase) {
        for (int i = threadIdx.x; i < n2; i += blockDim.x) {
            float t = a.logsCur[i] - a.logsTgtBase[i];
            if (i >= n2 - 2 && a.logsTgtTrend) t -= a.ahead * (a.logsTgtBase[i] - a.logsTgtTrend[i]);
            a.target[i] = t;
        }
    }
    // 3. Next input: pooled histogram of this frame + camera delta.
    if (threadIdx.x < kHistCells * kHistCells) {
        const int c = threadIdx.x, cx = c % kHistCells, cy = c / kHistCells;
        const int bx0 = (cx * a.wb + kHistCells - 1) / kHistCells, bx1 = ((cx + 1) * a.wb + kHistCells - 1) / kHistCells;
        const int by0 = (cy * a.hb + kHistCells - 1) / kHistCells, by1 = ((cy + 1) * a.hb + kHistCells - 1) / kHistCells;
        float s = 0.0f;
        int n = 0;
        for (int by = by0; by < by1; by++)
            for (int bx = bx0; bx < bx1; bx++) {
                s += a.logsCur[by * a.wb + bx];
                n++;
            }
        const float v = n ? s / (float)n * kHistScale : 0.0f;
        sx[c] = v;
        a.xNext[c] = v;
    }
    if (threadIdx.x < 6) {
        sx[kHistCells * kHistCells + threadIdx.x] = a.camNext.v[threadIdx.x];
        a.xNext[kHistCells * kHistCells + threadIdx.x] = a.camNext.v[threadIdx.x];
    }
    __syncthreads();
    // 4. Hidden layers: one warp per unit, lanes over the inputs.
    for (int j = warp; j < h1; j += nw) {
        float s = 0.0f;
        for (int k = lane; k < in; k += 32) s = fmaf(__bfloat162float(w[oW1 + (long long)j * in + k]), sx[k], s);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
        if (lane == 0) sh1[j] = gelu(s + __bfloat162float(w[ob1 + j]));
    }
    __syncthreads();
    for (int j = warp; j < h2; j += nw) {
        float s = 0.0f;
        for (int k = lane; k < h1; k += 32) s = fmaf(__bfloat162float(w[oW2 + (long long)j * h1 + k]), sh1[k], s);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
        if (lane == 0) sh2[j] = gelu(s + __bfloat162float(w[ob2 + j]));
    }
    __syncthreads();
    // 5. Output layer and the plan of the next frame.
    double ps[2] = {0.0, 0.0};
    for (int o = threadIdx.x; o < out; o += blockDim.x) {
        float s = 0.0f;
        const __nv_bfloat16* row = w + oW3 + (long long)o * h2;
        for (int k = 0; k < h2; k++) s = fmaf(__bfloat162float(row[k]), sh2[k], s);
        const float y = s + __bfloat162float(w[ob3 + o]);
        if (o < 2 * nb) {
            const float p = fmaxf(expm1f(a.logsCur[o] + y), 0.0f);
            if (a.perBin) a.perBin[o] = p;
            ps[o >= nb] += (double)p;
        } else if (o < n2) {
            const double base = (double)a.logsCur[o] +
                                (a.logsPrev ? (double)a.ahead * ((double)a.logsCur[o] - (double)a.logsPrev[o]) : 0.0);
            a.fetch[o - 2 * nb] = fmax(expm1(base + (double)y), 0.0);
        }
    }
    for (int k = 0; k < 2; k++) {
        double v = ps[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
        if (lane == 0) sPlan[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        double t = 0.0;
        for (int i = 0; i < nw; i++) t += sPlan[i][threadIdx.x];
        a.fetch[2 + threadIdx.x] = t;
    }
    if (threadIdx.x < 8) reinterpret_cast<int32_t*>(a.fetch + 4)[threadIdx.x] = a.counters ? a.counters[threadIdx.x] : 0;
}

}  // namespace predictor
}  // namespace cr

using namespace cr::predictor;

// ---------------------------------------------------------------- the network
struct cr_predictor {
    int in = 0, h1 = 0, h2 = 0, out = 0, maxBatch = 0;
    long long numParams = 0;
    long long oW1 = 0, ob1 = 0, oW2 = 0, ob2 = 0, oW3 = 0, ob3 = 0;
    float* master = nullptr;        // FP32 parameters [numParams]
    __nv_bfloat16* w16 = nullptr;   // BF16 copy used by the kernels
    float* grad = nullptr;          // gradients of the last step
    float* adamM = nullptr;
    float* adamV = nullptr;
    float* act = nullptr;           // activations, see the offsets below
    long long step = 0;
    // activation buffer layout ([maxBatch x width] each)
    float *x = nullptr, *t = nullptr, *z1 = nullptr, *a1 = nullptr, *z2 = nullptr, *a2 = nullptr, *y = nullptr;
    float *dy = nullptr, *dz2 = nullptr, *dz1 = nullptr, *loss = nullptr;
    int* badRows = nullptr;         // set when a batch named a row outside its pool
    // Fused training step (sizes within the kFused* limits).
    bool fused = false;
    int slices = 0;                 // output slices of kFusedOutSlice rows
    float* da2Part = nullptr;       // [slices][maxBatch][h2]
    float* lossPart = nullptr;      // [slices]
    float* outWeights = nullptr;    // per-output loss weights (NULL: all 1)
    double sumWeights = 0.0;
};

namespace {

void freePredictor(cr_predictor* p) {
    if (!p) return;
    cudaFree(p->da2Part);
    cudaFree(p->outWeights);
    cudaFree(p->master);
    cudaFree(p->w16);
    cudaFree(p->grad);
    cudaFree(p->adamM);
    cudaFree(p->adamV);
    cudaFree(p->act);
    delete p;
}

// Forward pass of `batch` rows already in p->x; leaves z1, a1, z2, a2, y.
void forward(cr_predictor* p, int batch, cudaStream_t s) {
    const __nv_bfloat16* w = p->w16;
    gemm<float, __nv_bfloat16, kEpiBiasGelu>(s, batch, p->h1, p->in, p->x, p->in, 1, w + p->oW1, 1, p->in, p->z1, p->h1,
                                             w + p->ob1, nullptr, 0, p->a1);
    gemm<float, __nv_bfloat16, kEpiBiasGelu>(s, batch, p->h2, p->h1, p->a1, p->h1, 1, w + p->oW2, 1, p->h1, p->z2, p->h2,
                                             w + p->ob2, nullptr, 0, p->a2);
    gemm<float, __nv_bfloat16, kEpiBias>(s, batch, p->out, p->h2, p->a2, p->h2, 1, w + p->oW3, 1, p->h2, p->y, p->out,
                                         w + p->ob3);
}

// Backward pass from dy (in p->dy); gradients into p->grad (parameter layout).
void backward(cr_predictor* p, int batch, cudaStream_t s) {
    const __nv_bfloat16* w = p->w16;
    float* g = p->grad;
    // Output layer: dW3[o][j] = sum_b dy[b][o] a2[b][j]; db3 = column sums of dy.
    gemm<float, float, kEpiPlain>(s, p->out, p->h2, batch, p->dy, 1, p->out, p->a2, p->h2, 1, g + p->oW3, p->h2);
    colSumKernel<<<(p->out + 255) / 256, 256, 0, s>>>(p->dy, batch, p->out, p->out, g + p->ob3);
    // dz2 = (dy . W3) * GELU'(z2)
    gemm<float, __nv_bfloat16, kEpiGeluGrad>(s, batch, p->h2, p->out, p->dy, p->out, 1, w + p->oW3, p->h2, 1, p->dz2,
                                             p->h2, nullptr, p->z2, p->h2);
    gemm<float, float, kEpiPlain>(s, p->h2, p->h1, batch, p->dz2, 1, p->h2, p->a1, p->h1, 1, g + p->oW2, p->h1);
    colSumKernel<<<(p->h2 + 255) / 256, 256, 0, s>>>(p->dz2, batch, p->h2, p->h2, g + p->ob2);
    // dz1 = (dz2 . W2) * GELU'(z1)
    gemm<float, __nv_bfloat16, kEpiGeluGrad>(s, batch, p->h1, p->h2, p->dz2, p->h2, 1, w + p->oW2, p->h1, 1, p->dz1,
                                             p->h1, nullptr, p->z1, p->h1);
    gemm<float, float, kEpiPlain>(s, p->h1, p->in, batch, p->dz1, 1, p->h1, p->x, p->in, 1, g + p->oW1, p->in);
    colSumKernel<<<(p->h1 + 255) / 256, 256, 0, s>>>(p->dz1, batch, p->h1, p->h1, g + p->ob1);
}

// The fused step: gradients of `batch` rows into p->grad and the loss into
// p->loss, and with adam the Adam update of every parameter (p->step already
// advanced).
cr_status trainFused(cr_predictor* p, const float* xPool, const float* tPool, int poolRows, const int32_t* rows,
                     int batch, bool adam, float lr, float beta1, float beta2, float eps, cudaStream_t s) {
    FusedNet n;
    memset(&n, 0, sizeof(n));
    n.in = p->in;
    n.h1 = p->h1;
    n.h2 = p->h2;
    n.out = p->out;
    n.batch = batch;
    n.oW1 = p->oW1;
    n.ob1 = p->ob1;
    n.oW2 = p->oW2;
    n.ob2 = p->ob2;
    n.oW3 = p->oW3;
    n.ob3 = p->ob3;
    n.w16 = p->w16;
    n.w16Out = p->w16;
    n.master = p->master;
    n.grad = p->grad;
    n.adamM = p->adamM;
    n.adamV = p->adamV;
    n.adam = adam ? 1 : 0;
    n.lr = lr;
    n.b1 = beta1;
    n.b2 = beta2;
    n.eps = eps;
    n.c1 = adam ? (float)(1.0 - std::pow((double)beta1, (double)p->step)) : 1.0f;
    n.c2 = adam ? (float)(1.0 - std::pow((double)beta2, (double)p->step)) : 1.0f;
    n.xPool = xPool;
    n.tPool = tPool;
    n.poolRows = poolRows;
    n.rows = rows;
    n.outWeights = p->outWeights;
    n.lossScale = (float)(1.0 / ((double)batch * (p->outWeights ? p->sumWeights : (double)p->out)));
    n.x = p->x;
    n.z1 = p->z1;
    n.a1 = p->a1;
    n.z2 = p->z2;
    n.dz1 = p->dz1;
    n.dz2 = p->dz2;
    n.da2Part = p->da2Part;
    n.lossPart = p->lossPart;
    n.loss = p->loss;
    n.badRows = p->badRows;
    static cr::OncePerDevice attribute;
    attribute.run([] {
        cudaFuncSetAttribute(trainForwardKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)fusedSmemF(kFusedMaxIn, kFusedMaxBatch));
        cudaFuncSetAttribute(trainOutputKernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)fusedSmemA(kFusedMaxHidden, kFusedMaxHidden, kFusedMaxBatch));
    });
    cudaError_t e = cr::launchKernel(trainForwardKernel, (n.h1 + kFusedUnits - 1) / kFusedUnits, 256,
                                     fusedSmemF(n.in, batch), s, false, n);
    if (e == cudaSuccess)
        e = cr::launchKernel(trainOutputKernel, p->slices, kFusedThreads, fusedSmemA(n.h1, n.h2, batch), s, true, n);
    if (e == cudaSuccess) e = cr::launchKernel(trainHiddenKernel, batch, kFusedMaxHidden, 0, s, true, n, p->slices);
    if (e == cudaSuccess)
        e = cr::launchKernel(trainWeightsKernel, (unsigned)((p->oW3 + 255) / 256), 256, 0, s, true, n);
    return e == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

cr_status gatherBatch(cr_predictor* p, const float* xPool, const float* tPool, int poolRows, const int32_t* rows,
                      int batch, cudaStream_t s) {
    long long nx = (long long)batch * p->in, nt = (long long)batch * p->out;
    gatherRowsKernel<<<(unsigned)((nx + 255) / 256), 256, 0, s>>>(xPool, poolRows, rows, batch, p->in, p->x,
                                                                 p->badRows);
    if (tPool)
        gatherRowsKernel<<<(unsigned)((nt + 255) / 256), 256, 0, s>>>(tPool, poolRows, rows, batch, p->out, p->t,
                                                                     p->badRows);
    return cudaGetLastError() == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

}  // namespace

extern "C" {

cr_status cr_predictor_create(cr_predictor** out, int32_t inputs, int32_t hidden1, int32_t hidden2, int32_t outputs,
                              int32_t max_batch) {
    if (!out) return CR_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (inputs <= 0 || hidden1 <= 0 || hidden2 <= 0 || outputs <= 0 || max_batch <= 0 || inputs > (1 << 20) ||
        hidden1 > 4096 || hidden2 > 4096 || outputs > (1 << 20) || max_batch > 4096)
        return CR_ERR_INVALID_ARGUMENT;
    cr_predictor* p = new (std::nothrow) cr_predictor();
    if (!p) return CR_ERR_OUT_OF_MEMORY;
    p->in = inputs;
    p->h1 = hidden1;
    p->h2 = hidden2;
    p->out = outputs;
    p->maxBatch = max_batch;
    p->oW1 = 0;
    p->ob1 = p->oW1 + (long long)hidden1 * inputs;
    p->oW2 = p->ob1 + hidden1;
    p->ob2 = p->oW2 + (long long)hidden2 * hidden1;
    p->oW3 = p->ob2 + hidden2;
    p->ob3 = p->oW3 + (long long)outputs * hidden2;
    p->numParams = p->ob3 + outputs;
    const long long P = p->numParams, B = max_batch;
    const long long actFloats = B * (inputs + outputs /*t*/ + 2LL * hidden1 + 2LL * hidden2 + outputs /*y*/ +
                                     outputs /*dy*/ + hidden2 + hidden1) + 2;
    cudaError_t e = cudaMalloc(&p->master, P * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&p->w16, P * sizeof(__nv_bfloat16));
    if (e == cudaSuccess) e = cudaMalloc(&p->grad, P * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&p->adamM, P * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&p->adamV, P * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&p->act, actFloats * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(p->master, 0, P * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(p->w16, 0, P * sizeof(__nv_bfloat16));
    if (e == cudaSuccess) e = cudaMemset(p->grad, 0, P * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(p->adamM, 0, P * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(p->adamV, 0, P * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(p->act, 0, actFloats * sizeof(float));
    if (e != cudaSuccess) {
        freePredictor(p);
        return e == cudaErrorMemoryAllocation ? CR_ERR_OUT_OF_MEMORY : CR_ERR_CUDA;
    }
    p->fused = inputs <= kFusedMaxIn && hidden1 <= kFusedMaxHidden && hidden2 <= kFusedMaxHidden &&
               max_batch <= kFusedMaxBatch;
    if (p->fused) {
        p->slices = (outputs + kFusedOutSlice - 1) / kFusedOutSlice;
        e = cudaMalloc(&p->da2Part, ((size_t)p->slices * max_batch * hidden2 + p->slices) * sizeof(float));
        if (e != cudaSuccess) {
            freePredictor(p);
            return e == cudaErrorMemoryAllocation ? CR_ERR_OUT_OF_MEMORY : CR_ERR_CUDA;
        }
        p->lossPart = p->da2Part + (size_t)p->slices * max_batch * hidden2;
    }
    float* a = p->act;
    p->x = a;   a += B * inputs;
    p->t = a;   a += B * outputs;
    p->z1 = a;  a += B * hidden1;
    p->a1 = a;  a += B * hidden1;
    p->z2 = a;  a += B * hidden2;
    p->a2 = a;  a += B * hidden2;
    p->y = a;   a += B * outputs;
    p->dy = a;  a += B * outputs;
    p->dz2 = a; a += B * hidden2;
    p->dz1 = a; a += B * hidden1;
    p->loss = a; a += 1;
    p->badRows = reinterpret_cast<int*>(a);
    *out = p;
    return CR_OK;
}

void cr_predictor_destroy(cr_predictor* p) {
    if (p) cudaDeviceSynchronize();
    freePredictor(p);
}

int64_t cr_predictor_num_params(const cr_predictor* p) { return p ? p->numParams : 0; }

cr_status cr_predictor_set_params(cr_predictor* p, const float* host, int64_t n) {
    if (!p || !host || n != p->numParams) return CR_ERR_INVALID_ARGUMENT;
    const size_t bytes = (size_t)n * sizeof(float);
    cudaError_t e = cudaMemcpy(p->master, host, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(p->adamM, 0, bytes);
    if (e == cudaSuccess) e = cudaMemset(p->adamV, 0, bytes);
    if (e != cudaSuccess) return CR_ERR_CUDA;
    roundBf16Kernel<<<(unsigned)((n + 255) / 256), 256>>>(p->master, p->w16, n);
    p->step = 0;
    return cudaDeviceSynchronize() == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

cr_status cr_predictor_get_params(const cr_predictor* p, float* host, int64_t n) {
    if (!p || !host || n != p->numParams) return CR_ERR_INVALID_ARGUMENT;
    return cudaMemcpy(host, p->master, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess ? CR_OK
                                                                                                          : CR_ERR_CUDA;
}

cr_status cr_predictor_get_params_bf16(const cr_predictor* p, uint16_t* host, int64_t n) {
    if (!p || !host || n != p->numParams) return CR_ERR_INVALID_ARGUMENT;
    return cudaMemcpy(host, p->w16, (size_t)n * 2, cudaMemcpyDeviceToHost) == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

cr_status cr_predictor_forward(cr_predictor* p, const float* x, int32_t batch, float* y, void* stream) {
    if (!p || !x || !y || batch <= 0 || batch > p->maxBatch) return CR_ERR_INVALID_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    if (gatherBatch(p, x, nullptr, batch, nullptr, batch, s) != CR_OK) return CR_ERR_CUDA;
    forward(p, batch, s);
    if (cudaMemcpyAsync(y, p->y, (size_t)batch * p->out * sizeof(float), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return CR_ERR_CUDA;
    return cudaGetLastError() == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

cr_status cr_predictor_gradients(cr_predictor* p, const float* x_pool, const float* target_pool, int32_t pool_rows,
                                 const int32_t* rows, int32_t batch, float* grads, float* loss, void* stream) {
    if (!p || !x_pool || !target_pool || batch <= 0 || batch > p->maxBatch || pool_rows <= 0 ||
        (!rows && batch > pool_rows))
        return CR_ERR_INVALID_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    if (p->fused) {
        if (trainFused(p, x_pool, target_pool, pool_rows, rows, batch, false, 0.0f, 0.0f, 0.0f, 1.0f, s) != CR_OK)
            return CR_ERR_CUDA;
    } else {
        if (p->outWeights) return CR_ERR_UNSUPPORTED;
        if (gatherBatch(p, x_pool, target_pool, pool_rows, rows, batch, s) != CR_OK) return CR_ERR_CUDA;
        forward(p, batch, s);
        mseKernel<<<1, 1024, 0, s>>>(p->y, p->t, batch * p->out, p->dy, p->loss);
        backward(p, batch, s);
    }
    cudaError_t e = cudaSuccess;
    if (grads) e = cudaMemcpyAsync(grads, p->grad, (size_t)p->numParams * sizeof(float), cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && loss) e = cudaMemcpyAsync(loss, p->loss, sizeof(float), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return CR_ERR_CUDA;
    return cudaGetLastError() == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

cr_status cr_predictor_train_step(cr_predictor* p, const float* x_pool, const float* target_pool, int32_t pool_rows,
                                  const int32_t* rows, int32_t batch, float lr, float beta1, float beta2, float eps,
                                  float* loss, void* stream) {
    if (!(lr >= 0.0f) || !(beta1 >= 0.0f && beta1 < 1.0f) || !(beta2 >= 0.0f && beta2 < 1.0f) || !(eps > 0.0f))
        return CR_ERR_INVALID_ARGUMENT;
    if (p && p->fused) {
        if (!x_pool || !target_pool || batch <= 0 || batch > p->maxBatch || pool_rows <= 0 ||
            (!rows && batch > pool_rows))
            return CR_ERR_INVALID_ARGUMENT;
        p->step++;
        cudaStream_t s = (cudaStream_t)stream;
        if (trainFused(p, x_pool, target_pool, pool_rows, rows, batch, true, lr, beta1, beta2, eps, s) != CR_OK)
            return CR_ERR_CUDA;
        if (loss && cudaMemcpyAsync(loss, p->loss, sizeof(float), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            return CR_ERR_CUDA;
        return CR_OK;
    }
    cr_status st = cr_predictor_gradients(p, x_pool, target_pool, pool_rows, rows, batch, nullptr, loss, stream);
    if (st != CR_OK) return st;
    p->step++;
    const float c1 = (float)(1.0 - std::pow((double)beta1, (double)p->step));
    const float c2 = (float)(1.0 - std::pow((double)beta2, (double)p->step));
    const long long n = p->numParams;
    adamKernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(p->master, p->w16, p->grad, p->adamM,
                                                                            p->adamV, n, lr, beta1, beta2, eps, c1, c2);
    return cudaGetLastError() == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

int64_t cr_predictor_steps(const cr_predictor* p) { return p ? p->step : 0; }

cr_status cr_predictor_set_loss_weights(cr_predictor* p, const float* host, int64_t n) {
    if (!p) return CR_ERR_INVALID_ARGUMENT;
    if (!host) {
        cudaFree(p->outWeights);
        p->outWeights = nullptr;
        p->sumWeights = 0.0;
        return CR_OK;
    }
    if (n != p->out) return CR_ERR_INVALID_ARGUMENT;
    double sum = 0.0;
    for (int64_t i = 0; i < n; i++) {
        if (!(host[i] >= 0.0f) || !std::isfinite(host[i])) return CR_ERR_INVALID_ARGUMENT;
        sum += host[i];
    }
    if (!(sum > 0.0)) return CR_ERR_INVALID_ARGUMENT;
    if (!p->fused) return CR_ERR_UNSUPPORTED;
    if (!p->outWeights && cudaMalloc(&p->outWeights, (size_t)n * sizeof(float)) != cudaSuccess)
        return CR_ERR_OUT_OF_MEMORY;
    if (cudaMemcpy(p->outWeights, host, (size_t)n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
        return CR_ERR_CUDA;
    p->sumWeights = sum;
    return CR_OK;
}

cr_status cr_predictor_bad_rows(cr_predictor* p, int32_t* flag, int32_t reset) {
    if (!p || !flag) return CR_ERR_INVALID_ARGUMENT;
    if (cudaMemcpy(flag, p->badRows, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return CR_ERR_CUDA;
    if (reset && cudaMemset(p->badRows, 0, sizeof(int)) != cudaSuccess) return CR_ERR_CUDA;
    return CR_OK;
}

cr_status cr_predictor_frame(cr_predictor* p, const int32_t* bin_counts, const int32_t* tile_counts,
                             const int32_t* counters, const cr_queue_layout* layout, int32_t ahead,
                             const float* logs_prev, float* logs_cur, const float* logs_target_base,
                             const float* logs_target_trend, float* target, const float* camera_delta_ahead,
                             float* x_next, float* per_bin, void* fetch, void* stream) {
    if (!p || !bin_counts || !tile_counts || !layout || !logs_cur || !camera_delta_ahead || !x_next || !fetch ||
        ahead < 1 || ahead > 64)
        return CR_ERR_INVALID_ARGUMENT;
    const cr_queue_layout& l = *layout;
    if (l.bins_x <= 0 || l.bins_y <= 0 || l.tiles_x <= 0 || l.tiles_y <= 0 || l.bin_log2 < 0 || l.bin_log2 > 8 ||
        ((l.tiles_x + (1 << l.bin_log2) - 1) >> l.bin_log2) != l.bins_x ||
        ((l.tiles_y + (1 << l.bin_log2) - 1) >> l.bin_log2) != l.bins_y)
        return CR_ERR_INVALID_ARGUMENT;
    if (p->in != kHistCells * kHistCells + 6 || p->out != 2 * l.bins_x * l.bins_y + 2 || p->h1 > 256 || p->h2 > 256)
        return CR_ERR_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(fetch) & 7) return CR_ERR_INVALID_ARGUMENT;
    FrameArgs a;
    a.binCounts = bin_counts;
    a.tileCounts = tile_counts;
    a.counters = counters;
    a.wb = l.bins_x;
    a.hb = l.bins_y;
    a.wt = l.tiles_x;
    a.ht = l.tiles_y;
    a.binLog2 = l.bin_log2;
    a.ahead = (float)ahead;
    a.logsPrev = logs_prev;
    a.logsCur = logs_cur;
    a.logsTgtBase = logs_target_base;
    a.logsTgtTrend = logs_target_base ? logs_target_trend : nullptr;
    a.target = target;
    a.xNext = x_next;
    memcpy(a.camNext.v, camera_delta_ahead, sizeof(a.camNext.v));
    a.perBin = per_bin;
    a.fetch = static_cast<double*>(fetch);
    predictorFrameKernel<<<1, 1024, 0, (cudaStream_t)stream>>>(a, p->w16, p->in, p->h1, p->h2, p->out, p->oW1, p->ob1,
                                                             p->oW2, p->ob2, p->oW3, p->ob3);
    return cudaGetLastError() == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

cr_status cr_queue_features(const int32_t* bin_counts, int32_t bins_x, int32_t bins_y, const float* camera_delta,
                            float* x, void* stream) {
    if (!bin_counts || !camera_delta || !x || bins_x <= 0 || bins_y <= 0) return CR_ERR_INVALID_ARGUMENT;
    Cam6 cam;
    memcpy(cam.v, camera_delta, sizeof(cam.v));
    queueFeaturesKernel<<<1, kHistCells * kHistCells, 0, (cudaStream_t)stream>>>(bin_counts, bins_x, bins_y, cam, x);
    return cudaGetLastError() == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

cr_status cr_queue_log_counts(const int32_t* bin_counts, const int32_t* tile_counts, int32_t bins_x, int32_t bins_y,
                              int32_t tiles_x, int32_t tiles_y, int32_t bin_log2, float* logs, void* stream) {
    if (!bin_counts || !tile_counts || !logs || bins_x <= 0 || bins_y <= 0 || tiles_x <= 0 || tiles_y <= 0 ||
        bin_log2 < 0 || bin_log2 > 8 || ((tiles_x + (1 << bin_log2) - 1) >> bin_log2) != bins_x ||
        ((tiles_y + (1 << bin_log2) - 1) >> bin_log2) != bins_y)
        return CR_ERR_INVALID_ARGUMENT;
    if (reinterpret_cast<uintptr_t>(logs) & 7) return CR_ERR_INVALID_ARGUMENT;
    const int nb = bins_x * bins_y;
    cudaStream_t s = (cudaStream_t)stream;
    // The two 64-bit totals live in the 16 bytes behind the 2nb + 2 floats.
    unsigned long long* totals = reinterpret_cast<unsigned long long*>(logs + 2 * nb + 2);
    if (cudaMemsetAsync(totals, 0, 16, s) != cudaSuccess) return CR_ERR_CUDA;
    queueLogKernel<<<(nb * 32 + 255) / 256, 256, 0, s>>>(bin_counts, tile_counts, bins_x, bins_y, tiles_x, tiles_y,
                                                         bin_log2, logs, totals);
    totalLogKernel<<<1, 32, 0, s>>>(totals, logs + 2 * nb);
    return cudaGetLastError() == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

cr_status cr_queue_targets(const float* logs_prevprev, const float* logs_prev, const float* logs_cur, int32_t n,
                           int32_t n_trend, float* target, void* stream) {
    if (!logs_prev || !logs_cur || !target || n <= 0 || n_trend < 0 || n_trend > n) return CR_ERR_INVALID_ARGUMENT;
    targetsKernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(logs_prevprev, logs_prev, logs_cur, n, n_trend,
                                                                      target);
    return cudaGetLastError() == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

cr_status cr_queue_plan(const float* logs_prevprev, const float* logs_prev, const float* prediction, int32_t num_bins,
                        float* per_bin, double* totals, void* stream) {
    if (!logs_prev || !prediction || !totals || num_bins <= 0) return CR_ERR_INVALID_ARGUMENT;
    queuePlanKernel<<<1, 1024, 0, (cudaStream_t)stream>>>(logs_prevprev, logs_prev, prediction, num_bins, per_bin,
                                                         totals);
    return cudaGetLastError() == cudaSuccess ? CR_OK : CR_ERR_CUDA;
}

}  // extern "C"
