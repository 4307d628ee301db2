// Denoiser tensor-core kernels (tcgen05, BF16 operands, FP32 accumulation in TMEM).
//
// k_tc_gemm: D[M x N] (FP32) = A[M x K] (BF16, row-major) x B[N x K]^T (BF16, row-major).  One CTA
// of 128 threads computes 128 rows x N columns (N <= 256): the K loop runs in chunks of 64 through
// two shared-memory stages; each thread stages one row of A per chunk, the B rows are spread over
// the threads; thread 0 issues four K16 MMAs per chunk and commits them to the stage's mbarrier,
// which the threads wait on before refilling that stage.  The epilogue reads the accumulator rows
// from TMEM (warp w owns lanes 32w..32w+31).
#include <algorithm>

#include <cuda_bf16.h>

#include "agb_kernels.h"
#include "agb_tc.cuh"

namespace agb
{

// Set by a kernel whose bounded wait ran out; read and cleared by the host after the launch.
__device__ int g_tcError;

namespace
{

constexpr int kGemmRows  = 128;
constexpr int kGemmChunk = 64; // K per pipeline stage (4 MMAs)

__global__ void __launch_bounds__(128) k_tc_gemm(const uint16_t* A, const uint16_t* B, float* D, int N,
    int K)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t bar[2];
    __shared__ uint32_t tmemBase;
    const int tid  = threadIdx.x;
    const int warp = tid >> 5;
    const uint32_t aBytes = kGemmRows * kGemmChunk * 2;
    const uint32_t bBytes = uint32_t(N) * kGemmChunk * 2;
    uint8_t* aS[2] = { smem, smem + aBytes + bBytes };
    uint8_t* bS[2] = { smem + aBytes, smem + 2 * aBytes + bBytes };
    const uint32_t cols = tc::tmemCols(uint32_t(N));
    if (warp == 0)
        tc::tmemAlloc(&tmemBase, cols);
    if (tid == 0)
    {
        tc::mbarInit(&bar[0], 1);
        tc::mbarInit(&bar[1], 1);
        tc::fenceMbarInit();
    }
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    const uint32_t tmem  = tmemBase;
    const uint32_t idesc = tc::idescBf16(kGemmRows, uint32_t(N));
    const size_t m0      = size_t(blockIdx.x) * kGemmRows;
    const int chunks     = K / kGemmChunk;
    uint32_t parity[2]   = { 0, 0 };
    bool ok              = true;
    for (int c = 0; c < chunks; c++)
    {
        const int s = c & 1;
        if (c >= 2)
        {
            ok = tc::mbarWait(&bar[s], parity[s]) && ok;
            parity[s] ^= 1u;
        }
        // A: this thread's row, 64 K values = 8 chunks of 8 elements (16 bytes).
        const uint4* arow = reinterpret_cast<const uint4*>(A + (m0 + tid) * size_t(K) + size_t(c) * kGemmChunk);
#pragma unroll
        for (int j = 0; j < 8; j++)
        {
            uint4 v = __ldg(arow + j);
            *reinterpret_cast<uint4*>(aS[s] + (j >> 1) * (kGemmRows * 32) + tc::sliceOffset(tid, (j & 1) * 8)) = v;
        }
        for (int r = tid; r < N; r += 128)
        {
            const uint4* brow = reinterpret_cast<const uint4*>(B + size_t(r) * K + size_t(c) * kGemmChunk);
#pragma unroll
            for (int j = 0; j < 8; j++)
            {
                uint4 v = __ldg(brow + j);
                *reinterpret_cast<uint4*>(bS[s] + (j >> 1) * (N * 32) + tc::sliceOffset(r, (j & 1) * 8)) = v;
            }
        }
        tc::fenceProxyAsync();
        __syncthreads();
        if (tid == 0)
        {
            tc::fenceAfterSync();
#pragma unroll
            for (int sl = 0; sl < 4; sl++)
            {
                uint64_t ad = tc::smemDesc(tc::smemAddr(aS[s] + sl * (kGemmRows * 32)), tc::kSliceLbo, tc::kSliceSbo);
                uint64_t bd = tc::smemDesc(tc::smemAddr(bS[s] + sl * (N * 32)), tc::kSliceLbo, tc::kSliceSbo);
                tc::mma(tmem, ad, bd, idesc, (c > 0 || sl > 0) ? 1u : 0u);
            }
            tc::commit(&bar[s]);
        }
        __syncwarp();
    }
    if (chunks > 0)
    {
        const int sl = (chunks - 1) & 1;
        ok           = tc::mbarWait(&bar[sl], parity[sl]) && ok;
    }
    tc::fenceAfterSync();
    const size_t row = m0 + size_t(warp) * 32 + (tid & 31);
    for (int c0 = 0; c0 < N; c0 += 16)
    {
        uint32_t r[16];
        tc::tmemLoad16(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0), r);
        tc::tmemWaitLoad();
        float4* out = reinterpret_cast<float4*>(D + row * N + c0);
#pragma unroll
        for (int j = 0; j < 4; j++)
            out[j] = make_float4(__uint_as_float(r[4 * j]), __uint_as_float(r[4 * j + 1]),
                __uint_as_float(r[4 * j + 2]), __uint_as_float(r[4 * j + 3]));
    }
    tc::fenceBeforeSync();
    __syncthreads();
    if (warp == 0)
        tc::tmemDealloc(tmem, cols);
    if (!ok && tid == 0)
        atomicExch(&g_tcError, 1);
}

// ------------------------------------------------------------------ weight gradient
// dW[tap][ci][co] += sum over pixels p of X[p + d(tap)][ci] * dY[p][co], X = concat(up(in0), in1) as
// in the forward pass.  GEMM with rows = input channels (128 per CTA, grid.z blocks), columns =
// Cout, K = pixels: grid.x splits the pixels (each CTA sums its range in TMEM and adds it to dW
// with FP32 reductions), grid.y is the tap.  NHWC stores a pixel's channels contiguously, which is
// the MN-major operand layout: both operands are staged as 16-byte rows of 8 channels of one
// pixel, no transpose.  Core matrix (channel group m, pixel group k) of a K16 slice sits at byte
// (m * 2 + k) * 128 with its 8 pixel rows 16 bytes apart; the MN-major descriptors give 128 (the
// leading byte offset) between pixel groups and 256 (the stride byte offset) between channel
// groups.

struct WgradArgs
{
    const uint16_t* in0;
    const uint16_t* in1;
    const uint16_t* dy;  // [B][H][W][Cout]
    float* dw;           // [9][Cin][Cout], accumulated
    int B, H, W, C0, C1, Cout, up0;
    int chunksPerSplit;  // 64-pixel chunks per CTA
};

// Byte offset of channel group `group` (8 channels) of pixel k (k in [0, 16)) in an MN-major K16
// slice.
__device__ __forceinline__ uint32_t mnOffset(uint32_t group, uint32_t k)
{
    return (group * 2 + (k >> 3)) * tc::kCoreBytes + (k & 7) * 16;
}

__global__ void __launch_bounds__(128) k_conv_wgrad(WgradArgs a)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t mmaBar[2];
    __shared__ uint32_t tmemBase;
    const int tid  = threadIdx.x;
    const int warp = tid >> 5;
    const int Cin  = a.C0 + a.C1;
    const int N    = a.Cout;
    const uint32_t aStage = 4 * 128 * 32;
    const uint32_t bSlice = uint32_t(N) * 32;
    const uint32_t bStage = 4 * bSlice;
    uint8_t* aS[2] = { smem, smem + aStage + bStage };
    uint8_t* bS[2] = { smem + aStage, smem + 2 * aStage + bStage };
    const long P         = long(a.B) * a.H * a.W;
    const long total     = (P + 63) / 64;
    const long first     = long(blockIdx.x) * a.chunksPerSplit;
    const int chunks     = int(min(long(a.chunksPerSplit), total - first));
    if (chunks <= 0)
        return;
    const uint32_t cols = tc::tmemCols(uint32_t(N));
    if (warp == 0)
        tc::tmemAlloc(&tmemBase, cols);
    if (tid == 0)
    {
        tc::mbarInit(&mmaBar[0], 1);
        tc::mbarInit(&mmaBar[1], 1);
        tc::fenceMbarInit();
    }
    tc::fenceBeforeSync();
    __syncthreads();
    tc::fenceAfterSync();
    const uint32_t tmem  = tmemBase;
    // MN-major A and B (instruction descriptor bits 15 and 16).
    const uint32_t idesc = tc::idescBf16(128, uint32_t(N)) | (1u << 15) | (1u << 16);
    const int tap = blockIdx.y, oy = tap / 3 - 1, ox = tap % 3 - 1;
    const int ci0 = blockIdx.z * 128;
    const int j   = tid & 63, hh = tid >> 6;
    uint32_t parity[2] = { 0, 0 };
    bool ok = true;
    for (int c = 0; c < chunks; c++)
    {
        const int s = c & 1;
        if (c >= 2)
        {
            ok = tc::mbarWait(&mmaBar[s], parity[s]) && ok;
            parity[s] ^= 1u;
        }
        const long p = (first + c) * 64 + j;
        uint8_t* aSl = aS[s] + (j >> 4) * (128 * 32);
        uint8_t* bSl = bS[s] + (j >> 4) * bSlice;
        const int k  = j & 15;
        // A rows: input channels ci0 + hh * 64 + [0, 64) at the tap-shifted pixel.
        bool inImg = false;
        int b = 0, yy = 0, xx = 0;
        if (p < P)
        {
            int x  = int(p % a.W);
            long t = p / a.W;
            int y  = int(t % a.H);
            b      = int(t / a.H);
            yy     = y + oy;
            xx     = x + ox;
            inImg  = yy >= 0 && yy < a.H && xx >= 0 && xx < a.W;
        }
#pragma unroll
        for (int g = 0; g < 8; g++)
        {
            int ci  = ci0 + hh * 64 + g * 8;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (inImg && ci < Cin)
            {
                const uint16_t* src;
                if (ci < a.C0)
                {
                    int h0 = a.up0 ? a.H >> 1 : a.H, w0 = a.up0 ? a.W >> 1 : a.W;
                    int y0 = a.up0 ? yy >> 1 : yy, x0 = a.up0 ? xx >> 1 : xx;
                    src = a.in0 + ((size_t(b) * h0 + y0) * w0 + x0) * a.C0 + ci;
                }
                else
                    src = a.in1 + ((size_t(b) * a.H + yy) * a.W + xx) * a.C1 + (ci - a.C0);
                v = __ldg(reinterpret_cast<const uint4*>(src));
            }
            *reinterpret_cast<uint4*>(aSl + mnOffset(uint32_t(hh * 8 + g), uint32_t(k))) = v;
        }
        // B rows: output channels hh * N / 2 + [0, N / 2) at the pixel itself.
        for (int g = 0; g < N / 16; g++)
        {
            int co  = hh * (N / 2) + g * 8;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (p < P)
                v = __ldg(reinterpret_cast<const uint4*>(a.dy + size_t(p) * N + co));
            *reinterpret_cast<uint4*>(bSl + mnOffset(uint32_t(co / 8), uint32_t(k))) = v;
        }
        tc::fenceProxyAsync();
        __syncthreads();
        if (tid == 0)
        {
            tc::fenceAfterSync();
#pragma unroll
            for (int sl = 0; sl < 4; sl++)
            {
                uint64_t ad = tc::smemDesc(tc::smemAddr(aS[s] + sl * (128 * 32)), 128, 256);
                uint64_t bd = tc::smemDesc(tc::smemAddr(bS[s] + sl * bSlice), 128, 256);
                tc::mma(tmem, ad, bd, idesc, (c > 0 || sl > 0) ? 1u : 0u);
            }
            tc::commit(&mmaBar[s]);
        }
        __syncwarp();
    }
    {
        const int sl = (chunks - 1) & 1;
        ok           = tc::mbarWait(&mmaBar[sl], parity[sl]) && ok;
    }
    tc::fenceAfterSync();
    const int ci = ci0 + warp * 32 + (tid & 31);
    for (int c0 = 0; c0 < N; c0 += 16)
    {
        uint32_t r[16];
        tc::tmemLoad16(tmem + (uint32_t(warp * 32) << 16) + uint32_t(c0), r);
        tc::tmemWaitLoad();
        if (ci < Cin)
        {
            float* dst = a.dw + (size_t(tap) * Cin + ci) * N + c0;
#pragma unroll
            for (int q = 0; q < 16; q++)
                atomicAdd(dst + q, __uint_as_float(r[q]));
        }
    }
    tc::fenceBeforeSync();
    __syncthreads();
    if (warp == 0)
        tc::tmemDealloc(tmem, cols);
    if (!ok && tid == 0)
        atomicExch(&g_tcError, 1);
}

} // namespace

cudaError_t launchConvWgrad(const ConvLaunch& c, const uint16_t* dy, float* dw, int smCount, cudaStream_t st)
{
    int Cin = c.C0 + c.C1;
    WgradArgs a{ c.in0, c.in1, dy, dw, c.B, c.H, c.W, c.C0, c.C1, c.Cout, c.up0, 1 };
    long P      = long(c.B) * c.H * c.W;
    long chunks = (P + 63) / 64;
    int mblocks = (Cin + 127) / 128;
    long want   = std::max(1L, long(smCount) * 2 / (9L * mblocks));
    long splits = std::min(chunks, want);
    a.chunksPerSplit = int((chunks + splits - 1) / splits);
    splits           = (chunks + a.chunksPerSplit - 1) / a.chunksPerSplit;
    size_t smem = 2 * (size_t(4) * 128 * 32 + size_t(4) * c.Cout * 32);
    cudaError_t e = cudaFuncSetAttribute(k_conv_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess)
        return e;
    k_conv_wgrad<<<dim3(unsigned(splits), 9, unsigned(mblocks)), 128, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launchTcGemm(const uint16_t* A, const uint16_t* B, float* D, int M, int N, int K, cudaStream_t st)
{
    size_t smem = 2 * (size_t(kGemmRows) * kGemmChunk * 2 + size_t(N) * kGemmChunk * 2);
    cudaError_t e = cudaFuncSetAttribute(k_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess)
        return e;
    k_tc_gemm<<<M / kGemmRows, 128, smem, st>>>(A, B, D, N, K);
    return cudaGetLastError();
}

cudaError_t takeTcError(int* flag)
{
    cudaError_t e = cudaMemcpyFromSymbol(flag, g_tcError, sizeof(int));
    if (e != cudaSuccess || *flag == 0)
        return e;
    int zero = 0;
    return cudaMemcpyToSymbol(g_tcError, &zero, sizeof(int));
}

cudaError_t tcErrorFlag(int** flag) { return cudaGetSymbolAddress(reinterpret_cast<void**>(flag), g_tcError); }

} // namespace agb
