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

} // namespace

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
