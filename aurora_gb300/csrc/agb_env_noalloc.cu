// Environment alias-table build that allocates no device memory.
//
// The regular build (agb_environment_set) grows cudaMalloc'd scratch to the size of the light
// image.  Some callers cannot allocate at that point: a host that hands the whole device to its
// own allocator or to a fixed memory budget (a serving loop that admits work against an HBM
// budget cannot let a table rebuild take memory it did not plan for), and a host that must not
// stall its other streams (cudaMalloc and cudaFree can synchronise the device).  This variant
// runs the same kernels on one fixed scratch array that is part of the library's device image.
//
// The array lives in this file alone so that only processes that use this entry point carry it:
// the CUDA driver reserves a module's __device__ storage when it loads the module (at context
// creation with eager module loading, on first use with lazy loading).
#include "agb_kernels.h"

namespace agb
{
namespace
{

constexpr size_t kScratchAlign = 256;
constexpr size_t alignUp(size_t v) { return (v + kScratchAlign - 1) & ~(kScratchAlign - 1); }

// Sub-array layout of the scratch for at most kMax texels (and at most kMax rows).  The tile
// arrays follow the regular build's sizing: 3 doubles per 1024-texel tile + 8, one count per
// tile + 8.
constexpr uint32_t kMax        = AGB_ENV_NOALLOC_MAX_TEXELS;
constexpr size_t kTiles        = (size_t(kMax) + 1023) / 1024;
constexpr size_t kOffWeights   = 0;
constexpr size_t kOffScanA     = alignUp(kOffWeights + sizeof(double) * kMax);
constexpr size_t kOffRanks     = alignUp(kOffScanA + sizeof(double) * kMax);
constexpr size_t kOffHeavyIdx  = alignUp(kOffRanks + sizeof(uint32_t) * 2 * size_t(kMax));
constexpr size_t kOffHeavyIncl = alignUp(kOffHeavyIdx + sizeof(uint32_t) * kMax);
constexpr size_t kOffLightIncl = alignUp(kOffHeavyIncl + sizeof(double) * kMax);
constexpr size_t kOffBlockSums = alignUp(kOffLightIncl + sizeof(double) * kMax);
constexpr size_t kOffBlockCnt  = alignUp(kOffBlockSums + sizeof(double) * (kTiles * 3 + 8));
constexpr size_t kOffRowSA     = alignUp(kOffBlockCnt + sizeof(uint32_t) * (kTiles + 8));
constexpr size_t kScratchBytes = alignUp(kOffRowSA + sizeof(float) * (size_t(kMax) + 16));

} // namespace

// Nothing in it has to start at zero: every kernel of the build writes each scratch entry it
// later reads within the same call.
static __device__ __align__(256) unsigned char g_envNoAllocScratch[kScratchBytes];

namespace
{

// Device address of the scratch in the current device's context.  Looked up on every call (the
// lookup allocates nothing): a cached address would outlive a context reset (cudaDeviceReset, or
// a primary context released and retained again), after which the module's storage is reloaded
// at another address.
cudaError_t scratchAddress(unsigned char** out)
{
    unsigned char* p = nullptr;
    cudaError_t e    = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_envNoAllocScratch);
    if (e != cudaSuccess)
        return e;
    *out = p;
    return cudaSuccess;
}

} // namespace

cudaError_t buildEnvAliasNoAlloc(const float4* rgba, uint32_t width, uint32_t height, int layout,
    agb_alias_entry* out, double* integralFP64Out, float* integralShadingOut, cudaStream_t st)
{
    static_assert(kScratchBytes % kScratchAlign == 0, "scratch layout");
    uint64_t n = uint64_t(width) * height;
    if (width == 0 || height == 0 || n > kMax)
        return cudaErrorInvalidValue;
    if (envScratchTileDoubles(uint32_t(n)) > kTiles * 3 + 8 ||
        envScratchTileCounts(uint32_t(n)) > kTiles + 8)
        return cudaErrorInvalidValue;
    unsigned char* base = nullptr;
    cudaError_t e       = scratchAddress(&base);
    if (e != cudaSuccess)
        return e;
    EnvBuildScratch s;
    s.weights     = reinterpret_cast<double*>(base + kOffWeights);
    s.scanA       = reinterpret_cast<double*>(base + kOffScanA);
    s.ranks       = reinterpret_cast<uint32_t*>(base + kOffRanks);
    s.heavyIdx    = reinterpret_cast<uint32_t*>(base + kOffHeavyIdx);
    s.heavyIncl   = reinterpret_cast<double*>(base + kOffHeavyIncl);
    s.lightIncl   = reinterpret_cast<double*>(base + kOffLightIncl);
    s.blockSums   = reinterpret_cast<double*>(base + kOffBlockSums);
    s.blockCounts = reinterpret_cast<uint32_t*>(base + kOffBlockCnt);
    s.rowSA       = reinterpret_cast<float*>(base + kOffRowSA);
    s.capacity    = kMax;
    s.rows        = kMax;
    if (layout == AGB_ENV_TABLE_REFERENCE)
    {
        // Per-row solid angles with the reference's host arithmetic (AliasMap.cpp:101-110: FP32
        // increments, FP32 running latitude, float sin), staged through a stack buffer in
        // chunks.  A copy from pageable memory returns once the source has been consumed, so the
        // buffer can be refilled at once.
        constexpr uint32_t kChunk = 512;
        float rows[kChunk];
        const double kPi   = 3.14159265358979323846;
        float lonIncrement = static_cast<float>(2.0f * kPi / width);
        float latIncrement = static_cast<float>(kPi / height);
        float latAngle     = static_cast<float>(kPi / 2.0);
        for (uint32_t y0 = 0; y0 < height; y0 += kChunk)
        {
            uint32_t m = height - y0 < kChunk ? height - y0 : kChunk;
            for (uint32_t i = 0; i < m; i++)
            {
                rows[i] = (std::sin(latAngle) - std::sin(latAngle - latIncrement)) * lonIncrement;
                latAngle -= latIncrement;
            }
            e = cudaMemcpyAsync(s.rowSA + y0, rows, sizeof(float) * m, cudaMemcpyHostToDevice, st);
            if (e != cudaSuccess)
                return e;
        }
    }
    return launchEnvAliasBuild(rgba, width, height, layout, nullptr, out, integralFP64Out,
        integralShadingOut, s, st);
}

} // namespace agb
