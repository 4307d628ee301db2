// Environment importance-sampling table built on the GPU from FP64 prefix sums.
//
// Replaces the CPU AliasMap::build (AliasMap.cpp:71-166, called from HGI/HGIImage.cpp:45-90
// after a GPU->CPU readback).  Same texel weights (luminance x solid angle of the texel's
// latitude row, luminance weights 0.2125/0.7154/0.0721), same per-texel pdf
// (luminance / integral of luminance over the sphere), and the same entry layout and sampling
// procedure, so Environment.slang:137-186 samples it unchanged.
//
// The table is built in parallel instead of by the reference's sequential sweep.  With the
// normalised weights p_i = N w_i / W, "light" texels (p < 1) and "heavy" texels (p >= 1) in index
// order, deficit prefix sums D (lights, 1 - p) and surplus prefix sums S (heavies, p - 1):
//   light k is aliased to the heavy j whose surplus interval contains D_k (S_j < D_k <= S_{j+1});
//   heavy j is exhausted by the light whose deficit interval crosses S_{j+1}, keeps probability
//   1 + S_{j+1} - D_after and aliases heavy j + 1.
// This is the greedy sweep of Vose's method with the state expressed through prefix sums, so each
// entry is independent: one binary search per texel.  All prefix sums are FP64.
#include "agb_kernels.h"

namespace agb
{

namespace
{

constexpr int kScanThreads = 256;
constexpr int kScanItems   = 4;
constexpr int kScanTile    = kScanThreads * kScanItems;

// Exclusive block scan of one double per thread (fixed summation order); the block total is
// returned through `total`.
__device__ double blockExclusiveScan(double v, double& total)
{
    constexpr int kWarps = kScanThreads / 32;
    __shared__ double warpOffset[kWarps];
    __shared__ double blockTotal;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double incl = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1)
    {
        double t = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off)
            incl += t;
    }
    double exw = __shfl_up_sync(0xffffffffu, incl, 1);
    if (lane == 0)
        exw = 0.0;
    if (lane == 31)
        warpOffset[warp] = incl;
    __syncthreads();
    if (warp == 0)
    {
        double ws = lane < kWarps ? warpOffset[lane] : 0.0;
        double wi = ws;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1)
        {
            double t = __shfl_up_sync(0xffffffffu, wi, off);
            if (lane >= off)
                wi += t;
        }
        double we = __shfl_up_sync(0xffffffffu, wi, 1);
        if (lane == 0)
            we = 0.0;
        if (lane < kWarps)
            warpOffset[lane] = we;
        if (lane == kWarps - 1)
            blockTotal = wi;
    }
    __syncthreads();
    double excl = warpOffset[warp] + exw;
    total       = blockTotal;
    __syncthreads();
    return excl;
}

// Per texel: luminance (FP32, reference arithmetic) and weight = luminance x solid angle (FP64).
__global__ void k_env_weights(const float4* rgba, uint32_t width, uint32_t height, float* lum,
    double* weight, double* blockSum)
{
    uint32_t n    = width * height;
    uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    double local  = 0.0;
    const double kPiD   = 3.14159265358979323846;
    const double lonInc = 2.0 * kPiD / double(width);
    const double latInc = kPiD / double(height);
    for (int q = 0; q < kScanItems; q++)
    {
        uint32_t i = base + q;
        if (i >= n)
            break;
        float4 c = rgba[i];
        // glm::dot order: (r * 0.2125 + g * 0.7154) + b * 0.0721, no contraction.
        float l = __fadd_rn(__fadd_rn(__fmul_rn(c.x, 0.2125f), __fmul_rn(c.y, 0.7154f)),
            __fmul_rn(c.z, 0.0721f));
        uint32_t y   = i / width;
        double upper = 0.5 * kPiD - double(y) * latInc;
        double sa    = (sin(upper) - sin(upper - latInc)) * lonInc;
        double w     = double(l) * sa;
        lum[i]    = l;
        weight[i] = w;
        local += w;
    }
    double total;
    blockExclusiveScan(local, total);
    if (threadIdx.x == 0)
        blockSum[blockIdx.x] = total;
}

// Single block: exclusive scan over the per-tile values (in place), total to out[count].
__global__ void k_scan_tiles(double* v, uint32_t count, double* totalOut)
{
    double carry = 0.0;
    for (uint32_t b = 0; b < count; b += kScanThreads)
    {
        uint32_t i = b + threadIdx.x;
        double x   = i < count ? v[i] : 0.0;
        double total;
        double e = blockExclusiveScan(x, total);
        if (i < count)
            v[i] = carry + e;
        carry += total;
    }
    if (threadIdx.x == 0 && totalOut)
        *totalOut = carry;
}
__global__ void k_scan_tiles_u32(uint32_t* v, uint32_t count, uint32_t* totalOut)
{
    uint32_t carry = 0;
    for (uint32_t b = 0; b < count; b += kScanThreads)
    {
        uint32_t i = b + threadIdx.x;
        uint32_t x = i < count ? v[i] : 0u;
        double total;
        double e = blockExclusiveScan(double(x), total); // exact: counts are far below 2^53
        if (i < count)
            v[i] = carry + uint32_t(e);
        carry += uint32_t(total);
    }
    if (threadIdx.x == 0 && totalOut)
        *totalOut = carry;
}

// Classifies texels and computes per-tile sums of deficits, surpluses and light counts.
__global__ void k_env_classify(const double* weight, uint32_t n, const double* integral,
    double* p, double* tileDef, double* tileSur, uint32_t* tileLights)
{
    uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    double W      = *integral;
    double def = 0.0, sur = 0.0;
    uint32_t lights = 0;
    for (int q = 0; q < kScanItems; q++)
    {
        uint32_t i = base + q;
        if (i >= n)
            break;
        double pi = W > 0.0 ? weight[i] * double(n) / W : 1.0;
        p[i]      = pi;
        if (pi < 1.0)
        {
            def += 1.0 - pi;
            lights++;
        }
        else
            sur += pi - 1.0;
    }
    double t;
    blockExclusiveScan(def, t);
    if (threadIdx.x == 0)
        tileDef[blockIdx.x] = t;
    blockExclusiveScan(sur, t);
    if (threadIdx.x == 0)
        tileSur[blockIdx.x] = t;
    blockExclusiveScan(double(lights), t);
    if (threadIdx.x == 0)
        tileLights[blockIdx.x] = uint32_t(t);
}

// Element-level exclusive scans with tile offsets; scatters light / heavy prefix arrays.
__global__ void k_env_scatter(const double* p, uint32_t n, const double* tileDef,
    const double* tileSur, const uint32_t* tileLights, uint32_t* rankOut, double* lightIncl,
    double* heavyIncl, uint32_t* heavyIdx)
{
    uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    double pv[kScanItems];
    double def = 0.0, sur = 0.0;
    uint32_t lights = 0;
    for (int q = 0; q < kScanItems; q++)
    {
        uint32_t i = base + q;
        pv[q]      = i < n ? p[i] : 1.0;
        if (i < n)
        {
            if (pv[q] < 1.0)
            {
                def += 1.0 - pv[q];
                lights++;
            }
            else
                sur += pv[q] - 1.0;
        }
    }
    double t;
    double defE = blockExclusiveScan(def, t) + tileDef[blockIdx.x];
    double surE = blockExclusiveScan(sur, t) + tileSur[blockIdx.x];
    uint32_t lightE = uint32_t(blockExclusiveScan(double(lights), t)) + tileLights[blockIdx.x];
    for (int q = 0; q < kScanItems; q++)
    {
        uint32_t i = base + q;
        if (i >= n)
            break;
        if (pv[q] < 1.0)
        {
            defE += 1.0 - pv[q];
            lightIncl[lightE] = defE;
            rankOut[i]        = lightE;
            lightE++;
        }
        else
        {
            uint32_t h = i - lightE;
            surE += pv[q] - 1.0;
            heavyIncl[h] = surE;
            heavyIdx[h]  = i;
            rankOut[i]   = h;
        }
    }
}

// First index in a[0, count) with a[idx] >= x (strict: a[idx] > x), or count.
__device__ uint32_t lowerBound(const double* a, uint32_t count, double x, bool strict)
{
    uint32_t lo = 0, hi = count;
    while (lo < hi)
    {
        uint32_t mid = (lo + hi) >> 1;
        bool go      = strict ? (a[mid] <= x) : (a[mid] < x);
        if (go)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

__global__ void k_env_alias(const double* p, const float* lum, uint32_t n, const double* integral,
    const uint32_t* rank, const double* lightIncl,
    const double* heavyIncl, const uint32_t* heavyIdx, const uint32_t* lightCountPtr,
    agb_alias_entry* out)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double W        = *integral;
    uint32_t lights = *lightCountPtr;
    uint32_t heavies = n - lights;
    agb_alias_entry e;
    e._padding1 = 0.f;
    e.pdf       = W > 0.0 ? lum[i] / float(W) : 0.f;
    double pi   = p[i];
    if (W <= 0.0 || heavies == 0)
    {
        e.alias = i;
        e.prob  = 1.f;
    }
    else if (pi < 1.0)
    {
        // The deficit consumed before light k is the previous light's inclusive prefix, so light
        // and heavy searches read the same FP64 values.
        uint32_t k = rank[i];
        double Dk  = k == 0 ? 0.0 : lightIncl[k - 1];
        uint32_t j = lowerBound(heavyIncl, heavies, Dk, false);
        j          = j < heavies ? j : heavies - 1;
        e.alias    = heavyIdx[j];
        e.prob     = float(pi);
    }
    else
    {
        uint32_t j = rank[i];
        e.alias    = i;
        e.prob     = 1.f;
        if (j + 1 < heavies)
        {
            double X   = heavyIncl[j];
            uint32_t k = lowerBound(lightIncl, lights, X, true);
            if (k < lights)
            {
                double r = 1.0 + X - lightIncl[k];
                e.prob   = float(r < 0.0 ? 0.0 : r);
                e.alias  = heavyIdx[j + 1];
            }
        }
    }
    out[i] = e;
}

// ---------------------------------------------------------------- reference table layout
// The reference's table (AliasMap.cpp:71-166) rebuilt bit for bit: FP32 luminance x row solid
// angle (row angles from the host, as the reference computes them), FP32 sequential integral, the
// same index map (below-average texels first in index order, the others from the end), and the
// same sequential sweep.  The sweep is inherently sequential; one warp runs it, lanes prefetching
// the next windows of the small and large queues into shared memory while lane 0 consumes them.

__global__ void k_ref_lum(const float4* rgba, uint32_t width, uint32_t n, const float* rowSA,
    float* lum, float* lumArea)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float4 c = rgba[i];
    float l  = __fadd_rn(__fadd_rn(__fmul_rn(c.x, 0.2125f), __fmul_rn(c.y, 0.7154f)),
        __fmul_rn(c.z, 0.0721f));
    lum[i]     = l;
    lumArea[i] = __fmul_rn(rowSA[i / width], l);
}

// One warp: FP32 sum of v[0, n) in index order, as a sequential loop would compute it.
__global__ void k_ref_seq_sum(const float* v, uint32_t n, float* out)
{
    constexpr uint32_t kChunk = 4096;
    __shared__ float buf[kChunk];
    int lane  = threadIdx.x;
    float acc = 0.f;
    for (uint32_t base = 0; base < n; base += kChunk)
    {
        uint32_t cnt = n - base < kChunk ? n - base : kChunk;
        for (uint32_t k = lane; k < cnt; k += 32)
            buf[k] = v[base + k];
        __syncwarp();
        if (lane == 0)
            for (uint32_t k = 0; k < cnt; k++)
                acc = __fadd_rn(acc, buf[k]);
        __syncwarp();
    }
    if (lane == 0)
        *out = acc;
}

__global__ void k_ref_probs(const float* lum, const float* lumArea, uint32_t n,
    const float* integral, float* prob, float* pdf, uint32_t* alias, uint32_t* tileSmall)
{
    uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    float I       = *integral;
    float average = __fdiv_rn(I, float(n));
    uint32_t smalls = 0;
    for (int q = 0; q < kScanItems; q++)
    {
        uint32_t i = base + q;
        if (i >= n)
            break;
        float pr = __fdiv_rn(lumArea[i], average);
        prob[i]  = pr;
        pdf[i]   = __fdiv_rn(lum[i], I);
        alias[i] = i;
        smalls += pr < 1.f ? 1u : 0u;
    }
    double t;
    blockExclusiveScan(double(smalls), t);
    if (threadIdx.x == 0)
        tileSmall[blockIdx.x] = uint32_t(t);
}

__global__ void k_ref_index(const float* prob, uint32_t n, const uint32_t* tileSmallExcl,
    uint32_t* indexMap)
{
    uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t smalls = 0;
    bool isSmall[kScanItems];
    for (int q = 0; q < kScanItems; q++)
    {
        uint32_t i = base + q;
        isSmall[q] = i < n && prob[i] < 1.f;
        smalls += isSmall[q] ? 1u : 0u;
    }
    double t;
    uint32_t before = uint32_t(blockExclusiveScan(double(smalls), t)) + tileSmallExcl[blockIdx.x];
    for (int q = 0; q < kScanItems; q++)
    {
        uint32_t i = base + q;
        if (i >= n)
            break;
        if (isSmall[q])
            indexMap[before++] = i;
        else
            indexMap[n - 1 - (i - before)] = i; // k-th large (index order) at position n-1-k
    }
}

// The sweep: for (sml = 0; sml < lrg && lrg < n; sml++) pair indexMap[sml] with indexMap[lrg].
__global__ void k_ref_sweep(const uint32_t* indexMap, float* prob, uint32_t* alias, uint32_t n,
    const uint32_t* smallCount)
{
    constexpr int kWin = 256; // queue window per batch (8 entries per lane)
    __shared__ uint32_t sIdx[kWin], lIdx[kWin];
    __shared__ float sProb[kWin], lProb[kWin];
    __shared__ uint8_t sFinal[kWin];
    __shared__ uint32_t st[3]; // sml, lrg, done
    int lane = threadIdx.x;
    uint32_t S = *smallCount;
    uint32_t curLarge = 0;
    float w = 0.f;
    if (lane == 0)
    {
        st[0] = 0;
        st[1] = S;
        st[2] = (S == 0 || S >= n) ? 1u : 0u;
        if (!st[2])
        {
            curLarge = indexMap[S];
            w        = prob[curLarge];
        }
    }
    __syncwarp();
    while (!st[2])
    {
        uint32_t sml = st[0], lrg = st[1];
        // Prefetch the small-queue window [sml, sml + kWin) and the large-queue window
        // (lrg, lrg + kWin].  Small entries below S never change; entries at positions in
        // [S, lrg) are larges already exhausted, whose probability is final.
        for (int k = lane; k < kWin; k += 32)
        {
            uint32_t ps = sml + uint32_t(k);
            if (ps < n)
            {
                uint32_t idx = indexMap[ps];
                sIdx[k]      = idx;
                bool fin     = ps < S || ps < lrg;
                sFinal[k]    = fin ? 1 : 0;
                sProb[k]     = fin ? prob[idx] : 0.f;
            }
            uint32_t pl = lrg + 1u + uint32_t(k);
            if (pl < n)
            {
                uint32_t idx = indexMap[pl];
                lIdx[k]      = idx;
                lProb[k]     = prob[idx]; // untouched until it becomes the current large
            }
        }
        __syncwarp();
        if (lane == 0)
        {
            int si = 0, li = 0;
            while (si < kWin && li < kWin)
            {
                if (!(sml < lrg && lrg < n))
                {
                    st[2] = 1;
                    break;
                }
                uint32_t small = sIdx[si];
                float ps       = sFinal[si] ? sProb[si] : prob[small];
                alias[small]   = curLarge;
                w              = __fsub_rn(w, __fsub_rn(1.f, ps));
                if (w < 1.f)
                {
                    prob[curLarge] = w;
                    lrg++;
                    if (lrg < n)
                    {
                        curLarge = lIdx[li];
                        w        = lProb[li];
                        li++;
                    }
                }
                sml++;
                si++;
            }
            st[0] = sml;
            st[1] = lrg;
            if (lrg >= n || sml >= lrg)
                st[2] = 1;
            if (st[2] && lrg < n)
                prob[curLarge] = w;
        }
        __syncwarp();
    }
}

__global__ void k_ref_pack(const uint32_t* alias, const float* prob, const float* pdf, uint32_t n,
    agb_alias_entry* out)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    agb_alias_entry e;
    e.alias     = alias[i];
    e.prob      = prob[i];
    e.pdf       = pdf[i];
    e._padding1 = 0.f;
    out[i]      = e;
}

} // namespace

void freeEnvScratch(EnvBuildScratch& s)
{
    cudaFree(s.weights);
    cudaFree(s.scanA);
    cudaFree(s.ranks);
    cudaFree(s.heavyIdx);
    cudaFree(s.heavyIncl);
    cudaFree(s.lightIncl);
    cudaFree(s.blockSums);
    cudaFree(s.blockCounts);
    cudaFree(s.rowSA);
    s = EnvBuildScratch();
}

size_t envScratchTileDoubles(uint32_t texels) { return size_t((texels + kScanTile - 1) / kScanTile) * 3 + 8; }
size_t envScratchTileCounts(uint32_t texels) { return size_t((texels + kScanTile - 1) / kScanTile) + 8; }

cudaError_t buildEnvAlias(const float4* rgba, uint32_t width, uint32_t height, int layout,
    const float* rowSolidAngle, agb_alias_entry* out, double* integralFP64Out,
    float* integralShadingOut, EnvBuildScratch& s, cudaStream_t st)
{
    uint32_t n     = width * height;
    uint32_t tiles = (n + kScanTile - 1) / kScanTile;
    if (s.capacity < n || s.rows < height)
    {
        freeEnvScratch(s);
        size_t tileCap = envScratchTileDoubles(n);
        cudaError_t e  = cudaSuccess;
        if ((e = cudaMalloc(&s.weights, sizeof(double) * n)) != cudaSuccess ||
            (e = cudaMalloc(&s.scanA, sizeof(double) * n)) != cudaSuccess ||
            (e = cudaMalloc(&s.ranks, sizeof(uint32_t) * n * 2)) != cudaSuccess ||
            (e = cudaMalloc(&s.heavyIdx, sizeof(uint32_t) * n)) != cudaSuccess ||
            (e = cudaMalloc(&s.heavyIncl, sizeof(double) * n)) != cudaSuccess ||
            (e = cudaMalloc(&s.lightIncl, sizeof(double) * n)) != cudaSuccess ||
            (e = cudaMalloc(&s.blockSums, sizeof(double) * tileCap)) != cudaSuccess ||
            (e = cudaMalloc(&s.blockCounts, sizeof(uint32_t) * envScratchTileCounts(n))) != cudaSuccess ||
            (e = cudaMalloc(&s.rowSA, sizeof(float) * height + 16)) != cudaSuccess)
        {
            freeEnvScratch(s);
            return e;
        }
        s.capacity = n;
        s.rows     = height;
    }
    return launchEnvAliasBuild(rgba, width, height, layout, rowSolidAngle, out, integralFP64Out,
        integralShadingOut, s, st);
}

cudaError_t launchEnvAliasBuild(const float4* rgba, uint32_t width, uint32_t height, int layout,
    const float* rowSolidAngle, agb_alias_entry* out, double* integralFP64Out,
    float* integralShadingOut, const EnvBuildScratch& s, cudaStream_t st)
{
    uint32_t n       = width * height;
    uint32_t tiles   = (n + kScanTile - 1) / kScanTile;
    float* lum       = reinterpret_cast<float*>(s.ranks + n); // second half of ranks
    double* tileW    = s.blockSums;
    double* tileDef  = s.blockSums + tiles;
    double* tileSur  = s.blockSums + 2 * tiles;
    double* integral = s.blockSums + 3 * tiles;
    uint32_t* lightCount = s.blockCounts + tiles;
    // FP64 luminance integral (always): prefix sums over luminance x solid angle.
    k_env_weights<<<tiles, kScanThreads, 0, st>>>(rgba, width, height, lum, s.weights, tileW);
    k_scan_tiles<<<1, kScanThreads, 0, st>>>(tileW, tiles, integral);
    float* shadingIntegral = reinterpret_cast<float*>(s.blockSums + 3 * tiles + 1);
    if (layout == 1)
    {
        k_env_classify<<<tiles, kScanThreads, 0, st>>>(s.weights, n, integral, s.scanA, tileDef,
            tileSur, s.blockCounts);
        k_scan_tiles<<<1, kScanThreads, 0, st>>>(tileDef, tiles, nullptr);
        k_scan_tiles<<<1, kScanThreads, 0, st>>>(tileSur, tiles, nullptr);
        k_scan_tiles_u32<<<1, kScanThreads, 0, st>>>(s.blockCounts, tiles, lightCount);
        k_env_scatter<<<tiles, kScanThreads, 0, st>>>(s.scanA, n, tileDef, tileSur, s.blockCounts,
            s.ranks, s.lightIncl, s.heavyIncl, s.heavyIdx);
        k_env_alias<<<(n + 255) / 256, 256, 0, st>>>(s.scanA, lum, n, integral, s.ranks,
            s.lightIncl, s.heavyIncl, s.heavyIdx, lightCount, out);
    }
    else
    {
        // Reference layout.  Scratch reuse: lumArea / prob / pdf in the FP64 weight arrays,
        // alias / index map in the FP64 prefix arrays.
        float* lumArea    = reinterpret_cast<float*>(s.scanA);
        float* prob       = reinterpret_cast<float*>(s.scanA) + n;
        float* pdf        = reinterpret_cast<float*>(s.heavyIncl);
        uint32_t* alias   = reinterpret_cast<uint32_t*>(s.heavyIncl) + n;
        uint32_t* indexMap = reinterpret_cast<uint32_t*>(s.lightIncl);
        uint32_t* smallCount = lightCount;
        if (rowSolidAngle)
        {
            cudaError_t e = cudaMemcpyAsync(s.rowSA, rowSolidAngle, sizeof(float) * height,
                cudaMemcpyHostToDevice, st);
            if (e != cudaSuccess)
                return e;
        }
        k_ref_lum<<<(n + 255) / 256, 256, 0, st>>>(rgba, width, n, s.rowSA, lum, lumArea);
        k_ref_seq_sum<<<1, 32, 0, st>>>(lumArea, n, shadingIntegral);
        k_ref_probs<<<tiles, kScanThreads, 0, st>>>(lum, lumArea, n, shadingIntegral, prob, pdf,
            alias, s.blockCounts);
        k_scan_tiles_u32<<<1, kScanThreads, 0, st>>>(s.blockCounts, tiles, smallCount);
        k_ref_index<<<tiles, kScanThreads, 0, st>>>(prob, n, s.blockCounts, indexMap);
        k_ref_sweep<<<1, 32, 0, st>>>(indexMap, prob, alias, n, smallCount);
        k_ref_pack<<<(n + 255) / 256, 256, 0, st>>>(alias, prob, pdf, n, out);
    }
    cudaError_t e = cudaMemcpyAsync(integralFP64Out, integral, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess)
        return e;
    if (layout != 1)
    {
        e = cudaMemcpyAsync(integralShadingOut, shadingIntegral, sizeof(float), cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess)
            return e;
    }
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return e;
    if (layout == 1)
        *integralShadingOut = float(*integralFP64Out);
    return cudaGetLastError();
}

} // namespace agb
