// Batched entry points over device arrays, used to check the device code against the oracle one
// function at a time (BSDF eval / sample / pdf, ray casts, environment sampling, random numbers),
// and the post-processing pass (HGI/Shaders/PostProcessing.glsl:37-64).
#include "agb_kernels.h"

namespace agb
{

namespace
{

__device__ Mat matFromBlock(const agb_material& b)
{
    Mat m;
    m.b                 = &b;
    m.baseColor         = ld3(b.base_color);
    m.specularRoughness = b.specular_roughness;
    m.coatRoughness     = b.coat_roughness;
    m.emissionColor     = ld3(b.emission_color);
    m.opacity           = ld3(b.opacity);
    return m;
}

__global__ void k_bsdf_batch(int op, const agb_material* mats, const int32_t* mi,
    const float* frames, const float* V, const float* L, const float* rnd, int64_t n,
    float* outValue, float* outDir, float* outPdf, int32_t* outLobe)
{
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    Mat m    = matFromBlock(mats[mi[i]]);
    Frame fr = Frame{ ld3(frames + 12 * i), ld3(frames + 12 * i + 3), ld3(frames + 12 * i + 6) };
    v3 v     = ld3(V + 3 * i);
    v3 res;
    if (op == 0)
        res = evaluateMaterial(m, fr, v, ld3(L + 3 * i));
    else if (op == 1)
    {
        v3 lw;
        float pdf;
        int lobe;
        res = sampleMaterial(m, fr, v, v2{ rnd[2 * i], rnd[2 * i + 1] }, lw, pdf, lobe);
        outDir[3 * i]     = lw.x;
        outDir[3 * i + 1] = lw.y;
        outDir[3 * i + 2] = lw.z;
        outPdf[i]         = pdf;
        outLobe[i]        = lobe;
    }
    else
    {
        float pdf;
        int lobe;
        res = evaluateMaterialAndPDF(m, fr, v, ld3(L + 3 * i), v2{ rnd[2 * i], rnd[2 * i + 1] },
            pdf, lobe);
        outPdf[i]  = pdf;
        outLobe[i] = lobe;
    }
    outValue[3 * i]     = res.x;
    outValue[3 * i + 1] = res.y;
    outValue[3 * i + 2] = res.z;
}

extern __shared__ int32_t u_stack[];

struct BatchRayLoader
{
    const float* rays;
    AGB_D void operator()(uint32_t i, v3& o, v3& d, float& tmin, float& tmax) const
    {
        const float* r = rays + 8 * size_t(i);
        o    = v3{ r[0], r[1], r[2] };
        d    = v3{ r[4], r[5], r[6] };
        tmin = fmaxf(r[3], 0.f); // a negative tmin is taken as 0, as TraceRay requires TMin >= 0
        tmax = r[7];
    }
};
struct BatchHitWriter
{
    float* tuv;
    int32_t* ip;
    AGB_D void operator()(uint32_t i, bool hit, const RayHit& h) const
    {
        tuv[3 * size_t(i)]     = hit ? h.t : -1.f;
        tuv[3 * size_t(i) + 1] = hit ? h.u : 0.f;
        tuv[3 * size_t(i) + 2] = hit ? h.v : 0.f;
        ip[2 * size_t(i)]      = hit ? h.inst : -1;
        ip[2 * size_t(i) + 1]  = hit ? h.prim : -1;
    }
};

// Same persistent traversal as the renderer's trace kernels.
template <bool kAnyHit>
__global__ void __launch_bounds__(kTraceBlock) k_intersect_batch(DevScene s, const float* rays,
    uint32_t n, uint32_t* work, float* outTUV, int32_t* outIP, unsigned long long* overflowCount)
{
    TraceCounters c = { 0, 0 };
    bool overflow   = false;
    persistentTrace<kAnyHit, false>(s, n, work, BatchRayLoader{ rays }, BatchHitWriter{ outTUV, outIP },
        u_stack + threadIdx.x, kTraceBlock, c, overflow);
    if (overflow)
        atomicAdd(overflowCount, 1ull);
}

__global__ void k_env_sample_batch(DevScene s, const float* rnd, int64_t n, float* outR,
    float* outD, float* outPdf)
{
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    v3 L;
    float pdf;
    v3 r = sampleEnvironment(s, v2{ rnd[2 * i], rnd[2 * i + 1] }, L, pdf);
    outR[3 * i]     = r.x;
    outR[3 * i + 1] = r.y;
    outR[3 * i + 2] = r.z;
    outD[3 * i]     = L.x;
    outD[3 * i + 1] = L.y;
    outD[3 * i + 2] = L.z;
    outPdf[i]       = pdf;
}

__global__ void k_random_stream(uint32_t sampleIndex, uint32_t width, uint32_t px, uint32_t py,
    int n, float* out)
{
    if (blockIdx.x != 0 || threadIdx.x != 0)
        return;
    Rng r = rngInit(sampleIndex, width, px, py);
    for (int i = 0; i < n; i++)
    {
        v2 v           = random2D(r);
        out[2 * i]     = v.x;
        out[2 * i + 1] = v.y;
    }
}

// Colors.slang:33-53 / PostProcessing.glsl:15-64
__device__ float srgbApprox(float c)
{
    float s1 = sqrtf(c), s2 = sqrtf(s1), s3 = sqrtf(s2);
    return 0.662002687f * s1 + 0.684122060f * s2 - 0.323583601f * s3 - 0.0225411470f * c;
}
__device__ float aces(float c)
{
    return clampf((c * (2.51f * c + 0.03f)) / (c * (2.43f * c + 0.59f) + 0.14f), 0.f, 1.f);
}
__global__ void k_post(const float4* accum, const float4* comp, int mode, float invCount,
    uint32_t pixels, float3 brightness, int toneMap, int gamma, float4* out32, uchar4* out8)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= pixels)
        return;
    float4 a = accum[i];
    if (mode == AGB_ACCUM_KAHAN)
        a = make_float4(a.x * invCount, a.y * invCount, a.z * invCount, a.w * invCount);
    float c[3] = { a.x * brightness.x, a.y * brightness.y, a.z * brightness.z };
    for (int k = 0; k < 3; k++)
    {
        if (toneMap)
            c[k] = aces(c[k]);
        if (gamma)
            c[k] = srgbApprox(clampf(c[k], 0.f, 1.f));
    }
    if (out32)
        out32[i] = make_float4(c[0], c[1], c[2], 1.f);
    if (out8)
        out8[i] = make_uchar4((unsigned char)(clampf(c[0], 0.f, 1.f) * 255.f + 0.5f),
            (unsigned char)(clampf(c[1], 0.f, 1.f) * 255.f + 0.5f),
            (unsigned char)(clampf(c[2], 0.f, 1.f) * 255.f + 0.5f), 255);
}

} // namespace

cudaError_t launchBsdfBatch(int op, const agb_material* mats, const int32_t* matIndex,
    const float* frames, const float* V, const float* L, const float* rnd, int64_t n,
    float* outValue, float* outDir, float* outPdf, int32_t* outLobe, cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    k_bsdf_batch<<<unsigned((n + 127) / 128), 128, 0, st>>>(op, mats, matIndex, frames, V, L, rnd,
        n, outValue, outDir, outPdf, outLobe);
    return cudaGetLastError();
}

cudaError_t launchIntersectBatch(const DevScene& s, const float* rays, int64_t n, int anyHit,
    float* outTUV, int32_t* outInstPrim, uint32_t* work, unsigned long long* overflowCount,
    cudaStream_t st, int smCount)
{
    if (n <= 0)
        return cudaSuccess;
    size_t smem = kTraceStackBytes;
    int64_t blocks = (n + kTraceBlock - 1) / kTraceBlock;
    int grid       = int(blocks < int64_t(smCount) * 8 ? blocks : int64_t(smCount) * 8);
    cudaError_t e = cudaMemsetAsync(work, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess)
        return e;
    if (anyHit)
        k_intersect_batch<true><<<grid, kTraceBlock, smem, st>>>(s, rays, uint32_t(n), work, outTUV,
            outInstPrim, overflowCount);
    else
        k_intersect_batch<false><<<grid, kTraceBlock, smem, st>>>(s, rays, uint32_t(n), work, outTUV,
            outInstPrim, overflowCount);
    return cudaGetLastError();
}

cudaError_t launchEnvSampleBatch(const DevScene& s, const float* rnd, int64_t n,
    float* outRadiance, float* outDir, float* outPdf, cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    k_env_sample_batch<<<unsigned((n + 127) / 128), 128, 0, st>>>(s, rnd, n, outRadiance, outDir, outPdf);
    return cudaGetLastError();
}

cudaError_t launchRandomStream(uint32_t sampleIndex, uint32_t width, uint32_t px, uint32_t py,
    int n, float* out, cudaStream_t st)
{
    k_random_stream<<<1, 32, 0, st>>>(sampleIndex, width, px, py, n, out);
    return cudaGetLastError();
}

cudaError_t launchPostProcess(const float4* accum, const float* accumComp, int mode,
    float invCount, uint32_t pixels, float3 brightness, int toneMap, int gamma, float4* out32,
    uchar4* out8, cudaStream_t st)
{
    (void)accumComp;
    k_post<<<(pixels + 255) / 256, 256, 0, st>>>(accum, nullptr, mode, invCount, pixels, brightness,
        toneMap, gamma, out32, out8);
    return cudaGetLastError();
}

// relMSE of an accumulation against a reference: mean over pixels and RGB of (x - r)^2 / (r^2 + eps),
// x = accum * scale.  FP64 block sums, one atomic per block.
__global__ void k_rel_mse(const float4* accum, float scale, const float4* ref, uint32_t pixels, double eps,
    double* out)
{
    __shared__ double part[8];
    double s = 0.0;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < pixels; p += gridDim.x * blockDim.x)
    {
        float4 a = accum[p], r = ref[p];
        double x[3] = { double(a.x) * scale, double(a.y) * scale, double(a.z) * scale };
        double y[3] = { r.x, r.y, r.z };
        for (int k = 0; k < 3; k++)
            s += (x[k] - y[k]) * (x[k] - y[k]) / (y[k] * y[k] + eps);
    }
    for (int o = 16; o > 0; o >>= 1)
        s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0)
        part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        double t = 0.0;
        for (int w = 0; w < int(blockDim.x >> 5); w++)
            t += part[w];
        atomicAdd(out, t);
    }
}

cudaError_t launchRelMse(const float4* accum, float scale, const float4* ref, uint32_t pixels, double eps,
    double* out, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), st);
    if (e != cudaSuccess)
        return e;
    k_rel_mse<<<304, 256, 0, st>>>(accum, scale, ref, pixels, eps, out);
    return cudaGetLastError();
}

} // namespace agb
