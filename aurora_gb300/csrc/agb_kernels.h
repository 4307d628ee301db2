// Internal declarations shared by the CUDA translation units of libagb_cuda.
#pragma once

#include <string>
#include <vector>

#include "agb_wavefront.cuh"

namespace agb
{

constexpr int kTraceBlock       = 128; // threads per traversal block
#ifndef AGB_TRACE_BLOCKS
#define AGB_TRACE_BLOCKS 8
#endif
constexpr int kTraceBlocksPerSM = AGB_TRACE_BLOCKS; // x 128 threads x kSmemStack entries x 4 B of shared memory per SM
// Dynamic shared memory of a traversal block (its threads' shared-memory stacks).
constexpr size_t kTraceStackBytes = size_t(kSmemStack) * kTraceBlock * sizeof(int32_t);
// Shared-memory carveout (percent of the SM's 228 KB) that holds kTraceBlocksPerSM blocks' stacks
// (plus 1 KB reserved per block); the rest of the SM's L1 / shared storage stays L1 cache.
inline int traceCarveoutPercent()
{
    size_t need = size_t(kTraceBlocksPerSM) * (kTraceStackBytes + 1024);
    size_t pct  = (need * 100 + 228 * 1024 - 1) / (228 * 1024);
    return int(pct > 100 ? 100 : pct);
}
constexpr int kShadeBlock       = 128;
#ifndef AGB_SHADE_MIN_BLOCKS
#define AGB_SHADE_MIN_BLOCKS 16
#endif
// Resident shading blocks per SM the register budget is sized for.  The shading kernel waits on
// scattered loads (vertices, materials, textures, environment); full occupancy hides more of that
// latency than the registers it gives up (measured: 16 blocks of 128 threads beat 8 by 1.3x).
constexpr int kShadeMinBlocks   = AGB_SHADE_MIN_BLOCKS;

// Kernel categories for per-kernel device timing.
enum KernelCategory
{
    KC_CAMERA = 0,
    KC_CLOSEST,
    KC_SHADE,
    KC_SHADOW,
    KC_RESOLVE,
    KC_FINALIZE,
    KC_END,
    KC_COUNT
};

// CUDA events recorded before each launch; interval i is charged to the launch after mark i.
struct KernelMarks
{
    std::vector<cudaEvent_t> pool;
    std::vector<int> category;
    size_t used = 0;
    void reset() { used = 0, category.clear(); }
    void record(int cat, cudaStream_t st)
    {
        if (used == pool.size())
        {
            cudaEvent_t e;
            cudaEventCreate(&e);
            pool.push_back(e);
        }
        cudaEventRecord(pool[used], st);
        category.push_back(cat);
        used++;
    }
    // Milliseconds per category (call after the stream has completed).
    void sum(double ms[KC_COUNT]) const
    {
        for (int k = 0; k < KC_COUNT; k++)
            ms[k] = 0.0;
        for (size_t i = 0; i + 1 < used; i++)
        {
            if (category[i] == KC_END)
                continue;
            float t = 0.f;
            cudaEventElapsedTime(&t, pool[i], pool[i + 1]);
            ms[category[i]] += t;
        }
    }
    ~KernelMarks()
    {
        for (auto e : pool)
            cudaEventDestroy(e);
    }
};

// agb_pt.cu
// DevMesh::verts from the mesh's attribute arrays (normals / texcoords may be null).
cudaError_t launchVertexRecords(const float* positions, const float* normals, const float* texcoords,
    uint32_t vertexCount, float4* verts, cudaStream_t stream);
void launchWave(const DevScene& s, const agb_frame_data& f, const WaveParams& wp,
    const WaveBuffers& wb, cudaStream_t st, int smCount, uint64_t& launches, KernelMarks* marks);
// A batched wave over several requests (BatchTables): `shared` is the scenes' shared namespace,
// maxDepth the deepest request's trace depth.
void launchBatchWave(const DevScene& shared, const agb_frame_data& anyFrame, const WaveParams& wp,
    const WaveBuffers& wb, const BatchTables& bt, int maxDepth, bool forceOpaque, cudaStream_t st, int smCount,
    uint64_t& launches, KernelMarks* marks);
void setTraceAttributes();

// agb_env_build.cu: environment sampling table on the device.  rgba: device RGBA32F texels.
// layout 0: the reference's table bit for bit (rowSolidAngle: host, one FP32 solid angle per row
// computed as the reference does); layout 1: FP64 prefix-sum sweep.  integralFP64Out receives the
// FP64 luminance integral, integralShadingOut the integral the shading divides by (the
// reference's FP32 sum for layout 0).  scratch is reused across calls.
struct EnvBuildScratch
{
    double* weights   = nullptr; // per texel (luminance x solid angle), then normalised p
    double* scanA     = nullptr;
    uint32_t* ranks   = nullptr;
    uint32_t* heavyIdx = nullptr;
    double* heavyIncl = nullptr;
    double* lightIncl = nullptr;
    double* blockSums = nullptr;
    uint32_t* blockCounts = nullptr;
    float* rowSA      = nullptr;
    size_t capacity   = 0;
    uint32_t rows     = 0;
};
cudaError_t buildEnvAlias(const float4* rgba, uint32_t width, uint32_t height, int layout,
    const float* rowSolidAngle, agb_alias_entry* out, double* integralFP64Out,
    float* integralShadingOut, EnvBuildScratch& scratch, cudaStream_t st);
void freeEnvScratch(EnvBuildScratch& s);
// The kernel sequence of buildEnvAlias on scratch that is already large enough (capacity >= texels,
// rows >= height; the tile arrays sized by the two helpers below).  rowSolidAngle: host array of
// per-row solid angles copied into scratch.rowSA, or null when scratch.rowSA already holds them.
// Synchronises the stream before returning.
cudaError_t launchEnvAliasBuild(const float4* rgba, uint32_t width, uint32_t height, int layout,
    const float* rowSolidAngle, agb_alias_entry* out, double* integralFP64Out,
    float* integralShadingOut, const EnvBuildScratch& scratch, cudaStream_t st);
size_t envScratchTileDoubles(uint32_t texels); // blockSums entries
size_t envScratchTileCounts(uint32_t texels);  // blockCounts entries

// agb_env_noalloc.cu: the same build on a fixed scratch array in the library's device image.
// Returns cudaErrorInvalidValue when width * height exceeds AGB_ENV_NOALLOC_MAX_TEXELS.
cudaError_t buildEnvAliasNoAlloc(const float4* rgba, uint32_t width, uint32_t height, int layout,
    agb_alias_entry* out, double* integralFP64Out, float* integralShadingOut, cudaStream_t st);

// agb_bvh_build.cpp: host binned-SAH builder producing the device layout.
struct BuiltBVH
{
    std::vector<BNode> nodes;
    std::vector<uint32_t> order; // primitive index per leaf slot
    int32_t root  = 0;
    int32_t depth = 0;
};
// boxes: 6 floats per primitive (lo xyz, hi xyz).
void buildBVH2(const float* boxes, uint32_t count, int maxLeaf, int maxDepth, BuiltBVH& out);
// Double-precision inverse of a 3x4 affine transform rounded to float.
void invertAffine(const float* m, float* out);

// agb_temporal.cu
struct TemporalSettings
{
    uint32_t isReset;
    float blendAlphaMin, blendAlphaMax, speedReference;
};
cudaError_t launchTemporalResolve(const float4* accum, const float4* history, const float4* motion,
    const float* depthView, int W, int H, const TemporalSettings& s, float4* out, cudaStream_t st);

// agb_conv.cu: the 3x3 convolution (TMA-fed, warp-specialised tcgen05 implicit GEMM).
struct ConvLaunch
{
    const uint16_t* in0;
    const uint16_t* in1;
    const uint16_t* wpack;
    const float* bias;
    uint16_t* out;
    float* out32;
    int B, H, W, C0, C1, Cout, up0, relu;
    uint16_t* pool = nullptr; // [B][H/2][W/2][Cout]: 2x2 average of the BF16 outputs (H, W even)
    // The denoiser's output layer: RGBA radiance max(expm1(out[c] + radianceInput[c]), 0) for
    // c = 0..2 (radianceInput: the BF16 features, 16 per pixel, log1p noisy radiance in 0..2).
    float* radiance                = nullptr;
    const uint16_t* radianceInput  = nullptr;
    // Data-gradient split (the FP32 result is added, not stored): output channels [0, gradC0) go
    // to grad0 - summed over 2x2 blocks into half resolution when gradUp (the gradient of a
    // nearest upsample) -, channels [gradC0, Cout) to grad1 at full resolution.
    float* grad0 = nullptr;
    float* grad1 = nullptr;
    int gradC0   = 0;
    int gradUp   = 0;
};
// W even (and H even with up0 or pool), outputs 32-byte aligned; cudaErrorInvalidValue otherwise.
cudaError_t launchConv3x3(const ConvLaunch& c, cudaStream_t st);
cudaError_t launchPackConvWeights(const float* w, int Cin, int Cout, int flip, uint16_t* out, cudaStream_t st);
// Packs several layers' weights in one launch, each both ways (forward into out, data-gradient
// into outFlip; either may be null).
struct PackJob
{
    const float* w;
    uint16_t* out;
    uint16_t* outFlip;
    int cin, cout;
};
constexpr int kMaxPackJobs = 16;
cudaError_t launchPackConvWeightsMany(const PackJob* jobs, int count, cudaStream_t st);
// dW[tap][ci][co] += sum over pixels of X[p + d][ci] dY[p][co] (X as c.in0 / c.in1 / c.up0; c.Cout
// the layer's output channels: up to 128, or a multiple of 64 / 128 beyond; W even).
cudaError_t launchConvWgrad(const ConvLaunch& c, const uint16_t* dy, float* dw, int smCount, cudaStream_t st);

// agb_denoise.cu

cudaError_t launchTcGemm(const uint16_t* A, const uint16_t* B, float* D, int M, int N, int K, cudaStream_t st);
// Reads and clears the tensor-core kernels' timeout flag (1 = a bounded wait ran out).
cudaError_t takeTcError(int* flag);
// Device address of that flag on the current device (kernels in other translation units set it).
cudaError_t tcErrorFlag(int** flag);

// agb_unet.cu: the U-Net denoiser (layer graph, training state, elementwise kernels).
class UnetDenoiser
{
public:
    static constexpr int kLayers = 15;
    static constexpr int kActs   = 18;
    ~UnetDenoiser();
    cudaError_t init(uint64_t seed, cudaStream_t st, int smCount);
    static size_t paramCount();
    // x: [B][H][W][16] BF16 features (H, W multiples of 8).  Keeps the activations for backward.
    // rgba (inference): the denoised RGBA radiance, written by the output layer's epilogue.
    cudaError_t forward(const uint16_t* x, int B, int H, int W, bool training, float* rgba = nullptr);
    // Inference (forward with rgba) replayed from a CUDA graph of its 15 launches, captured on first
    // use for each (x, rgba, B, H, W) and kept while the activation buffers stay (a few graphs).
    // The tensor-core timeout flag is copied to host memory behind it on the stream: after the
    // stream is synchronised, inferTimedOut() says whether a wait ran out (the flag is then cleared).
    cudaError_t infer(const uint16_t* x, int B, int H, int W, float* rgba);
    bool inferTimedOut();
    // After forward(training): L1 loss against target RGBA (FP32) and all parameter gradients.
    cudaError_t backward(const float* target);
    cudaError_t adam(float lr);
    cudaError_t setParams(const float* host);
    const float* params() const { return params_; }
    const float* grads() const { return grads_; }
    const float* lossDevice() const { return loss_; }
    size_t nParams() const { return nParams_; }
    static double flopsPerPixel(bool training);
    void release();

private:
    cudaError_t alloc(void** p, size_t bytes, std::vector<void*>& list);
    cudaError_t repack();
    cudaError_t ensureShape(int B, int H, int W, bool training);
    static size_t pixels(int B, int H, int W, int level);
    ConvLaunch layerLaunch(int i, const uint16_t* x) const;
    void dropGraphs();
    cudaError_t inferLaunch(const uint16_t* x, int B, int H, int W, float* rgba);

    cudaStream_t stream_ = nullptr;
    int smCount_         = 0;
    size_t nParams_      = 0;
    float* params_ = nullptr;
    float* grads_  = nullptr;
    float* adamM_  = nullptr;
    float* adamV_  = nullptr;
    float* loss_   = nullptr;
    uint16_t* pack_     = nullptr;
    uint16_t* packFlip_ = nullptr;
    size_t wOff_[kLayers] = {}, bOff_[kLayers] = {}, packOff_[kLayers] = {};
    uint16_t* act_[kActs] = {};
    float* grad_[kActs]   = {};
    float* out32_ = nullptr;
    float* gOut_  = nullptr;
    uint16_t* dpre_        = nullptr;
    const uint16_t* input_ = nullptr;
    int B_ = 0, H_ = 0, W_ = 0;
    long step_ = 0;
    std::vector<void*> allocs_, shapeAllocs_;
    struct Graph
    {
        const uint16_t* x = nullptr;
        float* rgba       = nullptr;
        int B = 0, H = 0, W = 0;
        cudaGraphExec_t exec = nullptr;
    };
    std::vector<Graph> graphs_; // most recently used last
    Graph pending_{};           // buffers seen once, captured when seen again
    int* flagHost_ = nullptr;   // pinned copy of the tensor-core timeout flag
};
cudaError_t launchDenoiseFeatures(const float4* mean, const float2* moments, float samples, const float4* albedo,
    const float4* normal, const float* depth, float skyZ, long P, uint16_t* out, cudaStream_t st);

// agb_bvh_gpu.cu: binned-SAH BLAS build on the GPU.
struct GpuBvhScratch
{
    float* boxes      = nullptr;
    size_t boxesBytes = 0;
    uint32_t* order   = nullptr;
    size_t orderBytes = 0;
    uint32_t* scratch = nullptr;
    size_t scratchBytes = 0;
    void* tasksA      = nullptr;
    size_t tasksABytes = 0;
    void* tasksB      = nullptr;
    size_t tasksBBytes = 0;
    void* counters    = nullptr;
    size_t countersBytes = 0;
    BNode* nodes      = nullptr;
    size_t nodesBytes = 0;
};
// positions / indices: device arrays of the mesh.  Writes up to nodeCapacity nodes, the triangles
// in leaf order (3 float4 each), the root ref, the depth and the interior node count.
cudaError_t buildBlasGpu(const float* positions, const uint32_t* indices, uint32_t ntri, int maxDepth,
    GpuBvhScratch& s, BNode* nodes, uint32_t nodeCapacity, float4* tris, int32_t* rootOut, int32_t* depthOut,
    uint32_t* nodeCountOut, cudaStream_t st);
// TLAS over count instance boxes (6 floats each, host memory; staged through the scratch): one
// instance per leaf; orderOut (device, count entries) gets the instance index of each leaf slot.
cudaError_t buildTlasGpu(const float* boxesHost, uint32_t count, int maxDepth, GpuBvhScratch& s, BNode* nodes,
    uint32_t nodeCapacity, int32_t* orderOut, int32_t* rootOut, int32_t* depthOut, uint32_t* nodeCountOut,
    cudaStream_t st);
void freeGpuBvhScratch(GpuBvhScratch& s);

// agb_unit.cu
cudaError_t launchBsdfBatch(int op, const agb_material* mats, const int32_t* matIndex,
    const float* frames, const float* V, const float* L, const float* rnd, int64_t n,
    float* outValue, float* outDir, float* outPdf, int32_t* outLobe, cudaStream_t st);
cudaError_t launchIntersectBatch(const DevScene& s, const float* rays, int64_t n, int anyHit,
    float* outTUV, int32_t* outInstPrim, uint32_t* work, unsigned long long* overflowCount,
    cudaStream_t st, int smCount);
cudaError_t launchEnvSampleBatch(const DevScene& s, const float* rnd, int64_t n,
    float* outRadiance, float* outDir, float* outPdf, cudaStream_t st);
cudaError_t launchRandomStream(uint32_t sampleIndex, uint32_t width, uint32_t px, uint32_t py,
    int n, float* out, cudaStream_t st);
cudaError_t launchRelMse(const float4* accum, float scale, const float4* ref, uint32_t pixels, double eps,
    double* out, cudaStream_t st);
cudaError_t launchPostProcess(const float4* accum, const float* accumComp, int mode,
    float invCount, uint32_t pixels, float3 brightness, int toneMap, int gamma, float4* out32,
    uchar4* out8, cudaStream_t st);

} // namespace agb
