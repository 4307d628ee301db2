// C ABI of the GB300 path-tracing backend (include/agb.h): context, scene upload, environment,
// rendering, readback.  All inputs are validated on the host before any kernel sees them, so no
// kernel indexes memory with an unchecked value.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "agb_kernels.h"

using namespace agb;

namespace
{

thread_local std::string g_lastError;

float bitsToFloat(int32_t v)
{
    float f;
    memcpy(&f, &v, sizeof f);
    return f;
}

agb_status fail(agb_status code, const std::string& msg)
{
    g_lastError = msg;
    return code;
}

agb_status cudaFail(cudaError_t e, const char* what)
{
    agb_status code = (e == cudaErrorMemoryAllocation) ? AGB_ERR_OOM : AGB_ERR_CUDA;
    return fail(code, std::string(what) + ": " + cudaGetErrorString(e));
}

#define AGB_CUDA(call, what)                                                                       \
    do                                                                                             \
    {                                                                                              \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return cudaFail(e_, what);                                                             \
    } while (0)

// A device allocation owned by the context.
struct DevBuf
{
    void* ptr    = nullptr;
    size_t bytes = 0;
    DevBuf()     = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (ptr)
            cudaFree(ptr);
        ptr   = nullptr;
        bytes = 0;
    }
    cudaError_t ensure(size_t n)
    {
        if (bytes >= n && ptr)
            return cudaSuccess;
        release();
        if (n == 0)
            return cudaSuccess;
        cudaError_t e = cudaMalloc(&ptr, n);
        if (e == cudaSuccess)
            bytes = n;
        else
            ptr = nullptr;
        return e;
    }
    template <class T>
    T* as() const
    {
        return static_cast<T*>(ptr);
    }
};

struct Geometry
{
    DevBuf positions, normals, texcoords, verts, indices, tris, nodes;
    DevMesh mesh{};
    uint32_t nodeCount = 0;
    // Boxes that together cover the mesh (6 floats each): the child boxes of the BLAS's top
    // levels.  Instance boxes are built from them, which is much tighter than the mesh box for
    // rotated instances.
    std::vector<float> cover;
    float bounds[6]; // lo, hi in object space
};

struct Image
{
    DevBuf data;
    DevImage view{};
};

} // namespace

struct agb_context
{
    // A view (agb_view_create) renders its parent's scene with its own stream, frame and render
    // buffers; it holds no scene data of its own.
    agb_context* parent = nullptr;
    int viewCount       = 0;
    int device          = 0;
    cudaStream_t stream = nullptr;
    bool ownsStream     = false;
    int smCount         = 0;
    size_t deviceBytes  = 0; // total device memory
    bool counting       = false;
    bool profiling      = false;
    KernelMarks marks;

    std::vector<std::unique_ptr<Geometry>> geometries;
    DevBuf meshTable;
    std::vector<std::unique_ptr<Image>> images;
    DevBuf imageTable;

    DevBuf materials, matTex;
    uint32_t materialCount = 0;
    bool hasMatTex         = false;
    DevBuf matGraph, graphOps, graphConsts; // material node-graph programs
    bool hasGraphs = false;

    DevBuf instances, tlasNodes, tlasOrder, layers;
    std::vector<std::unique_ptr<DevBuf>> layerUVs;
    uint32_t instanceCount = 0;
    int32_t tlasRoot       = 0;
    int32_t tlasDepth      = 0;
    uint32_t tlasNodeCount = 0;

    agb_environment_data env{};
    int32_t envLight = -1, envBackground = -1;
    DevBuf alias;
    EnvBuildScratch envScratch;
    GpuBvhScratch bvhScratch;
    int32_t bvhBuilder = AGB_BVH_GPU;
    double envIntegral     = 0.0; // FP64 luminance integral
    double envShadingIntegral = 0.0;
    int32_t envLayout      = AGB_ENV_TABLE_REFERENCE;
    DevGroundPlane ground{}; // disabled until agb_ground_plane_set

    agb_frame_data frame{};
    bool frameSet = false;

    // Host mirrors of the scene tables (batched rendering builds the shared namespace from them)
    // and a counter bumped by every scene change.
    std::vector<DevInstance> hostInstances;
    std::vector<DevLayer> hostLayers;
    std::vector<agb_material> hostMaterials;
    std::vector<agb_material_textures> hostMatTex;
    uint64_t sceneVersion = 0;
    // Union of the instances' world boxes (ray binning's grid).
    float sceneLo[3] = { 0.f, 0.f, 0.f }, sceneHi[3] = { 0.f, 0.f, 0.f };
    bool binRays = false;
    DevBuf bins;

    // Wave buffers.
    size_t pathCapacity = 0;
    DevBuf pathState, queues, counters, stats;
    WaveBuffers wb{};
    // Accumulation.
    uint32_t accW = 0, accH = 0;
    DevBuf accMean, accSum, accComp, lastSample, accMoments;
    // Denoising AOVs of the last render that enabled them (accW x accH).
    DevBuf aovDepth, aovNormal, aovAlbedo, aovMotion;
    bool aovValid = false;
    // Temporal-resolve histories (ping-pong) and the index of the one written last.
    DevBuf taaHistory[2];
    uint32_t taaW = 0, taaH = 0;
    int taaLast     = -1;
    uint32_t accumulatedSamples = 0;
    uint32_t lastAccumMode      = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    ~agb_context()
    {
        freeEnvScratch(envScratch);
        freeGpuBvhScratch(bvhScratch);
        if (ev0)
            cudaEventDestroy(ev0);
        if (ev1)
            cudaEventDestroy(ev1);
        if (ownsStream && stream)
            cudaStreamDestroy(stream);
    }

    DevScene scene() const
    {
        if (parent)
            return parent->scene();
        DevScene s{};
        s.meshes        = meshTable.as<DevMesh>();
        s.instances     = instances.as<DevInstance>();
        s.tlas          = tlasNodes.as<BNode>();
        s.tlasRoot      = tlasRoot;
        s.instanceCount = int32_t(instanceCount);
        s.tlasOrder     = tlasOrder.as<int32_t>();
        s.materials     = materials.as<agb_material>();
        s.matTex        = hasMatTex ? matTex.as<agb_material_textures>() : nullptr;
        s.materialCount = int32_t(materialCount);
        s.imageCount    = int32_t(images.size());
        s.images        = imageTable.as<DevImage>();
        s.layers        = layers.as<DevLayer>();
        s.matGraph      = hasGraphs ? matGraph.as<int2>() : nullptr;
        s.graphOps      = hasGraphs ? graphOps.as<agb_graph_op>() : nullptr;
        s.graphConsts   = hasGraphs ? graphConsts.as<float4>() : nullptr;
        s.env           = env;
        s.envLight      = DevImage{};
        s.envBackground = DevImage{};
        if (envLight >= 0 && size_t(envLight) < images.size())
            s.envLight = images[envLight]->view;
        if (envBackground >= 0 && size_t(envBackground) < images.size())
            s.envBackground = images[envBackground]->view;
        s.alias  = alias.as<agb_alias_entry>();
        s.ground = ground;
        return s;
    }
};

namespace
{

agb_status setDevice(agb_context* ctx)
{
    AGB_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    return AGB_OK;
}

// Device bytes per path in flight: path state, and the ray / hit / shadow queues.
constexpr size_t kPathStateBytes = sizeof(uint2) + sizeof(float4) * 7 + sizeof(uint32_t) * 3 +
                                   sizeof(float4) * kMaxShadowSlots * 2 + sizeof(float4);
constexpr size_t kPathQueueBytes = 2 * (2 * sizeof(float4) + sizeof(uint32_t)) + sizeof(float4) +
                                   sizeof(int32_t) + sizeof(uint32_t) * kMaxShadowSlots + sizeof(uint32_t) +
                                   sizeof(float4) * (kShadePointWords + kMisWords);

// Carves the wave buffers for `paths` paths and `depth` bounces out of a few allocations.
agb_status ensureWave(agb_context* ctx, size_t paths, int depth, size_t waves)
{
    if (paths > ctx->pathCapacity)
    {
        // The buffers are reallocated below; if that fails the context holds none.
        ctx->pathCapacity = 0;
        size_t P = paths;
        size_t stateBytes = P * kPathStateBytes;
        size_t queueBytes = P * kPathQueueBytes + 1024;
        AGB_CUDA(ctx->pathState.ensure(stateBytes + 4096), "allocate path state");
        AGB_CUDA(ctx->queues.ensure(queueBytes + 4096), "allocate ray queues");
        char* s = ctx->pathState.as<char>();
        auto take = [&](size_t bytes) {
            char* r = s;
            s += (bytes + 255) & ~size_t(255);
            return r;
        };
        WaveBuffers& w   = ctx->wb;
        w.rng            = reinterpret_cast<uint2*>(take(P * sizeof(uint2)));
        w.contrib        = reinterpret_cast<float4*>(take(P * sizeof(float4)));
        w.flags          = reinterpret_cast<uint32_t*>(take(P * sizeof(uint32_t)));
        w.outDirect      = reinterpret_cast<float4*>(take(P * sizeof(float4)));
        w.outDiffuse     = reinterpret_cast<float4*>(take(P * sizeof(float4)));
        w.outGlossy      = reinterpret_cast<float4*>(take(P * sizeof(float4)));
        w.lastIndirect   = reinterpret_cast<float4*>(take(P * sizeof(float4)));
        w.pendEmission   = reinterpret_cast<float4*>(take(P * sizeof(float4)));
        w.pendSegContrib = reinterpret_cast<float4*>(take(P * sizeof(float4)));
        w.pendSlot       = reinterpret_cast<float4*>(take(P * kMaxShadowSlots * sizeof(float4)));
        w.pendBits       = reinterpret_cast<uint32_t*>(take(P * sizeof(uint32_t)));
        w.occluded       = reinterpret_cast<uint32_t*>(take(P * sizeof(uint32_t)));
        w.shOrg          = reinterpret_cast<float4*>(take(P * sizeof(float4)));
        w.shDir          = reinterpret_cast<float4*>(take(P * kMaxShadowSlots * sizeof(float4)));
        if (size_t(s - ctx->pathState.as<char>()) > ctx->pathState.bytes)
            return fail(AGB_ERR_LIMIT, "internal: path state carve overflow");
        s = ctx->queues.as<char>();
        for (int b = 0; b < 2; b++)
        {
            w.rayOrg[b]  = reinterpret_cast<float4*>(take(P * sizeof(float4)));
            w.rayDir[b]  = reinterpret_cast<float4*>(take(P * sizeof(float4)));
            w.rayPath[b] = reinterpret_cast<uint32_t*>(take(P * sizeof(uint32_t)));
        }
        w.hitTUV      = reinterpret_cast<float4*>(take(P * sizeof(float4)));
        w.hitInst     = reinterpret_cast<int32_t*>(take(P * sizeof(int32_t)));
        w.shTag       = reinterpret_cast<uint32_t*>(take(P * kMaxShadowSlots * sizeof(uint32_t)));
        w.resolveList = reinterpret_cast<uint32_t*>(take(P * sizeof(uint32_t)));
        w.shadePoint  = reinterpret_cast<float4*>(take(P * kShadePointWords * sizeof(float4)));
        w.misPoint    = reinterpret_cast<float4*>(take(P * kMisWords * sizeof(float4)));
        if (size_t(s - ctx->queues.as<char>()) > ctx->queues.bytes)
            return fail(AGB_ERR_LIMIT, "internal: queue carve overflow");
        ctx->pathCapacity = P;
    }
    size_t counterWords = size_t(depth + 2) * kCounterStride * waves;
    AGB_CUDA(ctx->counters.ensure(counterWords * sizeof(uint32_t)), "allocate counters");
    if (!ctx->bins.ptr)
    {
        AGB_CUDA(ctx->bins.ensure(2 * kRayBins * sizeof(uint32_t)), "allocate ray bins");
        AGB_CUDA(cudaMemsetAsync(ctx->bins.ptr, 0, 2 * kRayBins * sizeof(uint32_t), ctx->stream), "clear ray bins");
    }
    ctx->wb.binCount  = ctx->bins.as<uint32_t>();
    ctx->wb.binOffset = ctx->bins.as<uint32_t>() + kRayBins;
    AGB_CUDA(ctx->stats.ensure(8 * sizeof(unsigned long long)), "allocate stats");
    ctx->wb.stats = ctx->stats.as<unsigned long long>();
    return AGB_OK;
}

agb_status ensureAccum(agb_context* ctx, uint32_t W, uint32_t H)
{
    if (ctx->accW == W && ctx->accH == H && ctx->accMean.ptr)
        return AGB_OK;
    size_t n = size_t(W) * H;
    AGB_CUDA(ctx->accMean.ensure(n * sizeof(float4)), "allocate accumulation");
    AGB_CUDA(ctx->accSum.ensure(n * sizeof(float4)), "allocate accumulation");
    AGB_CUDA(ctx->accComp.ensure(n * sizeof(float4)), "allocate accumulation");
    AGB_CUDA(ctx->lastSample.ensure(n * sizeof(float4)), "allocate accumulation");
    AGB_CUDA(ctx->accMoments.ensure(n * sizeof(float2)), "allocate accumulation");
    AGB_CUDA(cudaMemsetAsync(ctx->accMoments.ptr, 0, n * sizeof(float2), ctx->stream), "clear");
    AGB_CUDA(cudaMemsetAsync(ctx->accMean.ptr, 0, n * sizeof(float4), ctx->stream), "clear");
    AGB_CUDA(cudaMemsetAsync(ctx->accSum.ptr, 0, n * sizeof(float4), ctx->stream), "clear");
    AGB_CUDA(cudaMemsetAsync(ctx->accComp.ptr, 0, n * sizeof(float4), ctx->stream), "clear");
    ctx->accW = W;
    ctx->accH = H;
    ctx->accumulatedSamples = 0;
    return AGB_OK;
}

// Collects the child boxes of the BLAS down to kCoverDepth levels (or to a leaf, or to a node that
// is not among the `avail` nodes at hand) into out; a mesh whose root is a leaf keeps its bounds.
// BLAS node order in memory.  The GPU builder numbers nodes level by level.  AGB_BLAS_LAYOUT=dfs
// lays them out depth first with a node's two interior children side by side (a path's nodes
// close together, both children of a node in one or two cache lines): the children of node n are
// placed together, and the pairs of child 0's subtree follow before child 1's.  The tree (and so
// every hit) is the same.  Measured on the large configuration: closest-hit 138.2 -> 137.8 ms,
// shadow 97.8 -> 97.5 ms per frame, for a host round trip of the nodes per build, so the builder's
// order stays the default.
bool blasLayoutDepthFirst()
{
    const char* v = getenv("AGB_BLAS_LAYOUT");
    return v && std::strcmp(v, "dfs") == 0;
}

void layoutDepthFirst(const std::vector<BNode>& in, int32_t root, std::vector<BNode>& out)
{
    out.clear();
    out.reserve(in.size());
    out.push_back(in[size_t(root)]);
    std::vector<std::pair<int32_t, int32_t>> stack; // (node in `in`, its slot in `out`)
    stack.push_back({ root, 0 });
    while (!stack.empty())
    {
        const auto [old, slot] = stack.back();
        stack.pop_back();
        const int4 r     = in[size_t(old)].ref;
        const int32_t c0 = r.x, c1 = r.y;
        int4 nr          = r;
        if (c0 >= 0)
        {
            nr.x = int32_t(out.size());
            out.push_back(in[size_t(c0)]);
        }
        if (c1 >= 0)
        {
            nr.y = int32_t(out.size());
            out.push_back(in[size_t(c1)]);
        }
        out[size_t(slot)].ref = nr;
        if (c1 >= 0)
            stack.push_back({ c1, nr.y });
        if (c0 >= 0)
            stack.push_back({ c0, nr.x });
    }
}

void coverBoxes(const BNode* nodes, uint32_t avail, int32_t root, const float* bounds, std::vector<float>& out)
{
    const int kCoverDepth = 5;
    out.clear();
    if (root < 0 || uint32_t(root) >= avail)
    {
        out.assign(bounds, bounds + 6);
        return;
    }
    struct Item
    {
        int32_t node;
        int depth;
    };
    std::vector<Item> stack = { { root, 0 } };
    while (!stack.empty())
    {
        Item it = stack.back();
        stack.pop_back();
        const BNode& n = nodes[it.node];
        for (int side = 0; side < 2; side++)
        {
            int32_t ref     = side == 0 ? n.ref.x : n.ref.y;
            const float4 xy = side == 0 ? n.c0xy : n.c1xy;
            float z0 = side == 0 ? n.cz.x : n.cz.z, z1 = side == 0 ? n.cz.y : n.cz.w;
            if (ref >= 0 && uint32_t(ref) < avail && it.depth + 1 < kCoverDepth)
                stack.push_back({ ref, it.depth + 1 });
            else
            {
                const float b[6] = { xy.x, xy.z, z0, xy.y, xy.w, z1 };
                out.insert(out.end(), b, b + 6);
            }
        }
    }
}

agb_status rebuildMeshTable(agb_context* ctx)
{
    std::vector<DevMesh> t(ctx->geometries.size());
    for (size_t i = 0; i < t.size(); i++)
        t[i] = ctx->geometries[i]->mesh;
    if (t.empty())
        return AGB_OK;
    AGB_CUDA(ctx->meshTable.ensure(t.size() * sizeof(DevMesh)), "allocate mesh table");
    AGB_CUDA(cudaMemcpyAsync(ctx->meshTable.ptr, t.data(), t.size() * sizeof(DevMesh),
                 cudaMemcpyHostToDevice, ctx->stream),
        "upload mesh table");
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "upload mesh table");
    return AGB_OK;
}

agb_status upload(agb_context* ctx, DevBuf& dst, const void* src, size_t bytes, const char* what)
{
    AGB_CUDA(dst.ensure(bytes), what);
    if (bytes)
        AGB_CUDA(cudaMemcpyAsync(dst.ptr, src, bytes, cudaMemcpyHostToDevice, ctx->stream), what);
    return AGB_OK;
}

} // namespace

extern "C" {

AGB_API const char* agb_version(void) { return "aurora-gb300 0.1 (sm_103a)"; }

AGB_API const char* agb_last_error(void) { return g_lastError.c_str(); }

AGB_API agb_status agb_context_create(int32_t device, void* cuda_stream, agb_context** out)
{
    if (!out)
        return fail(AGB_ERR_INVALID_ARG, "agb_context_create: out is null");
    *out = nullptr;
    int count = 0;
    AGB_CUDA(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
    if (device < 0 || device >= count)
        return fail(AGB_ERR_INVALID_ARG, "agb_context_create: no CUDA device " + std::to_string(device));
    std::unique_ptr<agb_context> ctx(new agb_context());
    ctx->device = device;
    AGB_CUDA(cudaSetDevice(device), "cudaSetDevice");
    AGB_CUDA(cudaDeviceGetAttribute(&ctx->smCount, cudaDevAttrMultiProcessorCount, device),
        "query SM count");
    size_t freeBytes = 0;
    AGB_CUDA(cudaMemGetInfo(&freeBytes, &ctx->deviceBytes), "query device memory");
    if (cuda_stream)
        ctx->stream = static_cast<cudaStream_t>(cuda_stream);
    else
    {
        AGB_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "create stream");
        ctx->ownsStream = true;
    }
    AGB_CUDA(cudaEventCreate(&ctx->ev0), "create event");
    AGB_CUDA(cudaEventCreate(&ctx->ev1), "create event");
    setTraceAttributes();
    if (const char* e = std::getenv("AGB_BIN_RAYS"))
        ctx->binRays = e[0] == '1';
    // Default environment: the reference's gradient defaults (EnvironmentBase.cpp:33-45),
    // identity transforms.
    agb_environment_data& e = ctx->env;
    const float lt[3] = { 1.f, 1.f, 1.f }, lb[3] = { 0.f, 0.f, 0.f };
    const float bt[3] = { 0.02f, 0.25f, 0.60f }, bb[3] = { 0.32f, 0.79f, 1.0f };
    memcpy(e.light_top, lt, sizeof lt);
    memcpy(e.light_bottom, lb, sizeof lb);
    memcpy(e.background_top, bt, sizeof bt);
    memcpy(e.background_bottom, bb, sizeof bb);
    for (int k = 0; k < 4; k++)
    {
        e.light_transform[5 * k] = e.light_transform_inv[5 * k] = e.background_transform[5 * k] = 1.f;
    }
    *out = ctx.release();
    return AGB_OK;
}

AGB_API agb_status agb_context_destroy(agb_context* ctx)
{
    if (!ctx)
        return AGB_OK;
    if (ctx->viewCount > 0)
        return fail(AGB_ERR_INVALID_ARG, "agb_context_destroy: destroy the context's views first");
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->parent)
        ctx->parent->viewCount--;
    delete ctx;
    return AGB_OK;
}

AGB_API agb_status agb_view_create(agb_context* ctx, void* cuda_stream, agb_context** out)
{
    if (!ctx || !out)
        return fail(AGB_ERR_INVALID_ARG, "agb_view_create: null argument");
    if (ctx->parent)
        return fail(AGB_ERR_INVALID_ARG, "agb_view_create: a view cannot have views");
    *out = nullptr;
    std::unique_ptr<agb_context> v(new agb_context());
    v->parent  = ctx;
    v->device  = ctx->device;
    v->smCount = ctx->smCount;
    v->deviceBytes = ctx->deviceBytes;
    v->envLayout = ctx->envLayout;
    v->binRays   = ctx->binRays;
    AGB_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (cuda_stream)
        v->stream = static_cast<cudaStream_t>(cuda_stream);
    else
    {
        AGB_CUDA(cudaStreamCreateWithFlags(&v->stream, cudaStreamNonBlocking), "create stream");
        v->ownsStream = true;
    }
    AGB_CUDA(cudaEventCreate(&v->ev0), "create event");
    AGB_CUDA(cudaEventCreate(&v->ev1), "create event");
    ctx->viewCount++;
    *out = v.release();
    return AGB_OK;
}

AGB_API agb_status agb_context_memory(agb_context* ctx, uint64_t* bytes)
{
    if (!ctx || !bytes)
        return fail(AGB_ERR_INVALID_ARG, "agb_context_memory: null argument");
    uint64_t b = ctx->meshTable.bytes + ctx->imageTable.bytes + ctx->materials.bytes +
        ctx->matTex.bytes + ctx->instances.bytes + ctx->tlasNodes.bytes + ctx->tlasOrder.bytes +
        ctx->layers.bytes + ctx->alias.bytes + ctx->pathState.bytes + ctx->queues.bytes +
        ctx->counters.bytes + ctx->accMean.bytes + ctx->accSum.bytes + ctx->accComp.bytes +
        ctx->lastSample.bytes + ctx->accMoments.bytes + ctx->aovDepth.bytes + ctx->aovNormal.bytes +
        ctx->aovAlbedo.bytes + ctx->aovMotion.bytes + ctx->taaHistory[0].bytes + ctx->taaHistory[1].bytes +
        uint64_t(ctx->envScratch.capacity) * 44 + ctx->stats.bytes;
    for (auto& g : ctx->geometries)
        b += g->positions.bytes + g->normals.bytes + g->texcoords.bytes + g->verts.bytes + g->indices.bytes +
            g->tris.bytes + g->nodes.bytes;
    for (auto& i : ctx->images)
        b += i->data.bytes;
    for (auto& l : ctx->layerUVs)
        b += l->bytes;
    *bytes = b;
    return AGB_OK;
}

AGB_API agb_status agb_set_counting(agb_context* ctx, int32_t enabled)
{
    if (!ctx)
        return fail(AGB_ERR_INVALID_ARG, "agb_set_counting: null context");
    ctx->counting = enabled != 0;
    return AGB_OK;
}

AGB_API agb_status agb_set_profiling(agb_context* ctx, int32_t enabled)
{
    if (!ctx)
        return fail(AGB_ERR_INVALID_ARG, "agb_set_profiling: null context");
    ctx->profiling = enabled != 0;
    return AGB_OK;
}

AGB_API agb_status agb_geometry_create(agb_context* ctx, const float* positions,
    const float* normals, const float* texcoords, const uint32_t* indices, uint32_t vertex_count,
    uint32_t index_count, int32_t* out_geometry)
{
    if (ctx && !ctx->parent)
        ctx->sceneVersion++;
    if (ctx && ctx->parent)
        return fail(AGB_ERR_INVALID_ARG, "agb_geometry_create: a view shares its parent's scene; change the parent");
    if (!ctx || !positions || !out_geometry)
        return fail(AGB_ERR_INVALID_ARG, "agb_geometry_create: null argument");
    if (vertex_count == 0 || index_count == 0 || index_count % 3 != 0)
        return fail(AGB_ERR_INVALID_ARG, "agb_geometry_create: index count must be a positive multiple of 3");
    if (!indices && index_count != vertex_count)
        return fail(AGB_ERR_INVALID_ARG, "agb_geometry_create: non-indexed geometry needs index_count == vertex_count");
    if (uint64_t(index_count / 3) >= (1ull << 28))
        return fail(AGB_ERR_LIMIT, "agb_geometry_create: more than 2^28 triangles");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    std::vector<uint32_t> idx;
    if (indices)
    {
        idx.assign(indices, indices + index_count);
        for (uint32_t i = 0; i < index_count; i++)
            if (idx[i] >= vertex_count)
                return fail(AGB_ERR_INVALID_ARG, "agb_geometry_create: index " + std::to_string(i) +
                        " = " + std::to_string(idx[i]) + " out of range");
    }
    else
    {
        // Sequential indices for non-indexed geometry (HGIGeometry.cpp:37-47).
        idx.resize(index_count);
        for (uint32_t i = 0; i < index_count; i++)
            idx[i] = i;
    }
    uint32_t ntri = index_count / 3;
    std::unique_ptr<Geometry> g(new Geometry());
    if (ctx->bvhBuilder == AGB_BVH_GPU)
    {
        for (int k = 0; k < 3; k++)
        {
            g->bounds[k]     = INFINITY;
            g->bounds[3 + k] = -INFINITY;
        }
        for (uint32_t v = 0; v < vertex_count; v++)
            for (int k = 0; k < 3; k++)
            {
                float x = positions[3 * size_t(v) + k];
                if (!std::isfinite(x))
                    return fail(AGB_ERR_INVALID_ARG, "agb_geometry_create: non-finite position");
            }
        for (uint32_t i = 0; i < index_count; i++)
            for (int k = 0; k < 3; k++)
            {
                float x          = positions[3 * size_t(idx[i]) + k];
                g->bounds[k]     = std::min(g->bounds[k], x);
                g->bounds[3 + k] = std::max(g->bounds[3 + k], x);
            }
        st = upload(ctx, g->positions, positions, size_t(vertex_count) * 3 * sizeof(float), "upload positions");
        if (!st && normals)
            st = upload(ctx, g->normals, normals, size_t(vertex_count) * 3 * sizeof(float), "upload normals");
        if (!st && texcoords)
            st = upload(ctx, g->texcoords, texcoords, size_t(vertex_count) * 2 * sizeof(float), "upload texcoords");
        if (!st)
            st = upload(ctx, g->indices, idx.data(), idx.size() * sizeof(uint32_t), "upload indices");
        if (st)
            return st;
        AGB_CUDA(g->tris.ensure(size_t(ntri) * 3 * sizeof(float4)), "allocate triangles");
        GpuBvhScratch& s = ctx->bvhScratch;
        size_t capNodes  = std::max<size_t>(1, ntri);
        if (s.nodesBytes < capNodes * sizeof(BNode))
        {
            cudaFree(s.nodes);
            s.nodes      = nullptr;
            s.nodesBytes = 0;
            AGB_CUDA(cudaMalloc(&s.nodes, capNodes * sizeof(BNode)), "allocate BVH scratch");
            s.nodesBytes = capNodes * sizeof(BNode);
        }
        int32_t root = 0, depth = 0;
        uint32_t nodeCount = 0;
        AGB_CUDA(buildBlasGpu(g->positions.as<float>(), g->indices.as<uint32_t>(), ntri, kBlasMaxDepth, s, s.nodes,
                     uint32_t(capNodes), g->tris.as<float4>(), &root, &depth, &nodeCount, ctx->stream),
            "agb_geometry_create: GPU BVH build");
        if (depth > kBlasMaxDepth)
            return fail(AGB_ERR_LIMIT, "agb_geometry_create: BLAS deeper than the traversal stack allows");
        // The builder numbers nodes level by level, so the first ones are the top of the tree.
        std::vector<BNode> top(std::min<uint32_t>(nodeCount, 255));
        if (!top.empty())
            AGB_CUDA(cudaMemcpyAsync(top.data(), s.nodes, top.size() * sizeof(BNode), cudaMemcpyDeviceToHost,
                         ctx->stream),
                "read BVH top");
        AGB_CUDA(cudaStreamSynchronize(ctx->stream), "upload geometry");
        coverBoxes(top.data(), uint32_t(top.size()), root, g->bounds, g->cover);
        if (nodeCount && blasLayoutDepthFirst())
        {
            // Depth-first order with each node's interior children side by side (see layoutDepthFirst).
            std::vector<BNode> level(nodeCount), dfs;
            AGB_CUDA(cudaMemcpyAsync(level.data(), s.nodes, size_t(nodeCount) * sizeof(BNode), cudaMemcpyDeviceToHost,
                         ctx->stream),
                "read BVH");
            AGB_CUDA(cudaStreamSynchronize(ctx->stream), "read BVH");
            layoutDepthFirst(level, root, dfs);
            root      = 0;
            nodeCount = uint32_t(dfs.size());
            AGB_CUDA(g->nodes.ensure(size_t(nodeCount) * sizeof(BNode)), "allocate BVH");
            AGB_CUDA(cudaMemcpyAsync(g->nodes.ptr, dfs.data(), size_t(nodeCount) * sizeof(BNode),
                         cudaMemcpyHostToDevice, ctx->stream),
                "upload BVH");
            AGB_CUDA(cudaStreamSynchronize(ctx->stream), "upload BVH");
        }
        else if (nodeCount)
        {
            AGB_CUDA(g->nodes.ensure(size_t(nodeCount) * sizeof(BNode)), "allocate BVH");
            AGB_CUDA(cudaMemcpyAsync(g->nodes.ptr, s.nodes, size_t(nodeCount) * sizeof(BNode),
                         cudaMemcpyDeviceToDevice, ctx->stream),
                "copy BVH");
            AGB_CUDA(cudaStreamSynchronize(ctx->stream), "upload geometry");
        }
        AGB_CUDA(g->verts.ensure(size_t(vertex_count) * 2 * sizeof(float4)), "allocate vertex records");
        AGB_CUDA(launchVertexRecords(g->positions.as<float>(), normals ? g->normals.as<float>() : nullptr,
                     texcoords ? g->texcoords.as<float>() : nullptr, vertex_count, g->verts.as<float4>(), ctx->stream),
            "build vertex records");
        AGB_CUDA(cudaStreamSynchronize(ctx->stream), "build vertex records");
        DevMesh& m      = g->mesh;
        m.positions     = g->positions.as<float>();
        m.normals       = normals ? g->normals.as<float>() : nullptr;
        m.texcoords     = texcoords ? g->texcoords.as<float>() : nullptr;
        m.verts         = g->verts.as<float4>();
        m.indices       = g->indices.as<uint32_t>();
        m.tris          = g->tris.as<float4>();
        m.nodes         = g->nodes.as<BNode>();
        m.vertexCount   = vertex_count;
        m.triangleCount = ntri;
        m.root          = root;
        m.depth         = depth;
        g->nodeCount    = nodeCount;
        ctx->geometries.push_back(std::move(g));
        *out_geometry = int32_t(ctx->geometries.size() - 1);
        return rebuildMeshTable(ctx);
    }
    for (int k = 0; k < 3; k++)
    {
        g->bounds[k]     = INFINITY;
        g->bounds[3 + k] = -INFINITY;
    }
    std::vector<float> boxes(size_t(ntri) * 6);
    for (uint32_t t = 0; t < ntri; t++)
    {
        float* b = &boxes[6 * size_t(t)];
        for (int k = 0; k < 3; k++)
        {
            b[k]     = INFINITY;
            b[3 + k] = -INFINITY;
        }
        for (int v = 0; v < 3; v++)
        {
            const float* p = positions + 3 * size_t(idx[3 * size_t(t) + v]);
            for (int k = 0; k < 3; k++)
            {
                if (!std::isfinite(p[k]))
                    return fail(AGB_ERR_INVALID_ARG, "agb_geometry_create: non-finite position");
                b[k]     = std::min(b[k], p[k]);
                b[3 + k] = std::max(b[3 + k], p[k]);
            }
        }
        for (int k = 0; k < 3; k++)
        {
            g->bounds[k]     = std::min(g->bounds[k], b[k]);
            g->bounds[3 + k] = std::max(g->bounds[3 + k], b[3 + k]);
        }
    }
    BuiltBVH bvh;
    buildBVH2(boxes.data(), ntri, 4, kBlasMaxDepth, bvh);
    if (bvh.depth > kBlasMaxDepth)
        return fail(AGB_ERR_LIMIT, "agb_geometry_create: BLAS deeper than the traversal stack allows");
    std::vector<float4> tris(size_t(ntri) * 3);
    for (uint32_t s = 0; s < ntri; s++)
    {
        uint32_t t = bvh.order[s];
        for (int v = 0; v < 3; v++)
        {
            const float* p = positions + 3 * size_t(idx[3 * size_t(t) + v]);
            tris[3 * size_t(s) + v] =
                make_float4(p[0], p[1], p[2], v == 0 ? bitsToFloat(int32_t(t)) : 0.f);
        }
    }
    st = upload(ctx, g->positions, positions, size_t(vertex_count) * 3 * sizeof(float), "upload positions");
    if (!st && normals)
        st = upload(ctx, g->normals, normals, size_t(vertex_count) * 3 * sizeof(float), "upload normals");
    if (!st && texcoords)
        st = upload(ctx, g->texcoords, texcoords, size_t(vertex_count) * 2 * sizeof(float), "upload texcoords");
    if (!st)
        st = upload(ctx, g->indices, idx.data(), idx.size() * sizeof(uint32_t), "upload indices");
    if (!st)
        st = upload(ctx, g->tris, tris.data(), tris.size() * sizeof(float4), "upload triangles");
    if (!st && !bvh.nodes.empty())
        st = upload(ctx, g->nodes, bvh.nodes.data(), bvh.nodes.size() * sizeof(BNode), "upload BVH");
    if (st)
        return st;
    AGB_CUDA(g->verts.ensure(size_t(vertex_count) * 2 * sizeof(float4)), "allocate vertex records");
    AGB_CUDA(launchVertexRecords(g->positions.as<float>(), normals ? g->normals.as<float>() : nullptr,
                 texcoords ? g->texcoords.as<float>() : nullptr, vertex_count, g->verts.as<float4>(), ctx->stream),
        "build vertex records");
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "upload geometry");
    DevMesh& m      = g->mesh;
    m.positions     = g->positions.as<float>();
    m.normals       = normals ? g->normals.as<float>() : nullptr;
    m.texcoords     = texcoords ? g->texcoords.as<float>() : nullptr;
    m.verts         = g->verts.as<float4>();
    m.indices       = g->indices.as<uint32_t>();
    m.tris          = g->tris.as<float4>();
    m.nodes         = g->nodes.as<BNode>();
    m.vertexCount   = vertex_count;
    m.triangleCount = ntri;
    m.root          = bvh.root;
    m.depth         = bvh.depth;
    g->nodeCount    = uint32_t(bvh.nodes.size());
    coverBoxes(bvh.nodes.data(), uint32_t(bvh.nodes.size()), bvh.root, g->bounds, g->cover);
    ctx->geometries.push_back(std::move(g));
    *out_geometry = int32_t(ctx->geometries.size() - 1);
    return rebuildMeshTable(ctx);
}

AGB_API uint64_t agb_bytes_per_path(void)
{
    return kPathStateBytes + kPathQueueBytes;
}

AGB_API agb_status agb_set_bvh_builder(agb_context* ctx, int32_t builder)
{
    if (!ctx || (builder != AGB_BVH_HOST && builder != AGB_BVH_GPU))
        return fail(AGB_ERR_INVALID_ARG, "agb_set_bvh_builder: bad builder");
    ctx->bvhBuilder = builder;
    return AGB_OK;
}

AGB_API agb_status agb_geometry_bvh(agb_context* ctx, int32_t geometry, float* nodes_out,
    uint64_t node_capacity, float* tris_out, uint64_t tri_capacity, int32_t* root, int32_t* depth,
    uint32_t* node_count)
{
    if (!ctx || geometry < 0 || geometry >= int32_t(ctx->geometries.size()))
        return fail(AGB_ERR_INVALID_ARG, "agb_geometry_bvh: bad geometry");
    const Geometry& g = *ctx->geometries[geometry];
    if ((nodes_out && node_capacity < g.nodeCount) || (tris_out && tri_capacity < g.mesh.triangleCount))
        return fail(AGB_ERR_INVALID_ARG, "agb_geometry_bvh: output too small");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    if (nodes_out && g.nodeCount)
        AGB_CUDA(cudaMemcpyAsync(nodes_out, g.nodes.ptr, size_t(g.nodeCount) * sizeof(BNode), cudaMemcpyDeviceToHost,
                     ctx->stream), "agb_geometry_bvh");
    if (tris_out)
        AGB_CUDA(cudaMemcpyAsync(tris_out, g.tris.ptr, size_t(g.mesh.triangleCount) * 3 * sizeof(float4),
                     cudaMemcpyDeviceToHost, ctx->stream), "agb_geometry_bvh");
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "agb_geometry_bvh");
    if (root)
        *root = g.mesh.root;
    if (depth)
        *depth = g.mesh.depth;
    if (node_count)
        *node_count = g.nodeCount;
    return AGB_OK;
}

AGB_API agb_status agb_tlas_read(agb_context* ctx, float* nodes_out, uint64_t node_capacity,
    int32_t* order_out, uint64_t order_capacity, int32_t* root, int32_t* depth, uint32_t* node_count)
{
    if (!ctx || ctx->parent)
        return fail(AGB_ERR_INVALID_ARG, "agb_tlas_read: a context with a scene is required");
    if ((nodes_out && node_capacity < ctx->tlasNodeCount) || (order_out && order_capacity < ctx->instanceCount))
        return fail(AGB_ERR_INVALID_ARG, "agb_tlas_read: output too small");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    if (nodes_out && ctx->tlasNodeCount)
        AGB_CUDA(cudaMemcpyAsync(nodes_out, ctx->tlasNodes.ptr, size_t(ctx->tlasNodeCount) * sizeof(BNode),
                     cudaMemcpyDeviceToHost, ctx->stream), "agb_tlas_read");
    if (order_out && ctx->instanceCount)
        AGB_CUDA(cudaMemcpyAsync(order_out, ctx->tlasOrder.ptr, size_t(ctx->instanceCount) * sizeof(int32_t),
                     cudaMemcpyDeviceToHost, ctx->stream), "agb_tlas_read");
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "agb_tlas_read");
    if (root)
        *root = ctx->tlasRoot;
    if (depth)
        *depth = ctx->tlasDepth;
    if (node_count)
        *node_count = ctx->tlasNodeCount;
    return AGB_OK;
}

AGB_API agb_status agb_image_create(agb_context* ctx, const void* pixels, uint32_t width,
    uint32_t height, int32_t format, int32_t linear, int32_t* out_image)
{
    if (ctx && !ctx->parent)
        ctx->sceneVersion++;
    if (ctx && ctx->parent)
        return fail(AGB_ERR_INVALID_ARG, "agb_image_create: a view shares its parent's scene; change the parent");
    if (!ctx || !pixels || !out_image || width == 0 || height == 0)
        return fail(AGB_ERR_INVALID_ARG, "agb_image_create: invalid argument");
    if (format != AGB_FORMAT_RGBA8_UNORM && format != AGB_FORMAT_RGBA32F && format != AGB_FORMAT_RGB32F)
        return fail(AGB_ERR_INVALID_ARG, "agb_image_create: unsupported format");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    std::unique_ptr<Image> im(new Image());
    size_t n = size_t(width) * height;
    if (format == AGB_FORMAT_RGB32F)
    {
        std::vector<float4> rgba(n);
        const float* p = static_cast<const float*>(pixels);
        for (size_t i = 0; i < n; i++)
            rgba[i] = make_float4(p[3 * i], p[3 * i + 1], p[3 * i + 2], 1.f);
        st = upload(ctx, im->data, rgba.data(), n * sizeof(float4), "upload image");
        format = AGB_FORMAT_RGBA32F;
        if (!st)
            AGB_CUDA(cudaStreamSynchronize(ctx->stream), "upload image");
    }
    else
    {
        size_t texel = format == AGB_FORMAT_RGBA8_UNORM ? 4 : 16;
        st = upload(ctx, im->data, pixels, n * texel, "upload image");
        if (!st)
            AGB_CUDA(cudaStreamSynchronize(ctx->stream), "upload image");
    }
    if (st)
        return st;
    im->view = DevImage{ im->data.ptr, width, height, format, linear ? 1 : 0 };
    ctx->images.push_back(std::move(im));
    std::vector<DevImage> table(ctx->images.size());
    for (size_t i = 0; i < table.size(); i++)
        table[i] = ctx->images[i]->view;
    st = upload(ctx, ctx->imageTable, table.data(), table.size() * sizeof(DevImage), "upload image table");
    if (st)
        return st;
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "upload image table");
    *out_image = int32_t(ctx->images.size() - 1);
    return AGB_OK;
}

AGB_API agb_status agb_materials_set(agb_context* ctx, const agb_material* materials,
    const agb_material_textures* textures, uint32_t count)
{
    if (ctx && !ctx->parent)
        ctx->sceneVersion++;
    if (ctx && ctx->parent)
        return fail(AGB_ERR_INVALID_ARG, "agb_materials_set: a view shares its parent's scene; change the parent");
    if (!ctx || (!materials && count))
        return fail(AGB_ERR_INVALID_ARG, "agb_materials_set: null argument");
    if (textures)
        for (uint32_t i = 0; i < count; i++)
            for (int k = 0; k < AGB_TEX_SLOTS; k++)
                if (textures[i].image[k] >= int32_t(ctx->images.size()))
                    return fail(AGB_ERR_INVALID_ARG, "agb_materials_set: texture image index out of range");
    agb_status st = setDevice(ctx);
    if (!st)
        st = upload(ctx, ctx->materials, materials, size_t(count) * sizeof(agb_material), "upload materials");
    if (!st && textures)
        st = upload(ctx, ctx->matTex, textures, size_t(count) * sizeof(agb_material_textures), "upload material textures");
    if (st)
        return st;
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "upload materials");
    ctx->materialCount = count;
    ctx->hasMatTex     = textures != nullptr;
    ctx->hostMaterials.assign(materials, materials + count);
    if (textures)
        ctx->hostMatTex.assign(textures, textures + count);
    else
        ctx->hostMatTex.clear();
    ctx->hasGraphs = false; // programs belong to the material table they were set for
    return AGB_OK;
}

AGB_API agb_status agb_material_graphs_set(agb_context* ctx, const int32_t* first, const int32_t* count,
    uint32_t material_count, const agb_graph_op* ops, uint32_t op_count, const float* constants,
    uint32_t constant_count)
{
    if (ctx && !ctx->parent)
        ctx->sceneVersion++;
    if (ctx && ctx->parent)
        return fail(AGB_ERR_INVALID_ARG, "agb_material_graphs_set: a view shares its parent's scene; change the parent");
    if (!ctx || (material_count && (!first || !count)) || (op_count && !ops) || (constant_count && !constants))
        return fail(AGB_ERR_INVALID_ARG, "agb_material_graphs_set: null argument");
    if (material_count != ctx->materialCount)
        return fail(AGB_ERR_INVALID_ARG, "agb_material_graphs_set: one (first, count) pair per material of the current table");
    if (constant_count > 65536u)
        return fail(AGB_ERR_LIMIT, "agb_material_graphs_set: at most 65536 constants");
    bool any = false;
    for (uint32_t m = 0; m < material_count; m++)
    {
        if (count[m] == 0)
            continue;
        if (count[m] < 0 || count[m] > AGB_GRAPH_MAX_OPS || first[m] < 0 || int64_t(first[m]) + count[m] > int64_t(op_count))
            return fail(AGB_ERR_INVALID_ARG, "agb_material_graphs_set: program range of material " + std::to_string(m));
        any = true;
    }
    const uint32_t images = uint32_t(ctx->images.size());
    for (uint32_t k = 0; k < op_count; k++)
    {
        const agb_graph_op& o = ops[k];
        bool ok = o.op < AGB_GOP_COUNT && o.dst < AGB_GRAPH_REGS && o.a < AGB_GRAPH_REGS && o.b < AGB_GRAPH_REGS &&
            o.c < AGB_GRAPH_REGS && o.d < AGB_GRAPH_REGS;
        if (ok && o.op == AGB_GOP_CONST)
            ok = o.imm < constant_count;
        if (ok && o.op == AGB_GOP_INPUT)
            ok = o.imm < AGB_GIN_COUNT;
        if (ok && o.op == AGB_GOP_IMAGE)
            ok = o.imm < images;
        if (ok && o.op == AGB_GOP_OUTPUT)
            ok = o.imm < AGB_GOUT_COUNT;
        if (ok && o.op == AGB_GOP_SELECT)
            ok = o.imm <= 2;
        if (ok && o.op == AGB_GOP_NOISE)
            ok = o.imm <= 3;
        if (ok && (o.op == AGB_GOP_DOT || o.op == AGB_GOP_NORMALIZE || o.op == AGB_GOP_LENGTH))
            ok = o.d >= 1 && o.d <= 4;
        if (!ok)
            return fail(AGB_ERR_INVALID_ARG, "agb_material_graphs_set: invalid operation " + std::to_string(k));
    }
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    if (!any)
    {
        ctx->hasGraphs = false;
        return AGB_OK;
    }
    std::vector<int2> table(material_count);
    for (uint32_t m = 0; m < material_count; m++)
        table[m] = make_int2(first[m], count[m]);
    std::vector<float> k4(size_t(std::max(constant_count, 1u)) * 4, 0.f);
    if (constant_count)
        std::memcpy(k4.data(), constants, size_t(constant_count) * 16);
    if ((st = upload(ctx, ctx->matGraph, table.data(), table.size() * sizeof(int2), "upload material graphs")) ||
        (st = upload(ctx, ctx->graphOps, ops, size_t(op_count) * sizeof(agb_graph_op), "upload material graphs")) ||
        (st = upload(ctx, ctx->graphConsts, k4.data(), k4.size() * sizeof(float), "upload material graphs")))
        return st;
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "upload material graphs");
    ctx->hasGraphs = true;
    return AGB_OK;
}

AGB_API agb_status agb_instances_set(agb_context* ctx, const agb_instance* inst, uint32_t count)
{
    if (ctx && !ctx->parent)
        ctx->sceneVersion++;
    if (ctx && ctx->parent)
        return fail(AGB_ERR_INVALID_ARG, "agb_instances_set: a view shares its parent's scene; change the parent");
    if (!ctx || (!inst && count))
        return fail(AGB_ERR_INVALID_ARG, "agb_instances_set: null argument");
    if (count >= (1u << 27))
        return fail(AGB_ERR_LIMIT, "agb_instances_set: too many instances");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    std::vector<DevInstance> di(count);
    std::vector<DevLayer> dl;
    std::vector<std::unique_ptr<DevBuf>> uvs;
    std::map<std::pair<const float*, size_t>, const float*> uvUploads;
    std::vector<float> boxes(size_t(count) * 6);
    for (uint32_t i = 0; i < count; i++)
    {
        const agb_instance& s = inst[i];
        if (s.geometry < 0 || size_t(s.geometry) >= ctx->geometries.size())
            return fail(AGB_ERR_INVALID_ARG, "agb_instances_set: instance " + std::to_string(i) + " geometry out of range");
        if (s.material < 0 || uint32_t(s.material) >= ctx->materialCount)
            return fail(AGB_ERR_INVALID_ARG, "agb_instances_set: instance " + std::to_string(i) + " material out of range");
        if (s.layer_count < 0 || s.layer_count > 64 || (s.layer_count > 0 && !s.layers))
            return fail(AGB_ERR_INVALID_ARG, "agb_instances_set: bad layer list");
        for (int k = 0; k < 12; k++)
            if (!std::isfinite(s.object_to_world[k]))
                return fail(AGB_ERR_INVALID_ARG, "agb_instances_set: non-finite transform");
        DevInstance& d = di[i];
        memcpy(d.o2w, s.object_to_world, sizeof d.o2w);
        invertAffine(d.o2w, d.w2o);
        for (int k = 0; k < 12; k++)
            if (!std::isfinite(d.w2o[k]))
                return fail(AGB_ERR_INVALID_ARG, "agb_instances_set: singular transform");
        d.mesh        = s.geometry;
        d.material    = s.material;
        d.layerCount  = s.layer_count;
        d.layerOffset = int32_t(dl.size());
        const Geometry& g = *ctx->geometries[s.geometry];
        for (int l = 0; l < s.layer_count; l++)
        {
            const agb_layer& L = s.layers[l];
            if (L.material < 0 || uint32_t(L.material) >= ctx->materialCount || !L.texcoords)
                return fail(AGB_ERR_INVALID_ARG, "agb_instances_set: bad layer material or UVs");
            // Instances that share a layer UV array (one per BLAS, typically) share its upload.
            const size_t bytes = size_t(g.mesh.vertexCount) * 2 * sizeof(float);
            auto key           = std::make_pair(L.texcoords, bytes);
            auto hit           = uvUploads.find(key);
            const float* dev   = nullptr;
            if (hit != uvUploads.end())
                dev = hit->second;
            else
            {
                std::unique_ptr<DevBuf> b(new DevBuf());
                st = upload(ctx, *b, L.texcoords, bytes, "upload layer UVs");
                if (st)
                    return st;
                dev = b->as<float>();
                uvUploads.emplace(key, dev);
                uvs.push_back(std::move(b));
            }
            // Layers are applied outermost first: the reference loops li = count .. 1 over
            // layer index li - 1, so store them in the given order.
            dl.push_back(DevLayer{ L.material, 0, dev });
        }
        float* box = &boxes[6 * size_t(i)];
        for (int k = 0; k < 3; k++)
        {
            box[k]     = INFINITY;
            box[3 + k] = -INFINITY;
        }
        // Union of the transformed corners of the mesh's cover boxes.
        for (size_t cb = 0; cb < g.cover.size(); cb += 6)
        {
            const float* gb = &g.cover[cb];
            for (int c = 0; c < 8; c++)
            {
                float p[3] = { (c & 1) ? gb[3] : gb[0], (c & 2) ? gb[4] : gb[1], (c & 4) ? gb[5] : gb[2] };
                for (int r = 0; r < 3; r++)
                {
                    float w = d.o2w[4 * r] * p[0] + d.o2w[4 * r + 1] * p[1] + d.o2w[4 * r + 2] * p[2] +
                        d.o2w[4 * r + 3];
                    box[r]     = std::min(box[r], w);
                    box[3 + r] = std::max(box[3 + r], w);
                }
            }
        }
        for (int k = 0; k < 3; k++)
        {
            float pad = 1e-5f * (std::fabs(box[k]) + std::fabs(box[3 + k])) + 1e-6f;
            box[k] -= pad;
            box[3 + k] += pad;
        }
    }
    for (int k = 0; k < 3; k++)
    {
        float lo = INFINITY, hi = -INFINITY;
        for (uint32_t i = 0; i < count; i++)
        {
            lo = std::min(lo, boxes[6 * size_t(i) + k]);
            hi = std::max(hi, boxes[6 * size_t(i) + 3 + k]);
        }
        ctx->sceneLo[k] = count ? lo : 0.f;
        ctx->sceneHi[k] = count ? hi : 0.f;
    }
    // TLAS depth budget: the traversal stack holds the TLAS path, an instance-exit marker and the
    // deepest BLAS path.  Near the budget the builders split at the index midpoint, so any tree
    // with ceil(log2(count)) + 2 levels to spare fits; beyond that the stack cannot hold the scene.
    int maxBlas = 0;
    for (auto& g : ctx->geometries)
        maxBlas = std::max(maxBlas, g->mesh.depth);
    const int tlasBudget = kStackSize - 2 - maxBlas;
    int need = 0;
    while ((1u << need) < count)
        need++;
    if (count > 1 && need + 2 > tlasBudget)
        return fail(AGB_ERR_LIMIT, "agb_instances_set: " + std::to_string(count) +
            " instances need a TLAS deeper than the traversal stack leaves beside the deepest BLAS (" +
            std::to_string(maxBlas) + " levels)");
    st = upload(ctx, ctx->instances, di.data(), di.size() * sizeof(DevInstance), "upload instances");
    if (!st && !dl.empty())
        st = upload(ctx, ctx->layers, dl.data(), dl.size() * sizeof(DevLayer), "upload layers");
    if (st)
        return st;
    int32_t tlasRoot = 0, tlasDepth = 0;
    uint32_t nodeCount = 0;
    if (ctx->bvhBuilder == AGB_BVH_GPU && count > 0)
    {
        // Binned SAH over the instance boxes on the GPU (the BLAS builder's kernel, one instance
        // per leaf); nodes and leaf order are written straight into the scene's arrays.
        AGB_CUDA(ctx->tlasNodes.ensure(std::max<size_t>(1, count) * sizeof(BNode)), "allocate TLAS");
        AGB_CUDA(ctx->tlasOrder.ensure(size_t(count) * sizeof(int32_t)), "allocate TLAS order");
        AGB_CUDA(buildTlasGpu(boxes.data(), count, tlasBudget, ctx->bvhScratch, ctx->tlasNodes.as<BNode>(),
                     std::max<uint32_t>(1, count), ctx->tlasOrder.as<int32_t>(), &tlasRoot, &tlasDepth,
                     &nodeCount, ctx->stream),
            "agb_instances_set: GPU TLAS build");
    }
    else
    {
        BuiltBVH tl;
        buildBVH2(boxes.data(), count, 1, tlasBudget, tl);
        std::vector<int32_t> order(tl.order.begin(), tl.order.end());
        if (!tl.nodes.empty())
            st = upload(ctx, ctx->tlasNodes, tl.nodes.data(), tl.nodes.size() * sizeof(BNode), "upload TLAS");
        if (!st)
            st = upload(ctx, ctx->tlasOrder, order.data(), order.size() * sizeof(int32_t), "upload TLAS order");
        if (st)
            return st;
        tlasRoot  = tl.root;
        tlasDepth = tl.depth;
        nodeCount = uint32_t(tl.nodes.size());
    }
    if (tlasDepth + maxBlas + 2 > kStackSize)
        return fail(AGB_ERR_LIMIT, "agb_instances_set: TLAS + BLAS depth exceeds the traversal stack");
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "upload instances");
    ctx->layerUVs      = std::move(uvs);
    ctx->instanceCount = count;
    ctx->tlasRoot      = tlasRoot;
    ctx->tlasDepth     = tlasDepth;
    ctx->tlasNodeCount = nodeCount;
    ctx->hostInstances = std::move(di);
    ctx->hostLayers    = std::move(dl);
    return AGB_OK;
}

AGB_API agb_status agb_environment_set(agb_context* ctx, const agb_environment_data* env,
    int32_t light_image, int32_t background_image)
{
    if (ctx && !ctx->parent)
        ctx->sceneVersion++;
    if (ctx && ctx->parent)
        return fail(AGB_ERR_INVALID_ARG, "agb_environment_set: a view shares its parent's scene; change the parent");
    if (!ctx || !env)
        return fail(AGB_ERR_INVALID_ARG, "agb_environment_set: null argument");
    if (light_image >= int32_t(ctx->images.size()) || background_image >= int32_t(ctx->images.size()))
        return fail(AGB_ERR_INVALID_ARG, "agb_environment_set: image index out of range");
    if (light_image >= 0 && ctx->images[light_image]->view.format != AGB_FORMAT_RGBA32F)
        return fail(AGB_ERR_INVALID_ARG, "agb_environment_set: light image must be float RGB(A)");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    ctx->env           = *env;
    ctx->envLight      = light_image;
    ctx->envBackground = background_image;
    ctx->env.has_light_tex      = light_image >= 0 ? 1 : 0;
    ctx->env.has_background_tex = background_image >= 0 ? 1 : 0;
    if (light_image >= 0)
    {
        const DevImage& v = ctx->images[light_image]->view;
        uint64_t n = uint64_t(v.width) * v.height;
        if (n >= (1ull << 31))
            return fail(AGB_ERR_LIMIT, "agb_environment_set: light image too large");
        AGB_CUDA(ctx->alias.ensure(n * sizeof(agb_alias_entry)), "allocate alias table");
        // Per-row solid angles exactly as the reference computes them on the host
        // (AliasMap.cpp:101-110): FP32 increments, FP32 running latitude, float sin.
        std::vector<float> rowSA(v.height);
        {
            const double kPi   = 3.14159265358979323846;
            float lonIncrement = static_cast<float>(2.0f * kPi / v.width);
            float latIncrement = static_cast<float>(kPi / v.height);
            float latAngle     = static_cast<float>(kPi / 2.0);
            for (uint32_t y = 0; y < v.height; y++)
            {
                rowSA[y] = (std::sin(latAngle) - std::sin(latAngle - latIncrement)) * lonIncrement;
                latAngle -= latIncrement;
            }
        }
        double integral = 0.0;
        float shadingIntegral = 0.f;
        AGB_CUDA(buildEnvAlias(static_cast<const float4*>(v.data), v.width, v.height, ctx->envLayout,
                     rowSA.data(), ctx->alias.as<agb_alias_entry>(), &integral, &shadingIntegral,
                     ctx->envScratch, ctx->stream),
            "build environment alias table");
        ctx->envIntegral        = integral;
        ctx->envShadingIntegral = shadingIntegral;
        ctx->env.light_tex_luminance_integral = shadingIntegral;
    }
    return AGB_OK;
}

AGB_API agb_status agb_set_environment_table(agb_context* ctx, int32_t layout)
{
    if (ctx && !ctx->parent)
        ctx->sceneVersion++;
    if (ctx && ctx->parent)
        return fail(AGB_ERR_INVALID_ARG, "agb_set_environment_table: a view shares its parent's scene; change the parent");
    if (!ctx || (layout != AGB_ENV_TABLE_REFERENCE && layout != AGB_ENV_TABLE_FP64))
        return fail(AGB_ERR_INVALID_ARG, "agb_set_environment_table: bad layout");
    ctx->envLayout = layout;
    return AGB_OK;
}

AGB_API agb_status agb_ground_plane_set(agb_context* ctx, const agb_ground_plane* plane)
{
    if (ctx && !ctx->parent)
        ctx->sceneVersion++;
    if (ctx && ctx->parent)
        return fail(AGB_ERR_INVALID_ARG, "agb_ground_plane_set: a view shares its parent's scene; change the parent");
    if (!ctx)
        return fail(AGB_ERR_INVALID_ARG, "agb_ground_plane_set: null context");
    DevGroundPlane g{};
    if (plane)
    {
        const float* n = plane->normal;
        if (!(n[0] * n[0] + n[1] * n[1] + n[2] * n[2] > 0.f))
            return fail(AGB_ERR_INVALID_ARG, "agb_ground_plane_set: zero or non-finite normal");
        g.enabled = plane->enabled ? 1 : 0;
        for (int k = 0; k < 3; k++)
        {
            g.position[k]        = plane->position[k];
            g.normal[k]          = n[k];
            g.shadowColor[k]     = plane->shadow_color[k];
            g.reflectionColor[k] = plane->reflection_color[k];
        }
        g.shadowOpacity       = plane->shadow_opacity;
        g.reflectionOpacity   = plane->reflection_opacity;
        g.reflectionRoughness = plane->reflection_roughness;
        // Tangent frame from the normal (PTGroundPlane.cpp:23-28): bitangent +Y unless the normal
        // is within 0.999 of it, then +X; tangent = normalize(cross(bitangent, normal)),
        // bitangent = cross(normal, tangent).
        float b[3] = { 0.f, 1.f, 0.f };
        if (!(std::fabs(n[1]) < 0.999f))
        {
            b[0] = 1.f;
            b[1] = 0.f;
        }
        float t[3] = { b[1] * n[2] - b[2] * n[1], b[2] * n[0] - b[0] * n[2], b[0] * n[1] - b[1] * n[0] };
        float inv  = 1.f / std::sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
        for (int k = 0; k < 3; k++)
            g.tangent[k] = t[k] * inv;
        const float* u = g.tangent;
        g.bitangent[0] = n[1] * u[2] - n[2] * u[1];
        g.bitangent[1] = n[2] * u[0] - n[0] * u[2];
        g.bitangent[2] = n[0] * u[1] - n[1] * u[0];
    }
    ctx->ground = g;
    return AGB_OK;
}

AGB_API agb_status agb_environment_alias(agb_context* ctx, agb_alias_entry* host_out,
    uint64_t capacity, double* shading_integral, double* fp64_integral)
{
    if (!ctx || ctx->envLight < 0)
        return fail(AGB_ERR_NOT_READY, "agb_environment_alias: no light image");
    const DevImage& v = ctx->images[ctx->envLight]->view;
    uint64_t n = uint64_t(v.width) * v.height;
    if (!host_out || capacity < n)
        return fail(AGB_ERR_INVALID_ARG, "agb_environment_alias: output too small");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    AGB_CUDA(cudaMemcpyAsync(host_out, ctx->alias.ptr, n * sizeof(agb_alias_entry),
                 cudaMemcpyDeviceToHost, ctx->stream),
        "read alias table");
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "read alias table");
    if (shading_integral)
        *shading_integral = ctx->envShadingIntegral;
    if (fp64_integral)
        *fp64_integral = ctx->envIntegral;
    return AGB_OK;
}

AGB_API agb_status agb_environment_alias_build_noalloc(const float* rgba_device, uint32_t width,
    uint32_t height, int32_t layout, agb_alias_entry* table_device, double* shading_integral,
    double* fp64_integral, void* stream)
{
    if (!rgba_device || !table_device)
        return fail(AGB_ERR_INVALID_ARG, "agb_environment_alias_build_noalloc: null device pointer");
    if (width == 0 || height == 0)
        return fail(AGB_ERR_INVALID_ARG, "agb_environment_alias_build_noalloc: empty image");
    if (layout != AGB_ENV_TABLE_REFERENCE && layout != AGB_ENV_TABLE_FP64)
        return fail(AGB_ERR_INVALID_ARG, "agb_environment_alias_build_noalloc: bad layout");
    if (uint64_t(width) * height > AGB_ENV_NOALLOC_MAX_TEXELS)
        return fail(AGB_ERR_LIMIT, "agb_environment_alias_build_noalloc: " + std::to_string(width) +
                                       "x" + std::to_string(height) + " = " +
                                       std::to_string(uint64_t(width) * height) +
                                       " texels exceeds the limit of " +
                                       std::to_string(AGB_ENV_NOALLOC_MAX_TEXELS) +
                                       " texels (AGB_ENV_NOALLOC_MAX_TEXELS)");
    if ((reinterpret_cast<uintptr_t>(rgba_device) & 15u) || (reinterpret_cast<uintptr_t>(table_device) & 15u))
        return fail(AGB_ERR_INVALID_ARG, "agb_environment_alias_build_noalloc: device pointers must be "
                                         "16-byte aligned");
    double integral       = 0.0;
    float shadingIntegral = 0.f;
    AGB_CUDA(buildEnvAliasNoAlloc(reinterpret_cast<const float4*>(rgba_device), width, height, layout,
                 table_device, &integral, &shadingIntegral, static_cast<cudaStream_t>(stream)),
        "agb_environment_alias_build_noalloc");
    if (shading_integral)
        *shading_integral = shadingIntegral;
    if (fp64_integral)
        *fp64_integral = integral;
    return AGB_OK;
}

AGB_API agb_status agb_frame_set(agb_context* ctx, const agb_frame_data* frame)
{
    if (!ctx || !frame)
        return fail(AGB_ERR_INVALID_ARG, "agb_frame_set: null argument");
    ctx->frame = *frame;
    // RendererBase.cpp:280-282 clamps the trace depth to [1, kMaxTraceDepth = 10].
    ctx->frame.trace_depth = std::max(1, std::min(10, ctx->frame.trace_depth));
    if (ctx->frame.distant_light_count < 0 || ctx->frame.distant_light_count > 4)
        return fail(AGB_ERR_INVALID_ARG, "agb_frame_set: distant_light_count must be 0..4");
    ctx->frameSet = true;
    return AGB_OK;
}

AGB_API agb_status agb_render(agb_context* ctx, const agb_render_options* opt,
    uint32_t sample_start, uint32_t sample_count, agb_render_stats* stats)
{
    if (!ctx || !opt)
        return fail(AGB_ERR_INVALID_ARG, "agb_render: null argument");
    if (!ctx->frameSet)
        return fail(AGB_ERR_NOT_READY, "agb_render: frame data not set");
    if (opt->width == 0 || opt->height == 0 || uint64_t(opt->width) * opt->height > (1ull << 26))
        return fail(AGB_ERR_INVALID_ARG, "agb_render: bad image size");
    const agb_context* sc = ctx->parent ? ctx->parent : ctx;
    if (sc->instanceCount > 0 && sc->materialCount == 0)
        return fail(AGB_ERR_NOT_READY, "agb_render: no materials");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    uint32_t accumMode = opt->accumulation ? opt->accumulation : AGB_ACCUM_RUNNING_MEAN;
    uint32_t pixels    = opt->width * opt->height;
    uint32_t spw = 1;
    const bool explicitWave = opt->max_paths_in_flight && opt->max_paths_in_flight != AGB_WAVE_LARGEST;
    if (explicitWave)
    {
        spw = uint32_t(std::max<uint64_t>(1, opt->max_paths_in_flight / pixels));
        spw = std::min(spw, std::max(1u, sample_count));
    }
    else
    {
        // The call's samples in as few waves as fit, split evenly.  Default: wave buffers of at
        // most AGB_WAVE_DEFAULT_BYTES (a library that shares the device with its host takes a
        // bounded amount).  AGB_WAVE_LARGEST: half of the device memory that is free (counting
        // this context's wave buffers as free) and at most a third of the device: one wave of
        // 82 GB for 64 samples of 1920x1080 on an idle 288 GB device.  Fewer, larger waves keep
        // every bounce's launch full and pay each launch's tail once per bounce instead of once
        // per wave and bounce (about 4 % at that size).
        size_t freeBytes = 0, totalBytes = ctx->deviceBytes;
        if (cudaMemGetInfo(&freeBytes, &totalBytes) != cudaSuccess)
            freeBytes = totalBytes / 4;
        const uint64_t perPath = kPathStateBytes + kPathQueueBytes;
        uint64_t held   = uint64_t(ctx->pathCapacity) * perPath;
        uint64_t bytes  = std::min<uint64_t>((uint64_t(freeBytes) + held) / 2, uint64_t(totalBytes) / 3);
        if (!opt->max_paths_in_flight)
            bytes = std::min<uint64_t>(bytes, AGB_WAVE_DEFAULT_BYTES);
        uint64_t budget = std::max<uint64_t>(pixels, bytes / perPath);
        budget          = std::min<uint64_t>(budget, (1ull << 29) - 1);
        uint32_t most   = uint32_t(std::max<uint64_t>(1, budget / pixels));
        uint32_t count  = std::max(1u, sample_count);
        uint32_t n      = (count + most - 1) / most;
        spw             = (count + n - 1) / n;
    }
    if (uint64_t(spw) * pixels >= (1ull << 29))
        return fail(AGB_ERR_LIMIT, "agb_render: wave too large");
    int depth = ctx->frame.trace_depth;
    st = ensureAccum(ctx, opt->width, opt->height);
    if (st)
        return st;
    uint32_t waves = 0;
    for (;;)
    {
        waves = sample_count ? (sample_count + spw - 1) / spw : 0;
        st    = ensureWave(ctx, size_t(spw) * pixels, depth, std::max(1u, waves));
        if (st != AGB_ERR_OOM || explicitWave || spw == 1)
            break;
        // The default wave did not fit after all (memory taken meanwhile): halve it.
        cudaGetLastError();
        spw = (spw + 1) / 2;
    }
    if (st)
        return st;
    if (sample_start == 0)
        ctx->accumulatedSamples = 0;
    else if (ctx->accumulatedSamples != sample_start || (ctx->lastAccumMode & accumMode) != accumMode)
        return fail(AGB_ERR_INVALID_ARG, "agb_render: sample_start must continue the accumulated "
                                         "sequence in the same accumulation mode");
    // Denoising AOVs: written by the primary paths of the call's last sample.
    uint32_t aovSample = ~0u;
    if (ctx->frame.is_denoising_aovs_enabled)
    {
        AGB_CUDA(ctx->aovDepth.ensure(size_t(pixels) * sizeof(float)), "allocate AOVs");
        AGB_CUDA(ctx->aovNormal.ensure(size_t(pixels) * sizeof(float4)), "allocate AOVs");
        AGB_CUDA(ctx->aovAlbedo.ensure(size_t(pixels) * sizeof(float4)), "allocate AOVs");
        AGB_CUDA(ctx->aovMotion.ensure(size_t(pixels) * sizeof(float4)), "allocate AOVs");
        ctx->wb.aovDepth  = ctx->aovDepth.as<float>();
        ctx->wb.aovNormal = ctx->aovNormal.as<float4>();
        ctx->wb.aovAlbedo = ctx->aovAlbedo.as<float4>();
        ctx->wb.aovMotion = ctx->aovMotion.as<float4>();
        aovSample         = sample_start + sample_count - 1;
    }
    ctx->aovValid = ctx->frame.is_denoising_aovs_enabled != 0;
    size_t counterWords = size_t(depth + 2) * kCounterStride;
    AGB_CUDA(cudaMemsetAsync(ctx->counters.ptr, 0, counterWords * waves * sizeof(uint32_t), ctx->stream),
        "clear counters");
    AGB_CUDA(cudaMemsetAsync(ctx->stats.ptr, 0, 8 * sizeof(unsigned long long), ctx->stream), "clear stats");
    DevScene scene = ctx->scene();
    WaveBuffers wb = ctx->wb;
    wb.accumMean  = ctx->accMean.as<float4>();
    wb.accumSum   = ctx->accSum.as<float4>();
    wb.accumComp  = ctx->accComp.as<float4>();
    wb.lastSample = ctx->lastSample.as<float4>();
    wb.accumMoments = ctx->accMoments.as<float2>();
    uint64_t launches = 0;
    ctx->marks.reset();
    KernelMarks* marks = ctx->profiling ? &ctx->marks : nullptr;
    AGB_CUDA(cudaEventRecord(ctx->ev0, ctx->stream), "record event");
    for (uint32_t w = 0; w < waves; w++)
    {
        WaveParams wp{};
        wp.width          = opt->width;
        wp.height         = opt->height;
        wp.pixels         = pixels;
        wp.sampleBase     = sample_start + w * spw;
        wp.samples        = std::min(spw, sample_start + sample_count - wp.sampleBase);
        wp.paths          = wp.samples * pixels;
        wp.accumMode      = accumMode;
        wp.countTraversal = ctx->counting ? 1 : 0;
        wp.aovSample      = aovSample;
        wp.seedOffset     = opt->seed_offset;
        wp.binRays        = ctx->binRays ? 1 : 0;
        for (int k = 0; k < 3; k++)
        {
            wp.binLo[k]    = sc->sceneLo[k];
            float ext      = sc->sceneHi[k] - sc->sceneLo[k];
            wp.binScale[k] = ext > 0.f ? 16.f / ext : 0.f;
        }
        wb.counters       = ctx->counters.as<uint32_t>() + counterWords * w;
        launchWave(scene, ctx->frame, wp, wb, ctx->stream, ctx->smCount, launches, marks);
        AGB_CUDA(cudaGetLastError(), "launch wave");
    }
    AGB_CUDA(cudaEventRecord(ctx->ev1, ctx->stream), "record event");
    ctx->accumulatedSamples = sample_start + sample_count;
    ctx->lastAccumMode      = sample_start == 0 ? accumMode : ctx->lastAccumMode;
    if (stats)
    {
        AGB_CUDA(cudaEventSynchronize(ctx->ev1), "render");
        std::vector<uint32_t> c(counterWords * waves);
        AGB_CUDA(cudaMemcpy(c.data(), ctx->counters.ptr, c.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost),
            "read counters");
        unsigned long long s[8];
        AGB_CUDA(cudaMemcpy(s, ctx->stats.ptr, sizeof s, cudaMemcpyDeviceToHost), "read stats");
        if (s[4])
            return fail(AGB_ERR_LIMIT, "agb_render: traversal stack overflow");
        agb_render_stats r{};
        r.paths = uint64_t(sample_count) * pixels;
        for (uint32_t w = 0; w < waves; w++)
        {
            for (int b = 0; b < depth; b++)
            {
                const uint64_t cr = c[counterWords * w + kCounterStride * b + CNT_RAYS];
                const uint64_t sr = uint64_t(c[counterWords * w + kCounterStride * b + CNT_SHADOW]) +
                    c[counterWords * w + kCounterStride * b + CNT_GROUND_SHADOW];
                r.closest_rays += cr;
                r.shading_points += c[counterWords * w + kCounterStride * b + CNT_SCATTER];
                r.shadow_rays += sr;
                if (b < 16)
                {
                    r.closest_rays_per_bounce[b] += cr;
                    r.shadow_rays_per_bounce[b] += sr;
                }
            }
        }
        r.node_visits        = s[2];
        r.tri_tests          = s[3];
        r.shadow_node_visits = s[5];
        r.shadow_tri_tests   = s[6];
        r.kernel_launches    = launches;
        if (marks)
        {
            double ms[KC_COUNT];
            marks->sum(ms);
            for (int k = 0; k < 6; k++)
                r.kernel_ms[k] = ms[k];
            for (size_t i = 0; i < marks->category.size(); i++)
                if (marks->category[i] < 6)
                    r.kernel_count[marks->category[i]]++;
        }
        float ms = 0.f;
        AGB_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1), "event time");
        r.gpu_ms = ms;
        *stats   = r;
    }
    return AGB_OK;
}

// ------------------------------------------------------------------------- batched rendering
// Several requests (views or contexts, of one or several scenes, any resolutions) rendered by
// one wavefront: every stage is one launch over all of their paths (BatchTables in
// agb_wavefront.cuh).  The scenes' tables are concatenated into a shared namespace, rebuilt when
// the set of scenes or any of them changes.
struct agb_batch
{
    agb_context* work = nullptr; // wave buffers, counters, stats, events and the stream; no scene
    uint64_t maxPaths = 0;
    // Shared namespace of the scenes of the last call.
    std::vector<const agb_context*> scenes;
    std::vector<uint64_t> versions;
    DevBuf meshes, instances, tlas, tlasOrder, materials, matTex, images, layers;
    std::vector<DevScene> sceneTable;
    DevBuf sceneTableDev, reqTable, frameTable, pathReq;
    cudaEvent_t done = nullptr;
    ~agb_batch()
    {
        if (done)
            cudaEventDestroy(done);
        delete work;
    }
};

namespace
{

int32_t remapTlasRef(int32_t ref, uint32_t nodeOff, uint32_t orderOff)
{
    if (ref >= 0)
        return ref + int32_t(nodeOff);
    uint32_t code  = uint32_t(~ref);
    uint32_t first = code >> 3, cnt = code & 7u;
    return ~int32_t(((first + orderOff) << 3) | cnt);
}

agb_status buildSharedScenes(agb_batch* b, const std::vector<agb_context*>& scenes)
{
    bool same = scenes.size() == b->scenes.size();
    for (size_t k = 0; same && k < scenes.size(); k++)
        same = scenes[k] == b->scenes[k] && scenes[k]->sceneVersion == b->versions[k];
    if (same)
        return AGB_OK;
    cudaStream_t st = b->work->stream;
    std::vector<DevMesh> M;
    std::vector<DevInstance> I;
    std::vector<DevLayer> L;
    std::vector<agb_material> Mt;
    std::vector<agb_material_textures> T;
    std::vector<DevImage> Im;
    std::vector<BNode> N;
    std::vector<int32_t> O;
    std::vector<DevScene> table;
    bool anyTex = false;
    for (agb_context* sc : scenes)
        anyTex = anyTex || sc->hasMatTex;
    for (agb_context* sc : scenes)
    {
        if (sc->ground.enabled)
            return fail(AGB_ERR_INVALID_ARG, "agb_batch_render: scenes with a ground plane render alone");
        if (sc->hasGraphs)
            return fail(AGB_ERR_INVALID_ARG, "agb_batch_render: scenes with material node graphs render alone");
        if (sc->hostMaterials.size() != sc->materialCount || sc->hostInstances.size() != sc->instanceCount)
            return fail(AGB_ERR_NOT_READY, "agb_batch_render: a scene has no materials or instances set");
        const uint32_t meshOff = uint32_t(M.size()), instOff = uint32_t(I.size()), layerOff = uint32_t(L.size());
        const uint32_t matOff = uint32_t(Mt.size()), imgOff = uint32_t(Im.size()), nodeOff = uint32_t(N.size());
        const uint32_t orderOff = uint32_t(O.size());
        for (auto& g : sc->geometries)
            M.push_back(g->mesh);
        for (auto& im : sc->images)
            Im.push_back(im->view);
        Mt.insert(Mt.end(), sc->hostMaterials.begin(), sc->hostMaterials.end());
        for (uint32_t m = 0; m < sc->materialCount; m++)
        {
            agb_material_textures t;
            for (int k = 0; k < AGB_TEX_SLOTS; k++)
            {
                int32_t v  = sc->hasMatTex ? sc->hostMatTex[m].image[k] : -1;
                t.image[k] = v >= 0 ? v + int32_t(imgOff) : -1;
            }
            T.push_back(t);
        }
        for (DevLayer l : sc->hostLayers)
        {
            l.material += int32_t(matOff);
            L.push_back(l);
        }
        for (DevInstance in : sc->hostInstances)
        {
            in.mesh += int32_t(meshOff);
            in.material += int32_t(matOff);
            in.layerOffset += int32_t(layerOff);
            I.push_back(in);
        }
        std::vector<BNode> nodes(sc->tlasNodeCount);
        std::vector<int32_t> order(sc->instanceCount);
        if (!nodes.empty())
            AGB_CUDA(cudaMemcpy(nodes.data(), sc->tlasNodes.ptr, nodes.size() * sizeof(BNode), cudaMemcpyDeviceToHost),
                "agb_batch_render: read TLAS");
        if (!order.empty())
            AGB_CUDA(cudaMemcpy(order.data(), sc->tlasOrder.ptr, order.size() * sizeof(int32_t),
                         cudaMemcpyDeviceToHost),
                "agb_batch_render: read TLAS order");
        for (BNode& nd : nodes)
        {
            nd.ref.x = remapTlasRef(nd.ref.x, nodeOff, orderOff);
            nd.ref.y = remapTlasRef(nd.ref.y, nodeOff, orderOff);
            N.push_back(nd);
        }
        for (int32_t o : order)
            O.push_back(o + int32_t(instOff));
        DevScene e      = sc->scene();
        e.tlasRoot      = sc->instanceCount > 0 ? remapTlasRef(sc->tlasRoot, nodeOff, orderOff) : kDone;
        e.instanceCount = int32_t(sc->instanceCount);
        table.push_back(e);
    }
    auto put = [&](DevBuf& buf, const void* src, size_t bytes, const char* what) -> agb_status {
        AGB_CUDA(buf.ensure(std::max<size_t>(bytes, 16)), what);
        if (bytes)
            AGB_CUDA(cudaMemcpyAsync(buf.ptr, src, bytes, cudaMemcpyHostToDevice, st), what);
        return AGB_OK;
    };
    agb_status r;
    if ((r = put(b->meshes, M.data(), M.size() * sizeof(DevMesh), "batch meshes")) ||
        (r = put(b->instances, I.data(), I.size() * sizeof(DevInstance), "batch instances")) ||
        (r = put(b->layers, L.data(), L.size() * sizeof(DevLayer), "batch layers")) ||
        (r = put(b->materials, Mt.data(), Mt.size() * sizeof(agb_material), "batch materials")) ||
        (r = put(b->matTex, T.data(), T.size() * sizeof(agb_material_textures), "batch textures")) ||
        (r = put(b->images, Im.data(), Im.size() * sizeof(DevImage), "batch images")) ||
        (r = put(b->tlas, N.data(), N.size() * sizeof(BNode), "batch TLAS")) ||
        (r = put(b->tlasOrder, O.data(), O.size() * sizeof(int32_t), "batch TLAS order")))
        return r;
    for (DevScene& e : table)
    {
        e.meshes        = b->meshes.as<DevMesh>();
        e.instances     = b->instances.as<DevInstance>();
        e.tlas          = b->tlas.as<BNode>();
        e.tlasOrder     = b->tlasOrder.as<int32_t>();
        e.materials     = b->materials.as<agb_material>();
        e.matTex        = anyTex ? b->matTex.as<agb_material_textures>() : nullptr;
        e.materialCount = int32_t(Mt.size());
        e.imageCount    = int32_t(Im.size());
        e.images        = b->images.as<DevImage>();
        e.layers        = b->layers.as<DevLayer>();
    }
    if ((r = put(b->sceneTableDev, table.data(), table.size() * sizeof(DevScene), "batch scene table")))
        return r;
    AGB_CUDA(cudaStreamSynchronize(st), "agb_batch_render: shared scenes");
    b->sceneTable = table;
    b->scenes.assign(scenes.begin(), scenes.end());
    b->versions.clear();
    for (agb_context* sc : scenes)
        b->versions.push_back(sc->sceneVersion);
    return AGB_OK;
}

} // namespace

AGB_API agb_status agb_batch_create(int32_t device, void* cuda_stream, uint64_t max_paths_in_flight,
    agb_batch** out)
{
    if (!out || max_paths_in_flight == 0 || max_paths_in_flight >= (1ull << 29))
        return fail(AGB_ERR_INVALID_ARG, "agb_batch_create: bad argument");
    *out = nullptr;
    std::unique_ptr<agb_batch> b(new agb_batch());
    agb_status st = agb_context_create(device, cuda_stream, &b->work);
    if (st)
        return st;
    b->maxPaths = max_paths_in_flight;
    AGB_CUDA(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming), "create event");
    *out = b.release();
    return AGB_OK;
}

AGB_API agb_status agb_batch_destroy(agb_batch* b)
{
    if (!b)
        return AGB_OK;
    cudaSetDevice(b->work->device);
    cudaStreamSynchronize(b->work->stream);
    delete b;
    return AGB_OK;
}

AGB_API agb_status agb_batch_render(agb_batch* b, agb_context* const* views, const agb_render_options* options,
    const uint32_t* sample_starts, const uint32_t* sample_counts, uint32_t count, agb_render_stats* stats)
{
    if (!b || !views || !options || !sample_counts || count == 0 || count > 65535)
        return fail(AGB_ERR_INVALID_ARG, "agb_batch_render: bad argument");
    agb_context* W = b->work;
    agb_status st  = setDevice(W);
    if (st)
        return st;
    // Requests, their scenes and options.
    std::vector<agb_context*> scenes;
    std::vector<int32_t> sceneOf(count);
    int maxDepth = 0;
    int forceOpaque = -1;
    for (uint32_t i = 0; i < count; i++)
    {
        agb_context* v = views[i];
        const agb_render_options& o = options[i];
        if (!v || !v->frameSet)
            return fail(AGB_ERR_NOT_READY, "agb_batch_render: a view has no frame data");
        if (v->device != W->device)
            return fail(AGB_ERR_INVALID_ARG, "agb_batch_render: views on another device");
        if (o.width == 0 || o.height == 0 || uint64_t(o.width) * o.height > (1ull << 26) || sample_counts[i] == 0)
            return fail(AGB_ERR_INVALID_ARG, "agb_batch_render: bad image size or sample count");
        agb_context* sc = v->parent ? v->parent : v;
        if (sc->instanceCount > 0 && sc->materialCount == 0)
            return fail(AGB_ERR_NOT_READY, "agb_batch_render: no materials");
        size_t k = std::find(scenes.begin(), scenes.end(), sc) - scenes.begin();
        if (k == scenes.size())
            scenes.push_back(sc);
        sceneOf[i] = int32_t(k);
        maxDepth   = std::max(maxDepth, int(v->frame.trace_depth));
        int fo     = v->frame.is_force_opaque_shadows_enabled ? 1 : 0;
        if (forceOpaque >= 0 && fo != forceOpaque)
            return fail(AGB_ERR_INVALID_ARG, "agb_batch_render: views differ in opaque-shadow forcing");
        forceOpaque = fo;
        for (uint32_t j = 0; j < i; j++)
            if (views[j] == v)
                return fail(AGB_ERR_INVALID_ARG, "agb_batch_render: a view appears twice");
    }
    // The namespace set by agb_batch_set_scenes when it holds every scene of the call (and none
    // changed); otherwise one over this call's scenes.
    bool covered = !b->scenes.empty();
    for (size_t k = 0; covered && k < scenes.size(); k++)
        covered = std::find(b->scenes.begin(), b->scenes.end(), scenes[k]) != b->scenes.end();
    if (covered)
    {
        std::vector<agb_context*> keep;
        for (const agb_context* c : b->scenes)
            keep.push_back(const_cast<agb_context*>(c));
        if ((st = buildSharedScenes(b, keep)))
            return st;
        for (uint32_t i = 0; i < count; i++)
        {
            agb_context* sc = views[i]->parent ? views[i]->parent : views[i];
            sceneOf[i]      = int32_t(std::find(b->scenes.begin(), b->scenes.end(), sc) - b->scenes.begin());
        }
    }
    else if ((st = buildSharedScenes(b, scenes)))
        return st;
    // Render targets, accumulation bookkeeping and AOVs of every view (on its own stream, which the
    // batch then waits for).
    std::vector<BatchRequest> reqs(count);
    std::vector<uint32_t> remaining(count);
    for (uint32_t i = 0; i < count; i++)
    {
        agb_context* v = views[i];
        const agb_render_options& o = options[i];
        uint32_t start = sample_starts ? sample_starts[i] : 0;
        uint32_t accumMode = o.accumulation ? o.accumulation : AGB_ACCUM_RUNNING_MEAN;
        if ((st = setDevice(v)) || (st = ensureAccum(v, o.width, o.height)))
            return st;
        if (start == 0)
            v->accumulatedSamples = 0;
        else if (v->accumulatedSamples != start || (v->lastAccumMode & accumMode) != accumMode)
            return fail(AGB_ERR_INVALID_ARG, "agb_batch_render: sample_start must continue the view's accumulated "
                                             "sequence in the same accumulation mode");
        uint32_t pixels = o.width * o.height;
        BatchRequest& q = reqs[i];
        q               = BatchRequest{};
        q.pixels        = pixels;
        q.width         = o.width;
        q.height        = o.height;
        q.sampleBase    = start;
        q.seedOffset    = o.seed_offset;
        q.accumMode     = accumMode;
        q.scene         = sceneOf[i];
        q.traceDepth    = v->frame.trace_depth;
        q.tlasRoot      = b->sceneTable[sceneOf[i]].tlasRoot;
        q.aovSample     = ~0u;
        q.accumMean     = v->accMean.as<float4>();
        q.accumSum      = v->accSum.as<float4>();
        q.accumComp     = v->accComp.as<float4>();
        q.lastSample    = v->lastSample.as<float4>();
        q.accumMoments  = v->accMoments.as<float2>();
        if (v->frame.is_denoising_aovs_enabled)
        {
            AGB_CUDA(v->aovDepth.ensure(size_t(pixels) * sizeof(float)), "allocate AOVs");
            AGB_CUDA(v->aovNormal.ensure(size_t(pixels) * sizeof(float4)), "allocate AOVs");
            AGB_CUDA(v->aovAlbedo.ensure(size_t(pixels) * sizeof(float4)), "allocate AOVs");
            AGB_CUDA(v->aovMotion.ensure(size_t(pixels) * sizeof(float4)), "allocate AOVs");
            q.aovDepth  = v->aovDepth.as<float>();
            q.aovNormal = v->aovNormal.as<float4>();
            q.aovAlbedo = v->aovAlbedo.as<float4>();
            q.aovMotion = v->aovMotion.as<float4>();
            q.aovSample = start + sample_counts[i] - 1;
        }
        v->aovValid  = v->frame.is_denoising_aovs_enabled != 0;
        remaining[i] = sample_counts[i];
        AGB_CUDA(cudaEventRecord(v->ev0, v->stream), "record event");
        AGB_CUDA(cudaStreamWaitEvent(W->stream, v->ev0, 0), "order view work before the batch");
    }
    if ((st = setDevice(W)))
        return st;
    // Waves: every unfinished request takes a share of the path budget in proportion to what it
    // still needs (at least one sample), so small requests are not held back by large ones.
    uint64_t launches = 0;
    uint64_t closest = 0, shadow = 0;
    uint32_t waves = 0;
    W->marks.reset();
    KernelMarks* marks = W->profiling ? &W->marks : nullptr;
    AGB_CUDA(cudaEventRecord(W->ev0, W->stream), "record event");
    std::vector<BatchRequest> round;
    std::vector<agb_frame_data> frames;
    std::vector<uint32_t> chunk(count);
    for (;;)
    {
        uint64_t need = 0;
        for (uint32_t i = 0; i < count; i++)
            need += uint64_t(reqs[i].pixels) * remaining[i];
        if (need == 0)
            break;
        double scale = need > b->maxPaths ? double(b->maxPaths) / double(need) : 1.0;
        round.clear();
        frames.clear();
        uint64_t paths = 0, pixelsTotal = 0;
        for (uint32_t i = 0; i < count; i++)
        {
            if (!remaining[i])
                continue;
            uint32_t c = std::max<uint32_t>(1, uint32_t(double(remaining[i]) * scale));
            c = std::min(c, remaining[i]);
            // Keep the wave within the budget (and the path index range) once it holds a request.
            if (!round.empty() && paths + uint64_t(reqs[i].pixels) * c > std::max<uint64_t>(b->maxPaths, 1))
                c = uint32_t(std::min<uint64_t>(c, (b->maxPaths - std::min(b->maxPaths, paths)) / reqs[i].pixels));
            if (c == 0)
                continue;
            BatchRequest q = reqs[i];
            q.samples      = c;
            q.pathOffset   = uint32_t(paths);
            q.pixelOffset  = uint32_t(pixelsTotal);
            round.push_back(q);
            frames.push_back(views[i]->frame);
            chunk[i] = c;
            paths += uint64_t(q.pixels) * c;
            pixelsTotal += q.pixels;
        }
        if (paths >= (1ull << 29))
            return fail(AGB_ERR_LIMIT, "agb_batch_render: wave too large");
        if ((st = ensureWave(W, size_t(paths), maxDepth, 1)))
            return st;
        AGB_CUDA(b->pathReq.ensure(size_t(paths) * sizeof(uint16_t)), "allocate batch path table");
        AGB_CUDA(b->reqTable.ensure(round.size() * sizeof(BatchRequest)), "allocate batch requests");
        AGB_CUDA(b->frameTable.ensure(frames.size() * sizeof(agb_frame_data)), "allocate batch frames");
        AGB_CUDA(cudaMemcpyAsync(b->reqTable.ptr, round.data(), round.size() * sizeof(BatchRequest),
                     cudaMemcpyHostToDevice, W->stream),
            "upload batch requests");
        AGB_CUDA(cudaMemcpyAsync(b->frameTable.ptr, frames.data(), frames.size() * sizeof(agb_frame_data),
                     cudaMemcpyHostToDevice, W->stream),
            "upload batch frames");
        size_t counterWords = size_t(maxDepth + 2) * kCounterStride;
        AGB_CUDA(cudaMemsetAsync(W->counters.ptr, 0, counterWords * sizeof(uint32_t), W->stream), "clear counters");
        AGB_CUDA(cudaMemsetAsync(W->stats.ptr, 0, 8 * sizeof(unsigned long long), W->stream), "clear stats");
        BatchTables bt{};
        bt.req          = b->reqTable.as<BatchRequest>();
        bt.frames       = b->frameTable.as<agb_frame_data>();
        bt.scenes       = b->sceneTableDev.as<DevScene>();
        bt.pathReq      = b->pathReq.as<uint16_t>();
        bt.requestCount = uint32_t(round.size());
        bt.pixelsTotal  = uint32_t(pixelsTotal);
        WaveParams wp{};
        wp.paths          = uint32_t(paths);
        wp.countTraversal = W->counting ? 1 : 0;
        WaveBuffers wb    = W->wb;
        wb.counters       = W->counters.as<uint32_t>();
        DevScene shared   = b->sceneTable[0];
        shared.ground     = DevGroundPlane{};
        launchBatchWave(shared, frames[0], wp, wb, bt, maxDepth, forceOpaque != 0, W->stream, W->smCount, launches,
            marks);
        AGB_CUDA(cudaGetLastError(), "launch batch wave");
        if (stats)
        {
            std::vector<uint32_t> c(counterWords);
            AGB_CUDA(cudaMemcpyAsync(c.data(), W->counters.ptr, c.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                         W->stream),
                "read counters");
            AGB_CUDA(cudaStreamSynchronize(W->stream), "batch wave");
            for (int bb = 0; bb < maxDepth; bb++)
            {
                closest += c[kCounterStride * bb + CNT_RAYS];
                shadow += c[kCounterStride * bb + CNT_SHADOW];
            }
        }
        for (uint32_t i = 0; i < count; i++)
            if (remaining[i] && chunk[i])
            {
                reqs[i].sampleBase += chunk[i];
                remaining[i] -= chunk[i];
                chunk[i] = 0;
            }
        // The next wave's tables and counters are written by copies on the same stream, after
        // this wave's kernels (a pageable upload stages its source before returning).
        waves++;
    }
    AGB_CUDA(cudaEventRecord(W->ev1, W->stream), "record event");
    AGB_CUDA(cudaEventRecord(b->done, W->stream), "record event");
    for (uint32_t i = 0; i < count; i++)
    {
        agb_context* v = views[i];
        uint32_t start = sample_starts ? sample_starts[i] : 0;
        uint32_t accumMode = options[i].accumulation ? options[i].accumulation : AGB_ACCUM_RUNNING_MEAN;
        v->accumulatedSamples = start + sample_counts[i];
        v->lastAccumMode      = start == 0 ? accumMode : v->lastAccumMode;
        // Work on the view's own stream (reads, denoising) follows the batch.
        AGB_CUDA(cudaStreamWaitEvent(v->stream, b->done, 0), "order the batch before view work");
    }
    if (stats)
    {
        AGB_CUDA(cudaEventSynchronize(W->ev1), "batch render");
        unsigned long long sv[8];
        AGB_CUDA(cudaMemcpy(sv, W->stats.ptr, sizeof sv, cudaMemcpyDeviceToHost), "read stats");
        if (sv[4])
            return fail(AGB_ERR_LIMIT, "agb_batch_render: traversal stack overflow");
        agb_render_stats r{};
        for (uint32_t i = 0; i < count; i++)
            r.paths += uint64_t(options[i].width) * options[i].height * sample_counts[i];
        r.closest_rays    = closest;
        r.shadow_rays     = shadow;
        r.kernel_launches = launches;
        if (marks)
        {
            double ms[KC_COUNT];
            marks->sum(ms);
            for (int k = 0; k < 6; k++)
                r.kernel_ms[k] = ms[k];
            for (size_t i = 0; i < marks->category.size(); i++)
                if (marks->category[i] < 6)
                    r.kernel_count[marks->category[i]]++;
        }
        float ms = 0.f;
        AGB_CUDA(cudaEventElapsedTime(&ms, W->ev0, W->ev1), "event time");
        r.gpu_ms = ms;
        *stats   = r;
    }
    (void)waves;
    return AGB_OK;
}

AGB_API agb_status agb_batch_set_scenes(agb_batch* b, agb_context* const* scenes, uint32_t count)
{
    if (!b || (!scenes && count))
        return fail(AGB_ERR_INVALID_ARG, "agb_batch_set_scenes: bad argument");
    std::vector<agb_context*> list;
    for (uint32_t i = 0; i < count; i++)
    {
        if (!scenes[i] || scenes[i]->parent)
            return fail(AGB_ERR_INVALID_ARG, "agb_batch_set_scenes: contexts with scenes required");
        if (std::find(list.begin(), list.end(), scenes[i]) == list.end())
            list.push_back(scenes[i]);
    }
    agb_status st = setDevice(b->work);
    if (st)
        return st;
    AGB_CUDA(cudaStreamSynchronize(b->work->stream), "agb_batch_set_scenes");
    return buildSharedScenes(b, list);
}

AGB_API agb_status agb_batch_poll(agb_batch* b)
{
    if (!b)
        return AGB_ERR_INVALID_ARG;
    cudaError_t e = cudaEventQuery(b->done);
    if (e == cudaSuccess)
        return AGB_OK;
    if (e == cudaErrorNotReady)
        return AGB_ERR_NOT_READY;
    return fail(AGB_ERR_CUDA, std::string("agb_batch_poll: ") + cudaGetErrorString(e));
}

AGB_API agb_status agb_batch_set_profiling(agb_batch* b, int32_t enabled)
{
    if (!b)
        return AGB_ERR_INVALID_ARG;
    return agb_set_profiling(b->work, enabled);
}

AGB_API agb_status agb_wait_poll(agb_context* ctx)
{
    if (!ctx)
        return AGB_ERR_INVALID_ARG;
    cudaError_t e = cudaStreamQuery(ctx->stream);
    if (e == cudaSuccess)
        return AGB_OK;
    if (e == cudaErrorNotReady)
        return AGB_ERR_NOT_READY;
    return cudaFail(e, "agb_wait_poll");
}

AGB_API agb_status agb_wait(agb_context* ctx)
{
    if (!ctx)
        return fail(AGB_ERR_INVALID_ARG, "agb_wait: null context");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "agb_wait");
    unsigned long long s[8] = { 0 };
    if (ctx->stats.ptr)
    {
        AGB_CUDA(cudaMemcpy(s, ctx->stats.ptr, sizeof s, cudaMemcpyDeviceToHost), "read stats");
        if (s[4])
            return fail(AGB_ERR_LIMIT, "traversal stack overflow during render");
    }
    return AGB_OK;
}

AGB_API agb_status agb_accum_device(agb_context* ctx, int32_t mode, float** device_rgba)
{
    if (!ctx || !device_rgba || !ctx->accMean.ptr)
        return fail(AGB_ERR_NOT_READY, "agb_accum_device: nothing rendered");
    *device_rgba = mode == AGB_ACCUM_KAHAN ? ctx->accSum.as<float>() : ctx->accMean.as<float>();
    return AGB_OK;
}

AGB_API agb_status agb_last_sample_device(agb_context* ctx, float** device_rgba)
{
    if (!ctx || !device_rgba || !ctx->lastSample.ptr)
        return fail(AGB_ERR_NOT_READY, "agb_last_sample_device: nothing rendered");
    *device_rgba = ctx->lastSample.as<float>();
    return AGB_OK;
}

AGB_API agb_status agb_accum_read(agb_context* ctx, int32_t mode, float* host_rgba,
    uint64_t capacity_floats)
{
    if (!ctx || !host_rgba || !ctx->accMean.ptr)
        return fail(AGB_ERR_NOT_READY, "agb_accum_read: nothing rendered");
    size_t n = size_t(ctx->accW) * ctx->accH * 4;
    if (capacity_floats < n)
        return fail(AGB_ERR_INVALID_ARG, "agb_accum_read: buffer too small");
    if (mode != AGB_ACCUM_RUNNING_MEAN && mode != AGB_ACCUM_KAHAN)
        return fail(AGB_ERR_INVALID_ARG, "agb_accum_read: bad mode");
    if (!(ctx->lastAccumMode & uint32_t(mode)))
        return fail(AGB_ERR_NOT_READY, "agb_accum_read: mode was not accumulated");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    const void* src = mode == AGB_ACCUM_KAHAN ? ctx->accSum.ptr : ctx->accMean.ptr;
    AGB_CUDA(cudaMemcpyAsync(host_rgba, src, n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream),
        "read accumulation");
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "read accumulation");
    if (mode == AGB_ACCUM_KAHAN && ctx->accumulatedSamples)
    {
        float inv = 1.f / float(ctx->accumulatedSamples);
        for (size_t i = 0; i < n; i++)
            host_rgba[i] *= inv;
    }
    return AGB_OK;
}

AGB_API agb_status agb_accum_read_rect(agb_context* ctx, int32_t mode, uint32_t x0, uint32_t y0,
    uint32_t width, uint32_t height, float* host_rgba, uint64_t capacity_floats)
{
    if (!ctx || !host_rgba || !ctx->accMean.ptr)
        return fail(AGB_ERR_NOT_READY, "agb_accum_read_rect: nothing rendered");
    if (width == 0 || height == 0 || uint64_t(x0) + width > ctx->accW || uint64_t(y0) + height > ctx->accH)
        return fail(AGB_ERR_INVALID_ARG, "agb_accum_read_rect: rectangle outside the image");
    size_t n = size_t(width) * height * 4;
    if (capacity_floats < n)
        return fail(AGB_ERR_INVALID_ARG, "agb_accum_read_rect: buffer too small");
    if (mode != AGB_ACCUM_RUNNING_MEAN && mode != AGB_ACCUM_KAHAN)
        return fail(AGB_ERR_INVALID_ARG, "agb_accum_read_rect: bad mode");
    if (!(ctx->lastAccumMode & uint32_t(mode)))
        return fail(AGB_ERR_NOT_READY, "agb_accum_read_rect: mode was not accumulated");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    const float4* src = (mode == AGB_ACCUM_KAHAN ? ctx->accSum.as<float4>() : ctx->accMean.as<float4>()) +
        size_t(y0) * ctx->accW + x0;
    AGB_CUDA(cudaMemcpy2DAsync(host_rgba, size_t(width) * sizeof(float4), src, size_t(ctx->accW) * sizeof(float4),
                 size_t(width) * sizeof(float4), height, cudaMemcpyDeviceToHost, ctx->stream),
        "read accumulation rectangle");
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "read accumulation rectangle");
    if (mode == AGB_ACCUM_KAHAN && ctx->accumulatedSamples)
    {
        float inv = 1.f / float(ctx->accumulatedSamples);
        for (size_t i = 0; i < n; i++)
            host_rgba[i] *= inv;
    }
    return AGB_OK;
}

AGB_API agb_status agb_accum_rel_mse(agb_context* ctx, int32_t mode, const float* reference_device,
    double eps, double* out)
{
    if (!ctx || !reference_device || !out || !(eps > 0.0))
        return fail(AGB_ERR_INVALID_ARG, "agb_accum_rel_mse: null argument or eps <= 0");
    if (!ctx->accMean.ptr || (mode != AGB_ACCUM_RUNNING_MEAN && mode != AGB_ACCUM_KAHAN))
        return fail(AGB_ERR_NOT_READY, "agb_accum_rel_mse: nothing rendered or bad mode");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    AGB_CUDA(ctx->stats.ensure(8 * sizeof(unsigned long long)), "allocate stats");
    double* d = reinterpret_cast<double*>(ctx->stats.as<unsigned long long>() + 7);
    uint32_t pixels = ctx->accW * ctx->accH;
    const float4* src = mode == AGB_ACCUM_KAHAN ? ctx->accSum.as<float4>() : ctx->accMean.as<float4>();
    float scale = (mode == AGB_ACCUM_KAHAN && ctx->accumulatedSamples) ? 1.f / float(ctx->accumulatedSamples) : 1.f;
    AGB_CUDA(launchRelMse(src, scale, reinterpret_cast<const float4*>(reference_device), pixels, eps, d, ctx->stream),
        "agb_accum_rel_mse");
    double sum = 0.0;
    AGB_CUDA(cudaMemcpyAsync(&sum, d, sizeof sum, cudaMemcpyDeviceToHost, ctx->stream), "agb_accum_rel_mse");
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "agb_accum_rel_mse");
    *out = pixels ? sum / (3.0 * pixels) : 0.0;
    return AGB_OK;
}

AGB_API agb_status agb_post_process(agb_context* ctx, int32_t mode, const float brightness[3],
    int32_t tone_map, int32_t gamma, float* out_rgba32f, uint8_t* out_rgba8)
{
    if (!ctx || !ctx->accMean.ptr || !brightness)
        return fail(AGB_ERR_NOT_READY, "agb_post_process: nothing rendered");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    size_t pixels = size_t(ctx->accW) * ctx->accH;
    DevBuf o32, o8;
    AGB_CUDA(o32.ensure(pixels * sizeof(float4)), "allocate post output");
    AGB_CUDA(o8.ensure(pixels * sizeof(uchar4)), "allocate post output");
    if (mode == AGB_POST_SOURCE_TEMPORAL && (ctx->taaLast < 0 || ctx->taaW != ctx->accW || ctx->taaH != ctx->accH))
        return fail(AGB_ERR_NOT_READY, "agb_post_process: no temporal resolve of this size");
    const float4* src = mode == AGB_ACCUM_KAHAN ? ctx->accSum.as<float4>()
        : mode == AGB_POST_SOURCE_TEMPORAL      ? ctx->taaHistory[ctx->taaLast].as<float4>()
                                                : ctx->accMean.as<float4>();
    if (mode == AGB_POST_SOURCE_TEMPORAL)
        mode = AGB_ACCUM_RUNNING_MEAN;
    float inv = ctx->accumulatedSamples ? 1.f / float(ctx->accumulatedSamples) : 1.f;
    AGB_CUDA(launchPostProcess(src, nullptr, mode, inv, uint32_t(pixels),
                 make_float3(brightness[0], brightness[1], brightness[2]), tone_map, gamma,
                 o32.as<float4>(), o8.as<uchar4>(), ctx->stream),
        "post-process");
    if (out_rgba32f)
        AGB_CUDA(cudaMemcpyAsync(out_rgba32f, o32.ptr, pixels * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream),
            "read post output");
    if (out_rgba8)
        AGB_CUDA(cudaMemcpyAsync(out_rgba8, o8.ptr, pixels * sizeof(uchar4), cudaMemcpyDeviceToHost, ctx->stream),
            "read post output");
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "post-process");
    return AGB_OK;
}

AGB_API agb_status agb_aov_read(agb_context* ctx, float* depth_view, float* normal_roughness,
    float* base_color_metalness, float* motion)
{
    if (!ctx || !ctx->aovValid || !ctx->aovDepth.ptr)
        return fail(AGB_ERR_NOT_READY, "agb_aov_read: the last render did not enable the AOVs");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    size_t n = size_t(ctx->accW) * ctx->accH;
    if (depth_view)
        AGB_CUDA(cudaMemcpyAsync(depth_view, ctx->aovDepth.ptr, n * sizeof(float), cudaMemcpyDeviceToHost,
                     ctx->stream), "read AOVs");
    if (normal_roughness)
        AGB_CUDA(cudaMemcpyAsync(normal_roughness, ctx->aovNormal.ptr, n * sizeof(float4),
                     cudaMemcpyDeviceToHost, ctx->stream), "read AOVs");
    if (base_color_metalness)
        AGB_CUDA(cudaMemcpyAsync(base_color_metalness, ctx->aovAlbedo.ptr, n * sizeof(float4),
                     cudaMemcpyDeviceToHost, ctx->stream), "read AOVs");
    if (motion)
        AGB_CUDA(cudaMemcpyAsync(motion, ctx->aovMotion.ptr, n * sizeof(float4), cudaMemcpyDeviceToHost,
                     ctx->stream), "read AOVs");
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "read AOVs");
    return AGB_OK;
}

AGB_API agb_status agb_aov_device(agb_context* ctx, agb_aov_buffers* out)
{
    if (!ctx || !out)
        return fail(AGB_ERR_INVALID_ARG, "agb_aov_device: null argument");
    if (!ctx->aovValid || !ctx->aovDepth.ptr)
        return fail(AGB_ERR_NOT_READY, "agb_aov_device: the last render did not enable the AOVs");
    out->depth_view           = ctx->aovDepth.as<float>();
    out->normal_roughness     = ctx->aovNormal.as<float>();
    out->base_color_metalness = ctx->aovAlbedo.as<float>();
    out->motion               = ctx->aovMotion.as<float>();
    return AGB_OK;
}

AGB_API agb_status agb_temporal_resolve(agb_context* ctx, const agb_temporal_settings* settings)
{
    if (!ctx || !settings)
        return fail(AGB_ERR_INVALID_ARG, "agb_temporal_resolve: null argument");
    if (!ctx->accMean.ptr || !ctx->aovValid)
        return fail(AGB_ERR_NOT_READY, "agb_temporal_resolve: needs a render with the denoising AOVs "
                                       "enabled (motion vectors and view depth)");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    size_t n     = size_t(ctx->accW) * ctx->accH;
    bool resized = ctx->taaW != ctx->accW || ctx->taaH != ctx->accH || ctx->taaLast < 0;
    if (resized)
    {
        for (int k = 0; k < 2; k++)
        {
            AGB_CUDA(ctx->taaHistory[k].ensure(n * sizeof(float4)), "allocate temporal history");
            AGB_CUDA(cudaMemsetAsync(ctx->taaHistory[k].ptr, 0, n * sizeof(float4), ctx->stream),
                "clear temporal history");
        }
        ctx->taaW    = ctx->accW;
        ctx->taaH    = ctx->accH;
        ctx->taaLast = 1;
    }
    TemporalSettings ts{ settings->is_reset || resized ? 1u : 0u, settings->blend_alpha_min,
        settings->blend_alpha_max, settings->speed_reference };
    int write = ctx->taaLast ^ 1;
    AGB_CUDA(launchTemporalResolve(ctx->accMean.as<float4>(), ctx->taaHistory[ctx->taaLast].as<float4>(),
                 ctx->aovMotion.as<float4>(), ctx->aovDepth.as<float>(), int(ctx->accW), int(ctx->accH), ts,
                 ctx->taaHistory[write].as<float4>(), ctx->stream),
        "temporal resolve");
    ctx->taaLast = write;
    return AGB_OK;
}

AGB_API agb_status agb_temporal_read(agb_context* ctx, float* host_rgba, uint64_t capacity)
{
    if (!ctx || !host_rgba)
        return fail(AGB_ERR_INVALID_ARG, "agb_temporal_read: null argument");
    if (ctx->taaLast < 0)
        return fail(AGB_ERR_NOT_READY, "agb_temporal_read: no temporal resolve yet");
    size_t n = size_t(ctx->taaW) * ctx->taaH * 4;
    if (capacity < n)
        return fail(AGB_ERR_INVALID_ARG, "agb_temporal_read: output too small");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    AGB_CUDA(cudaMemcpyAsync(host_rgba, ctx->taaHistory[ctx->taaLast].ptr, n * sizeof(float),
                 cudaMemcpyDeviceToHost, ctx->stream),
        "read temporal history");
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "read temporal history");
    return AGB_OK;
}

AGB_API agb_status agb_temporal_resolve_batch(const float* accum, const float* history,
    const float* motion, const float* depth_view, uint32_t width, uint32_t height,
    const agb_temporal_settings* settings, float* out, void* cuda_stream)
{
    if (!settings || (uint64_t(width) * height > 0 && (!accum || !history || !motion || !depth_view || !out)))
        return fail(AGB_ERR_INVALID_ARG, "agb_temporal_resolve_batch: null argument");
    if (width > (1u << 15) || height > (1u << 15))
        return fail(AGB_ERR_LIMIT, "agb_temporal_resolve_batch: image larger than 32768 pixels a side");
    if (width == 0 || height == 0)
        return AGB_OK;
    TemporalSettings ts{ settings->is_reset, settings->blend_alpha_min, settings->blend_alpha_max,
        settings->speed_reference };
    AGB_CUDA(launchTemporalResolve(reinterpret_cast<const float4*>(accum),
                 reinterpret_cast<const float4*>(history), reinterpret_cast<const float4*>(motion),
                 depth_view, int(width), int(height), ts, reinterpret_cast<float4*>(out),
                 static_cast<cudaStream_t>(cuda_stream)),
        "agb_temporal_resolve_batch");
    return AGB_OK;
}

AGB_API agb_status agb_tc_gemm_bf16(const uint16_t* a, const uint16_t* b, float* d, int32_t m,
    int32_t n, int32_t k, void* cuda_stream)
{
    if (!a || !b || !d || m <= 0 || m % 128 || n < 16 || n > 256 || n % 16 || k <= 0 || k % 64)
        return fail(AGB_ERR_INVALID_ARG, "agb_tc_gemm_bf16: M % 128, 16 <= N <= 256, N % 16, K % 64");
    if ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) | reinterpret_cast<uintptr_t>(d)) & 15u)
        return fail(AGB_ERR_INVALID_ARG, "agb_tc_gemm_bf16: pointers must be 16-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    AGB_CUDA(launchTcGemm(a, b, d, m, n, k, st), "agb_tc_gemm_bf16");
    AGB_CUDA(cudaStreamSynchronize(st), "agb_tc_gemm_bf16");
    int flag = 0;
    AGB_CUDA(takeTcError(&flag), "agb_tc_gemm_bf16");
    if (flag)
        return fail(AGB_ERR_TIMEOUT, "agb_tc_gemm_bf16: tensor-core completion wait timed out");
    return AGB_OK;
}

static agb_status convCommon(const char* what, const uint16_t* in0, const uint16_t* in1, const uint16_t* wpack,
    const float* bias, uint16_t* out, float* out32, uint16_t* pool, int32_t batch, int32_t height, int32_t width,
    int32_t c0, int32_t c1, int32_t cout, int32_t up0, int32_t relu, void* cuda_stream)
{
    if (!in0 || !wpack || (c1 > 0 && !in1) || batch <= 0 || height <= 0 || width <= 0)
        return fail(AGB_ERR_INVALID_ARG, std::string(what) + ": null input or empty image");
    if (c0 < 16 || c0 % 16 || c1 < 0 || c1 % 16 || cout < 16 || cout % 16 || cout > 1024 || c0 + c1 > 1024)
        return fail(AGB_ERR_INVALID_ARG, std::string(what) + ": channel counts must be multiples of 16 up to 1024");
    if (width % 2)
        return fail(AGB_ERR_INVALID_ARG, std::string(what) + ": the width must be even");
    if ((up0 || pool) && height % 2)
        return fail(AGB_ERR_INVALID_ARG, std::string(what) + ": an upsampled input or a pooled output needs even sizes");
    if (int64_t(batch) * height * width >= (int64_t(1) << 31) / 128)
        return fail(AGB_ERR_LIMIT, std::string(what) + ": too many pixels");
    uintptr_t al = reinterpret_cast<uintptr_t>(in0) | reinterpret_cast<uintptr_t>(in1) |
        reinterpret_cast<uintptr_t>(wpack) | reinterpret_cast<uintptr_t>(bias);
    uintptr_t alOut = reinterpret_cast<uintptr_t>(out) | reinterpret_cast<uintptr_t>(out32) |
        reinterpret_cast<uintptr_t>(pool);
    if ((al & 15u) || (alOut & 31u))
        return fail(AGB_ERR_INVALID_ARG, std::string(what) + ": inputs and bias must be 16-byte and outputs 32-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    ConvLaunch c{ in0, c1 > 0 ? in1 : nullptr, wpack, bias, out, out32, batch, height, width, c0, c1, cout,
        up0 ? 1 : 0, relu ? 1 : 0 };
    c.pool = pool;
    AGB_CUDA(launchConv3x3(c, st), what);
    AGB_CUDA(cudaStreamSynchronize(st), what);
    int flag = 0;
    AGB_CUDA(takeTcError(&flag), what);
    if (flag)
        return fail(AGB_ERR_TIMEOUT, std::string(what) + ": tensor-core completion wait timed out");
    return AGB_OK;
}

AGB_API agb_status agb_conv3x3_bf16(const uint16_t* in0, const uint16_t* in1, const uint16_t* wpack,
    const float* bias, uint16_t* out, float* out32, int32_t batch, int32_t height, int32_t width,
    int32_t c0, int32_t c1, int32_t cout, int32_t up0, int32_t relu, void* cuda_stream)
{
    return convCommon("agb_conv3x3_bf16", in0, in1, wpack, bias, out, out32, nullptr, batch, height, width, c0, c1,
        cout, up0, relu, cuda_stream);
}

AGB_API agb_status agb_conv3x3_pool_bf16(const uint16_t* in0, const uint16_t* in1, const uint16_t* wpack,
    const float* bias, uint16_t* out, uint16_t* pool, int32_t batch, int32_t height, int32_t width,
    int32_t c0, int32_t c1, int32_t cout, int32_t up0, int32_t relu, void* cuda_stream)
{
    if (!pool)
        return fail(AGB_ERR_INVALID_ARG, "agb_conv3x3_pool_bf16: null pool output");
    return convCommon("agb_conv3x3_pool_bf16", in0, in1, wpack, bias, out, nullptr, pool, batch, height, width, c0,
        c1, cout, up0, relu, cuda_stream);
}

AGB_API agb_status agb_conv3x3_wgrad_bf16(const uint16_t* in0, const uint16_t* in1, const uint16_t* dy,
    float* dw, int32_t batch, int32_t height, int32_t width, int32_t c0, int32_t c1, int32_t cout,
    int32_t up0, void* cuda_stream)
{
    if (!in0 || !dy || !dw || (c1 > 0 && !in1) || batch <= 0 || height <= 0 || width <= 0)
        return fail(AGB_ERR_INVALID_ARG, "agb_conv3x3_wgrad_bf16: null input or empty image");
    if (c0 < 16 || c0 % 16 || c1 < 0 || c1 % 16 || cout < 16 || cout > 256 || cout % 16 || c0 + c1 > 1024)
        return fail(AGB_ERR_INVALID_ARG, "agb_conv3x3_wgrad_bf16: channel counts must be multiples of 16, cout <= 256");
    if (width % 2 || (up0 && height % 2))
        return fail(AGB_ERR_INVALID_ARG, "agb_conv3x3_wgrad_bf16: the width must be even (the height too with an upsampled input)");
    uintptr_t al = reinterpret_cast<uintptr_t>(in0) | reinterpret_cast<uintptr_t>(in1) | reinterpret_cast<uintptr_t>(dy);
    if (al & 15u)
        return fail(AGB_ERR_INVALID_ARG, "agb_conv3x3_wgrad_bf16: pointers must be 16-byte aligned");
    int dev = 0, sms = 0;
    AGB_CUDA(cudaGetDevice(&dev), "agb_conv3x3_wgrad_bf16");
    AGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "agb_conv3x3_wgrad_bf16");
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    ConvLaunch c{ in0, c1 > 0 ? in1 : nullptr, nullptr, nullptr, nullptr, nullptr, batch, height, width, c0, c1, cout,
        up0 ? 1 : 0, 0 };
    AGB_CUDA(launchConvWgrad(c, dy, dw, sms, st), "agb_conv3x3_wgrad_bf16");
    AGB_CUDA(cudaStreamSynchronize(st), "agb_conv3x3_wgrad_bf16");
    int flag = 0;
    AGB_CUDA(takeTcError(&flag), "agb_conv3x3_wgrad_bf16");
    if (flag)
        return fail(AGB_ERR_TIMEOUT, "agb_conv3x3_wgrad_bf16: tensor-core completion wait timed out");
    return AGB_OK;
}

AGB_API agb_status agb_pack_conv_weights(const float* w, int32_t cin, int32_t cout, int32_t flip,
    uint16_t* out, void* cuda_stream)
{
    if (!w || !out || cin < 16 || cin % 16 || cout < 16 || cout % 16)
        return fail(AGB_ERR_INVALID_ARG, "agb_pack_conv_weights: channel counts must be multiples of 16");
    AGB_CUDA(launchPackConvWeights(w, cin, cout, flip ? 1 : 0, out, static_cast<cudaStream_t>(cuda_stream)),
        "agb_pack_conv_weights");
    return AGB_OK;
}

struct agb_denoiser
{
    int device          = 0;
    cudaStream_t stream = nullptr;
    bool ownsStream     = false;
    UnetDenoiser net;
    ~agb_denoiser()
    {
        net.release();
        if (ownsStream && stream)
            cudaStreamDestroy(stream);
    }
};

namespace
{
agb_status denoiserCheck(agb_denoiser* dn, int32_t B, int32_t H, int32_t W, const char* what)
{
    if (!dn)
        return fail(AGB_ERR_INVALID_ARG, std::string(what) + ": null denoiser");
    if (B <= 0 || H <= 0 || W <= 0 || H % 8 || W % 8)
        return fail(AGB_ERR_INVALID_ARG, std::string(what) + ": batch > 0, height and width multiples of 8");
    if (int64_t(B) * H * W >= (int64_t(1) << 26))
        return fail(AGB_ERR_LIMIT, std::string(what) + ": too many pixels per batch");
    AGB_CUDA(cudaSetDevice(dn->device), "cudaSetDevice");
    return AGB_OK;
}
agb_status tcStatus(const char* what)
{
    int flag = 0;
    AGB_CUDA(takeTcError(&flag), what);
    if (flag)
        return fail(AGB_ERR_TIMEOUT, std::string(what) + ": tensor-core completion wait timed out");
    return AGB_OK;
}
} // namespace

AGB_API agb_status agb_denoiser_create(int32_t device, void* cuda_stream, uint64_t seed, agb_denoiser** out)
{
    if (!out)
        return fail(AGB_ERR_INVALID_ARG, "agb_denoiser_create: out is null");
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count)
        return fail(AGB_ERR_INVALID_ARG, "agb_denoiser_create: no CUDA device " + std::to_string(device));
    std::unique_ptr<agb_denoiser> dn(new agb_denoiser());
    dn->device = device;
    AGB_CUDA(cudaSetDevice(device), "cudaSetDevice");
    int sms = 0;
    AGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "agb_denoiser_create");
    if (cuda_stream)
        dn->stream = static_cast<cudaStream_t>(cuda_stream);
    else
    {
        AGB_CUDA(cudaStreamCreateWithFlags(&dn->stream, cudaStreamNonBlocking), "create stream");
        dn->ownsStream = true;
    }
    AGB_CUDA(dn->net.init(seed, dn->stream, sms), "agb_denoiser_create");
    AGB_CUDA(cudaStreamSynchronize(dn->stream), "agb_denoiser_create");
    *out = dn.release();
    return AGB_OK;
}

AGB_API agb_status agb_denoiser_destroy(agb_denoiser* dn)
{
    if (dn)
    {
        cudaSetDevice(dn->device);
        delete dn;
    }
    return AGB_OK;
}

AGB_API agb_status agb_denoiser_param_count(uint64_t* count)
{
    if (!count)
        return fail(AGB_ERR_INVALID_ARG, "agb_denoiser_param_count: null argument");
    *count = UnetDenoiser::paramCount();
    return AGB_OK;
}

AGB_API agb_status agb_denoiser_params(agb_denoiser* dn, float* host_out, uint64_t count)
{
    if (!dn || !host_out || count < dn->net.nParams())
        return fail(AGB_ERR_INVALID_ARG, "agb_denoiser_params: null argument or output too small");
    AGB_CUDA(cudaSetDevice(dn->device), "cudaSetDevice");
    AGB_CUDA(cudaMemcpyAsync(host_out, dn->net.params(), dn->net.nParams() * 4, cudaMemcpyDeviceToHost, dn->stream),
        "read parameters");
    AGB_CUDA(cudaStreamSynchronize(dn->stream), "read parameters");
    return AGB_OK;
}

AGB_API agb_status agb_denoiser_set_params(agb_denoiser* dn, const float* host, uint64_t count)
{
    if (!dn || !host || count != dn->net.nParams())
        return fail(AGB_ERR_INVALID_ARG, "agb_denoiser_set_params: null argument or wrong count");
    AGB_CUDA(cudaSetDevice(dn->device), "cudaSetDevice");
    AGB_CUDA(dn->net.setParams(host), "agb_denoiser_set_params");
    AGB_CUDA(cudaStreamSynchronize(dn->stream), "agb_denoiser_set_params");
    return AGB_OK;
}

AGB_API agb_status agb_denoiser_grads(agb_denoiser* dn, float* host_out, uint64_t count)
{
    if (!dn || !host_out || count < dn->net.nParams())
        return fail(AGB_ERR_INVALID_ARG, "agb_denoiser_grads: null argument or output too small");
    AGB_CUDA(cudaSetDevice(dn->device), "cudaSetDevice");
    AGB_CUDA(cudaMemcpyAsync(host_out, dn->net.grads(), dn->net.nParams() * 4, cudaMemcpyDeviceToHost, dn->stream),
        "read gradients");
    AGB_CUDA(cudaStreamSynchronize(dn->stream), "read gradients");
    return AGB_OK;
}

AGB_API agb_status agb_denoiser_forward(agb_denoiser* dn, const uint16_t* features, int32_t batch,
    int32_t height, int32_t width, float* out_rgba)
{
    agb_status st = denoiserCheck(dn, batch, height, width, "agb_denoiser_forward");
    if (st)
        return st;
    if (!features || !out_rgba || ((reinterpret_cast<uintptr_t>(features) | reinterpret_cast<uintptr_t>(out_rgba)) & 15u))
        return fail(AGB_ERR_INVALID_ARG, "agb_denoiser_forward: null or unaligned device pointer");
    AGB_CUDA(dn->net.infer(features, batch, height, width, out_rgba), "agb_denoiser_forward");
    AGB_CUDA(cudaStreamSynchronize(dn->stream), "agb_denoiser_forward");
    if (dn->net.inferTimedOut())
        return fail(AGB_ERR_TIMEOUT, "agb_denoiser_forward: tensor-core completion wait timed out");
    return AGB_OK;
}

AGB_API agb_status agb_denoiser_train_step(agb_denoiser* dn, const uint16_t* features,
    const float* target_rgba, int32_t batch, int32_t height, int32_t width, float learning_rate,
    int32_t update, float* loss)
{
    agb_status st = denoiserCheck(dn, batch, height, width, "agb_denoiser_train_step");
    if (st)
        return st;
    if (!features || !target_rgba || ((reinterpret_cast<uintptr_t>(features) | reinterpret_cast<uintptr_t>(target_rgba)) & 15u))
        return fail(AGB_ERR_INVALID_ARG, "agb_denoiser_train_step: null or unaligned device pointer");
    if (!(learning_rate >= 0.f))
        return fail(AGB_ERR_INVALID_ARG, "agb_denoiser_train_step: learning rate must be >= 0");
    AGB_CUDA(dn->net.forward(features, batch, height, width, true), "agb_denoiser_train_step");
    AGB_CUDA(dn->net.backward(target_rgba), "agb_denoiser_train_step");
    if (update)
        AGB_CUDA(dn->net.adam(learning_rate), "agb_denoiser_train_step");
    float l = 0.f;
    AGB_CUDA(cudaMemcpyAsync(&l, dn->net.lossDevice(), 4, cudaMemcpyDeviceToHost, dn->stream), "read loss");
    AGB_CUDA(cudaStreamSynchronize(dn->stream), "agb_denoiser_train_step");
    if (loss)
        *loss = l;
    return tcStatus("agb_denoiser_train_step");
}

AGB_API agb_status agb_denoiser_features(agb_context* ctx, uint16_t* out_features)
{
    if (!ctx || !out_features || (reinterpret_cast<uintptr_t>(out_features) & 15u))
        return fail(AGB_ERR_INVALID_ARG, "agb_denoiser_features: null or unaligned argument");
    if (!ctx->accMean.ptr || !ctx->aovValid || !(ctx->lastAccumMode & AGB_ACCUM_RUNNING_MEAN))
        return fail(AGB_ERR_NOT_READY, "agb_denoiser_features: needs a running-mean render with the denoising "
                                       "AOVs enabled");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    long P = long(ctx->accW) * ctx->accH;
    const float2* mom = (ctx->lastAccumMode & AGB_ACCUM_MOMENTS) ? ctx->accMoments.as<float2>() : nullptr;
    AGB_CUDA(launchDenoiseFeatures(ctx->accMean.as<float4>(), mom, float(ctx->accumulatedSamples),
                 ctx->aovAlbedo.as<float4>(), ctx->aovNormal.as<float4>(), ctx->aovDepth.as<float>(),
                 ctx->frame.sky_view_z, P, out_features, ctx->stream),
        "agb_denoiser_features");
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "agb_denoiser_features");
    return AGB_OK;
}

AGB_API void agb_temporal_jitter(uint32_t frame_index, uint32_t phase_count, float out[2])
{
    // PTRenderer.cpp:81-95 (halton) and :168-174: index = frame (mod phases) + 1, centred.
    uint32_t index = (phase_count > 0u ? frame_index % phase_count : frame_index) + 1u;
    for (int a = 0; a < 2; a++)
    {
        uint32_t base = a == 0 ? 2u : 3u, i = index;
        float result = 0.0f;
        float scale  = 1.0f / static_cast<float>(base);
        while (i > 0)
        {
            result += scale * static_cast<float>(i % base);
            i /= base;
            scale /= static_cast<float>(base);
        }
        out[a] = result - 0.5f;
    }
}

AGB_API agb_status agb_bsdf_batch(int32_t op, const agb_material* materials,
    const int32_t* material_index, const float* frames, const float* V, const float* L,
    const float* rnd, int64_t n, float* out_value, float* out_dir, float* out_pdf,
    int32_t* out_lobe, void* cuda_stream)
{
    if (op < 0 || op > 2 || n < 0 || (n > 0 && (!materials || !material_index || !frames || !V || !out_value)))
        return fail(AGB_ERR_INVALID_ARG, "agb_bsdf_batch: invalid argument");
    if ((op == 0 || op == 2) && n > 0 && !L)
        return fail(AGB_ERR_INVALID_ARG, "agb_bsdf_batch: L required");
    if (op >= 1 && n > 0 && (!rnd || !out_pdf || !out_lobe || (op == 1 && !out_dir)))
        return fail(AGB_ERR_INVALID_ARG, "agb_bsdf_batch: sampling outputs required");
    AGB_CUDA(launchBsdfBatch(op, materials, material_index, frames, V, L, rnd, n, out_value, out_dir,
                 out_pdf, out_lobe, static_cast<cudaStream_t>(cuda_stream)),
        "agb_bsdf_batch");
    return AGB_OK;
}

AGB_API agb_status agb_intersect_batch(agb_context* ctx, const float* rays, int64_t n,
    int32_t any_hit, float* out_tuv, int32_t* out_inst_prim)
{
    if (!ctx || n < 0 || (n > 0 && (!rays || !out_tuv || !out_inst_prim)))
        return fail(AGB_ERR_INVALID_ARG, "agb_intersect_batch: invalid argument");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    if (n >= (1ll << 31))
        return fail(AGB_ERR_LIMIT, "agb_intersect_batch: at most 2^31 - 1 rays per call");
    AGB_CUDA(ctx->stats.ensure(8 * sizeof(unsigned long long)), "allocate stats");
    AGB_CUDA(cudaMemsetAsync(ctx->stats.ptr, 0, 8 * sizeof(unsigned long long), ctx->stream), "clear stats");
    unsigned long long* st64 = ctx->stats.as<unsigned long long>();
    AGB_CUDA(launchIntersectBatch(ctx->scene(), rays, n, any_hit, out_tuv, out_inst_prim,
                 reinterpret_cast<uint32_t*>(st64 + 7), st64 + 4, ctx->stream, ctx->smCount),
        "agb_intersect_batch");
    unsigned long long ov = 0;
    AGB_CUDA(cudaMemcpyAsync(&ov, st64 + 4, sizeof ov, cudaMemcpyDeviceToHost, ctx->stream), "read overflow");
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "agb_intersect_batch");
    if (ov)
        return fail(AGB_ERR_LIMIT, "agb_intersect_batch: traversal stack overflow");
    return AGB_OK;
}

AGB_API agb_status agb_env_sample_batch(agb_context* ctx, const float* rnd, int64_t n,
    float* out_radiance, float* out_dir, float* out_pdf)
{
    if (!ctx || n < 0 || (n > 0 && (!rnd || !out_radiance || !out_dir || !out_pdf)))
        return fail(AGB_ERR_INVALID_ARG, "agb_env_sample_batch: invalid argument");
    agb_status st = setDevice(ctx);
    if (st)
        return st;
    AGB_CUDA(launchEnvSampleBatch(ctx->scene(), rnd, n, out_radiance, out_dir, out_pdf, ctx->stream),
        "agb_env_sample_batch");
    AGB_CUDA(cudaStreamSynchronize(ctx->stream), "agb_env_sample_batch");
    return AGB_OK;
}

AGB_API agb_status agb_random_stream(uint32_t sample_index, uint32_t screen_width, uint32_t px,
    uint32_t py, int32_t n, float* out, void* cuda_stream)
{
    if (!out || n < 0)
        return fail(AGB_ERR_INVALID_ARG, "agb_random_stream: invalid argument");
    AGB_CUDA(launchRandomStream(sample_index, screen_width, px, py, n, out,
                 static_cast<cudaStream_t>(cuda_stream)),
        "agb_random_stream");
    return AGB_OK;
}

} // extern "C"
