// GPU binned-SAH BVH2 builder, producing the same 64-byte node layout and leaf encoding as the host
// builder (agb_bvh_build.cpp): over the triangles of a mesh (BLAS, leaves of at most 4 triangles)
// and over instance boxes (TLAS, one instance per leaf).
//
// Top-down, one level of the tree per launch, one CTA per node (task) of the level:
//   1. the CTA reduces its primitives' box and centroid box and writes the box into its parent's
//      child slot (the node layout keeps both child boxes in the parent);
//   2. a node of at most leafMax primitives becomes a leaf (ref ~(first << 3 | count - 1));
//   3. otherwise 16 bins per axis over the centroid box collect counts and boxes (shared-memory
//      atomics on order-preserving integer encodings of the floats); one thread per axis sweeps the
//      15 split planes with the SAH cost area(L) n(L) + area(R) n(R);
//   4. the CTA partitions its range of the primitive order stably and in place (ballot ranks per
//      warp, warp offsets through shared memory, a scratch copy of the range), allocates its node
//      id and appends its two children to the next level's task list.
// Nodes that could exceed the depth budget (the traversal stack holds 48 entries for TLAS + BLAS)
// split at their index midpoint, which halves every subtree and bounds the depth: the tree is then
// at most maxDepth deep whenever ceil(log2(count / leafMax)) + 2 <= maxDepth.
#include <algorithm>

#include "agb_kernels.h"

namespace agb
{
namespace
{

constexpr int kBins        = 16;
constexpr int kBuildThreads = 128;
constexpr int kBlasLeaf    = 4;

struct BuildTask
{
    uint32_t first, count;
    int32_t parent; // node index, -1 for the root
    int32_t side;   // 0 / 1: which child slot of the parent
    int32_t depth;
};

__device__ __forceinline__ int32_t orderedFromFloat(float f)
{
    int32_t i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float floatFromOrdered(int32_t i)
{
    return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF);
}

__device__ __forceinline__ float boxArea(const float* lo, const float* hi)
{
    float d0 = fmaxf(0.f, hi[0] - lo[0]), d1 = fmaxf(0.f, hi[1] - lo[1]), d2 = fmaxf(0.f, hi[2] - lo[2]);
    return 2.f * (d0 * d1 + d1 * d2 + d2 * d0);
}

__device__ __forceinline__ int ceilLog2(uint32_t x)
{
    int r = 0;
    while ((1u << r) < x)
        r++;
    return r;
}

// Block-wide min / max reduction of 6 values (lo xyz, hi xyz) into s[0..5] (thread 0 reads).
__device__ void blockBox(float v[6], float* s)
{
    for (int o = 16; o > 0; o >>= 1)
        for (int k = 0; k < 6; k++)
        {
            float w = __shfl_xor_sync(0xffffffffu, v[k], o);
            v[k]    = k < 3 ? fminf(v[k], w) : fmaxf(v[k], w);
        }
    __shared__ float part[kBuildThreads / 32][6];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
        for (int k = 0; k < 6; k++)
            part[warp][k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < 6; k++)
        {
            float r = part[0][k];
            for (int w = 1; w < kBuildThreads / 32; w++)
                r = k < 3 ? fminf(r, part[w][k]) : fmaxf(r, part[w][k]);
            s[k] = r;
        }
    __syncthreads();
}

__global__ void __launch_bounds__(kBuildThreads) k_bvh_level(const float* boxes, uint32_t* order,
    uint32_t* scratch, const BuildTask* tasks, BuildTask* next, uint32_t* nextCount, BNode* nodes,
    uint32_t* nodeCount, int32_t* rootRef, uint32_t* depthSeen, uint32_t nodeCapacity, int maxDepth,
    uint32_t leafMax, int* err)
{
    const BuildTask t = tasks[blockIdx.x];
    const int tid     = threadIdx.x;
    __shared__ float box[6], cbox[6];
    __shared__ uint32_t binCount[3][kBins];
    __shared__ int32_t binLo[3][kBins][3], binHi[3][kBins][3];
    __shared__ float bestCost[3];
    __shared__ int bestSplit[3];
    __shared__ int mode, axisSel, splitSel;
    __shared__ uint32_t warpLeft[kBuildThreads / 32], nLeftTotal, chunkBase;

    // 1. Box and centroid box.
    float b[6] = { INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY };
    float c[6] = { INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY };
    for (uint32_t i = t.first + tid; i < t.first + t.count; i += kBuildThreads)
    {
        const float* p = boxes + 6 * size_t(order[i]);
        for (int k = 0; k < 3; k++)
        {
            float lo = p[k], hi = p[3 + k], ce = 0.5f * (lo + hi);
            b[k]     = fminf(b[k], lo);
            b[3 + k] = fmaxf(b[3 + k], hi);
            c[k]     = fminf(c[k], ce);
            c[3 + k] = fmaxf(c[3 + k], ce);
        }
    }
    blockBox(b, box);
    blockBox(c, cbox);
    if (tid == 0)
    {
        if (t.parent >= 0)
        {
            BNode& P = nodes[t.parent];
            if (t.side == 0)
            {
                P.c0xy   = make_float4(box[0], box[3], box[1], box[4]);
                P.cz.x   = box[2];
                P.cz.y   = box[5];
            }
            else
            {
                P.c1xy   = make_float4(box[0], box[3], box[1], box[4]);
                P.cz.z   = box[2];
                P.cz.w   = box[5];
            }
        }
        atomicMax(depthSeen, uint32_t(t.depth));
    }
    // 2. Small nodes are leaves.
    auto makeLeaf = [&]() {
        if (tid == 0)
        {
            int32_t ref = ~int32_t((t.first << 3) | (t.count - 1));
            if (t.parent >= 0)
            {
                if (t.side == 0)
                    nodes[t.parent].ref.x = ref;
                else
                    nodes[t.parent].ref.y = ref;
            }
            else
                *rootRef = ref;
        }
    };
    if (t.count <= leafMax)
    {
        makeLeaf();
        return;
    }
    const bool forceMid = t.depth + ceilLog2((t.count + leafMax - 1) / leafMax) + 2 >= maxDepth;
    // 3. Binned SAH.
    if (tid < 3 * kBins)
    {
        int a = tid / kBins, k = tid % kBins;
        binCount[a][k] = 0;
        for (int q = 0; q < 3; q++)
        {
            binLo[a][k][q] = orderedFromFloat(INFINITY);
            binHi[a][k][q] = orderedFromFloat(-INFINITY);
        }
    }
    __syncthreads();
    if (!forceMid)
    {
        for (uint32_t i = t.first + tid; i < t.first + t.count; i += kBuildThreads)
        {
            const float* p = boxes + 6 * size_t(order[i]);
            for (int a = 0; a < 3; a++)
            {
                float ext = cbox[3 + a] - cbox[a];
                if (!(ext > 0.f))
                    continue;
                float ce = 0.5f * (p[a] + p[3 + a]);
                int bin  = int((ce - cbox[a]) * (float(kBins) / ext));
                bin      = min(max(bin, 0), kBins - 1);
                atomicAdd(&binCount[a][bin], 1u);
                for (int q = 0; q < 3; q++)
                {
                    atomicMin(&binLo[a][bin][q], orderedFromFloat(p[q]));
                    atomicMax(&binHi[a][bin][q], orderedFromFloat(p[3 + q]));
                }
            }
        }
    }
    __syncthreads();
    if (tid < 3)
    {
        const int a = tid;
        float cost  = INFINITY;
        int split   = -1;
        float ext   = cbox[3 + a] - cbox[a];
        if (!forceMid && ext > 0.f)
        {
            float rArea[kBins];
            uint32_t rCnt[kBins];
            float lo[3] = { INFINITY, INFINITY, INFINITY }, hi[3] = { -INFINITY, -INFINITY, -INFINITY };
            uint32_t n = 0;
            for (int k = kBins - 1; k > 0; k--)
            {
                for (int q = 0; q < 3; q++)
                {
                    lo[q] = fminf(lo[q], floatFromOrdered(binLo[a][k][q]));
                    hi[q] = fmaxf(hi[q], floatFromOrdered(binHi[a][k][q]));
                }
                n += binCount[a][k];
                rArea[k] = boxArea(lo, hi);
                rCnt[k]  = n;
            }
            for (int q = 0; q < 3; q++)
            {
                lo[q] = INFINITY;
                hi[q] = -INFINITY;
            }
            n = 0;
            for (int k = 0; k < kBins - 1; k++)
            {
                for (int q = 0; q < 3; q++)
                {
                    lo[q] = fminf(lo[q], floatFromOrdered(binLo[a][k][q]));
                    hi[q] = fmaxf(hi[q], floatFromOrdered(binHi[a][k][q]));
                }
                n += binCount[a][k];
                if (n == 0 || rCnt[k + 1] == 0)
                    continue;
                float cc = boxArea(lo, hi) * float(n) + rArea[k + 1] * float(rCnt[k + 1]);
                if (cc < cost)
                {
                    cost  = cc;
                    split = k;
                }
            }
        }
        bestCost[a]  = cost;
        bestSplit[a] = split;
    }
    __syncthreads();
    if (tid == 0)
    {
        int best = -1;
        for (int a = 0; a < 3; a++)
            if (bestSplit[a] >= 0 && (best < 0 || bestCost[a] < bestCost[best]))
                best = a;
        if (best >= 0)
        {
            mode     = 1; // SAH split
            axisSel  = best;
            splitSel = bestSplit[best];
        }
        else
            mode = 2; // index midpoint
    }
    __syncthreads();
    // 4. Stable in-place partition through the scratch copy of the range.
    uint32_t nLeft = t.count / 2;
    if (mode == 1)
    {
        const int a     = axisSel;
        const float lo  = cbox[a];
        const float scl = float(kBins) / (cbox[3 + a] - cbox[a]);
        if (tid == 0)
            chunkBase = 0;
        __syncthreads();
        // Left items in order to scratch[first ...], right items to scratch[first + count - 1 ...]
        // backwards (item i is the (i - rank)-th right item); the right run is reversed back when
        // copied home, so the partition is stable.
        for (uint32_t base = 0; base < t.count; base += kBuildThreads)
        {
            uint32_t i  = base + tid;
            bool valid  = i < t.count;
            uint32_t p  = valid ? order[t.first + i] : 0;
            bool left   = false;
            if (valid)
            {
                const float* q = boxes + 6 * size_t(p);
                int bin        = int((0.5f * (q[a] + q[3 + a]) - lo) * scl);
                bin            = min(max(bin, 0), kBins - 1);
                left           = bin <= splitSel;
            }
            unsigned m    = __ballot_sync(0xffffffffu, left);
            int lane      = tid & 31, warp = tid >> 5;
            if (lane == 0)
                warpLeft[warp] = __popc(m);
            __syncthreads();
            uint32_t before = chunkBase;
            for (int w = 0; w < warp; w++)
                before += warpLeft[w];
            uint32_t chunkLeft = 0;
            for (int w = 0; w < kBuildThreads / 32; w++)
                chunkLeft += warpLeft[w];
            uint32_t rankL = before + __popc(m & ((1u << lane) - 1u));
            if (valid)
            {
                if (left)
                    scratch[t.first + rankL] = p;
                else
                    scratch[t.first + t.count - 1 - (i - rankL)] = p;
            }
            __syncthreads();
            if (tid == 0)
                chunkBase += chunkLeft;
            __syncthreads();
        }
        nLeft = chunkBase;
        if (nLeft == 0 || nLeft == t.count)
        {
            mode  = 2;
            nLeft = t.count / 2;
        }
        else
        {
            // Copy home: the left run as is, the right run reversed (restoring its order).
            for (uint32_t i = tid; i < t.count; i += kBuildThreads)
                order[t.first + i] = i < nLeft ? scratch[t.first + i] : scratch[t.first + t.count - 1 - (i - nLeft)];
        }
        __syncthreads();
    }
    // Node and children.
    if (tid == 0)
    {
        uint32_t id = atomicAdd(nodeCount, 1u);
        if (id >= nodeCapacity)
        {
            atomicExch(err, 1);
            return;
        }
        nodes[id].ref = make_int4(0, 0, 0, 0);
        if (t.parent >= 0)
        {
            if (t.side == 0)
                nodes[t.parent].ref.x = int32_t(id);
            else
                nodes[t.parent].ref.y = int32_t(id);
        }
        else
            *rootRef = int32_t(id);
        uint32_t slot = atomicAdd(nextCount, 2u);
        next[slot]     = BuildTask{ t.first, nLeft, int32_t(id), 0, t.depth + 1 };
        next[slot + 1] = BuildTask{ t.first + nLeft, t.count - nLeft, int32_t(id), 1, t.depth + 1 };
    }
}

__global__ void k_tri_boxes(const float* positions, const uint32_t* indices, uint32_t ntri, float* boxes)
{
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < ntri; t += gridDim.x * blockDim.x)
    {
        float lo[3] = { INFINITY, INFINITY, INFINITY }, hi[3] = { -INFINITY, -INFINITY, -INFINITY };
        for (int v = 0; v < 3; v++)
        {
            const float* p = positions + 3 * size_t(indices[3 * size_t(t) + v]);
            for (int k = 0; k < 3; k++)
            {
                lo[k] = fminf(lo[k], p[k]);
                hi[k] = fmaxf(hi[k], p[k]);
            }
        }
        for (int k = 0; k < 3; k++)
        {
            boxes[6 * size_t(t) + k]     = lo[k];
            boxes[6 * size_t(t) + 3 + k] = hi[k];
        }
    }
}

__global__ void k_iota(uint32_t* order, uint32_t n)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        order[i] = i;
}

// Triangles in leaf order: v0 (w = triangle id bits), v1, v2.
__global__ void k_reorder_tris(const float* positions, const uint32_t* indices, const uint32_t* order,
    uint32_t ntri, float4* tris)
{
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < ntri; s += gridDim.x * blockDim.x)
    {
        uint32_t t = order[s];
        for (int v = 0; v < 3; v++)
        {
            const float* p = positions + 3 * size_t(indices[3 * size_t(t) + v]);
            tris[3 * size_t(s) + v] = make_float4(p[0], p[1], p[2], v == 0 ? __int_as_float(int32_t(t)) : 0.f);
        }
    }
}

cudaError_t growScratch(void** p, size_t& cap, size_t bytes)
{
    if (cap >= bytes)
        return cudaSuccess;
    cudaFree(*p);
    *p  = nullptr;
    cap = 0;
    cudaError_t r = cudaMalloc(p, bytes);
    if (r == cudaSuccess)
        cap = bytes;
    return r;
}

// Scratch for n primitives (their boxes are written into s.boxes by the caller).
cudaError_t reserve(GpuBvhScratch& s, size_t n)
{
    cudaError_t e;
    if ((e = growScratch(reinterpret_cast<void**>(&s.boxes), s.boxesBytes, n * 24)) != cudaSuccess ||
        (e = growScratch(reinterpret_cast<void**>(&s.order), s.orderBytes, n * 4)) != cudaSuccess ||
        (e = growScratch(reinterpret_cast<void**>(&s.scratch), s.scratchBytes, n * 4)) != cudaSuccess ||
        (e = growScratch(&s.tasksA, s.tasksABytes, (n + 2) * sizeof(BuildTask))) != cudaSuccess ||
        (e = growScratch(&s.tasksB, s.tasksBBytes, (n + 2) * sizeof(BuildTask))) != cudaSuccess ||
        (e = growScratch(&s.counters, s.countersBytes, 64)) != cudaSuccess)
        return e;
    return cudaSuccess;
}

// The level-by-level build over s.boxes (n primitives); s.order ends in leaf order.
cudaError_t buildLevels(uint32_t n, uint32_t leafMax, int maxDepth, GpuBvhScratch& s, BNode* nodes,
    uint32_t nodeCapacity, int32_t* rootOut, int32_t* depthOut, uint32_t* nodeCountOut, cudaStream_t st)
{
    cudaError_t e;
    unsigned g = unsigned(std::min<size_t>((size_t(n) + 255) / 256, 4096));
    k_iota<<<g, 256, 0, st>>>(s.order, n);
    // counters: [0] next task count, [1] node count, [2] root ref, [3] depth seen, [4] error
    uint32_t* cnt = static_cast<uint32_t*>(s.counters);
    if ((e = cudaMemsetAsync(cnt, 0, 64, st)) != cudaSuccess)
        return e;
    BuildTask root{ 0, n, -1, 0, 0 };
    BuildTask* cur = static_cast<BuildTask*>(s.tasksA);
    BuildTask* nxt = static_cast<BuildTask*>(s.tasksB);
    if ((e = cudaMemcpyAsync(cur, &root, sizeof root, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return e;
    uint32_t taskCount = 1;
    for (int level = 0; taskCount > 0; level++)
    {
        if (level > maxDepth + 1)
            return cudaErrorInvalidValue;
        if ((e = cudaMemsetAsync(cnt, 0, 4, st)) != cudaSuccess)
            return e;
        k_bvh_level<<<taskCount, kBuildThreads, 0, st>>>(s.boxes, s.order, s.scratch, cur, nxt, cnt, nodes,
            cnt + 1, reinterpret_cast<int32_t*>(cnt + 2), cnt + 3, nodeCapacity, maxDepth, leafMax,
            reinterpret_cast<int*>(cnt + 4));
        if ((e = cudaGetLastError()) != cudaSuccess)
            return e;
        if ((e = cudaMemcpyAsync(&taskCount, cnt, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return e;
        std::swap(cur, nxt);
    }
    uint32_t h[5];
    if ((e = cudaMemcpyAsync(h, cnt, sizeof h, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return e;
    if (h[4])
        return cudaErrorInvalidValue;
    *nodeCountOut = h[1];
    *rootOut      = int32_t(h[2]);
    *depthOut     = int32_t(h[3]);
    return cudaSuccess;
}

} // namespace

cudaError_t buildBlasGpu(const float* positions, const uint32_t* indices, uint32_t ntri, int maxDepth,
    GpuBvhScratch& s, BNode* nodes, uint32_t nodeCapacity, float4* tris, int32_t* rootOut, int32_t* depthOut,
    uint32_t* nodeCountOut, cudaStream_t st)
{
    cudaError_t e = reserve(s, ntri);
    if (e != cudaSuccess)
        return e;
    unsigned g = unsigned(std::min<size_t>((size_t(ntri) + 255) / 256, 4096));
    k_tri_boxes<<<g, 256, 0, st>>>(positions, indices, ntri, s.boxes);
    if ((e = buildLevels(ntri, kBlasLeaf, maxDepth, s, nodes, nodeCapacity, rootOut, depthOut, nodeCountOut,
             st)) != cudaSuccess)
        return e;
    k_reorder_tris<<<g, 256, 0, st>>>(positions, indices, s.order, ntri, tris);
    return cudaGetLastError();
}

cudaError_t buildTlasGpu(const float* boxesHost, uint32_t count, int maxDepth, GpuBvhScratch& s, BNode* nodes,
    uint32_t nodeCapacity, int32_t* orderOut, int32_t* rootOut, int32_t* depthOut, uint32_t* nodeCountOut,
    cudaStream_t st)
{
    cudaError_t e = reserve(s, count);
    if (e != cudaSuccess)
        return e;
    if ((e = cudaMemcpyAsync(s.boxes, boxesHost, size_t(count) * 24, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return e;
    if ((e = buildLevels(count, 1, maxDepth, s, nodes, nodeCapacity, rootOut, depthOut, nodeCountOut, st)) !=
        cudaSuccess)
        return e;
    return cudaMemcpyAsync(orderOut, s.order, size_t(count) * 4, cudaMemcpyDeviceToDevice, st);
}

void freeGpuBvhScratch(GpuBvhScratch& s)
{
    cudaFree(s.nodes);
    cudaFree(s.boxes);
    cudaFree(s.order);
    cudaFree(s.scratch);
    cudaFree(s.tasksA);
    cudaFree(s.tasksB);
    cudaFree(s.counters);
    s = GpuBvhScratch();
}

} // namespace agb
