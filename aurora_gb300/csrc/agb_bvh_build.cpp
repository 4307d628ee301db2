// Host-side binned-SAH BVH2 builder producing the device node layout (BNode, 64 bytes with both
// child boxes).  Used for BLAS (triangles) and TLAS (instance boxes).  The reference has no BVH
// builder of its own: HGI/HGIGeometry.cpp:127-160 and HGI/HGIScene.cpp:377-420 hand geometry to the
// driver.  Depth is bounded so the device traversal stack (48 entries, TLAS + BLAS) never
// overflows: once a subtree could exceed the budget, splits fall back to object medians.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "agb_kernels.h"

namespace agb
{

namespace
{

struct Box
{
    float lo[3] = { INFINITY, INFINITY, INFINITY };
    float hi[3] = { -INFINITY, -INFINITY, -INFINITY };
    void grow(const Box& b)
    {
        for (int k = 0; k < 3; k++)
        {
            lo[k] = std::min(lo[k], b.lo[k]);
            hi[k] = std::max(hi[k], b.hi[k]);
        }
    }
    void growPoint(const float* p)
    {
        for (int k = 0; k < 3; k++)
        {
            lo[k] = std::min(lo[k], p[k]);
            hi[k] = std::max(hi[k], p[k]);
        }
    }
    float area() const
    {
        float d[3];
        for (int k = 0; k < 3; k++)
            d[k] = std::max(0.f, hi[k] - lo[k]);
        return 2.f * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
    }
};

struct TmpNode
{
    Box box;
    int32_t child[2] = { -1, -1 }; // tmp node indices; -1 for leaves
    uint32_t first = 0, count = 0;
};

int ceilLog2(uint32_t x)
{
    int r = 0;
    while ((1u << r) < x)
        r++;
    return r;
}

} // namespace

void buildBVH2(const float* boxesIn, uint32_t n, int maxLeaf, int maxDepth, BuiltBVH& out)
{
    out.nodes.clear();
    out.order.resize(n);
    out.depth = 0;
    if (n == 0)
    {
        out.root = 0;
        return;
    }
    std::vector<Box> boxes(n);
    std::vector<float> cen(size_t(n) * 3);
    for (uint32_t i = 0; i < n; i++)
    {
        for (int k = 0; k < 3; k++)
        {
            boxes[i].lo[k] = boxesIn[6 * size_t(i) + k];
            boxes[i].hi[k] = boxesIn[6 * size_t(i) + 3 + k];
            cen[3 * size_t(i) + k] = 0.5f * (boxes[i].lo[k] + boxes[i].hi[k]);
        }
        out.order[i] = i;
    }
    std::vector<TmpNode> tmp;
    tmp.reserve(2 * size_t(n) / std::max(1, maxLeaf) + 16);
    tmp.push_back(TmpNode());
    tmp[0].first = 0;
    tmp[0].count = n;
    struct Item
    {
        int32_t node;
        int depth;
    };
    std::vector<Item> stack = { { 0, 0 } };
    const int kBins = 16;
    while (!stack.empty())
    {
        Item it = stack.back();
        stack.pop_back();
        TmpNode& nd = tmp[it.node];
        out.depth   = std::max(out.depth, it.depth);
        Box box, cbox;
        for (uint32_t i = nd.first; i < nd.first + nd.count; i++)
        {
            box.grow(boxes[out.order[i]]);
            cbox.growPoint(&cen[3 * size_t(out.order[i])]);
        }
        nd.box = box;
        if (nd.count <= uint32_t(std::min(maxLeaf, 4)))
            continue;
        uint32_t first = nd.first, count = nd.count;
        uint32_t mid   = first;
        bool forceMedian = it.depth + ceilLog2((count + maxLeaf - 1) / maxLeaf) + 2 >= maxDepth;
        int bestAxis = -1, bestSplit = -1;
        float bestCost = INFINITY;
        if (!forceMedian)
        {
            for (int axis = 0; axis < 3; axis++)
            {
                float ext = cbox.hi[axis] - cbox.lo[axis];
                if (!(ext > 0.f))
                    continue;
                float scale = float(kBins) / ext;
                Box bb[kBins];
                uint32_t bc[kBins] = { 0 };
                for (uint32_t i = first; i < first + count; i++)
                {
                    uint32_t p = out.order[i];
                    int b = int((cen[3 * size_t(p) + axis] - cbox.lo[axis]) * scale);
                    b     = std::min(std::max(b, 0), kBins - 1);
                    bc[b]++;
                    bb[b].grow(boxes[p]);
                }
                float rArea[kBins];
                uint32_t rCount[kBins];
                Box acc;
                uint32_t cnt = 0;
                for (int b = kBins - 1; b > 0; b--)
                {
                    acc.grow(bb[b]);
                    cnt += bc[b];
                    rArea[b]  = acc.area();
                    rCount[b] = cnt;
                }
                acc = Box();
                cnt = 0;
                for (int b = 0; b < kBins - 1; b++)
                {
                    acc.grow(bb[b]);
                    cnt += bc[b];
                    if (cnt == 0 || rCount[b + 1] == 0)
                        continue;
                    float cost = acc.area() * float(cnt) + rArea[b + 1] * float(rCount[b + 1]);
                    if (cost < bestCost)
                    {
                        bestCost  = cost;
                        bestAxis  = axis;
                        bestSplit = b;
                    }
                }
            }
            // Leaf if splitting does not pay (and the primitives fit a leaf).
            if (count <= uint32_t(maxLeaf) && bestCost >= box.area() * float(count))
                continue;
        }
        if (bestAxis >= 0)
        {
            float scale = float(kBins) / (cbox.hi[bestAxis] - cbox.lo[bestAxis]);
            float lo    = cbox.lo[bestAxis];
            auto itMid  = std::partition(out.order.begin() + first, out.order.begin() + first + count,
                [&](uint32_t p) {
                    int b = int((cen[3 * size_t(p) + bestAxis] - lo) * scale);
                    b     = std::min(std::max(b, 0), kBins - 1);
                    return b <= bestSplit;
                });
            mid = uint32_t(itMid - out.order.begin());
        }
        if (bestAxis < 0 || mid == first || mid == first + count)
        {
            // Object median along the widest centroid extent.
            int axis = 0;
            for (int k = 1; k < 3; k++)
                if (cbox.hi[k] - cbox.lo[k] > cbox.hi[axis] - cbox.lo[axis])
                    axis = k;
            mid = first + count / 2;
            std::nth_element(out.order.begin() + first, out.order.begin() + mid,
                out.order.begin() + first + count, [&](uint32_t a, uint32_t b) {
                    float ca = cen[3 * size_t(a) + axis], cb = cen[3 * size_t(b) + axis];
                    return ca < cb || (ca == cb && a < b);
                });
        }
        int32_t l = int32_t(tmp.size());
        tmp.push_back(TmpNode());
        tmp.push_back(TmpNode());
        tmp[l].first     = first;
        tmp[l].count     = mid - first;
        tmp[l + 1].first = mid;
        tmp[l + 1].count = first + count - mid;
        tmp[it.node].child[0] = l;
        tmp[it.node].child[1] = l + 1;
        stack.push_back({ l + 1, it.depth + 1 });
        stack.push_back({ l, it.depth + 1 });
    }
    // Emit interior nodes in depth-first order; leaves become negative refs.
    std::vector<int32_t> remap(tmp.size(), -1);
    std::vector<int32_t> dfs = { 0 };
    std::vector<int32_t> orderInterior;
    while (!dfs.empty())
    {
        int32_t t = dfs.back();
        dfs.pop_back();
        if (tmp[t].child[0] < 0)
            continue;
        remap[t] = int32_t(orderInterior.size());
        orderInterior.push_back(t);
        dfs.push_back(tmp[t].child[1]);
        dfs.push_back(tmp[t].child[0]);
    }
    auto refOf = [&](int32_t t) -> int32_t {
        if (tmp[t].child[0] < 0)
            return leafRef(tmp[t].first, tmp[t].count);
        return remap[t];
    };
    out.nodes.resize(orderInterior.size());
    for (size_t i = 0; i < orderInterior.size(); i++)
    {
        const TmpNode& nd = tmp[orderInterior[i]];
        const Box& a      = tmp[nd.child[0]].box;
        const Box& b      = tmp[nd.child[1]].box;
        BNode& o          = out.nodes[i];
        o.c0xy = make_float4(a.lo[0], a.hi[0], a.lo[1], a.hi[1]);
        o.c1xy = make_float4(b.lo[0], b.hi[0], b.lo[1], b.hi[1]);
        o.cz   = make_float4(a.lo[2], a.hi[2], b.lo[2], b.hi[2]);
        o.ref  = make_int4(refOf(nd.child[0]), refOf(nd.child[1]), 0, 0);
    }
    out.root = refOf(0);
}

void invertAffine(const float* m, float* out)
{
    double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], i = m[10];
    double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    double det = a * A + b * B + c * C;
    double inv[9] = { A / det, -(b * i - c * h) / det, (b * f - c * e) / det, B / det,
        (a * i - c * g) / det, -(a * f - c * d) / det, C / det, -(a * h - b * g) / det,
        (a * e - b * d) / det };
    double tx = m[3], ty = m[7], tz = m[11];
    for (int r = 0; r < 3; r++)
    {
        out[4 * r + 0] = float(inv[3 * r + 0]);
        out[4 * r + 1] = float(inv[3 * r + 1]);
        out[4 * r + 2] = float(inv[3 * r + 2]);
        out[4 * r + 3] = float(-(inv[3 * r + 0] * tx + inv[3 * r + 1] * ty + inv[3 * r + 2] * tz));
    }
}

} // namespace agb
